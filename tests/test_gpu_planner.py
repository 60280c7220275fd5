"""Every candidate plan of a planning point computes the same words (so a
planner can change speed, never a result), and the autotuner times them."""
import ctypes

import numpy as np
import pytest

from omr_ntt import NttDomain, _lib
from omr_ntt.fields import BabyBear, Goldilocks, KoalaBear, TeddyBear
from omr_ntt.inputs import gen_input_seeded, random_indices
from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu
L = _lib.lib()


def _cands(field, log_n, pattern, count):
    n = L.omr_ntt_candidates(field.id, log_n, pattern, count, None, None, 0)
    st = (ctypes.c_int * n)()
    pa = (ctypes.c_int * n)()
    L.omr_ntt_candidates(field.id, log_n, pattern, count, st, pa, n)
    return list(zip(st, pa))


@pytest.mark.parametrize("field,log_n,pattern,count,batch", [
    (BabyBear, 12, 0, 1 << 12, 3),
    (BabyBear, 18, 0, 1 << 18, 2),
    (Goldilocks, 17, 0, 1 << 17, 1),
    (BabyBear, 16, 0, 64, 2),
    (Goldilocks, 16, 0, 1000, 1),
    (BabyBear, 18, 1, 256, 2),
    (Goldilocks, 16, 1, 4096, 1),
    (BabyBear, 16, 2, 300, 2),
    (BabyBear, 20, 0, 50, 1),
    (KoalaBear, 14, 0, 3, 1),
    (TeddyBear, 15, 0, 50, 2),
    (Goldilocks, 13, 0, 2048, 1),
    (BabyBear, 12, 0, 1, 1),
    (BabyBear, 13, 1, 4096, 1),
    (Goldilocks, 14, 1, 2, 1),
    (KoalaBear, 12, 1, 1, 2),
    (Goldilocks, 20, 1, 16, 1),
    (BabyBear, 16, 0, 1 << 16, 3),
    (Goldilocks, 13, 0, 1 << 13, 2),
    (TeddyBear, 15, 0, 1 << 15, 2),
    # index sets: the decomposition at every line length, then full + gather
    (Goldilocks, 18, 2, 4096, 1),
    (KoalaBear, 14, 2, 3, 1),
    (TeddyBear, 16, 2, 1000, 2),
    (BabyBear, 22, 2, 16, 1),
], ids=str)
def test_all_candidates_agree(oracle, field, log_n, pattern, count, batch):
    import torch

    n = 1 << log_n
    d = NttDomain(field, n)
    x = gen_input_seeded(field, n * batch, 99 + log_n)
    full = oracle.forward(field.id, x, batch=batch).reshape(batch, n)
    if count >= n:
        exp = full.reshape(-1)
        idx = None
    elif pattern == 0:
        exp = full[:, :count].reshape(-1)
        idx = None
    elif pattern == 1:
        exp = full[:, ::n // count].reshape(-1)
        idx = None
    else:
        idx = random_indices(n, count, 5)
        exp = full[:, idx.astype(np.int64)].reshape(-1)
    xd = to_dev(x)
    idt = torch.from_numpy(idx.view(np.int32)).cuda() if idx is not None else None
    outw = n if count >= n else count
    for s, p in _cands(field, log_n, pattern, count):
        out = torch.zeros(outw * batch, dtype=xd.dtype, device="cuda")
        _lib.check(L.omr_ntt_run_candidate(d.handle, s, p, pattern, count,
                                           ctypes.c_void_p(idt.data_ptr()) if idt is not None else None,
                                           ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                           batch, None))
        torch.cuda.synchronize()
        assert np.array_equal(to_host(out, field.dtype), exp), (s, p)


def test_tune_point_and_planner():
    n = L.omr_ntt_candidates(0, 16, 0, 64, None, None, 0)
    ms = (ctypes.c_float * n)()
    assert L.omr_ntt_tune_point(0, 16, 1, 0, 64, 3, 7, ms, n) == n
    times = list(ms)
    assert all(t > 0 for t in times)
    best = int(np.argmin(times))
    st = (ctypes.c_int * n)()
    pa = (ctypes.c_int * n)()
    L.omr_ntt_candidates(0, 16, 0, 64, st, pa, n)
    assert L.omr_ntt_planner_set(0, 16, 1, 0, 64, st[best], pa[best]) == 0
    # the auto path now takes the tuned strategy and still matches the oracle
    from oracle import oracle as o
    import omr_ntt

    d = NttDomain(BabyBear, 1 << 16)
    x = gen_input_seeded(BabyBear, 1 << 16, 3)
    assert np.array_equal(omr_ntt.partial(d, x, omr_ntt.PREFIX, 64), o.forward(0, x)[:64])
    L.omr_ntt_planner_clear()
