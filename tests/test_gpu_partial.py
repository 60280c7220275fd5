"""Partial-output transforms on the GPU: N = 2^22,
s in {2^4, 2^6, ..., 2^16}, contiguous / strided / random index sets, both
fields, bit-exact against the matching entries of the oracle's full
transform."""
import numpy as np
import pytest

import omr_ntt
from omr_ntt import INDICES, PREFIX, STRIDED, NttDomain, OmrNttError
from omr_ntt.fields import BabyBear, Goldilocks
from omr_ntt.inputs import gen_input_seeded, random_indices
from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu

S_VALUES = [1 << k for k in range(4, 17, 2)]


@pytest.fixture(scope="module", params=[BabyBear, Goldilocks], ids=lambda f: f.name)
def case(request, oracle):
    f = request.param
    n = 1 << 22
    x = gen_input_seeded(f, n, 2024)
    full = oracle.forward(f.id, x)
    return f, NttDomain(f, n), x, full


def test_prefix(case):
    f, d, x, full = case
    xd = to_dev(x)
    for s in S_VALUES:
        out = omr_ntt.partial(d, xd, PREFIX, s)
        assert np.array_equal(to_host(out, f.dtype), full[:s]), s
    assert np.array_equal(to_host(xd, f.dtype), x)  # input untouched


def test_strided(case):
    f, d, x, full = case
    xd = to_dev(x)
    n = d.N
    for s in S_VALUES:
        out = omr_ntt.partial(d, xd, STRIDED, s)
        assert np.array_equal(to_host(out, f.dtype), full[::n // s]), s


def test_random(case):
    import torch

    f, d, x, full = case
    xd = to_dev(x)
    for s in S_VALUES:
        idx = random_indices(d.N, s, seed=s)
        idt = torch.from_numpy(idx.view(np.int32)).cuda()
        out = omr_ntt.partial(d, xd, INDICES, s, indices=idt)
        assert np.array_equal(to_host(out, f.dtype), full[idx.astype(np.int64)]), s


def test_host_api_and_edges(case):
    f, d, x, full = case
    assert np.array_equal(omr_ntt.partial(d, x, PREFIX, 16), full[:16])
    idx = np.array([0, d.N - 1, 5, 5], dtype=np.uint32)  # repeats are well defined
    assert np.array_equal(omr_ntt.partial(d, x, INDICES, 4, indices=idx), full[idx.astype(np.int64)])
    assert np.array_equal(omr_ntt.partial(d, x, PREFIX, d.N), full)
    assert np.array_equal(omr_ntt.partial(d, x, STRIDED, d.N), full)
    with pytest.raises(OmrNttError):
        omr_ntt.partial(d, x, INDICES, 1, indices=np.array([d.N], dtype=np.uint32))
    with pytest.raises(OmrNttError):
        omr_ntt.partial(d, x, STRIDED, 3)
    with pytest.raises(OmrNttError):
        omr_ntt.partial(d, x, PREFIX, d.N + 1)


def test_strided_from_an_unaligned_pointer(oracle):
    """A device input that starts 4 bytes into an allocation (not 16-byte
    aligned) takes the scalar fold path and gives the same words."""
    import ctypes

    import torch
    from omr_ntt import _lib

    f, n = BabyBear, 1 << 16
    x = gen_input_seeded(f, n, 77)
    full = oracle.forward(f.id, x)
    d = NttDomain(f, n)
    big = torch.zeros(n + 4, dtype=torch.int32, device="cuda")
    big[1:n + 1] = torch.from_numpy(x.view(np.int32)).cuda()
    for s in (16, 256, 4096):
        out = torch.zeros(s, dtype=torch.int32, device="cuda")
        _lib.check(_lib.lib().omr_ntt_partial(d.handle, STRIDED, s, None, ctypes.c_void_p(big.data_ptr() + 4),
                                              ctypes.c_void_p(out.data_ptr()), None))
        torch.cuda.synchronize()
        assert np.array_equal(to_host(out, f.dtype), full[::n // s]), s


@pytest.mark.parametrize("field", [BabyBear, Goldilocks], ids=lambda f: f.name)
def test_index_set_decomposition_edges(oracle, field):
    """Index sets run through the pruned decomposition: any order, repeated
    indices, and an index past N (which yields 0, as the gather of the full
    transform gives it), for small and large sets."""
    import torch

    n = 1 << 18
    d = NttDomain(field, n)
    x = gen_input_seeded(field, n, 31)
    full = oracle.forward(field.id, x)
    xd = to_dev(x)
    rng = np.random.Generator(np.random.PCG64(5))
    for m in (1, 7, 64, 1000, 4096):
        idx = rng.integers(0, n, size=m).astype(np.uint32)  # unsorted, repeats
        idx[m // 2] = idx[0]
        if m > 1:
            idx[-1] = n + 3  # past N
        exp = np.where(idx < n, full[np.minimum(idx, n - 1).astype(np.int64)], 0).astype(field.dtype)
        idt = torch.from_numpy(idx.view(np.int32)).cuda()
        out = omr_ntt.partial(d, xd, INDICES, m, indices=idt)
        assert np.array_equal(to_host(out, field.dtype), exp), m
