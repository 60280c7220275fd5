"""Mixed batches in one persistent, graph-launched kernel: every request's
output is bit-exact against the oracle (small batch) and against the
per-request plain kernels (the full 4096-request mixed workload)."""
import numpy as np
import pytest

from omr_ntt import OmrNttError
from omr_ntt.batch import Batch, Request, fill_inputs, layout, mixed_requests
from omr_ntt.fields import BabyBear, Goldilocks

pytestmark = pytest.mark.gpu


def _canonical_arena(reqs, nbytes, seed):
    """Host input arena with seeded words uniform over the whole of [0, p) of
    each request's field (numpy's bounded integer generator)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    arena = np.zeros(nbytes, dtype=np.uint8)
    for r in reqs:
        x = rng.integers(0, r.field.p, size=r.n, dtype=r.field.dtype)
        arena[r.in_off:r.in_off + x.nbytes] = x.view(np.uint8)
    return arena


def _run(reqs, seed, per_request=False, host_in=None):
    import torch

    ib, ob = layout(reqs)
    if host_in is None:
        host_in = fill_inputs(reqs, ib, seed)
    d_in = torch.from_numpy(host_in).cuda()
    d_out = torch.zeros(max(ob, 1), dtype=torch.uint8, device="cuda")
    b = Batch(reqs)
    if per_request:
        b.run_per_request(d_in.data_ptr(), d_out.data_ptr())
    else:
        b.run(d_in.data_ptr(), d_out.data_ptr())
    b.check()
    torch.cuda.synchronize()
    return host_in, d_out.cpu().numpy(), b


def test_small_mixed_batch_against_oracle(oracle):
    reqs = mixed_requests(7, count=48, min_log=10, max_log=15)
    host_in, out, b = _run(reqs, 3)
    for i, r in enumerate(reqs):
        w = r.field.word_bytes
        x = host_in[r.in_off:r.in_off + r.n * w].view(r.field.dtype)
        full = oracle.inverse(r.field.id, x) if r.inverse else oracle.forward(r.field.id, x)
        exp = full if r.indices is None else full[r.indices.astype(np.int64)]
        got = out[r.out_off:r.out_off + r.out_words * w].view(r.field.dtype)
        assert np.array_equal(got, exp), (i, r.field, r.log_n, r.inverse, r.indices is not None)


def test_graph_replay_and_rerun(oracle):
    import torch

    reqs = [Request(BabyBear, 12, False), Request(Goldilocks, 11, True),
            Request(BabyBear, 20, True, np.array([0, 5, 77, (1 << 20) - 1], dtype=np.uint32))]
    ib, ob = layout(reqs)
    host_in = fill_inputs(reqs, ib, 11)
    d_in = torch.from_numpy(host_in).cuda()
    d_out = torch.zeros(ob, dtype=torch.uint8, device="cuda")
    b = Batch(reqs)
    for _ in range(3):  # replays of the captured graph give the same words
        d_out.zero_()
        b.run(d_in.data_ptr(), d_out.data_ptr())
        b.check()
        out = d_out.cpu().numpy()
        r = reqs[2]
        x = host_in[r.in_off:r.in_off + r.n * 4].view(np.uint32)
        exp = oracle.inverse(0, x)[r.indices.astype(np.int64)]
        assert np.array_equal(out[r.out_off:r.out_off + 16].view(np.uint32), exp)


def _check_against_oracle(oracle, reqs, host_in, out, which):
    for i in which:
        r = reqs[i]
        w = r.field.word_bytes
        x = host_in[r.in_off:r.in_off + r.n * w].view(r.field.dtype)
        assert int(x.max()) < r.field.p
        full = oracle.inverse(r.field.id, x) if r.inverse else oracle.forward(r.field.id, x)
        exp = full if r.indices is None else full[r.indices.astype(np.int64)]
        got = out[r.out_off:r.out_off + r.out_words * w].view(r.field.dtype)
        assert np.array_equal(got, exp), (i, r.field.name, r.log_n, r.inverse, r.indices is not None)


def test_full_mixed_workload_matches_per_request(oracle):
    """The 4096-request workload (inputs uniform over [0, p) of each field):
    the persistent batch equals the per-request kernels word for word, and a
    seeded sample of 64 requests with log n in [16, 20] -- both fields,
    forward and inverse, full and index-set outputs -- equals the oracle."""
    reqs = mixed_requests(2024, count=4096)
    ib, _ = layout(reqs)
    host_in, out_batch, b = _run(reqs, 5, host_in=_canonical_arena(reqs, ib, 5))
    info = b.info()
    assert info["requests"] == 4096 and info["tasks"] > 4096
    del b
    # eight requests of each field x direction x output-set kind, log n >= 16
    rng = np.random.Generator(np.random.PCG64(99))
    kinds = {}
    for i, r in enumerate(reqs):
        if r.log_n >= 16:
            kinds.setdefault((r.field.name, r.inverse, r.indices is not None), []).append(i)
    assert len(kinds) == 8, sorted(kinds)
    sample = sorted(j for v in kinds.values() for j in rng.choice(v, size=8, replace=False).tolist())
    assert {reqs[i].log_n for i in sample} == {16, 17, 18, 19, 20}
    _check_against_oracle(oracle, reqs, host_in, out_batch, sample)
    _, out_plain, _ = _run(reqs, 5, per_request=True, host_in=host_in)
    assert np.array_equal(out_batch, out_plain)


def test_batch_rejects_out_of_range_sizes():
    with pytest.raises(OmrNttError):
        Batch([Request(BabyBear, 22, False)])
    with pytest.raises(OmrNttError):
        Batch([Request(BabyBear, 12, False, np.array([1 << 12], dtype=np.uint32))])


def test_bounded_wait_reports_timeout_and_context_survives(oracle):
    """A dependency that can never complete (host-side injection: a row pass
    waiting for a column tile that does not exist) makes the persistent
    kernel's bounded waits give up: the run reports OMR_NTT_ERR_TIMEOUT and
    the next, correct run on the same context is bit-exact."""
    import time

    import torch
    from omr_ntt import _lib

    reqs = [Request(BabyBear, 12, False), Request(BabyBear, 14, False)]
    ib, ob = layout(reqs)
    host_in = fill_inputs(reqs, ib, 2)
    d_in = torch.from_numpy(host_in).cuda()
    d_out = torch.zeros(ob, dtype=torch.uint8, device="cuda")
    bad = Batch(reqs)
    assert _lib.lib().omr_ntt_batch_inject_stall(bad._h, 1) == 0
    t0 = time.time()
    bad.run(d_in.data_ptr(), d_out.data_ptr())
    with pytest.raises(OmrNttError) as e:
        bad.check()
    assert e.value.status == -6  # OMR_NTT_ERR_TIMEOUT
    assert time.time() - t0 < 60
    bad.close()
    good = Batch(reqs)
    d_out.zero_()
    good.run(d_in.data_ptr(), d_out.data_ptr())
    good.check()
    out = d_out.cpu().numpy()
    for r in reqs:
        x = host_in[r.in_off:r.in_off + r.n * 4].view(np.uint32)
        assert np.array_equal(out[r.out_off:r.out_off + r.n * 4].view(np.uint32), oracle.forward(0, x))
