"""GPU parity: forward / inverse NTTs through the C ABI against the oracle,
bit-exact, every field, every plan, sizes 2^0 .. 2^24 and batches."""
import numpy as np
import pytest

import omr_ntt
from omr_ntt import NttDomain, OmrNttError
from omr_ntt.fields import ALL, BabyBear, Goldilocks, KoalaBear, TeddyBear
from omr_ntt.inputs import gen_input_seeded
from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("field", ALL, ids=lambda f: f.name)
def test_forward_all_plans_small(oracle, field):
    for log_n in range(0, 15):
        n = 1 << log_n
        d = NttDomain(field, n)
        x = gen_input_seeded(field, n, 31 + log_n)
        exp = oracle.forward(field.id, x)
        for plan in range(omr_ntt.plan_count(field, log_n)):
            got = omr_ntt.forward(d, x, plan=plan)
            assert np.array_equal(got, exp), (field, log_n, plan)
            back = omr_ntt.inverse(d, got, plan=plan)
            assert np.array_equal(back, x), (field, log_n, plan)


def _edge_input(field, n, seed):
    """Words at the ends of the canonical range (0, 1, p-1, p-2, (p-1)/2,
    2^32 +- 1 for Goldilocks ...) so every carry / borrow / final-subtract
    branch of the field arithmetic is taken."""
    p = field.p
    pool = [0, 1, 2, p - 1, p - 2, p - 3, (p - 1) // 2, (p + 1) // 2]
    if p > 1 << 32:
        pool += [(1 << 32) - 1, 1 << 32, (1 << 32) + 1, p - (1 << 32), (1 << 63), (1 << 63) - 1]
    rng = np.random.default_rng(seed)
    return np.array(pool, dtype=field.dtype)[rng.integers(0, len(pool), n)]


@pytest.mark.parametrize("field", ALL, ids=lambda f: f.name)
def test_edge_values_all_plans(oracle, field):
    for log_n in (3, 12, 13, 16):
        n = 1 << log_n
        d = NttDomain(field, n)
        x = _edge_input(field, n, log_n)
        exp = oracle.forward(field.id, x)
        for plan in range(omr_ntt.plan_count(field, log_n)):
            got = omr_ntt.forward(d, x, plan=plan)
            assert np.array_equal(got, exp), (field, log_n, plan)
            assert np.array_equal(omr_ntt.inverse(d, got, plan=plan), x), (field, log_n, plan)
        y = np.full(n, field.p - 1, dtype=field.dtype)  # all p - 1
        assert np.array_equal(omr_ntt.forward(d, y), oracle.forward(field.id, y))


@pytest.mark.parametrize("field", [BabyBear, Goldilocks], ids=lambda f: f.name)
@pytest.mark.parametrize("log_n", [16, 18, 20, 22, 24])
def test_forward_inverse_large(oracle, field, log_n):
    n = 1 << log_n
    d = NttDomain(field, n)
    x = gen_input_seeded(field, n, 42)
    exp = oracle.forward(field.id, x)
    xd = to_dev(x)
    for plan in range(omr_ntt.plan_count(field, log_n)):
        yd = xd.clone()
        omr_ntt.forward(d, yd, plan=plan)
        assert np.array_equal(to_host(yd, field.dtype), exp), plan
        omr_ntt.inverse(d, yd, plan=plan)
        assert np.array_equal(to_host(yd, field.dtype), x), plan


@pytest.mark.parametrize("field", [KoalaBear, TeddyBear], ids=lambda f: f.name)
@pytest.mark.parametrize("log_n", [16, 20, 24])
def test_other_fields_every_plan(oracle, field, log_n):
    """KoalaBear and TeddyBear on every plan, the TMA tile passes included."""
    n = 1 << log_n
    d = NttDomain(field, n)
    x = gen_input_seeded(field, n, 5 + log_n)
    exp = oracle.forward(field.id, x)
    xd = to_dev(x)
    for plan in range(omr_ntt.plan_count(field, log_n)):
        yd = xd.clone()
        omr_ntt.forward(d, yd, plan=plan)
        assert np.array_equal(to_host(yd, field.dtype), exp), plan
        omr_ntt.inverse(d, yd, plan=plan)
        assert np.array_equal(to_host(yd, field.dtype), x), plan


@pytest.mark.parametrize("field", [KoalaBear, TeddyBear], ids=lambda f: f.name)
def test_other_fields_large(oracle, field):
    for log_n in (17, 21):
        n = 1 << log_n
        d = NttDomain(field, n)
        x = gen_input_seeded(field, n, 3)
        got = omr_ntt.forward(d, x)
        assert np.array_equal(got, oracle.forward(field.id, x))
        assert np.array_equal(omr_ntt.inverse(d, got), x)


@pytest.mark.parametrize("field", [BabyBear, Goldilocks], ids=lambda f: f.name)
def test_batch_64_of_2_20(oracle, field):
    log_n, batch = 20, 64
    n = 1 << log_n
    d = NttDomain(field, n)
    x = gen_input_seeded(field, n * batch, 77)
    xd = to_dev(x)
    yd = xd.clone()
    omr_ntt.forward(d, yd, batch=batch)
    y = to_host(yd, field.dtype)
    exp = oracle.forward(field.id, x, batch=batch)
    for b in range(batch):  # every segment of the batch
        seg = slice(b * n, (b + 1) * n)
        assert np.array_equal(y[seg], exp[seg]), b
    omr_ntt.inverse(d, yd, batch=batch)
    assert np.array_equal(to_host(yd, field.dtype), x)


@pytest.mark.parametrize("field", [BabyBear, Goldilocks, KoalaBear], ids=lambda f: f.name)
@pytest.mark.parametrize("log_n,batch", [(16, 2), (20, 3), (16, 8)])  # sizes with a 256-point pass
def test_wide_column_pass_twiddle_tables(oracle, field, log_n, batch):
    """Every wide plan whose 256-point column pass takes its four-step
    twiddles from the domain's [line][k] table (at most 8192 lines), in
    batches, forward and inverse (the two directions use separate tables),
    against the oracle -- and the same words from the allocation-free entry
    point, which reuses the tables the first call built."""
    import ctypes

    import torch

    from omr_ntt import _lib

    n = 1 << log_n
    d = NttDomain(field, n)
    x = gen_input_seeded(field, n * batch, 91 + log_n)
    exp = oracle.forward(field.id, x, batch=batch)
    wide = [p for p in range(omr_ntt.plan_count(field, log_n))
            if omr_ntt.plan_describe(field, log_n, p).endswith(" wide")]
    assert wide
    for plan in wide:
        xd = to_dev(x)
        yd = torch.empty_like(xd)
        omr_ntt.forward(d, xd, plan=plan, out=yd, batch=batch)
        assert np.array_equal(to_host(yd, field.dtype), exp), (log_n, plan)
        omr_ntt.inverse(d, yd, plan=plan, batch=batch)
        assert np.array_equal(to_host(yd, field.dtype), x), (log_n, plan)
    if n * batch * field.word_bytes <= 16 << 20:
        out = torch.empty_like(xd)
        sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _lib.check(_lib.lib().omr_ntt_forward_noalloc(d.handle, ctypes.c_void_p(xd.data_ptr()),
                                                      ctypes.c_void_p(out.data_ptr()), batch, sp))
        torch.cuda.synchronize()
        assert np.array_equal(to_host(out, field.dtype), exp)


@pytest.mark.parametrize("field,log_n,plan_word", [(BabyBear, 24, " wide"), (Goldilocks, 20, " wide"),
                                                   (BabyBear, 22, " slab"), (BabyBear, 16, " tma2cta")])
def test_graph_captured_transform(oracle, field, log_n, plan_word):
    """Transforms captured into a CUDA graph (after a warm-up call has built
    the domain's scratch and twiddle tables) and replayed: every pass kernel
    is launched with the programmatic stream-serialisation attribute, which
    capture turns into programmatic graph edges; replays are bit-exact."""
    import torch

    n = 1 << log_n
    d = NttDomain(field, n)
    plan = next(p for p in range(omr_ntt.plan_count(field, log_n))
                if omr_ntt.plan_describe(field, log_n, p).endswith(plan_word))
    x = gen_input_seeded(field, n, 123 + log_n)
    xd = to_dev(x)
    yd = torch.empty_like(xd)
    zd = torch.empty_like(xd)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        omr_ntt.forward(d, xd, plan=plan, out=yd)  # warm-up: allocations happen here
        omr_ntt.inverse(d, yd, plan=plan, out=zd)
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        omr_ntt.forward(d, xd, plan=plan, out=yd)
        omr_ntt.inverse(d, yd, plan=plan, out=zd)
    yd.zero_()
    zd.zero_()
    torch.cuda.synchronize()
    for _ in range(2):
        g.replay()
    torch.cuda.synchronize()
    assert np.array_equal(to_host(yd, field.dtype), oracle.forward(field.id, x))
    assert np.array_equal(to_host(zd, field.dtype), x)


@pytest.mark.parametrize("field", [BabyBear, Goldilocks], ids=lambda f: f.name)
def test_out_of_place_and_in_place_agree(oracle, field):
    n = 1 << 14
    d = NttDomain(field, n)
    x = gen_input_seeded(field, n, 5)
    xd = to_dev(x)
    out = xd.clone().zero_()
    omr_ntt.forward(d, xd, out=out)
    assert np.array_equal(to_host(xd, field.dtype), x)  # input untouched
    assert np.array_equal(to_host(out, field.dtype), oracle.forward(field.id, x))


def test_log_n_27_babybear(oracle):
    # the reference's own bench size (benches/ntt_bench_n.rs:7): 2^27, three passes
    n = 1 << 27
    d = NttDomain(BabyBear, n)
    x = gen_input_seeded(BabyBear, n, 42)
    xd = to_dev(x)
    omr_ntt.forward(d, xd)
    y = to_host(xd, BabyBear.dtype)
    oracle.set_threads(0)
    assert np.array_equal(y, oracle.forward(BabyBear.id, x))


def test_size_errors():
    with pytest.raises(OmrNttError):
        NttDomain(BabyBear, 1 << 28)
    with pytest.raises(OmrNttError):
        NttDomain(BabyBear, 12)
    with pytest.raises(OmrNttError):
        NttDomain(KoalaBear, 1 << 25)


def test_noncanonical_check():
    n = 1 << 12
    d = NttDomain(BabyBear, n)
    x = gen_input_seeded(BabyBear, n, 1)
    from omr_ntt import _lib
    import ctypes

    xd = to_dev(x)
    assert _lib.lib().omr_ntt_check_canonical(d.handle, ctypes.c_void_p(xd.data_ptr()), n, None) == 0
    x2 = x.copy()
    x2[100] = BabyBear.p
    xd2 = to_dev(x2)
    assert _lib.lib().omr_ntt_check_canonical(d.handle, ctypes.c_void_p(xd2.data_ptr()), n, None) == -7


def test_one_domain_shared_by_threads_on_their_own_streams(oracle):
    """The reference's encoders are Send + Sync and a domain is shared
    read-only; here four host threads drive one domain on four CUDA streams
    (per-stream scratch) and every result stays bit-exact."""
    import ctypes
    import threading

    import torch
    from omr_ntt import _lib

    f, log_n = BabyBear, 20
    n = 1 << log_n
    d = NttDomain(f, n)
    xs = [gen_input_seeded(f, n, 300 + t) for t in range(4)]
    exps = [oracle.forward(f.id, x) for x in xs]
    errors = []

    def work(t):
        try:
            st = torch.cuda.Stream()
            with torch.cuda.stream(st):
                for _ in range(5):
                    buf = torch.from_numpy(xs[t].view(np.int32)).cuda()
                    _lib.check(_lib.lib().omr_ntt_forward(d.handle, -1, ctypes.c_void_p(buf.data_ptr()),
                                                          ctypes.c_void_p(buf.data_ptr()), 1,
                                                          ctypes.c_void_p(st.cuda_stream)))
                    st.synchronize()
                    if not np.array_equal(buf.cpu().numpy().view(np.uint32), exps[t]):
                        errors.append(t)
        except Exception as e:  # surfaced below
            errors.append(repr(e))

    threads = [threading.Thread(target=work, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors


@pytest.mark.parametrize("field,log_n,batch", [(BabyBear, 16, 8), (BabyBear, 20, 5), (Goldilocks, 18, 3),
                                               (TeddyBear, 12, 2)], ids=str)
def test_host_buffer_batches_pipelined(oracle, field, log_n, batch):
    """Host-buffer batches run chunk by chunk through two device buffers on
    three streams (copy in / transform / copy out); the words match the
    oracle, forward and back."""
    n = 1 << log_n
    d = NttDomain(field, n)
    x = gen_input_seeded(field, n * batch, 11 + log_n)
    exp = oracle.forward(field.id, x, batch=batch)
    got = omr_ntt.forward(d, x, batch=batch)
    assert np.array_equal(got, exp)
    assert np.array_equal(omr_ntt.inverse(d, got, batch=batch), x)
