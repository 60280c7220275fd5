"""The allocation-free forward entry point, omr_ntt_forward_noalloc.

Some callers cannot let a call allocate device memory: a framework that has
reserved all device memory for its own caching allocator, or a latency-bound
loop that cannot afford the device-wide synchronisation a cudaMalloc/cudaFree
can cause.  omr_ntt_forward_noalloc serves them: it keeps the multi-pass
intermediate in a fixed 16 MiB array declared in device memory by the library
instead of the domain's cudaMalloc'd scratch.  These tests call it through
the C ABI and check it word for word against omr_ntt_forward, twice in a row
(the second call sees the array holding the first call's leftovers), against
the CPU oracle directly, that requests larger than the array are refused
without touching the buffers, and that a call allocates nothing even with
the learned planner installed (whose network allocates on its first use).

This file is collected last on purpose (tests/test_zz_*) and passes both on
its own in a fresh process and after the other tests.
"""
import ctypes

import numpy as np
import pytest

from omr_ntt import NttDomain, _lib
from omr_ntt.fields import BabyBear, Goldilocks
from omr_ntt.inputs import gen_input_seeded
from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu

CAPACITY = -9  # OMR_NTT_ERR_CAPACITY


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _reference_forward(domain, x, batch):
    import torch

    out = torch.empty_like(x)
    _lib.check(_lib.lib().omr_ntt_forward(domain.handle, -1, _ptr(x), _ptr(out), batch,
                                          ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return out


def _noalloc_forward(domain, x, batch):
    import torch

    out = torch.empty_like(x)
    rc = _lib.lib().omr_ntt_forward_noalloc(domain.handle, _ptr(x), _ptr(out), batch,
                                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc)
    return out


@pytest.mark.parametrize("field,log_n,batch", [
    (BabyBear, 20, 1),    # 4 MiB, two passes
    (BabyBear, 20, 4),    # 16 MiB, exactly the array's size
    (Goldilocks, 20, 2),  # 16 MiB
    (Goldilocks, 12, 3),  # short lines, odd batch
    (BabyBear, 14, 1),    # the built-in rule's one-launch cluster plan
], ids=lambda v: getattr(v, "name", str(v)))
def test_noalloc_matches_forward_twice(field, log_n, batch):
    import torch

    n = 1 << log_n
    d = NttDomain(field, n)
    for call, seed in enumerate((11, 12)):  # two calls in a row, different inputs
        x = to_dev(gen_input_seeded(field, n * batch, seed + log_n))
        ref = _reference_forward(d, x, batch)
        got = _noalloc_forward(d, x, batch)
        torch.cuda.synchronize()
        assert np.array_equal(to_host(got, field.dtype), to_host(ref, field.dtype)), f"call {call}"


def test_noalloc_in_place():
    import torch

    n = 1 << 21
    d = NttDomain(BabyBear, n)
    x = to_dev(gen_input_seeded(BabyBear, n, 5))
    ref = _reference_forward(d, x, 1)
    rc = _lib.lib().omr_ntt_forward_noalloc(d.handle, _ptr(x), _ptr(x), 1,
                                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc)
    torch.cuda.synchronize()
    assert np.array_equal(to_host(x, BabyBear.dtype), to_host(ref, BabyBear.dtype))


def test_noalloc_rejects_oversize_without_touching_buffers():
    import torch

    n = 1 << 23  # 32 MiB of BabyBear words > 16 MiB
    d = NttDomain(BabyBear, n)
    x = to_dev(gen_input_seeded(BabyBear, n, 3))
    out = torch.zeros_like(x)
    rc = _lib.lib().omr_ntt_forward_noalloc(d.handle, _ptr(x), _ptr(out), 1, None)
    assert rc == CAPACITY
    assert b"16 MiB" in _lib.lib().omr_ntt_last_error()
    torch.cuda.synchronize()
    assert int(out.abs().sum().item()) == 0


@pytest.mark.parametrize("field,log_n,batch", [(BabyBear, 18, 2), (Goldilocks, 16, 3)],
                         ids=lambda v: getattr(v, "name", str(v)))
def test_noalloc_matches_oracle(oracle, field, log_n, batch):
    import torch

    n = 1 << log_n
    d = NttDomain(field, n)
    x = gen_input_seeded(field, n * batch, 77 + log_n)
    got = _noalloc_forward(d, to_dev(x), batch)
    torch.cuda.synchronize()
    assert np.array_equal(to_host(got, field.dtype), oracle.forward(field.id, x, batch=batch))


def test_noalloc_skips_learned_planner_and_allocates_nothing(oracle):
    """With the learned planner installed, a call on a shape the planner has
    not seen neither consults the network (which would allocate its buffers
    and record its choice in the planner database) nor changes the device's
    free memory once the shape has been warmed up."""
    import torch

    from omr_ntt import planner

    field, log_n, batch = BabyBear, 19, 2  # inside the network's training domain
    n = 1 << log_n
    L = _lib.lib()
    planner.install_default()
    try:
        L.omr_ntt_planner_clear()
        d = NttDomain(field, n)
        x_host = gen_input_seeded(field, n * batch, 31)
        x = to_dev(x_host)
        out = torch.empty_like(x)
        sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

        def call():
            _lib.check(L.omr_ntt_forward_noalloc(d.handle, _ptr(x), _ptr(out), batch, sp))

        call()  # warm-up: loads the code and reserves the static array
        torch.cuda.synchronize()
        assert L.omr_ntt_planner_get(field.id, log_n, batch, -1, 0, None, None) == 0, \
            "the learned selector was consulted"
        assert np.array_equal(to_host(out, field.dtype), oracle.forward(field.id, x_host, batch=batch))
        free0, _ = torch.cuda.mem_get_info()
        for _ in range(3):
            call()
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0, f"device free memory changed by {free0 - free1} bytes"
        assert np.array_equal(to_host(out, field.dtype), oracle.forward(field.id, x_host, batch=batch))
    finally:
        planner.uninstall()
