"""Python mirror of the reference crate's API over the GB300 engine.

The names follow benbencik/omr-ntt so its tests and benches read the same:

    from omr_ntt import NttDomain, DefaultField, encoders
    domain = NttDomain(DefaultField, 1 << 16)          # src/encoder.rs:23-51
    for encoder in encoders.all(16):                    # src/encoders/mod.rs:32-46
        encoder.ntt(buf, domain)                        # src/encoder.rs:70-74

``buf`` is either a NumPy array of canonical words (host; the call copies
through the GPU and back, like the reference's in-place ``&mut [F]``) or a
CUDA tensor (device; runs asynchronously on torch's current stream).  All
compute runs in the CUDA library; there is no CPU path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import OmrNttError, check, lib
from .fields import BabyBear, DefaultField, Field, Goldilocks, KoalaBear, TeddyBear, field_by_id
from .inputs import gen_input_seeded, random_indices
from . import encoders

__all__ = [
    "NttDomain", "NttEncoder", "Field", "BabyBear", "Goldilocks", "KoalaBear", "TeddyBear",
    "DefaultField", "encoders", "forward", "inverse", "partial", "gen_input_seeded",
    "random_indices", "OmrNttError", "PREFIX", "STRIDED", "INDICES", "plan_count",
    "plan_describe", "plan_passes", "lib",
]

PREFIX, STRIDED, INDICES = 0, 1, 2


def _is_tensor(x) -> bool:
    return hasattr(x, "data_ptr") and hasattr(x, "is_cuda")


def _stream_of(x, stream):
    if stream is not None:
        return ctypes.c_void_p(int(stream))
    if _is_tensor(x):
        import torch

        return ctypes.c_void_p(torch.cuda.current_stream(x.device).cuda_stream)
    return ctypes.c_void_p(0)


class NttDomain:
    """Reusable NTT parameters (src/encoder.rs:9-51): N, log_N, omega and the
    device twiddle tables.  ``twiddles`` / ``bitrev_twiddles`` are fetched on
    first use (as NumPy arrays)."""

    def __init__(self, field: Field, N: int):
        if N <= 0 or N & (N - 1):
            # NttDomain::new asserts N.is_power_of_two() (src/encoder.rs:24)
            raise OmrNttError(-2, f"NTT size N={N} must be a power of 2")
        self.field = field
        self.N = int(N)
        self.log_N = self.N.bit_length() - 1
        h = ctypes.c_void_p()
        check(lib().omr_ntt_domain_create(field.id, self.log_N, ctypes.byref(h)))
        self._h = h
        om = ctypes.c_uint64()
        check(lib().omr_ntt_domain_info(h, None, None, None, ctypes.byref(om)))
        self.omega = int(om.value)
        self._tw = None
        self._brtw = None

    @property
    def handle(self):
        return self._h

    @property
    def twiddles(self):
        if self._tw is None:
            a = np.empty(self.N, dtype=self.field.dtype)
            check(lib().omr_ntt_domain_twiddles(self._h, 0, a.ctypes.data))
            self._tw = a
        return self._tw

    @property
    def bitrev_twiddles(self):
        if self._brtw is None:
            a = np.empty(self.N // 2, dtype=self.field.dtype)
            check(lib().omr_ntt_domain_twiddles(self._h, 1, a.ctypes.data))
            self._brtw = a
        return self._brtw

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().omr_ntt_domain_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


NttEncoder = encoders.NttEncoder


def _host_array(field: Field, x):
    a = np.ascontiguousarray(x, dtype=field.dtype)
    return a


def forward(domain: NttDomain, x, plan: int = -1, out=None, batch: int = 1, stream=None):
    """Forward NTT of ``batch`` transforms.  Host arrays return a new array;
    CUDA tensors are transformed into ``out`` (default: in place)."""
    return _transform(domain, x, plan, out, batch, stream, inverse=False)


def inverse(domain: NttDomain, x, plan: int = -1, out=None, batch: int = 1, stream=None):
    return _transform(domain, x, plan, out, batch, stream, inverse=True)


def _transform(domain, x, plan, out, batch, stream, inverse):
    L = lib()
    if _is_tensor(x):
        dst = x if out is None else out
        fn = L.omr_ntt_inverse if inverse else L.omr_ntt_forward
        check(fn(domain.handle, plan, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(dst.data_ptr()),
                 batch, _stream_of(x, stream)))
        return dst
    a = _host_array(domain.field, x).copy()
    fn = L.omr_ntt_inverse_host if inverse else L.omr_ntt_forward_host
    check(fn(domain.handle, plan, a.ctypes.data, batch))
    return a


def partial(domain: NttDomain, x, pattern: int, count: int, indices=None, out=None, stream=None):
    """Selected outputs of the forward NTT: X[0..count) (PREFIX),
    X[j N/count] (STRIDED) or X[indices] (INDICES)."""
    L = lib()
    if _is_tensor(x):
        import torch

        if out is None:
            out = torch.empty(count, dtype=x.dtype, device=x.device)
        idx_ptr = ctypes.c_void_p(indices.data_ptr()) if indices is not None else None
        check(L.omr_ntt_partial(domain.handle, pattern, count, idx_ptr, ctypes.c_void_p(x.data_ptr()),
                                ctypes.c_void_p(out.data_ptr()), _stream_of(x, stream)))
        return out
    a = _host_array(domain.field, x)
    res = np.empty(count, dtype=domain.field.dtype)
    idx = None
    if indices is not None:
        idx = np.ascontiguousarray(indices, dtype=np.uint32)
    check(L.omr_ntt_partial_host(domain.handle, pattern, count,
                                 idx.ctypes.data if idx is not None else None, a.ctypes.data,
                                 res.ctypes.data))
    return res


def plan_count(field: Field, log_n: int) -> int:
    n = lib().omr_ntt_plan_count(field.id, log_n)
    if n < 0:
        check(n)
    return n


def plan_describe(field: Field, log_n: int, plan: int) -> str:
    buf = ctypes.create_string_buffer(128)
    check(lib().omr_ntt_plan_describe(field.id, log_n, plan, buf, 128))
    return buf.value.decode()


def plan_passes(field: Field, log_n: int, plan: int = -1, batch: int = 1):
    rec = (ctypes.c_uint64 * (16 * 8))()
    n = lib().omr_ntt_plan_passes(field.id, log_n, plan, batch, rec, 8)
    if n < 0:
        check(n)
    keys = ["logT", "L_lo", "L_m", "L_b", "is_lo", "is_m", "is_b", "os_lo", "os_m", "os_b",
            "es_in", "es_out", "twiddle", "tw_scale", "tw_line_mul_m", "bufs"]
    out = []
    for i in range(n):
        r = dict(zip(keys, [int(rec[16 * i + k]) for k in range(16)]))
        r["in_buf"] = r["bufs"] & 0xFF
        r["out_buf"] = r.pop("bufs") >> 8
        out.append(r)
    return out
