"""Mixed batches (one persistent, graph-launched kernel) -- Python wrapper.

`mixed_requests(seed, count)` draws the mixed-batch workload: log2 N uniform
in [10, 20], BabyBear or Goldilocks with probability 1/2, 25% partial-output
requests with s = 2^k (k uniform in [4, log2 N - 2]) and a random index set,
forward or inverse with probability 1/2, all from one seed.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field as dfield

import numpy as np

from ._lib import check, lib
from .fields import BabyBear, Goldilocks, field_by_id
from .inputs import gen_input_seeded


@dataclass
class Request:
    field: object
    log_n: int
    inverse: bool
    indices: np.ndarray | None = None  # partial output set (None: full)
    in_off: int = 0
    out_off: int = 0

    @property
    def n(self):
        return 1 << self.log_n

    @property
    def out_words(self):
        return self.n if self.indices is None else len(self.indices)


def mixed_requests(seed: int, count: int = 4096, min_log: int = 10, max_log: int = 20):
    rng = np.random.Generator(np.random.PCG64(seed))
    reqs = []
    for _ in range(count):
        log_n = int(rng.integers(min_log, max_log + 1))
        fld = BabyBear if rng.random() < 0.5 else Goldilocks
        partial = rng.random() < 0.25
        inverse = bool(rng.random() < 0.5)
        idx = None
        if partial:
            k = int(rng.integers(4, log_n - 2 + 1))
            idx = np.sort(rng.choice(1 << log_n, size=1 << k, replace=False)).astype(np.uint32)
        reqs.append(Request(fld, log_n, inverse, idx))
    return reqs


def layout(reqs):
    """Byte offsets of every request in the input and output arenas."""
    ioff = ooff = 0
    for r in reqs:
        w = r.field.word_bytes
        ioff = (ioff + 255) // 256 * 256
        ooff = (ooff + 255) // 256 * 256
        r.in_off, r.out_off = ioff, ooff
        ioff += r.n * w
        ooff += r.out_words * w
    return ioff, ooff


def fill_inputs(reqs, in_bytes: int, seed: int) -> np.ndarray:
    """Host input arena (uint8) with seeded canonical words for every request."""
    arena = np.zeros(in_bytes, dtype=np.uint8)
    for i, r in enumerate(reqs):
        x = gen_input_seeded(r.field, r.n, seed * 100003 + i)
        arena[r.in_off:r.in_off + x.nbytes] = x.view(np.uint8)
    return arena


class Batch:
    def __init__(self, reqs):
        self.reqs = reqs
        h = ctypes.c_void_p()
        check(lib().omr_ntt_batch_create(ctypes.byref(h)))
        self._h = h
        for r in reqs:
            idx = r.indices
            rc = lib().omr_ntt_batch_add(
                h, r.field.id, r.log_n, 1 if r.inverse else 0, -1 if idx is None else 2,
                0 if idx is None else len(idx), idx.ctypes.data if idx is not None else None,
                r.in_off, r.out_off)
            if rc < 0:
                check(rc)
        check(lib().omr_ntt_batch_build(h))

    def info(self):
        a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        check(lib().omr_ntt_batch_info(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"requests": a.value, "tasks": b.value, "scratch_bytes": c.value}

    def run(self, d_in, d_out, stream=None):
        check(lib().omr_ntt_batch_run(self._h, ctypes.c_void_p(d_in), ctypes.c_void_p(d_out),
                                      ctypes.c_void_p(stream or 0)))

    def run_per_request(self, d_in, d_out, stream=None):
        check(lib().omr_ntt_batch_run_per_request(self._h, ctypes.c_void_p(d_in), ctypes.c_void_p(d_out),
                                                  ctypes.c_void_p(stream or 0)))

    def check(self, stream=None):
        check(lib().omr_ntt_batch_check(self._h, ctypes.c_void_p(stream or 0)))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().omr_ntt_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
