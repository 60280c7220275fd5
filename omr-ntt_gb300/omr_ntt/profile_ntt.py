"""Profiling harness (the GB300 counterpart of the reference's
examples/profile_ntt.rs, which runs TransformDecomposition(s = 50) at
log N = 27: two warm-up calls, then timed calls on seed 42).

    python -m omr_ntt.profile_ntt                              # the reference's case
    python -m omr_ntt.profile_ntt --mode forward --field BabyBear --log-n 24 --plan -1 --iters 2
    python -m omr_ntt.profile_ntt --mode partial --log-n 22 --pattern 1 --s 16
    python -m omr_ntt.profile_ntt --mode batch --requests 512   # mixed batch, graph launch
    python -m omr_ntt.profile_ntt --mode forward --log-n 16 --batch 64 --plan 15

Runs on device buffers through the C ABI with no host copies in the loop, so
that a profiler sees only the engine's kernels (plus one buffer fill).
"""
from __future__ import annotations

import argparse
import ctypes

from . import _lib
from .fields import field_by_name


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--mode", default="encode", choices=["encode", "forward", "inverse", "partial", "batch"])
    ap.add_argument("--field", default="BabyBear")
    ap.add_argument("--log-n", type=int, default=27)
    ap.add_argument("--encoder", default="TransformDecomposition")
    ap.add_argument("--s", type=int, default=50)
    ap.add_argument("--pattern", type=int, default=0)
    ap.add_argument("--plan", type=int, default=-1)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--iters", type=int, default=5)
    ap.add_argument("--requests", type=int, default=512)
    ap.add_argument("--batch", type=int, default=1, help="transforms per forward/inverse call")
    a = ap.parse_args(argv)

    import torch

    if a.mode == "batch":
        return run_batch(a)

    from . import NttDomain, encoders

    fld = field_by_name(a.field)
    n = 1 << a.log_n
    d = NttDomain(fld, n)
    dt = torch.int32 if fld.word_bytes == 4 else torch.int64
    g = torch.Generator(device="cuda").manual_seed(42)
    bt = a.batch if a.mode in ("forward", "inverse") else 1
    x = torch.randint(0, 1 << 30, (n * bt,), dtype=dt, device="cuda", generator=g)
    out = torch.empty(max(a.s, 1) if a.mode == "partial" else n, dtype=dt, device="cuda")
    L = _lib.lib()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    enc = {e.__name__: e for e in (encoders.ArkRadix2, encoders.Dft, encoders.DftPartial, encoders.LambdaBowers,
                                    encoders.LambdaRadix4, encoders.Plonky3Radix2LayerSplit,
                                    encoders.TfheStockhamRadix8, encoders.TransformDecomposition,
                                    encoders.TransformDecompositionV2, encoders.WinterfellFourStep)}

    idx = None
    if a.mode == "partial" and a.pattern == 2:
        from .inputs import random_indices

        idx = torch.from_numpy(random_indices(n, a.s, 3).view("int32")).cuda()

    def once():
        p = ctypes.c_void_p(x.data_ptr())
        if a.mode == "encode":
            cls = enc[a.encoder]
            e = cls(a.s) if cls.ID in (2, 7, 8) else cls()
            _lib.check(L.omr_ntt_encode(d.handle, e.ID, e.s, p, 1, st))
        elif a.mode == "forward":
            _lib.check(L.omr_ntt_forward(d.handle, a.plan, p, p, bt, st))
        elif a.mode == "inverse":
            _lib.check(L.omr_ntt_inverse(d.handle, a.plan, p, p, bt, st))
        else:
            ip = ctypes.c_void_p(idx.data_ptr()) if idx is not None else None
            _lib.check(L.omr_ntt_partial(d.handle, a.pattern, a.s, ip, p, ctypes.c_void_p(out.data_ptr()), st))

    for _ in range(a.warmup):
        once()
    torch.cuda.synchronize()
    for _ in range(a.iters):
        once()
    torch.cuda.synchronize()
    print("ok")


def run_batch(a):
    """The mixed batch of the bench (log n in [10, 20], both fields, 25%
    partial, fwd/inv) with `--requests` requests: one graph-launched
    persistent kernel per run."""
    import torch

    from .batch import Batch, layout, mixed_requests

    reqs = mixed_requests(2024, count=a.requests)
    ib, ob = layout(reqs)
    g = torch.Generator(device="cuda").manual_seed(5)
    d_in = torch.randint(0, 1 << 30, ((ib + 3) // 4,), dtype=torch.int32, device="cuda", generator=g)
    d_out = torch.empty(ob, dtype=torch.uint8, device="cuda")
    bt = Batch(reqs)
    st = torch.cuda.current_stream().cuda_stream
    for _ in range(a.warmup + a.iters):
        bt.run(d_in.data_ptr(), d_out.data_ptr(), st)
    torch.cuda.synchronize()
    bt.check(st)
    bt.close()
    print("ok")


if __name__ == "__main__":
    main()
