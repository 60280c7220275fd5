"""Benchmark: forward NTT, n = 2^24, BabyBear, on GB300 (one JSON line).

Contract: `python bench.py --gpus N --steps K --warmup W` (N > 1 under
torchrun, one rank per GPU; replicas of the same workload, weak scaling).
`--impl reference` times the reference algorithm's CPU implementation on the
host cores instead (the C restatement of WinterfellFourStep, the reference's
parallel full-NTT path; the Rust crate itself cannot be built here).

A step = one forward NTT of 2^24 BabyBear words (u32), inputs resident in
HBM.  The 64 MiB working set fits in L2, so L2 is flushed (a 256 MiB write)
before every timed step, outside the timed events.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "omr-ntt_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Gelem/s & %HBM roofline, n=2^24 NTT"
UNIT = "Gelem/s"
LOG_N = 24


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--field", default="BabyBear")
    ap.add_argument("--log-n", type=int, default=LOG_N)
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def job_throughput(local_ms, elems_per_step, steps, world, device=None):
    """Whole-job throughput of replicas (weak scaling): every rank transforms
    its own `steps` x `elems_per_step` words with no data exchange, the job
    time is the slowest rank's, so value = all ranks' elements / max time
    (Gelem/s).  Returns (value, max_ms); the only collective is the MAX."""
    total_ms = float(local_ms)
    if world > 1:
        import torch
        import torch.distributed as dist

        t = torch.tensor([total_ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return elems_per_step * world * steps / (total_ms / 1e3) / 1e9, total_ms


def replica_seed(rank):
    """Each replica transforms its own seeded input."""
    return 42 + rank


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                smax = float(r[1])
                for nm, v in zip(names, r[4:8]):
                    if v.lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def pass_kernel(plan_name: str) -> str:
    """The kernel that runs the passes of a plan (from its description)."""
    for key, kern in (("wide", "ntt_wide_pass"), ("slab", "ntt_slab_pass"), ("cluster", "ntt_cluster_kernel"),
                      ("tma", "ntt_tile_pass_tma")):
        if key in plan_name:
            return kern
    return "ntt_tile_pass"


def workload_config(field, log_n):
    """The `config` both arms print (the same workload, so the same dict)."""
    return {"workload": f"{field.name} forward NTT n=2^{log_n}, batch 1",
            "field": field.name, "log_n": log_n, "batch": 1}


def cpu_baseline(field, log_n, seconds, steps=None):
    """The oracle's WinterfellFourStep (the reference's parallel four-step,
    restated in C with OpenMP) on all host cores; bounded sample.  Returns
    (Gelem/s, cores, samples, times, compiler flags)."""
    import numpy as np
    from oracle import oracle

    flags = oracle.BUILD_FLAGS
    oracle.set_threads(0)
    cores = oracle.get_threads()
    n = 1 << log_n
    x = __import__("omr_ntt").gen_input_seeded(field, n, 42)
    oracle.ntt(field.id, x, "WinterfellFourStep")  # warm-up (page-in)
    times = []
    t_end = time.perf_counter() + seconds
    while (steps is None and (time.perf_counter() < t_end or not times)) or (steps is not None and len(times) < steps):
        t0 = time.perf_counter()
        oracle.ntt(field.id, x, "WinterfellFourStep")
        times.append(time.perf_counter() - t0)
    return n * len(times) / sum(times) / 1e9, cores, len(times), times, flags


def cpu_config_samples(extras, partial, headline_ms, field, log_n):
    """Each benchmark shape timed on the host cores with the oracle's C
    restatement of the reference encoder the crate's benches use for it
    (ArkRadix2 at 2^16, TfheStockhamRadix8 and WinterfellFourStep at 2^24,
    WinterfellFourStep on the 64 x 2^20 batch, TransformDecomposition for
    prefixes at 2^22), beside the GPU milliseconds of the same shape."""
    from omr_ntt.fields import BabyBear, Goldilocks
    from oracle import oracle

    oracle.set_threads(0)
    cores = oracle.get_threads()
    out = {"cores": cores, "kind": "port", "rows": {}}

    def best_ms(fn, reps=2):
        fn()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        return 1000 * min(ts)

    gpu = {f"{field.name} fwd 2^{log_n}x1": headline_ms}
    gpu.update({k: v["ms"] for k, v in extras.items()})
    rows = [("BabyBear fwd 2^16x1", BabyBear, 16, 1, "ArkRadix2", 0),
            ("BabyBear fwd 2^24x1", BabyBear, 24, 1, "TfheStockhamRadix8", 0),
            ("BabyBear fwd 2^24x1 (four-step)", BabyBear, 24, 1, "WinterfellFourStep", 0),
            ("Goldilocks fwd 2^24x1", Goldilocks, 24, 1, "WinterfellFourStep", 0),
            ("BabyBear fwd 2^20x64", BabyBear, 20, 64, "WinterfellFourStep", 0)]
    for k in (4, 8, 12, 16):
        rows.append((f"BabyBear s=2^{k} prefix", BabyBear, 22, 1, "TransformDecomposition", 1 << (k - 1)))
    for label, fld, lg, bt, enc, s in rows:
        x = __import__("omr_ntt").gen_input_seeded(fld, (1 << lg) * bt, 7)
        ms = best_ms(lambda: oracle.ntt(fld.id, x, enc, s=s, batch=bt), reps=1 if lg + (bt > 1) * 6 >= 24 else 3)
        key = label.replace(" (four-step)", "")
        g = partial.get(fld.name, {}).get(label.split(" ", 1)[1]) if "prefix" in label else gpu.get(key)
        out["rows"][label] = {"encoder": enc, "cpu_ms": round(ms, 3), "gpu_ms": g,
                              "gpu_speedup": round(ms / g, 1) if g else None}
    return out


def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return
    from omr_ntt.fields import field_by_name

    field = field_by_name(args.field)
    n = 1 << args.log_n
    cpu_baseline(field, args.log_n, 0, steps=max(1, args.warmup))
    val, cores, cnt, times, flags = cpu_baseline(field, args.log_n, 0, steps=args.steps)
    ms = 1000 * sum(times) / len(times)
    sample = (f"{cnt} x WinterfellFourStep {field.name} n=2^{args.log_n} forward (C restatement of "
              f"src/encoders/winterfell_four_step.rs, OpenMP {cores} threads, {flags})")
    line = {
        "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32" if field.word_bytes == 4 else "u64",
        "data": "synthetic (splitmix64 seed 42, uniform [0,p))",
        "config": workload_config(field, args.log_n),
        "impl": "reference",
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch

    import omr_ntt
    from omr_ntt import NttDomain, _lib
    from omr_ntt.fields import BabyBear, Goldilocks, field_by_name

    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # the learned planner trained on GB300 picks every plan = -1 below
    from omr_ntt import planner as lp

    planner_file = lp.install_default()

    field = field_by_name(args.field)
    log_n = args.log_n
    n = 1 << log_n
    w = field.word_bytes
    sdt = torch.int32 if w == 4 else torch.int64
    domain = NttDomain(field, n)
    x = omr_ntt.gen_input_seeded(field, n, replica_seed(rank))
    xd = torch.from_numpy(x.view(np.int32 if w == 4 else np.int64).copy()).cuda()
    buf = xd.clone()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    L = _lib.lib()
    plan = -1
    passes = omr_ntt.plan_passes(field, log_n, plan)

    def step():
        _lib.check(L.omr_ntt_forward(domain.handle, plan, ctypes.c_void_p(buf.data_ptr()),
                                     ctypes.c_void_p(buf.data_ptr()), 1, sp))

    assert args.warmup >= 3, "need >= 3 warm-up steps"
    for _ in range(args.warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize()

    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clk:
        for e0, e1 in evs:
            flush.zero_()
            e0.record(stream)
            step()
            e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    step_ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    value, total_ms = job_throughput(sum(step_ms), n, args.steps, world, device="cuda")
    ms_per_step = total_ms / args.steps

    # ---- per-pass timing (the dominant kernel's roofline), same stream, CUDA events
    scratch = torch.empty_like(buf)
    pass_ms = []
    for pi in range(len(passes)):
        ts = []
        for _ in range(max(3, args.steps // 2)):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _lib.check(L.omr_ntt_plan_run_pass(domain.handle, plan, pi, 0, ctypes.c_void_p(buf.data_ptr()),
                                               ctypes.c_void_p(scratch.data_ptr()),
                                               ctypes.c_void_p(buf.data_ptr()), 1, sp))
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        pass_ms.append(sum(ts) / len(ts))
    dom = max(range(len(pass_ms)), key=lambda i: pass_ms[i])
    peak, peak_src = peaks()
    alg_bytes = 2 * n * w  # one read + one write of the data per pass launch
    achieved = alg_bytes / (pass_ms[dom] / 1e3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        # DRAM bytes per launch from one ncu capture, valid only for the plan captured
        ent = json.load(open(tpath)).get(f"{field.name}:{log_n}")
        if ent and ent.get("plan") == omr_ntt.plan_describe(field, log_n, plan):
            traffic = ent["pass_traffic_bytes"][dom]

    # ---- end to end through the C ABI with host buffers (pinned), copies inside
    hbuf = torch.from_numpy(x.view(np.int32 if w == 4 else np.int64).copy()).pin_memory()
    hp = ctypes.c_void_p(hbuf.data_ptr())
    for _ in range(2):
        _lib.check(L.omr_ntt_forward_host(domain.handle, plan, hp, 1))
    e2e_t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _lib.check(L.omr_ntt_forward_host(domain.handle, plan, hp, 1))
        e2e_t.append(time.perf_counter() - t0)
    e2e_val = n * world * len(e2e_t) / sum(e2e_t) / 1e9

    # ---- extras: the other full-transform shapes (2^16..2^27, batch 64 x 2^20; a few steps each)
    extras = {}
    if not args.no_extras:
        def timed(fn, reps=5):
            for _ in range(2):
                flush.zero_()
                fn()
            ts = []
            for _ in range(reps):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            return sum(ts) / len(ts)

        def autotune(fld, lg, bt):
            # setup, untimed (the crate's benches build the domain outside the
            # timed loop): the exhaustive autotuner stores the fastest plan of
            # this shape in the planner database, which plan = -1 consults first
            pt = {"field": fld.id, "log_n": lg, "log_s": lg, "pattern": "contiguous", "batch": bt}
            ms = lp.tune(pt, reps=3, seed=11)
            st, pa = lp.candidates(pt)[int(np.argmin(ms))]
            _lib.check(L.omr_ntt_planner_set(fld.id, lg, bt, 0, 1 << lg, st, pa))

        for fld, lg, bt, inv in ((BabyBear, 16, 1, False), (BabyBear, 24, 1, True), (Goldilocks, 24, 1, False),
                                 (Goldilocks, 24, 1, True), (BabyBear, 20, 64, False),
                                 (Goldilocks, 20, 64, False), (BabyBear, 22, 1, False),
                                 (BabyBear, 20, 1, False), (BabyBear, 27, 1, False)):
            nn = 1 << lg
            autotune(fld, lg, bt)
            dd = NttDomain(fld, nn)
            t = torch.empty(nn * bt, dtype=torch.int32 if fld.word_bytes == 4 else torch.int64, device="cuda")
            t.random_(0, 1 << 30)
            fn_ = L.omr_ntt_inverse if inv else L.omr_ntt_forward
            ms = timed(lambda: _lib.check(fn_(dd.handle, -1, ctypes.c_void_p(t.data_ptr()),
                                              ctypes.c_void_p(t.data_ptr()), bt, sp)))
            gbs = 2 * nn * bt * fld.word_bytes / (ms / 1e3) / 1e9
            extras[f"{fld.name} {'inv' if inv else 'fwd'} 2^{lg}x{bt}"] = {
                "ms": round(ms, 4), "Gelem/s": round(nn * bt / (ms / 1e3) / 1e9, 2),
                "GB/s_alg": round(gbs, 1), "frac_hbm": round(gbs / peak, 3)}
            del t, dd

    # ---- partial outputs (n = 2^22, s = 2^4..2^16, three index patterns)
    partial = {}
    if not args.no_extras:
        import omr_ntt.inputs as oin

        for fld in (BabyBear, Goldilocks):
            nn = 1 << 22
            dd = NttDomain(fld, nn)
            t = torch.empty(nn, dtype=torch.int32 if fld.word_bytes == 4 else torch.int64, device="cuda")
            t.random_(0, 1 << 30)
            row = {}
            for k in range(4, 17, 2):
                sc = 1 << k
                o = torch.empty(sc, dtype=t.dtype, device="cuda")
                idx = torch.from_numpy(oin.random_indices(nn, sc, k).view(np.int32)).cuda()
                for pat, nm in ((0, "prefix"), (1, "strided"), (2, "random")):
                    ip = ctypes.c_void_p(idx.data_ptr()) if pat == 2 else None
                    ms = timed(lambda: _lib.check(L.omr_ntt_partial(dd.handle, pat, sc, ip, ctypes.c_void_p(t.data_ptr()),
                                                                    ctypes.c_void_p(o.data_ptr()), sp)), reps=5)
                    row[f"s=2^{k} {nm}"] = round(ms, 4)
            partial[fld.name] = row
            del t, dd

    # ---- mixed batch: one graph-launched persistent kernel vs per-request kernels
    mixed = None
    if not args.no_extras:
        from omr_ntt.batch import Batch, layout, mixed_requests

        reqs = mixed_requests(2024, count=4096)
        ib, ob = layout(reqs)
        g = torch.Generator(device="cuda").manual_seed(5)
        d_in = torch.randint(0, 1 << 30, ((ib + 3) // 4,), dtype=torch.int32, device="cuda", generator=g)
        d_out = torch.empty(ob, dtype=torch.uint8, device="cuda")
        bt = Batch(reqs)
        bt.run(d_in.data_ptr(), d_out.data_ptr(), stream.cuda_stream)  # capture + warm-up
        bt.run_per_request(d_in.data_ptr(), d_out.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()

        def tmix(fn, reps=5):
            ts = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            ts.sort()
            return ts[len(ts) // 2]

        ms_b = tmix(lambda: bt.run(d_in.data_ptr(), d_out.data_ptr(), stream.cuda_stream))
        ms_p = tmix(lambda: bt.run_per_request(d_in.data_ptr(), d_out.data_ptr(), stream.cuda_stream))
        bt.check(stream.cuda_stream)
        elems = sum(r.n for r in reqs)
        mixed = {"requests": len(reqs), "elements": elems, "tasks": bt.info()["tasks"],
                 "graph_persistent_ms": round(ms_b, 3), "per_request_ms": round(ms_p, 3),
                 "speedup": round(ms_p / ms_b, 2), "graph_Gelem/s": round(elems / ms_b / 1e6, 2)}
        bt.close()
        del d_in, d_out

    # ---- learned planner: stored held-out regret + a live re-tune of held-out points
    learned = None
    if not args.no_extras and rank == 0:
        params, meta = lp.load_params(os.path.join(lp.DATA_DIR, "planner_mlp.npz"))
        z = np.load(os.path.join(lp.DATA_DIR, "planner_dataset.npz"))
        pts = json.loads(str(z["points"]))
        net = lp.Mlp(seed=0)
        net.set_params(params)
        live = []
        for p in pts[1500:1500 + 50]:
            ms = lp.tune(p, reps=3, seed=7)
            cm = lp.class_map(p)
            pred = net.forward(lp.features(p)[None])[0]
            app = [c for c, j in enumerate(cm) if j >= 0]
            c = min(app, key=lambda c: pred[c])
            live.append(float(ms[cm[c]] / ms.min() - 1.0))
        net.close()
        # the built-in rule as the code has it now, on the stored held-out timings
        T = z["T"].astype(np.float64)
        best = z["best"].astype(np.float64)
        rule = np.array([lp.heuristic_class(p) for p in pts[1500:]])
        rule_regret = float(np.mean(lp.regret(T[1500:], best[1500:], rule)))
        s = meta["summary"]
        learned = {"held_out_points": s["held_out"], "classes": s["classes"],
                   "regret_mean": s["regret_mlp"]["mean"], "regret_median": s["regret_mlp"]["median"],
                   "regret_p90": s["regret_mlp"]["p90"], "within_5pct": s["regret_mlp"]["within_5pct"],
                   "builtin_rule_regret_mean": rule_regret,
                   "live_retune_points": len(live), "live_regret_mean": float(np.mean(live)),
                   "network": os.path.relpath(planner_file, ROOT)}

    # ---- CPU baseline (rank 0, N=1 only): the oracle port on the host cores
    cpu = None
    if rank == 0 and world == 1:
        cval, cores, cnt, _, flags = cpu_baseline(field, log_n, args.cpu_seconds)
        cpu = {"value": cval, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{cnt} x WinterfellFourStep {field.name} n=2^{log_n} forward, C restatement "
                         f"of src/encoders/winterfell_four_step.rs, OpenMP {cores} threads, {flags}"}

    # ---- CPU restatements of the reference's own encoders on the other configs
    # (rank 0, N=1): one bounded sample each, beside the GPU time of the same shape
    cpu_configs = None
    if not args.no_extras and rank == 0 and world == 1:
        cpu_configs = cpu_config_samples(extras, partial, ms_per_step, field, log_n)

    if rank == 0:
        clocks = clk.summary()
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32" if w == 4 else "u64",
            "data": "synthetic (splitmix64 seed 42+rank, uniform [0,p))",
            "config": workload_config(field, log_n),
            "setup": {"plan": omr_ntt.plan_describe(field, log_n, plan),
                      "l2": "flushed (256 MiB write) before every timed step",
                      "parallelism": f"replicas x{world} (batch 1 per GPU)"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": f"{pass_kernel(omr_ntt.plan_describe(field, log_n, plan))} pass {dom} "
                                   f"(logT={passes[dom]['logT']})",
                         "peak_source": peak_src,
                         "pass_ms": [round(t, 4) for t in pass_ms],
                         "transform_frac": (2 * n * w / (ms_per_step / 1e3) / 1e9) / peak},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": n * w,
                    "d2h_bytes_per_step": n * w,
                    "path": "omr_ntt_forward_host (pinned host buffer, H2D + NTT + D2H + sync)"},
            "gpu_launches": len(passes) * args.steps,
            "clocks": clocks,
            "extras": extras,
            "partial_ms": partial,
            "cpu_configs": cpu_configs,
            "mixed_batch": mixed,
            "learned_planner": learned,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
