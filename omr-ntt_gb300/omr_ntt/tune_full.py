"""Exhaustive tuning of full transforms into a planner database file.

    python -m omr_ntt.tune_full                 # writes omr-ntt_gb300/data/planner_full.db
    python -m omr_ntt.tune_full --out PATH --min-log 6 --max-log 24

For every field, log2 N in [min-log, max-log] and batch in (1, 8, 64, 512)
with batch * N <= 2^26 words, the exhaustive autotuner times every plan
(omr_ntt_tune_point: seeded canonical inputs, L2 flushed before each timed
run, median of `reps` CUDA-event timings) and the fastest goes into the
planner database, which is then written with omr_ntt_planner_save.
`planner.install_default()` loads the file beside the learned selector: the
database is consulted first, so plan = -1 -- and the full transform behind a
partial output's gather -- runs the measured-best plan for these shapes, and
the network plans the rest (partial outputs, other batch sizes).
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import planner as P
from ._lib import check, lib
from .fields import BabyBear, Goldilocks, KoalaBear, TeddyBear

BATCHES = (1, 8, 64, 512)
MAX_WORDS = 1 << 26


def shapes(min_log: int, max_log: int):
    for f in (BabyBear, Goldilocks, KoalaBear, TeddyBear):
        for log_n in range(min_log, max_log + 1):
            for batch in BATCHES:
                if batch << log_n <= MAX_WORDS:
                    yield f, log_n, batch


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(P.DATA_DIR, "planner_full.db"))
    ap.add_argument("--min-log", type=int, default=6)
    ap.add_argument("--max-log", type=int, default=24)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args(argv)
    L = lib()
    check(L.omr_ntt_planner_clear())
    t0 = time.time()
    rows = []
    for f, log_n, batch in shapes(a.min_log, a.max_log):
        p = {"field": f.id, "log_n": log_n, "log_s": log_n, "pattern": "contiguous", "batch": batch}
        ms = P.tune(p, reps=a.reps, seed=log_n * 1000 + batch)
        cands = P.candidates(p)
        i = int(np.nanargmin(ms))
        strategy, param = cands[i]
        check(L.omr_ntt_planner_set(f.id, log_n, batch, 0, 1 << log_n, strategy, param))
        rows.append((f.name, log_n, batch, param, float(ms[i])))
    check(L.omr_ntt_planner_save(a.out.encode()))
    print(json.dumps({"entries": len(rows), "seconds": round(time.time() - t0, 1), "out": a.out}))


if __name__ == "__main__":
    main()
