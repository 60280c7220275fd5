"""The learned plan selector: planning points, autotuner data, training, regret.

A planning point is (field, log2 n, log2 s, output pattern, batch).  The
exhaustive autotuner (omr_ntt_tune_point, native) times every candidate plan
of the point; the 64 plan classes (omr_ntt_plan_class_candidate) give a fixed
output vocabulary for the network.  The network (omr_ntt_mlp_*, trained on
the GPU by the library's own kernels) predicts each applicable class's log
time relative to the point's mean; its choice is the lowest prediction.
Regret of a choice = time(choice) / time(exhaustive optimum) - 1.

Points: field uniform in {BabyBear, Goldilocks}, log2 n uniform in [10, 24],
log2 s uniform in [4, log2 n] (s = n is the full transform), pattern uniform in
{contiguous, strided, random}, batch uniform in {1, 8, 64, 512}; points with
batch * n > 2^26 words are drawn again (they would hold tens of GB per point).
"""
from __future__ import annotations

import ctypes
import json
import math
import os

import numpy as np

from ._lib import check, lib
from .fields import BabyBear, Goldilocks, field_by_id

N_FEATURES = 10
N_HIDDEN = 64
PATTERNS = ("contiguous", "strided", "random")
PATTERN_ID = {"contiguous": 0, "strided": 1, "random": 2}
BATCHES = (1, 8, 64, 512)
MAX_WORDS = 1 << 26


def n_classes() -> int:
    return lib().omr_ntt_plan_class_count()


def planning_points(seed: int, count: int = 2000, min_log: int = 10, max_log: int = 24):
    rng = np.random.Generator(np.random.PCG64(seed))
    pts = []
    while len(pts) < count:
        field = BabyBear if rng.random() < 0.5 else Goldilocks
        log_n = int(rng.integers(min_log, max_log + 1))
        log_s = int(rng.integers(4, log_n + 1))
        pattern = PATTERNS[int(rng.integers(0, 3))]
        batch = BATCHES[int(rng.integers(0, 4))]
        if batch << log_n > MAX_WORDS:
            continue
        pts.append({"field": field.id, "log_n": log_n, "log_s": log_s, "pattern": pattern,
                    "batch": batch})
    return pts


def point_count(p) -> int:
    return 1 << p["log_s"]


def features(p) -> np.ndarray:
    f = (ctypes.c_float * N_FEATURES)()
    check_n = lib().omr_ntt_mlp_features(p["field"], p["log_n"], p["batch"], PATTERN_ID[p["pattern"]],
                                         point_count(p), f)
    assert check_n == N_FEATURES
    return np.frombuffer(f, dtype=np.float32).copy()


def candidates(p):
    L = lib()
    pat, cnt = PATTERN_ID[p["pattern"]], point_count(p)
    n = L.omr_ntt_candidates(p["field"], p["log_n"], pat, cnt, None, None, 0)
    st = (ctypes.c_int * n)()
    pa = (ctypes.c_int * n)()
    L.omr_ntt_candidates(p["field"], p["log_n"], pat, cnt, st, pa, n)
    return list(zip(list(st), list(pa)))


def class_map(p):
    """class -> index into candidates(p) (or -1 when not applicable)."""
    L = lib()
    cands = candidates(p)
    where = {c: i for i, c in enumerate(cands)}
    out = []
    s, q = ctypes.c_int(), ctypes.c_int()
    for c in range(n_classes()):
        ok = L.omr_ntt_plan_class_candidate(p["field"], p["log_n"], PATTERN_ID[p["pattern"]],
                                            point_count(p), c, ctypes.byref(s), ctypes.byref(q))
        out.append(where.get((s.value, q.value), -1) if ok else -1)
    return out


def tune(p, reps: int = 3, seed: int = 1):
    """Exhaustive autotuner on the GPU: median ms of every candidate."""
    cands = candidates(p)
    ms = (ctypes.c_float * len(cands))()
    rc = lib().omr_ntt_tune_point(p["field"], p["log_n"], p["batch"], PATTERN_ID[p["pattern"]],
                                  point_count(p), reps, seed, ms, len(cands))
    if rc < 0:
        check(rc)
    return np.array(list(ms), dtype=np.float64)


def collect(points, reps: int = 3, progress=None):
    """Dataset: features, class times (NaN: not applicable), exhaustive best."""
    K = n_classes()
    X = np.zeros((len(points), N_FEATURES), dtype=np.float32)
    T = np.full((len(points), K), np.nan)
    best = np.zeros(len(points))
    for i, p in enumerate(points):
        ms = tune(p, reps=reps, seed=1000 + i)
        cm = class_map(p)
        X[i] = features(p)
        for c, j in enumerate(cm):
            if j >= 0:
                T[i, c] = ms[j]
        best[i] = ms.min()
        if progress and (i + 1) % progress == 0:
            print(f"tuned {i + 1}/{len(points)}", flush=True)
    return {"X": X, "T": T, "best": best}


def targets(T):
    """Centred log times and the mask of applicable classes."""
    M = np.isfinite(T)
    logt = np.where(M, np.log(np.where(M, T, 1.0)), 0.0)
    mean = (logt * M).sum(1, keepdims=True) / np.maximum(M.sum(1, keepdims=True), 1)
    Y = np.where(M, logt - mean, 0.0)
    return Y.astype(np.float32), M.astype(np.float32)


class Mlp:
    """The library's MLP (device parameters, GPU training)."""

    def __init__(self, seed: int = 0, n_out: int | None = None):
        self.n_out = n_out or n_classes()
        h = ctypes.c_void_p()
        check(lib().omr_ntt_mlp_create(N_FEATURES, N_HIDDEN, self.n_out, seed, ctypes.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def params(self) -> np.ndarray:
        n = lib().omr_ntt_mlp_param_count(self._h)
        buf = (ctypes.c_float * n)()
        check(lib().omr_ntt_mlp_get_params(self._h, buf))
        return np.frombuffer(buf, dtype=np.float32).copy()

    def set_params(self, p):
        a = np.ascontiguousarray(p, dtype=np.float32)
        check(lib().omr_ntt_mlp_set_params(self._h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    def forward(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.zeros((X.shape[0], self.n_out), dtype=np.float32)
        check(lib().omr_ntt_mlp_forward(self._h, X.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                        X.shape[0], y.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return y

    def gradients(self, X, Y, M):
        X, Y, M = (np.ascontiguousarray(a, dtype=np.float32) for a in (X, Y, M))
        g = np.zeros(lib().omr_ntt_mlp_param_count(self._h), dtype=np.float32)
        loss = ctypes.c_float()
        f = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        check(lib().omr_ntt_mlp_gradients(self._h, f(X), f(Y), f(M), X.shape[0], f(g), ctypes.byref(loss)))
        return float(loss.value), g

    def fit(self, X, Y, M, epochs=300, batch=64, lr=3e-3, seed=0):
        X, Y, M = (np.ascontiguousarray(a, dtype=np.float32) for a in (X, Y, M))
        hist = np.zeros(epochs, dtype=np.float32)
        f = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        check(lib().omr_ntt_mlp_fit(self._h, f(X), f(Y), f(M), X.shape[0], epochs, batch, lr, seed, f(hist)))
        return hist

    def install(self):
        check(lib().omr_ntt_mlp_install(self._h))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().omr_ntt_mlp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def choose(pred, T):
    """Index of the applicable class with the lowest prediction, per row."""
    masked = np.where(np.isfinite(T), pred, np.inf)
    return masked.argmin(1)


# class layout (tuner.cu): 20 full-transform classes (4 x pass-kernel variant
# + split kind), 4 decomposition classes, 20 fold classes, 20 gather classes
FULL_CLASSES = 20
DECOMP_CLASS = FULL_CLASSES
FOLD_CLASS = DECOMP_CLASS + 4
GATHER_CLASS = FOLD_CLASS + FULL_CLASSES


def heuristic_class(p) -> int:
    """The class the planner picks without database or network (its built-in
    rule, tuner.cu heuristic_full_plan and partial.cu partial_dispatch): two
    passes of short lines at 2^10..2^12, the wide pass where the transform
    splits into 256-point passes only (2^24; batches of 2^16), the cluster
    plan for small or batched 2^13..2^16, else the TMA two-CTA pass on the
    balanced split (32-bit fields) or the slab pass with one more pass
    (Goldilocks); the decomposition for prefixes and index sets of <= 4096
    outputs above 2^20, the fold for strided sets (but for more than 2^16
    outputs of at most 8 cosets), else the full transform and a gather."""
    def full_class(log_n, batch):
        if 10 <= log_n <= 12:
            return 4 * 2 + 2  # two passes of short lines, TMA two-CTA variant
        if log_n < 10:
            return 0  # one launch
        if log_n == 24:
            return 4 * 4 + 2  # wide pass, 256 x 256 x 256 (one pass more than the fewest)
        if log_n == 16 and batch >= 8:
            return 4 * 4 + 0  # wide pass, 256 x 256
        if 13 <= log_n <= 16 and (log_n <= 14 or batch >= 8):
            return 3  # the one-launch cluster plan
        # BabyBear: TMA two CTAs per SM, balanced; Goldilocks: slab, one more pass
        return 4 * 3 + 2 if p["field"] == 1 else 4 * 2 + 0

    full_cls = full_class(p["log_n"], p["batch"])
    n, s = 1 << p["log_n"], point_count(p)
    if s >= n:
        return full_cls
    if p["pattern"] == "strided" and not (p["log_s"] > 16 and p["log_n"] - p["log_s"] <= 3):
        return FOLD_CLASS + full_class(p["log_s"], 1)
    if p["pattern"] in ("contiguous", "random") and s <= 4096 and n // s >= 2 and p["log_n"] > 20:
        return DECOMP_CLASS
    return GATHER_CLASS + full_class(p["log_n"], 1)  # the gather runs one transform at a time


def regret(T, best, choice):
    t = T[np.arange(len(choice)), choice]
    return t / best - 1.0


DATA_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "data")
DEFAULT_NETWORK = os.path.join(DATA_DIR, "planner_mlp.bin")
DEFAULT_DB = os.path.join(DATA_DIR, "planner_full.db")
_default = None


def install_default(path: str = DEFAULT_NETWORK, db: str | None = DEFAULT_DB):
    """Load the network trained on GB300 and make it the planner's learned
    selector (plan = -1 and the partial entry points then use it), and load
    the database of exhaustively tuned full-transform plans (`tune_full`),
    which the planner consults before the network."""
    global _default
    if db and os.path.exists(db):
        n = lib().omr_ntt_planner_load(db.encode())
        if n < 0:
            check(n)
    h = ctypes.c_void_p()
    check(lib().omr_ntt_mlp_load(path.encode(), ctypes.byref(h)))
    check(lib().omr_ntt_mlp_install(h))
    if _default is not None:
        lib().omr_ntt_mlp_destroy(_default)
    _default = h
    return path


def uninstall():
    global _default
    lib().omr_ntt_mlp_install(None)
    if _default is not None:
        lib().omr_ntt_mlp_destroy(_default)
        _default = None
    lib().omr_ntt_planner_clear()


def save_model(path, mlp: Mlp, meta: dict):
    np.savez(path, params=mlp.params(), meta=json.dumps(meta))


def save_weight_file(path, params):
    """The network file the library loads (omr_ntt_mlp_load): "OMRM", uint32
    n_in, n_hidden, n_out, then the float32 parameters (W1 b1 W2 b2 W3 b3)."""
    import struct

    k = (len(params) - (N_FEATURES + 1) * N_HIDDEN - (N_HIDDEN + 1) * N_HIDDEN) // (N_HIDDEN + 1)
    with open(path, "wb") as f:
        f.write(struct.pack("<4sIII", b"OMRM", N_FEATURES, N_HIDDEN, k))
        f.write(np.asarray(params, dtype="<f4").tobytes())


def load_params(path):
    z = np.load(path, allow_pickle=False)
    return z["params"], json.loads(str(z["meta"]))
