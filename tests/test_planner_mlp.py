"""What the learned planner gains (no GPU needed): the committed network
(omr-ntt_gb300/data/planner_mlp.npz, trained on GB300 by the library's own
kernels on 1500 autotuned planning points) is evaluated with the CPU
reference forward pass on the 500 held-out points of the committed dataset.
Its choices must stay within 5% of the exhaustive autotuner's optimum on
average and beat the planner's built-in rule (the method without the
network)."""
import json
import os

import numpy as np

from omr_ntt import planner as P
from oracle import mlp_ref

DATA = P.DATA_DIR


def _load():
    z = np.load(os.path.join(DATA, "planner_dataset.npz"))
    params, meta = P.load_params(os.path.join(DATA, "planner_mlp.npz"))
    pts = json.loads(str(z["points"]))
    return z["X"], z["T"].astype(np.float64), z["best"].astype(np.float64), pts, params, meta


def test_dataset_shape():
    X, T, best, pts, params, meta = _load()
    assert X.shape == (2000, P.N_FEATURES) and T.shape[0] == 2000 and len(pts) == 2000
    assert np.all(np.nanmin(T, 1) >= best - 1e-6)  # the exhaustive best bounds every class
    assert meta["summary"]["train"] == 1500


def test_held_out_regret_within_5pct_and_beats_builtin_rule():
    X, T, best, pts, params, meta = _load()
    k = T.shape[1]
    te = slice(1500, 2000)
    pred = mlp_ref.forward(params, X[te], P.N_FEATURES, P.N_HIDDEN, k)
    r_net = P.regret(T[te], best[te], P.choose(pred, T[te]))
    r_rule = P.regret(T[te], best[te], np.array([P.heuristic_class(p) for p in pts[1500:]]))
    assert np.isfinite(r_net).all()
    assert r_net.mean() <= 0.05, r_net.mean()
    assert r_net.mean() < r_rule.mean()
    assert np.median(r_net) <= np.median(r_rule)


def test_weight_file_matches_npz():
    import struct

    params, _ = P.load_params(os.path.join(DATA, "planner_mlp.npz"))
    raw = open(os.path.join(DATA, "planner_mlp.bin"), "rb").read()
    magic, n_in, n_h, n_out = struct.unpack("<4sIII", raw[:16])
    assert magic == b"OMRM" and (n_in, n_h) == (P.N_FEATURES, P.N_HIDDEN)
    assert np.array_equal(np.frombuffer(raw[16:], dtype="<f4"), params.astype("<f4"))
