"""Planner surface without a GPU: candidate enumeration per planning point and
the persisted planner database."""
import ctypes
import os

import omr_ntt
from omr_ntt import _lib
from omr_ntt.fields import BabyBear, Goldilocks

L = _lib.lib()


def cands(field, log_n, pattern, count):
    n = L.omr_ntt_candidates(field.id, log_n, pattern, count, None, None, 0)
    st = (ctypes.c_int * n)()
    pa = (ctypes.c_int * n)()
    assert L.omr_ntt_candidates(field.id, log_n, pattern, count, st, pa, n) == n
    return list(zip(st, pa))


def test_candidate_families():
    full = cands(BabyBear, 24, 0, 1 << 24)
    assert full and all(s == 0 for s, _ in full)
    pre = cands(BabyBear, 22, 0, 64)
    assert (1, 6) in pre and (1, 12) in pre and any(s == 3 for s, _ in pre)
    strided = cands(Goldilocks, 22, 1, 1024)
    assert any(s == 2 for s, _ in strided) and any(s == 3 for s, _ in strided)
    rnd = cands(BabyBear, 20, 2, 100)  # index sets: the decomposition, or full + gather
    assert (1, 7) in rnd and (1, 12) in rnd and any(s == 3 for s, _ in rnd)
    assert all(s in (1, 3) for s, _ in rnd)
    # the planning space of the learned selector: tens of plans per point
    assert 10 <= len(pre) <= 60


def test_planner_db_roundtrip(tmp_path):
    L.omr_ntt_planner_clear()
    assert L.omr_ntt_planner_set(0, 20, 64, -1, 0, 0, 3) == 0
    assert L.omr_ntt_planner_set(1, 22, 1, 0, 256, 1, 9) == 0
    s, p = ctypes.c_int(), ctypes.c_int()
    assert L.omr_ntt_planner_get(0, 20, 60, -1, 0, ctypes.byref(s), ctypes.byref(p)) == 1  # 60 -> bucket 64
    assert (s.value, p.value) == (0, 3)
    path = str(tmp_path / "db.txt").encode()
    assert L.omr_ntt_planner_save(path) == 0
    L.omr_ntt_planner_clear()
    assert L.omr_ntt_planner_get(1, 22, 1, 0, 256, ctypes.byref(s), ctypes.byref(p)) == 0
    assert L.omr_ntt_planner_load(path) == 2
    assert L.omr_ntt_planner_get(1, 22, 1, 0, 256, ctypes.byref(s), ctypes.byref(p)) == 1
    assert (s.value, p.value) == (1, 9)
    L.omr_ntt_planner_clear()


def test_encoder_plan_families_are_distinct():
    """The reference's full encoders map to distinct engine plan families
    (no GPU needed): at 2^24 five different plans, each named for its family."""
    import omr_ntt
    from omr_ntt import encoders as E

    fams = {"WinterfellFourStep": "4096x4096 slab", "Plonky3Radix2LayerSplit": "4096x4096 tma2buf",
            "LambdaBowers": "256x256x256 wide", "LambdaRadix4": "4096x4096 tma2cta",
            "TfheStockhamRadix8": "4096x4096 tile"}
    plans = {}
    for enc in (E.WinterfellFourStep(), E.Plonky3Radix2LayerSplit(), E.LambdaBowers(), E.LambdaRadix4(),
                E.TfheStockhamRadix8()):
        p = enc.plan(BabyBear, 24)
        assert omr_ntt.plan_describe(BabyBear, 24, p).endswith(fams[enc.name()]), enc.name()
        plans[enc.name()] = p
    assert len(set(plans.values())) == 5
    # the radix-4 family keeps to even-length passes where the balanced split is odd
    assert omr_ntt.plan_describe(BabyBear, 22, E.LambdaRadix4().plan(BabyBear, 22)).endswith("1024x4096 tma2cta")
    # one-pass sizes and the partial encoders
    assert E.WinterfellFourStep().plan(BabyBear, 12) == E.ArkRadix2().plan(BabyBear, 12)
    assert L.omr_ntt_encoder_plan(7, 0, 20) < 0 and L.omr_ntt_encoder_plan(4, 0, 21) < 0


def test_shipped_full_transform_db():
    """The database of exhaustively tuned full-transform plans that
    planner.install_default() loads: one entry per field, log2 N in [6, 24]
    and batch in (1, 8, 64, 512) within 2^26 words, each a valid plan id of
    its size (the wide 256^3 plan at 2^24 for both fields)."""
    from omr_ntt import planner
    from omr_ntt.tune_full import shapes

    L.omr_ntt_planner_clear()
    try:
        n = L.omr_ntt_planner_load(planner.DEFAULT_DB.encode())
        want = list(shapes(6, 24))
        assert n == len(want) == 256
        s, p = ctypes.c_int(), ctypes.c_int()
        for f, log_n, batch in want:
            assert L.omr_ntt_planner_get(f.id, log_n, batch, -1, 0, ctypes.byref(s), ctypes.byref(p)) == 1
            assert s.value == 0 and 0 <= p.value < omr_ntt.plan_count(f, log_n), (f.name, log_n, batch)
        for f in (BabyBear, Goldilocks):
            assert L.omr_ntt_planner_get(f.id, 24, 1, -1, 0, ctypes.byref(s), ctypes.byref(p)) == 1
            assert omr_ntt.plan_describe(f, 24, p.value) == "four-step 256x256x256 wide"
    finally:
        L.omr_ntt_planner_clear()
