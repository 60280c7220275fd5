"""Planner surface without a GPU: candidate enumeration per planning point and
the persisted planner database."""
import ctypes
import os

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
    rnd = cands(BabyBear, 20, 2, 100)
    assert all(s == 3 for s, _ in rnd)
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
