"""Host-side plan logic, checked on the CPU: the pass records the library
returns (omr_ntt_plan_passes) are emulated exactly (tests/plan_emulator.py
mirrors the tile-pass kernel's index arithmetic) and compared with the
oracle, for every plan of small sizes, forward and inverse, batched."""
import numpy as np
import pytest

import omr_ntt
from omr_ntt.fields import ALL, BabyBear, Goldilocks, TeddyBear
from omr_ntt.inputs import gen_input_seeded
from plan_emulator import emulate_plan


@pytest.mark.parametrize("field", [BabyBear, Goldilocks])
@pytest.mark.parametrize("log_n", list(range(1, 12)))
def test_every_plan_matches_oracle(oracle, field, log_n):
    n = 1 << log_n
    x = gen_input_seeded(field, n, 100 + log_n)
    exp = [int(v) for v in oracle.forward(field.id, x)]
    for plan in range(omr_ntt.plan_count(field, log_n)):
        passes = omr_ntt.plan_passes(field, log_n, plan)
        got = emulate_plan(field, passes, x, log_n)
        assert got == exp, (log_n, plan, omr_ntt.plan_describe(field, log_n, plan))


@pytest.mark.parametrize("field", [BabyBear, Goldilocks])
def test_three_pass_plans(oracle, field):
    for log_n in (13,):
        n = 1 << log_n
        x = gen_input_seeded(field, n, 5)
        exp = [int(v) for v in oracle.forward(field.id, x)]
        for plan in range(omr_ntt.plan_count(field, log_n)):
            passes = omr_ntt.plan_passes(field, log_n, plan)
            assert emulate_plan(field, passes, x, log_n) == exp, plan


@pytest.mark.parametrize("field", ALL)
def test_inverse_and_batch_plans(oracle, field):
    log_n, batch = 6, 3
    n = 1 << log_n
    x = gen_input_seeded(field, n * batch, 9)
    X = [int(v) for v in oracle.forward(field.id, x, batch=batch)]
    for plan in range(omr_ntt.plan_count(field, log_n)):
        passes = omr_ntt.plan_passes(field, log_n, plan, batch=batch)
        assert emulate_plan(field, passes, x, log_n, batch=batch) == X
        back = emulate_plan(field, passes, np.array(X, dtype=object), log_n, inverse=True, batch=batch)
        assert back == [int(v) for v in x]


def test_plan_geometry_large_sizes():
    # 2^24 and 2^27 plans: every pass line fits a tile, products cover N
    for field in (BabyBear, Goldilocks):
        for log_n in (16, 20, 22, 24, 27):
            for plan in range(omr_ntt.plan_count(field, log_n)):
                ps = omr_ntt.plan_passes(field, log_n, plan)
                assert sum(p["logT"] for p in ps) == log_n
                assert all(1 <= p["logT"] <= 12 for p in ps)
                assert ps[0]["in_buf"] == 0 and ps[-1]["out_buf"] == 2


def test_plan_errors():
    with pytest.raises(omr_ntt.OmrNttError):
        omr_ntt.plan_count(BabyBear, 28)  # > TWO_ADICITY
    assert omr_ntt.plan_count(TeddyBear, 30) >= 1


def test_tma_pass_preconditions():
    # the TMA-fed pass needs: column passes with a dense row pitch (es_in ==
    # L_lo) and 16-byte rows; row passes with 16-byte aligned line starts and
    # line lengths; tensor dimensions below 2^32
    for field in (BabyBear, Goldilocks):
        w = field.word_bytes
        for log_n in range(16, 28):
            for plan in range(omr_ntt.plan_count(field, log_n)):
                for batch in (1, 64):
                    for p in omr_ntt.plan_passes(field, log_n, plan, batch):
                        T = 1 << p["logT"]
                        if p["logT"] < 8 or p["twiddle"] == 0 and p["es_in"] != 1:
                            continue
                        if p["is_lo"] == 1:  # column pass
                            if (p["L_lo"] * w) % 16:
                                continue  # fewer than 16 bytes of columns: the plain tile pass runs it
                            assert p["es_in"] == p["L_lo"]
                            assert T * p["L_m"] * p["L_b"] < 2 ** 32
                        else:  # row pass
                            for stride in (p["is_lo"], p["is_m"], p["is_b"]):
                                assert (stride * w) % 16 == 0
                            assert (T * w) % 16 == 0
