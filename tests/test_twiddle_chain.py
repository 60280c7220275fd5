"""The four-step twiddle as the kernels form it, at full sizes (CPU).

The tile rounds (csrc/ntt_pass.cuh do_round, csrc/ntt_pass_tma.cuh
tma_round) give output k = d + q NS of a butterfly group the twiddle
omega_N^(line k scale) as base * step^q, with base = omega_N^(ls d) and
step = omega_N^(ls NS), ls = line * scale, all index products in 32-bit
arithmetic masked to N - 1.  This checks that exponent identity for every
twiddled pass of every plan up to each field's largest size, where the 32-bit
products wrap; the GPU parity tests check the words at the sizes they run.
"""
import random

import pytest

import omr_ntt
from omr_ntt.fields import BabyBear, Goldilocks, KoalaBear, TeddyBear

M32 = 0xFFFFFFFF


def _round_plan(log_t, maxr=4):
    rounds = (log_t + maxr - 1) // maxr
    logr = [log_t // rounds + (1 if i < log_t % rounds else 0) for i in range(rounds)]
    return [(logr[i], sum(logr[:i])) for i in range(rounds)]


@pytest.mark.parametrize("field,log_n", [(BabyBear, 24), (BabyBear, 27), (KoalaBear, 24),
                                         (TeddyBear, 30), (Goldilocks, 24), (Goldilocks, 32)])
def test_chain_exponent_matches_direct(field, log_n):
    rng = random.Random(log_n * 7 + field.id)
    N = 1 << log_n
    checked = 0
    for plan in range(omr_ntt.plan_count(field, log_n)):
        for pd in omr_ntt.plan_passes(field, log_n, plan, 1):
            if not pd["twiddle"]:
                continue
            T = 1 << pd["logT"]
            logr, logns = _round_plan(pd["logT"])[-1]  # the last round stores
            R, NS = 1 << logr, 1 << logns
            for _ in range(64):
                line = rng.randrange(pd["L_lo"]) + rng.randrange(pd["L_m"]) * pd["tw_line_mul_m"]
                j = rng.randrange(T // R)
                d = ((j >> logns) << (logns + logr)) | (j & (NS - 1))
                ls = (line * pd["tw_scale"]) & M32
                eb = ((ls * d) & M32) & (N - 1)
                es = ((ls * NS) & M32) & (N - 1)
                for q in range(R):
                    k = d + q * NS
                    assert k < T
                    assert (eb + q * es) % N == (line * k * pd["tw_scale"]) % N
                checked += 1
    assert checked > 0
