"""CPU oracle checks (no GPU): golden vectors, then the reference's own test
matrix (src/lib.rs:83-180) restated over the oracle's encoders."""
import json
import os

import numpy as np
import pytest

from omr_ntt.fields import ALL, BabyBear, Goldilocks, field_by_name
from omr_ntt.inputs import gen_input_seeded

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))

POWERS_OF_TWO = [2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192, 16384, 32768, 65536]
EVEN_POWERS_OF_TWO = [4, 16, 64, 256, 1024, 4096, 16384, 65536]
POWERS_OF_TWO_DIV_BY_3 = [8, 64, 512, 4096, 32768]


@pytest.mark.parametrize("fname", [f.name for f in ALL])
def test_roots_match_golden(oracle, fname):
    g = GOLDEN["fields"][fname]
    f = field_by_name(fname)
    for log_n, w in g["roots"].items():
        log_n = int(log_n)
        assert oracle.root_of_unity(f.id, log_n) == w
        assert f.root_of_unity(log_n) == w
        # omega^N = 1 and omega^(N/2) = -1 (primitive)
        assert pow(w, 1 << log_n, f.p) == 1
        if log_n:
            assert pow(w, 1 << (log_n - 1), f.p) == f.p - 1


def test_two_adic_generators_pinned():
    # 2^27-th root of BabyBear and 2^32-th root of Goldilocks under the
    # GEN^((p-1) >> TWO_ADICITY) convention
    assert BabyBear.root_of_unity(27) == 0x1A427A41
    assert Goldilocks.root_of_unity(32) == 0x185629DCDA58878C


@pytest.mark.parametrize("fname", [f.name for f in ALL])
@pytest.mark.parametrize("encoder", ["ArkRadix2", "Dft", "LambdaBowers", "WinterfellFourStep",
                                     "Plonky3Radix2LayerSplit"])
def test_oracle_against_golden(oracle, fname, encoder):
    f = field_by_name(fname)
    for case in GOLDEN["fields"][fname]["cases"]:
        x = np.array(case["x"], dtype=f.dtype)
        if case["log_n"] == 0 and encoder == "WinterfellFourStep":
            continue  # the reference's fft_in_place indexes out of bounds at N=1
        got = oracle.ntt(f.id, x, encoder)
        assert [int(v) for v in got] == case["X"], (encoder, case["log_n"])
        back = oracle.inverse(f.id, got)
        assert [int(v) for v in back] == case["x"]


@pytest.mark.parametrize("fname", [f.name for f in ALL])
def test_golden_inputs_reproducible(fname):
    f = field_by_name(fname)
    for case in GOLDEN["fields"][fname]["cases"]:
        x = gen_input_seeded(f, 1 << case["log_n"], case["seed"])
        assert [int(v) for v in x] == case["x"]


# ---- src/lib.rs:83-88  dft_agrees_with_ark
def test_dft_agrees_with_ark(oracle):
    for n in [64, 128, 256]:
        x = gen_input_seeded(BabyBear, n, n)
        assert np.array_equal(oracle.ntt(0, x, "Dft"), oracle.ntt(0, x, "ArkRadix2"))


# ---- src/lib.rs:90-112  ntt_linearity
def test_ntt_linearity(oracle):
    p = BabyBear.p
    n = 32
    x = gen_input_seeded(BabyBear, n, 1).astype(object)
    y = gen_input_seeded(BabyBear, n, 2).astype(object)
    a, b = 123456789, 987654321
    xy = np.array([(a * xi + b * yi) % p for xi, yi in zip(x, y)], dtype=np.uint32)
    nx = oracle.ntt(0, x.astype(np.uint32), "Dft").astype(object)
    ny = oracle.ntt(0, y.astype(np.uint32), "Dft").astype(object)
    comb = [(a * u + b * v) % p for u, v in zip(nx, ny)]
    assert [int(v) for v in oracle.ntt(0, xy, "Dft")] == comb


def _agrees(oracle, field, encoder, sizes):
    for n in sizes:
        x = gen_input_seeded(field, n, 7 * n + 1)
        exp = oracle.ntt(field.id, x, "ArkRadix2")
        got = oracle.ntt(field.id, x, encoder)
        assert np.array_equal(exp, got), f"{encoder}: ntt mismatch at N={n}"


# ---- src/lib.rs:114-139
@pytest.mark.parametrize("encoder,sizes", [
    ("LambdaBowers", POWERS_OF_TWO),
    ("WinterfellFourStep", POWERS_OF_TWO),
    ("Plonky3Radix2LayerSplit", POWERS_OF_TWO),
    ("LambdaRadix4", EVEN_POWERS_OF_TWO),
    ("TfheStockhamRadix8", POWERS_OF_TWO_DIV_BY_3),
])
def test_encoder_agrees_with_ark(oracle, encoder, sizes):
    _agrees(oracle, BabyBear, encoder, sizes)


@pytest.mark.parametrize("field", [Goldilocks] + [f for f in ALL if f.name in ("KoalaBear", "TeddyBear")])
@pytest.mark.parametrize("encoder", ["LambdaBowers", "WinterfellFourStep", "Plonky3Radix2LayerSplit",
                                     "LambdaRadix4", "TfheStockhamRadix8"])
def test_encoder_agrees_with_ark_other_fields(oracle, field, encoder):
    sizes = {"LambdaRadix4": [4, 64, 1024, 16384], "TfheStockhamRadix8": [8, 512, 4096]}.get(
        encoder, [2, 8, 32, 256, 2048, 16384])
    _agrees(oracle, field, encoder, sizes)


def _prefix(oracle, encoder, s, sizes, field=BabyBear):
    for n in sizes:
        m = min(2 * s, n)
        x = gen_input_seeded(field, n, 3 * n + s)
        exp = oracle.ntt(field.id, x, "ArkRadix2")[:m]
        got = oracle.ntt(field.id, x, encoder, s=s)[:m]
        assert np.array_equal(exp, got), f"{encoder}: first {m} outputs mismatch at N={n}"


# ---- src/lib.rs:141-165
@pytest.mark.parametrize("s", [2, 4, 8, 16, 50])
def test_partial_encoders_agree_with_ark(oracle, s):
    _prefix(oracle, "DftPartial", s, [64, 128, 256])
    _prefix(oracle, "TransformDecomposition", s, POWERS_OF_TWO)
    _prefix(oracle, "TransformDecompositionV2", s, [1024, 4096, 32768, 65536])


def test_partial_encoders_goldilocks(oracle):
    for s in [2, 50]:
        _prefix(oracle, "TransformDecomposition", s, [64, 4096], Goldilocks)
        _prefix(oracle, "TransformDecompositionV2", s, [1024, 4096], Goldilocks)


def test_partial_s_zero_is_noop(oracle):
    x = gen_input_seeded(BabyBear, 256, 5)
    for enc in ("DftPartial", "TransformDecomposition", "TransformDecompositionV2"):
        assert np.array_equal(oracle.ntt(0, x, enc, s=0), x)


def test_oracle_preconditions(oracle):
    x = gen_input_seeded(BabyBear, 8, 1)
    with pytest.raises(ValueError):
        oracle.ntt(0, x, "LambdaRadix4")  # log N = 3 is odd
    x = gen_input_seeded(BabyBear, 16, 1)
    with pytest.raises(ValueError):
        oracle.ntt(0, x, "TfheStockhamRadix8")  # log N = 4 not divisible by 3


def test_oracle_batch_and_inverse(oracle):
    for f in ALL:
        x = gen_input_seeded(f, 4 * 1024, 11)
        X = oracle.forward(f.id, x, batch=4)
        for b in range(4):
            assert np.array_equal(X[b * 1024:(b + 1) * 1024], oracle.forward(f.id, x[b * 1024:(b + 1) * 1024]))
        assert np.array_equal(oracle.inverse(f.id, X, batch=4), x)
