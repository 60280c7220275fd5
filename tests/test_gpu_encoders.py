"""The reference's own test matrix (src/lib.rs:24-180), run through the
GPU engine's encoder API: every encoder agrees with the oracle's ArkRadix2,
bit-exact; partial encoders agree on the prefix and leave the rest of buf
untouched; preconditions fail where the reference panics."""
import numpy as np
import pytest

from omr_ntt import NttDomain, OmrNttError, encoders
from omr_ntt.encoders import (ArkRadix2, Dft, DftPartial, LambdaBowers, LambdaRadix4,
                              Plonky3Radix2LayerSplit, TfheStockhamRadix8, TransformDecomposition,
                              TransformDecompositionV2, WinterfellFourStep)
from omr_ntt.fields import BabyBear, DefaultField, Goldilocks
from omr_ntt.inputs import gen_input_seeded
from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu

POWERS_OF_TWO = [2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192, 16384, 32768, 65536]
EVEN_POWERS_OF_TWO = [4, 16, 64, 256, 1024, 4096, 16384, 65536]
POWERS_OF_TWO_DIV_BY_3 = [8, 64, 512, 4096, 32768]


def assert_agrees_with_ark(oracle, encoder, sizes, field=DefaultField):
    for n in sizes:
        domain = NttDomain(field, n)
        inp = gen_input_seeded(field, n, n + 17)
        expected = oracle.ntt(field.id, inp, "ArkRadix2")
        actual = inp.copy()
        encoder.ntt(actual, domain)
        assert np.array_equal(expected, actual), f"{encoder.name()}: ntt mismatch at N={n}"


def assert_prefix_agrees_with_ark(oracle, encoder, s, cases, field=DefaultField):
    for n in cases:
        m = min(2 * s, n)
        domain = NttDomain(field, n)
        inp = gen_input_seeded(field, n, 3 * n + s)
        expected = oracle.ntt(field.id, inp, "ArkRadix2")
        actual = inp.copy()
        encoder.ntt(actual, domain)
        assert np.array_equal(actual[:m], expected[:m]), f"{encoder.name()}: first {m} outputs at N={n}"
        assert np.array_equal(actual[m:], inp[m:]), "partial encoder touched buf[m..]"


def test_dft_agrees_with_ark(oracle):
    assert_agrees_with_ark(oracle, Dft(), [64, 128, 256])


@pytest.mark.parametrize("enc,sizes", [
    (LambdaBowers(), POWERS_OF_TWO),
    (WinterfellFourStep(), POWERS_OF_TWO),
    (Plonky3Radix2LayerSplit(), POWERS_OF_TWO),
    (LambdaRadix4(), EVEN_POWERS_OF_TWO),
    (TfheStockhamRadix8(), POWERS_OF_TWO_DIV_BY_3),
    (ArkRadix2(), POWERS_OF_TWO),
], ids=lambda v: v.name() if hasattr(v, "name") else "sizes")
def test_encoder_agrees_with_ark(oracle, enc, sizes):
    assert_agrees_with_ark(oracle, enc, sizes)


def test_encoders_goldilocks(oracle):
    for enc in encoders.all(12):
        assert_agrees_with_ark(oracle, enc, [4096], Goldilocks)


def test_all_registry_at_2_24(oracle):
    n = 1 << 24
    domain = NttDomain(BabyBear, n)
    inp = gen_input_seeded(BabyBear, n, 42)
    expected = oracle.ntt(BabyBear.id, inp, "ArkRadix2")
    xd = to_dev(inp)
    for enc in encoders.all(24):
        buf = xd.clone()
        enc.ntt(buf, domain)
        assert np.array_equal(to_host(buf, BabyBear.dtype), expected), enc.name()


FAMILY = {"WinterfellFourStep": "slab", "Plonky3Radix2LayerSplit": "tma2buf",
          "LambdaBowers": "wide", "LambdaRadix4": "tma2cta", "TfheStockhamRadix8": "tile"}


@pytest.mark.parametrize("field", [BabyBear, Goldilocks], ids=lambda f: f.name)
def test_encoder_plan_families_agree(oracle, field):
    """Each reference algorithm runs its own plan family (its structure in
    engine plans) and every family gives the oracle's words."""
    import omr_ntt

    for log_n in (16, 18, 20, 21, 22, 24):
        n = 1 << log_n
        domain = NttDomain(field, n)
        inp = gen_input_seeded(field, n, 100 + log_n)
        expected = oracle.forward(field.id, inp)
        xd = to_dev(inp)
        for enc in (WinterfellFourStep(), Plonky3Radix2LayerSplit(), LambdaBowers(), LambdaRadix4(),
                    TfheStockhamRadix8()):
            if not enc.supports(log_n):
                continue
            name = omr_ntt.plan_describe(field, log_n, enc.plan(field, log_n))
            # LambdaBowers has a wide plan where a split has a 256-point pass
            if enc.name() != "LambdaBowers" or log_n in (16, 20, 22, 24):
                assert FAMILY[enc.name()] in name, (enc.name(), log_n, name)
            buf = xd.clone()
            enc.ntt(buf, domain)
            assert np.array_equal(to_host(buf, field.dtype), expected), (enc.name(), log_n, name)


@pytest.mark.parametrize("s", [2, 4, 8, 16, 50])
def test_dft_partial_agrees_with_ark(oracle, s):
    assert_prefix_agrees_with_ark(oracle, DftPartial(s), s, [64, 128, 256])


@pytest.mark.parametrize("s", [2, 4, 8, 16, 50])
def test_transform_decomposition_agrees_with_ark(oracle, s):
    assert_prefix_agrees_with_ark(oracle, TransformDecomposition(s), s, POWERS_OF_TWO)


@pytest.mark.parametrize("s", [2, 4, 8, 16, 50])
def test_transform_decomposition_v2_agrees_with_ark(oracle, s):
    assert_prefix_agrees_with_ark(oracle, TransformDecompositionV2(s), s, [1024, 4096, 32768, 65536])


def test_transform_decomposition_large_n(oracle):
    # src/lib.rs:167-180 (the reference marks it slow/ignored; here it runs)
    for s in [1, 2, 3, 50, 101, 16383, 16384]:
        assert_prefix_agrees_with_ark(oracle, TransformDecomposition(s), s,
                                      [1 << 14, 1 << 15, 1 << 22])


def test_partial_s_zero_leaves_buf(oracle):
    n = 1024
    d = NttDomain(BabyBear, n)
    x = gen_input_seeded(BabyBear, n, 2)
    y = x.copy()
    TransformDecomposition(0).ntt(y, d)
    assert np.array_equal(x, y)


def test_preconditions_raise():
    d = NttDomain(BabyBear, 1 << 5)
    buf = gen_input_seeded(BabyBear, 1 << 5, 1)
    with pytest.raises(OmrNttError):
        LambdaRadix4().ntt(buf, d)  # reference: assert log_N % 2 == 0
    with pytest.raises(OmrNttError):
        TfheStockhamRadix8().ntt(buf, d)  # reference: assert log_N % 3 == 0


def test_domain_tables_match_reference_definition():
    n = 1 << 10
    d = NttDomain(BabyBear, n)
    p = BabyBear.p
    assert d.omega == BabyBear.root_of_unity(10)
    tw = [int(v) for v in d.twiddles]
    assert tw == [pow(d.omega, k, p) for k in range(n)]
    br = [int(v) for v in d.bitrev_twiddles]
    rev = lambda i: int(format(i, "09b")[::-1], 2)
    assert br == [tw[rev(i)] for i in range(n // 2)]


def test_encode_host_batches_pipelined(oracle):
    """encode_host on a batch of host transforms (pipelined chunks): a full
    encoder and a partial one, each transform against the oracle."""
    f, log_n, batch = BabyBear, 18, 6
    n = 1 << log_n
    d = NttDomain(f, n)
    x = gen_input_seeded(f, n * batch, 808)
    full = oracle.forward(f.id, x, batch=batch).reshape(batch, n)
    y = x.copy()
    WinterfellFourStep().ntt(y, d, batch=batch)
    assert np.array_equal(y.reshape(batch, n), full)
    s = 50
    z = x.copy()
    TransformDecomposition(s).ntt(z, d, batch=batch)
    assert np.array_equal(z.reshape(batch, n)[:, :2 * s], full[:, :2 * s])
