"""CPU oracle for the GB300 NTT engine -- TEST INFRASTRUCTURE ONLY.

Only the tests, the smoke check and the CPU-baseline leg of ``bench.py`` may
import this module, and only as the checker (or as the timed CPU baseline).
The product library never routes through it.

It wraps ``oracle/_build/libntt_oracle.so`` (``oracle/ntt_oracle.c``), a plain-C
restatement of every encoder of the reference crate benbencik/omr-ntt:

    ArkRadix2 (src/encoders/ark_radix2.rs:12-19)
    Dft, DftPartial (src/encoders/dft.rs:9-89)
    LambdaBowers (src/encoders/lambdaworks_bowers.rs:13-173)
    LambdaRadix4 (src/encoders/lambdaworks_radix4.rs:14-75)
    Plonky3Radix2LayerSplit (src/encoders/plonky3_radix2_layer_split.rs:18-97)
    TfheStockhamRadix8 (src/encoders/tfhe_stockham_radix8.rs:15-140)
    TransformDecomposition (src/encoders/transform_decomposition.rs:10-97)
    TransformDecompositionV2 (src/encoders/transform_decomposition_v2.rs:8-100)
    WinterfellFourStep (src/encoders/winterfell_four_step.rs:19-130)

plus an inverse NTT and partial-output gathers that the reference lacks.

Parity pinning: the reference (Rust) cannot run here and its tests hold no
golden vectors; the oracle is pinned to the reference's agreement matrix
(src/lib.rs) and to independent big-integer DFT fixtures (tests/golden/).  The
absolute root of unity follows ark-ff's convention; beyond that, parity with
the reference's own outputs is unpinned.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libntt_oracle.so")
# compiler flags of the build (reported beside the timed CPU baseline)
BUILD_FLAGS = "gcc -O3 -fopenmp"

BABYBEAR, GOLDILOCKS, KOALABEAR, TEDDYBEAR = 0, 1, 2, 3
FIELDS = {
    "BabyBear": BABYBEAR,
    "Goldilocks": GOLDILOCKS,
    "KoalaBear": KOALABEAR,
    "TeddyBear": TEDDYBEAR,
}
MODULUS = {
    BABYBEAR: 2013265921,
    GOLDILOCKS: 18446744069414584321,
    KOALABEAR: 2130706433,
    TEDDYBEAR: 3221225473,
}
TWO_ADICITY = {BABYBEAR: 27, GOLDILOCKS: 32, KOALABEAR: 24, TEDDYBEAR: 30}
GENERATOR = {BABYBEAR: 31, GOLDILOCKS: 7, KOALABEAR: 3, TEDDYBEAR: 5}
DTYPE = {BABYBEAR: np.uint32, GOLDILOCKS: np.uint64, KOALABEAR: np.uint32, TEDDYBEAR: np.uint32}

ENCODERS = {
    "ArkRadix2": 0,
    "Dft": 1,
    "DftPartial": 2,
    "LambdaBowers": 3,
    "LambdaRadix4": 4,
    "Plonky3Radix2LayerSplit": 5,
    "TfheStockhamRadix8": 6,
    "TransformDecomposition": 7,
    "TransformDecompositionV2": 8,
    "WinterfellFourStep": 9,
}
PARTIAL_ENCODERS = ("DftPartial", "TransformDecomposition", "TransformDecompositionV2")

_lib = None


def field_id(field) -> int:
    return FIELDS[field] if isinstance(field, str) else int(field)


def build() -> str:
    """Compile the oracle library with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_ntt.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64]
        L.oracle_ntt.restype = ctypes.c_int
        L.oracle_ntt_batch.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_uint32,
                                       ctypes.c_uint64, ctypes.c_uint64]
        L.oracle_ntt_batch.restype = ctypes.c_int
        L.oracle_inverse.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_uint32]
        L.oracle_inverse.restype = ctypes.c_int
        L.oracle_root_of_unity.argtypes = [ctypes.c_int, ctypes.c_uint32]
        L.oracle_root_of_unity.restype = ctypes.c_uint64
        L.oracle_mul.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64]
        L.oracle_mul.restype = ctypes.c_uint64
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_set_threads.restype = ctypes.c_int
        L.oracle_get_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def set_threads(n: int) -> int:
    return lib().oracle_set_threads(int(n))


def get_threads() -> int:
    return lib().oracle_get_threads()


def root_of_unity(field, log_n: int) -> int:
    return int(lib().oracle_root_of_unity(field_id(field), log_n))


def mul(field, a: int, b: int) -> int:
    return int(lib().oracle_mul(field_id(field), a, b))


def _check(rc: int, what: str):
    if rc != 0:
        raise ValueError(f"oracle {what} failed with status {rc}")


def _prep(field, x):
    f = field_id(field)
    a = np.ascontiguousarray(np.array(x, dtype=DTYPE[f], copy=True))
    return f, a


def ntt(field, x, encoder: str = "ArkRadix2", s: int = 0, batch: int = 1):
    """Return ``encoder.ntt`` applied to a copy of ``x`` (the reference's
    in-place ``NttEncoder::ntt``).  ``x`` holds ``batch`` transforms of
    N = len(x) / batch canonical words each.  Partial encoders leave entries
    past ``min(2s, N)`` unspecified, as the reference does."""
    f, a = _prep(field, x)
    n = a.size // batch
    if n & (n - 1) or n * batch != a.size:
        raise ValueError("length must be batch * a power of two")
    log_n = n.bit_length() - 1
    rc = lib().oracle_ntt_batch(f, ENCODERS[encoder], a.ctypes.data, log_n, int(s), int(batch))
    _check(rc, encoder)
    return a


def forward(field, x, batch: int = 1):
    return ntt(field, x, "ArkRadix2", batch=batch)


def inverse(field, x, batch: int = 1):
    f, a = _prep(field, x)
    n = a.size // batch
    log_n = n.bit_length() - 1
    for b in range(batch):
        view = a[b * n:(b + 1) * n]
        _check(lib().oracle_inverse(f, view.ctypes.data, log_n), "inverse")
    return a


def partial(field, x, indices):
    """Outputs X[indices] of the full forward transform (the index-set
    partial transform has no reference path; its oracle is a gather from the
    full transform)."""
    full = forward(field, x)
    return full[np.asarray(indices, dtype=np.int64)]


def prefix(field, x, s: int, encoder: str = "TransformDecomposition"):
    """The reference's partial-output semantics: the first min(2s, N) outputs
    computed by one of the reference's partial encoders."""
    a = ntt(field, x, encoder, s=s)
    m = min(2 * s, a.size)
    return a[:m]
