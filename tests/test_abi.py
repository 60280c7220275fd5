"""The C-ABI library loads and exports every symbol include/omr_ntt.h
declares; GPU-free entry points behave (no compute call without a GPU)."""
import ctypes
import os
import re

import pytest

import omr_ntt
from omr_ntt import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(omr_ntt_[a-z0-9_]+)\s*\(", src)))


def test_header_symbols_exported():
    L = _lib.lib()
    names = _declared("omr_ntt.h")
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_binding_covers_header():
    """The ctypes binding declares exactly the header's entry points: none
    missing (the Python mirror could not call it) and none extra (a stale
    binding to a symbol the header no longer declares)."""
    names = set(_declared("omr_ntt.h"))
    bound = set(_lib.declared_symbols())
    assert not names - bound, sorted(names - bound)
    assert not bound - names, sorted(bound - names)


def test_encoder_registry_names():
    names = [e.name() for e in omr_ntt.encoders.all(24)]
    assert names == ["ArkRadix2", "LambdaBowers", "WinterfellFourStep", "Plonky3Radix2LayerSplit",
                     "LambdaRadix4", "TfheStockhamRadix8"]
    assert [e.name() for e in omr_ntt.encoders.all(22)][-1] == "LambdaRadix4"
    assert [e.name() for e in omr_ntt.encoders.all_partial(50)] == [
        "DftPartial", "TransformDecomposition", "TransformDecompositionV2"]
    L = _lib.lib()
    assert L.omr_ntt_encoder_name(99) is None
    assert L.omr_ntt_encoder_supports(4, 5) == 0 and L.omr_ntt_encoder_supports(6, 24) == 1


def test_domain_argument_errors_without_gpu():
    L = _lib.lib()
    h = ctypes.c_void_p()
    assert L.omr_ntt_domain_create(7, 10, ctypes.byref(h)) == -1    # unknown field
    assert L.omr_ntt_domain_create(0, 28, ctypes.byref(h)) == -2    # > 2-adicity
    assert L.omr_ntt_domain_create(0, 10, None) == -1
    assert L.omr_ntt_forward(None, -1, None, None, 1, None) == -1
    assert L.omr_ntt_partial(None, 0, 4, None, None, None, None) == -1
    assert b"TWO_ADICITY" in L.omr_ntt_last_error() or L.omr_ntt_last_error()


def test_version():
    assert b"sm_103a" in _lib.lib().omr_ntt_version()
