"""The reference's encoder registry (src/encoders/mod.rs) over the GPU engine.

Each class keeps the reference encoder's name, constructor and ``ntt`` /
``name`` methods (src/encoder.rs:70-74).  All of them compute the same
natural-order transform on the GPU (the id selects the plan family); the
partial encoders write only ``buf[..min(2s, N)]`` as the reference does.
Preconditions raise ``OmrNttError`` (status PRECONDITION) where the
reference panics (src/encoders/lambdaworks_radix4.rs:17-21,
src/encoders/tfhe_stockham_radix8.rs:17-21).
"""
from __future__ import annotations

import ctypes

from ._lib import check, lib

ARK_RADIX2, DFT, DFT_PARTIAL, LAMBDA_BOWERS, LAMBDA_RADIX4 = 0, 1, 2, 3, 4
PLONKY3_LAYER_SPLIT, TFHE_STOCKHAM_R8, TRANSFORM_DECOMPOSITION = 5, 6, 7
TRANSFORM_DECOMPOSITION_V2, WINTERFELL_FOUR_STEP = 8, 9


class NttEncoder:
    """trait NttEncoder<F> (src/encoder.rs:70-74)."""

    ID = -1
    s = 0

    def ntt(self, buf, domain, batch: int = 1, stream=None):
        """In-place forward NTT of ``buf`` (NumPy array or CUDA tensor)."""
        L = lib()
        if hasattr(buf, "data_ptr") and hasattr(buf, "is_cuda"):
            import torch

            st = stream if stream is not None else torch.cuda.current_stream(buf.device).cuda_stream
            check(L.omr_ntt_encode(domain.handle, self.ID, self.s, ctypes.c_void_p(buf.data_ptr()),
                                   batch, ctypes.c_void_p(int(st))))
            return buf
        if not buf.flags["C_CONTIGUOUS"] or buf.dtype != domain.field.dtype:
            raise TypeError("buf must be a C-contiguous array of the field's word type")
        check(L.omr_ntt_encode_host(domain.handle, self.ID, self.s, buf.ctypes.data, batch))
        return buf

    def name(self) -> str:
        return lib().omr_ntt_encoder_name(self.ID).decode()

    def supports(self, log_n: int) -> bool:
        return bool(lib().omr_ntt_encoder_supports(self.ID, log_n))

    def plan(self, field, log_n: int) -> int:
        """The engine plan this (full) encoder runs at 2^log_n: the plan
        family with the structure of the reference algorithm."""
        rc = lib().omr_ntt_encoder_plan(self.ID, field.id, log_n)
        if rc < 0:
            check(rc)
        return rc

    def __repr__(self):
        return self.name() if self.s == 0 else f"{self.name()}({self.s})"


class ArkRadix2(NttEncoder):
    ID = ARK_RADIX2


class Dft(NttEncoder):
    ID = DFT


class LambdaBowers(NttEncoder):
    ID = LAMBDA_BOWERS


class LambdaRadix4(NttEncoder):
    ID = LAMBDA_RADIX4


class Plonky3Radix2LayerSplit(NttEncoder):
    ID = PLONKY3_LAYER_SPLIT


class TfheStockhamRadix8(NttEncoder):
    ID = TFHE_STOCKHAM_R8


class WinterfellFourStep(NttEncoder):
    ID = WINTERFELL_FOUR_STEP


class _Partial(NttEncoder):
    def __init__(self, s: int):
        self.s = int(s)


class DftPartial(_Partial):
    ID = DFT_PARTIAL


class TransformDecomposition(_Partial):
    ID = TRANSFORM_DECOMPOSITION


class TransformDecompositionV2(_Partial):
    ID = TRANSFORM_DECOMPOSITION_V2


def all(log_n: int):  # noqa: A001  (mirrors encoders::all)
    """encoders::all(log_n) (src/encoders/mod.rs:32-46)."""
    v = [ArkRadix2(), LambdaBowers(), WinterfellFourStep(), Plonky3Radix2LayerSplit()]
    if log_n % 2 == 0:
        v.append(LambdaRadix4())
    if log_n % 3 == 0:
        v.append(TfheStockhamRadix8())
    return v


def all_partial(s: int):
    """encoders::all_partial(s) (src/encoders/mod.rs:48-54)."""
    return [DftPartial(s), TransformDecomposition(s), TransformDecompositionV2(s)]
