"""Device-buffer helpers for the GPU tests (torch is plumbing only)."""
import numpy as np


def to_dev(a: np.ndarray):
    import torch

    signed = a.view(np.int32 if a.dtype == np.uint32 else np.int64)
    return torch.from_numpy(signed.copy()).cuda()


def to_host(t, dtype):
    return t.cpu().numpy().view(dtype)
