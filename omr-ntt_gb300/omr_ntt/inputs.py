"""Seeded synthetic inputs.

The reference draws inputs with rand's SmallRng::seed_from_u64 + ark-ff's
F::rand (benches/common/mod.rs:54-57), which cannot be reproduced outside
Rust.  This engine's benches and tests use a documented generator instead:
the splitmix64 stream of `seed`, rejection-sampled into [0, p) (the top 32
bits of each draw for the 32-bit fields, the whole draw for Goldilocks).
Both the GPU path and the oracle consume the same arrays, so parity is
"same inputs in, same words out".
"""
from __future__ import annotations

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, start: int, count: int) -> np.ndarray:
    """Outputs start .. start+count-1 of splitmix64 seeded with `seed`."""
    with np.errstate(over="ignore"):
        i = np.arange(start + 1, start + count + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + i * _GAMMA
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def gen_input_seeded(field, n: int, seed: int) -> np.ndarray:
    """n canonical words of `field`, uniform in [0, p), from `seed`."""
    out = np.empty(n, dtype=field.dtype)
    filled, pos = 0, 0
    wide = np.dtype(field.dtype).itemsize == 8
    while filled < n:
        want = max(1024, int((n - filled) * (2.2 if not wide else 1.01)) + 64)
        z = splitmix64(seed, pos, want)
        pos += want
        cand = z if wide else (z >> np.uint64(32))
        keep = cand[cand < np.uint64(field.p)]
        take = min(n - filled, keep.size)
        out[filled:filled + take] = keep[:take].astype(field.dtype)
        filled += take
    return out


def random_indices(n: int, count: int, seed: int) -> np.ndarray:
    """`count` distinct indices in [0, n), uniformly at random (seeded)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.sort(rng.choice(n, size=count, replace=False)).astype(np.uint32)
