"""The four fields of the reference crate (src/fields.rs:4-19)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Field:
    name: str
    id: int            # omr_ntt_field
    p: int             # modulus
    generator: int
    two_adicity: int
    dtype: type        # canonical word type at the ABI

    @property
    def word_bytes(self) -> int:
        return np.dtype(self.dtype).itemsize

    def root_of_unity(self, log_n: int) -> int:
        """ark-ff's get_root_of_unity(2^log_n): GEN^((p-1) >> log_n)."""
        return pow(self.generator, (self.p - 1) >> log_n, self.p)

    def __repr__(self):
        return self.name


BabyBear = Field("BabyBear", 0, 2013265921, 31, 27, np.uint32)
Goldilocks = Field("Goldilocks", 1, 18446744069414584321, 7, 32, np.uint64)
KoalaBear = Field("KoalaBear", 2, 2130706433, 3, 24, np.uint32)
TeddyBear = Field("TeddyBear", 3, 3221225473, 5, 30, np.uint32)
DefaultField = BabyBear  # src/fields.rs:19

ALL = (BabyBear, Goldilocks, KoalaBear, TeddyBear)


def field_by_id(i: int) -> Field:
    return ALL[[f.id for f in ALL].index(i)]


def field_by_name(name: str) -> Field:
    for f in ALL:
        if f.name.lower() == name.lower():
            return f
    raise KeyError(name)
