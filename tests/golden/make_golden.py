"""Generate the golden known-answer vectors in tests/golden/golden.json.

The reference crate (benbencik/omr-ntt, Rust) cannot be built in this
environment and its tests hold no golden vectors (src/lib.rs only checks
encoders against each other).  These fixtures are therefore computed from
the definition, with arbitrary-precision Python integers and nothing else:

    omega_N = GEN^((p - 1) / N)            ark-ff's get_root_of_unity, as
                                           called by NttDomain::new
                                           (src/encoder.rs:34-35)
    X[k]    = sum_i x[i] omega_N^(ik)      the DFT that Dft computes
                                           (src/encoders/dft.rs:9-22)
    x[i]    = N^-1 sum_k X[k] omega_N^(-ik)

for every field of src/fields.rs, N = 2^0 .. 2^7, inputs from the seeded
generator of omr_ntt.inputs (splitmix64 + rejection into [0, p)), plus the
roots of unity for every log N up to each field's 2-adicity.

Run:  python tests/golden/make_golden.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "omr-ntt_gb300"))

from omr_ntt.fields import ALL  # noqa: E402
from omr_ntt.inputs import gen_input_seeded  # noqa: E402


def dft(x, w, p):
    n = len(x)
    return [sum(x[i] * pow(w, i * k, p) for i in range(n)) % p for k in range(n)]


def main():
    out = {"generator": "tests/golden/make_golden.py", "fields": {}}
    for f in ALL:
        p = f.p
        roots = {str(l): pow(f.generator, (p - 1) >> l, p) for l in range(f.two_adicity + 1)}
        cases = []
        for log_n in range(0, 8):
            n = 1 << log_n
            seed = 1000 + 17 * f.id + log_n
            x = [int(v) for v in gen_input_seeded(f, n, seed)]
            w = roots[str(log_n)]
            X = dft(x, w, p)
            winv = pow(w, p - 2, p)
            ninv = pow(n, p - 2, p)
            back = [(v * ninv) % p for v in dft(X, winv, p)]
            assert back == x
            cases.append({"log_n": log_n, "seed": seed, "x": x, "X": X})
        out["fields"][f.name] = {"p": p, "generator": f.generator,
                                 "two_adicity": f.two_adicity, "roots": roots, "cases": cases}
    with open(os.path.join(HERE, "golden.json"), "w") as fh:
        json.dump(out, fh, separators=(",", ":"))


if __name__ == "__main__":
    main()
