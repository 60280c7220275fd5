"""Exact CPU emulation of the engine's pass plans (test helper).

Mirrors ntt_tile_pass (omr-ntt_gb300/csrc/ntt_pass.cuh) index for index:
tile load, the Stockham rounds of RoundPlan (radix 2^4 for every field),
the four-step twiddle on the store (formed per butterfly group as the
kernels form it, base * step^q with 32-bit index arithmetic, and checked
against the direct exponent) and the inverse
scale, driven by the pass records that omr_ntt_plan_passes returns.  It
checks the host-side plan logic and the kernel's index arithmetic on the CPU.
"""
from __future__ import annotations


def round_plan(log_t: int, maxr: int):
    rounds = (log_t + maxr - 1) // maxr
    logr = [log_t // rounds + (1 if i < log_t % rounds else 0) for i in range(rounds)]
    logns = [sum(logr[:i]) for i in range(rounds)]
    return list(zip(logr, logns))


def emulate_plan(field, passes, x, log_n, inverse=False, batch=1):
    p = field.p
    N = 1 << log_n
    C = 32 // field.word_bytes
    maxr = 4
    wN = field.root_of_unity(log_n)
    if inverse:
        wN = pow(wN, p - 2, p)
    ninv = pow(N, p - 2, p)
    bufs = {0: [int(v) for v in x], 1: [0] * (N * batch), 2: [0] * (N * batch)}
    for pi, pd in enumerate(passes):
        last = pi == len(passes) - 1
        T = 1 << pd["logT"]
        wT = pow(wN, N // T, p)
        src, dst = bufs[pd["in_buf"]], bufs[pd["out_buf"]]
        out_vals = []
        groups = (pd["L_lo"] + C - 1) // C
        for lb in range(pd["L_b"]):
            for lm in range(pd["L_m"]):
                for g in range(groups):
                    llo0 = g * C
                    ib = lb * pd["is_b"] + lm * pd["is_m"] + llo0 * pd["is_lo"]
                    ob = lb * pd["os_b"] + lm * pd["os_m"] + llo0 * pd["os_lo"]
                    tile = [[(src[ib + c * pd["is_lo"] + t * pd["es_in"]] if llo0 + c < pd["L_lo"] else 0)
                             for c in range(C)] for t in range(T)]
                    if pd["in_buf"] == pd["out_buf"]:
                        # an in-place pass is race-free only if every CTA writes
                        # exactly the words it read
                        rd = {ib + c * pd["is_lo"] + t * pd["es_in"] for t in range(T) for c in range(C)
                              if llo0 + c < pd["L_lo"]}
                        wr = {ob + c * pd["os_lo"] + t * pd["es_out"] for t in range(T) for c in range(C)
                              if llo0 + c < pd["L_lo"]}
                        assert rd == wr, "in-place pass with mismatched read/write sets"
                    rp = round_plan(pd["logT"], maxr)
                    chain_e = {}  # (k, c) -> four-step exponent as the kernels' chain forms it
                    for ri, (logr, logns) in enumerate(rp):
                        R, NS = 1 << logr, 1 << logns
                        wR = pow(wT, T // R, p)
                        new = [row[:] for row in tile]
                        for b in range((T // R) * C):
                            c, j = b % C, b // C
                            v = [tile[j + q * (T // R)][c] for q in range(R)]
                            jm = j & (NS - 1)
                            if logns > 0:
                                sc = T // (NS * R)
                                v = [v[q] * pow(wT, q * jm * sc, p) % p for q in range(R)]
                            v = [sum(v[q] * pow(wR, q * k, p) for q in range(R)) % p for k in range(R)]
                            d = ((j >> logns) << (logns + logr)) | jm
                            for q in range(R):
                                new[d + q * NS][c] = v[q]
                            if pd["twiddle"] and ri == len(rp) - 1:
                                # base omega^(ls d) times step omega^(ls NS), q times;
                                # ls and the products wrap in 32 bits as in the kernels
                                ls = ((llo0 + c + lm * pd["tw_line_mul_m"]) * pd["tw_scale"]) & 0xFFFFFFFF
                                eb = ((ls * d) & 0xFFFFFFFF) & (N - 1)
                                es = ((ls * NS) & 0xFFFFFFFF) & (N - 1)
                                for q in range(R):
                                    chain_e[(d + q * NS, c)] = (eb + q * es) % N
                        tile = new
                    for k in range(T):
                        for c in range(C):
                            if llo0 + c >= pd["L_lo"]:
                                continue
                            y = tile[k][c]
                            if pd["twiddle"]:
                                line = llo0 + c + lm * pd["tw_line_mul_m"]
                                e = (line * k * pd["tw_scale"]) & (N - 1)
                                assert chain_e[(k, c)] == e, "four-step twiddle chain exponent"
                                y = y * pow(wN, chain_e[(k, c)], p) % p
                            if inverse and last:
                                y = y * ninv % p
                            out_vals.append((ob + c * pd["os_lo"] + k * pd["es_out"], y))
        for addr, y in out_vals:
            dst[addr] = y
    return bufs[passes[-1]["out_buf"]] if passes else bufs[0]
