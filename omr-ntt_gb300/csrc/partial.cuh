// partial.cuh -- partial-output transforms (selected outputs of one forward NTT).
//
// Reference semantics (prefix): TransformDecomposition / V2 / DftPartial
// (src/encoders/transform_decomposition.rs:25-97,
//  src/encoders/transform_decomposition_v2.rs:23-100, src/encoders/dft.rs:40-89)
// return X[0..m).  Strided and arbitrary index sets have no reference path;
// their oracle is a gather from the full transform.
//
// Algorithms (each exact, so any of them gives the same words):
//   PREFIX m <= 4096 : X[k] = sum_r omega_N^{rk} DFT_m(x[r + (N/m) c])[k]
//                      -- the reference's decomposition with n1 = m: one
//                      tile pass over the N/m stride-(N/m) columns fused with
//                      the twiddle and a per-CTA column sum, then a reduction
//                      over CTAs (reads N words once, writes m).
//   STRIDED s        : X[j N/s] = DFT_s(y)[j], y[n'] = sum_q x[n' + s q]
//                      (fold N -> s by coset sums, then one s-point NTT).
//   INDICES m <= 4096: the prefix decomposition with the index list:
//                      X[j] = sum_r omega_N^{rj} Y_r[j mod T] for any j.
//   otherwise        : full transform into scratch + gather.
#pragma once
#include "engine.cuh"

namespace omr {

int run_partial(omr_ntt_domain_s* d, int pattern, uint64_t count, const uint32_t* indices,
                const void* in, void* out, cudaStream_t stream);

// One explicit partial strategy (1 decomposition with line 2^param, 2 strided
// fold with sub-plan param, 3 full plan param + gather).
int run_partial_strategy(omr_ntt_domain_s* d, int strategy, int param, int pattern,
                         uint64_t count, const uint32_t* indices, const void* in, void* out,
                         cudaStream_t stream);

// out[j] = full[idx[j]] (j < count) on `stream`.
template <class F>
int launch_gather_indices(const void* full, uint64_t n, uint64_t count, const uint32_t* idx,
                          void* out, cudaStream_t stream);

template <class F>
int partial_dispatch(omr_ntt_domain_s* d, int pattern, uint64_t count, const uint32_t* indices,
                     const void* in, void* out, cudaStream_t stream);

}  // namespace omr
