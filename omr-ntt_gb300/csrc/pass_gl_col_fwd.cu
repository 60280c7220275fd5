// pass_gl_col_fwd.cu -- Goldilocks tile passes, MODE_COL, forward
// (one translation unit per field, mode and direction: parallel compiles).
#include "launch_pass.cuh"

namespace omr {
template int launch_pass_dir<Goldilocks, MODE_COL, false>(int, int, const PassArgs<Goldilocks>&, uint64_t, int*,
                                                     cudaStream_t);
template int launch_pass<Goldilocks>(const omr_ntt_domain_s*, const PassDesc&, bool, const void*, void*,
                             bool, cudaStream_t, bool);
}  // namespace omr
