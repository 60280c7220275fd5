// pass_tb_col_fwd.cu -- TeddyBear tile passes, MODE_COL, forward
// (one translation unit per field, mode and direction: parallel compiles).
#include "launch_pass.cuh"

namespace omr {
template int launch_pass_dir<TeddyBear, MODE_COL, false>(int, int, const PassArgs<TeddyBear>&, uint64_t, int*,
                                                     cudaStream_t);
template int launch_pass<TeddyBear>(const omr_ntt_domain_s*, const PassDesc&, bool, const void*, void*,
                             bool, cudaStream_t, bool);
}  // namespace omr
