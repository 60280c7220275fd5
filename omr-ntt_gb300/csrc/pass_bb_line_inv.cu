// pass_bb_line_inv.cu -- BabyBear tile passes, MODE_LINE, inverse
// (one translation unit per field, mode and direction: parallel compiles).
#include "launch_pass.cuh"

namespace omr {
template int launch_pass_dir<BabyBear, MODE_LINE, true>(int, int, const PassArgs<BabyBear>&, uint64_t, int*,
                                                     cudaStream_t);
}  // namespace omr
