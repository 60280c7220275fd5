// pass_bb_line_fwd.cu -- BabyBear tile passes, MODE_LINE, forward
// (one translation unit per field, mode and direction: parallel compiles).
#include "launch_pass.cuh"

namespace omr {
template int launch_pass_dir<BabyBear, MODE_LINE, false>(int, int, const PassArgs<BabyBear>&, uint64_t, int*,
                                                     cudaStream_t);
}  // namespace omr
