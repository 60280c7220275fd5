// pass_bb_row_fwd.cu -- BabyBear tile passes, MODE_ROW, forward
// (one translation unit per field, mode and direction: parallel compiles).
#include "launch_pass.cuh"

namespace omr {
template int launch_pass_dir<BabyBear, MODE_ROW, false>(int, int, const PassArgs<BabyBear>&, uint64_t, int*,
                                                     cudaStream_t);
}  // namespace omr
