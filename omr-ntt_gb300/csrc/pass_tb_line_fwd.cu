// pass_tb_line_fwd.cu -- TeddyBear tile passes, MODE_LINE, forward
// (one translation unit per field, mode and direction: parallel compiles).
#include "launch_pass.cuh"

namespace omr {
template int launch_pass_dir<TeddyBear, MODE_LINE, false>(int, int, const PassArgs<TeddyBear>&, uint64_t, int*,
                                                     cudaStream_t);
}  // namespace omr
