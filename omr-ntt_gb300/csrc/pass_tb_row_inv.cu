// pass_tb_row_inv.cu -- TeddyBear tile passes, MODE_ROW, inverse
// (one translation unit per field, mode and direction: parallel compiles).
#include "launch_pass.cuh"

namespace omr {
template int launch_pass_dir<TeddyBear, MODE_ROW, true>(int, int, const PassArgs<TeddyBear>&, uint64_t, int*,
                                                     cudaStream_t);
}  // namespace omr
