// pass_gl_row_inv.cu -- Goldilocks tile passes, MODE_ROW, inverse
// (one translation unit per field, mode and direction: parallel compiles).
#include "launch_pass.cuh"

namespace omr {
template int launch_pass_dir<Goldilocks, MODE_ROW, true>(int, int, const PassArgs<Goldilocks>&, uint64_t, int*,
                                                     cudaStream_t);
}  // namespace omr
