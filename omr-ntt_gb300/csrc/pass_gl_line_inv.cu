// pass_gl_line_inv.cu -- Goldilocks tile passes, MODE_LINE, inverse
// (one translation unit per field, mode and direction: parallel compiles).
#include "launch_pass.cuh"

namespace omr {
template int launch_pass_dir<Goldilocks, MODE_LINE, true>(int, int, const PassArgs<Goldilocks>&, uint64_t, int*,
                                                     cudaStream_t);
}  // namespace omr
