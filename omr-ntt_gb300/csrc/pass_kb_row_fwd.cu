// pass_kb_row_fwd.cu -- KoalaBear tile passes, MODE_ROW, forward
// (one translation unit per field, mode and direction: parallel compiles).
#include "launch_pass.cuh"

namespace omr {
template int launch_pass_dir<KoalaBear, MODE_ROW, false>(int, int, const PassArgs<KoalaBear>&, uint64_t, int*,
                                                     cudaStream_t);
}  // namespace omr
