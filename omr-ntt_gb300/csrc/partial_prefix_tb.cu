// partial_prefix_tb.cu -- TeddyBear pruned prefix kernels (one translation unit
// per field: parallel compiles).
#include "partial_prefix.cuh"

namespace omr {
template int launch_prefix<TeddyBear>(omr_ntt_domain_s*, uint32_t, int, const void*, void*, cudaStream_t,
                             const uint32_t*);
}  // namespace omr
