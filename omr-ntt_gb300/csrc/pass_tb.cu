// pass_tb.cu -- tile-pass launches for TeddyBear (one translation unit per field
// so the fields compile in parallel).
#include "launch_pass.cuh"

namespace omr {
template int launch_pass<TeddyBear>(const omr_ntt_domain_s*, const PassDesc&, bool, const void*, void*,
                             bool, cudaStream_t);
}  // namespace omr
