// noalloc.cu -- a forward NTT entry point that allocates nothing.
//
// omr_ntt_forward keeps the intermediate of its multi-pass plans in scratch
// memory that the domain allocates with cudaMalloc the first time a stream
// needs it (and grows later).  Some callers cannot allow that: a framework
// that has reserved all device memory for its own caching allocator, or a
// latency-bound serving loop for which a cudaMalloc/cudaFree (which can
// synchronise the whole device) is unacceptable.  omr_ntt_forward_noalloc
// runs the same passes but keeps the intermediate in a fixed array of
// kNoAllocScratchBytes in device global memory, declared at file scope below;
// every GPU that loads this library holds that array until the process exits.
//
// Rules of use:
//   * N * batch * word_bytes must not exceed kNoAllocScratchBytes (16 MiB);
//     larger requests fail with OMR_NTT_ERR_CAPACITY and touch no buffer;
//   * the array is shared by every call: calls whose work overlaps on the GPU
//     (different streams, or different host threads without ordering) race
//     on it and produce garbage; serialise them (one stream, or events);
//   * the array keeps the previous call's contents; the first pass overwrites
//     every word the later passes read, so nothing needs clearing;
//   * the first call on each device looks up the array's device address
//     (cudaGetSymbolAddress, with that device current).  With CUDA's lazy
//     module loading that lookup is also when the driver loads this code and
//     reserves the 16 MiB on the device, and the first launch of each kernel
//     loads that kernel: make one warm-up call per device and shape before
//     the region that must not allocate (and before any stream capture);
//   * the plan is the planner database's entry for the shape, else the
//     built-in rule; the learned selector is not consulted, because its first
//     evaluation allocates the network's device buffers.  Plans are
//     tabulated once per log N, so choosing one allocates nothing.
// The domain itself (its twiddle tables) is created beforehand with
// omr_ntt_domain_create, outside the allocation-free region.
#include <cuda_runtime.h>

#include <mutex>

#include "engine.cuh"
#include "launch_pass.cuh"

namespace omr {

constexpr size_t kNoAllocScratchBytes = 16ull << 20;  // 16 MiB

// Host code must not use this name as a device pointer: on the host it is a
// stand-in symbol; its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[64];  // device address of g_noalloc_scratch, per device

static int noalloc_scratch_address(int dev, void** out) {
  if (dev < 0 || dev >= 64) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "device index out of range");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr)
      return fail(OMR_NTT_ERR_CUDA, std::string("cudaGetSymbolAddress(static scratch): ") +
                                        cudaGetErrorString(e));
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return OMR_NTT_OK;
}

}  // namespace omr

using namespace omr;

extern "C" int omr_ntt_forward_noalloc(omr_ntt_domain_t d, const void* in, void* out,
                                       uint64_t batch, void* stream) {
  if (!d || !in || !out) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null argument");
  if (batch == 0) return OMR_NTT_OK;
  // capacity by division first: N * batch * word could wrap for a huge batch
  const uint64_t per = d->n * (uint64_t)word_bytes(d->field);
  if (batch > kNoAllocScratchBytes / per)
    return fail(OMR_NTT_ERR_CAPACITY,
                "omr_ntt_forward_noalloc: N * batch * word = " + std::to_string(per) + " * " +
                    std::to_string(batch) + " bytes exceeds the 16 MiB static scratch; use omr_ntt_forward");
  const size_t bytes = (size_t)(per * batch);
  DeviceGuard g(d->device);
  cudaStream_t st = (cudaStream_t)stream;
  if (d->log_n == 0) {
    if (in != out) OMR_CUDA_TRY(cudaMemcpyAsync(out, in, bytes, cudaMemcpyDeviceToDevice, st));
    return OMR_NTT_OK;
  }
  const int plan = planned_full_plan(d->field, d->log_n, batch, /*use_learned=*/false);
  const std::vector<PassDesc> ps = build_passes(d->log_n, batch, d->plans[plan]);
  if (d->plans[plan].variant == kClusterVariant) {
    // the one-launch cluster plan keeps its intermediate in shared memory
    int rc = launch_cluster_transform(d, ps, false, in, out, batch, st);
    if (rc <= 0) return rc;  // launched, or an error; 1: run the passes below
  }
  void* scratch = nullptr;
  if (ps.size() > 1) {
    int rc = noalloc_scratch_address(d->device, &scratch);
    if (rc) return rc;
  }
  for (size_t i = 0; i < ps.size(); i++) {
    const PassDesc& p = ps[i];
    const void* src = p.in_buf == 0 ? in : (p.in_buf == 1 ? scratch : out);
    void* dst = p.out_buf == 1 ? scratch : out;
    const bool last = i + 1 == ps.size();
    int rc = with_field(d->field, [&](auto f) {
      return launch_pass<decltype(f)>(d, p, false, src, dst, last, st, false);
    });
    if (rc) return rc;
  }
  return OMR_NTT_OK;
}
