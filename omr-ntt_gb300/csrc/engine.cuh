// engine.cuh -- host-side engine internals shared by the translation units:
// domain objects, device tables, pass plans and launch helpers.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "../../include/omr_ntt.h"
#include "fields.cuh"
#include "ntt_pass.cuh"

namespace omr {

// ------------------------------------------------------------------ errors
void set_error(const std::string& msg);
int fail(int status, const std::string& msg);
#define OMR_CUDA_TRY(expr)                                                        \
  do {                                                                            \
    cudaError_t err__ = (expr);                                                   \
    if (err__ != cudaSuccess)                                                     \
      return ::omr::fail(OMR_NTT_ERR_CUDA, std::string(#expr) + ": " +          \
                                               cudaGetErrorString(err__));       \
  } while (0)

inline int word_bytes(int field) { return field == GOLDILOCKS ? 8 : 4; }

// Launch with the programmatic stream-serialisation attribute: the kernel's
// CTAs may be scheduled while the previous kernel of the stream drains, and
// wait in griddepcontrol.wait (grid_dep_wait, ntt_pass.cuh) until it has
// completed.  Every kernel launched this way calls grid_dep_wait() before
// its first global access.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                       Args&&... args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}
int two_adicity(int field);
uint64_t modulus(int field);
bool valid_field(int field);

// ------------------------------------------------------------------ plans
// One pass of a plan (see ntt_pass.cuh for the meaning of the fields).
struct PassDesc {
  int logT;
  uint32_t L_lo, L_m;
  uint64_t L_b;
  uint64_t is_lo, is_m, is_b, os_lo, os_m, os_b, es_in, es_out;
  bool twiddle;
  uint64_t tw_scale;
  uint32_t tw_line_mul_m;
  int in_buf, out_buf;  // 0 source, 1 scratch, 2 destination
  int mode;             // PassMode (ntt_pass.cuh)
  int variant;          // 0: ntt_tile_pass; 1, 2: ntt_tile_pass_tma (two thread counts)
};

// A plan = a split of log N into pass sizes (each 1..12, at most 3 passes).
struct PlanShape {
  std::vector<int> split;  // log2 of each pass's line length, first pass first
  int variant = 0;         // pass kernel variant of the multi-pass plans (3: one cluster launch)
};

std::vector<PlanShape> enumerate_plans(uint32_t log_n);
// enumerate_plans(log_n) for log_n <= 32, built once (no allocation per call)
const std::vector<PlanShape>& plan_table(uint32_t log_n);
std::vector<PassDesc> build_passes(uint32_t log_n, uint64_t batch, const PlanShape& shape);
int default_plan(int field, uint32_t log_n, uint64_t batch);
// The planner's full-transform plan: planner database, learned selector, else
// built-in heuristic (tuner.cu).  use_learned = false skips the learned
// selector, whose first evaluation allocates its device buffers.
int planned_full_plan(int field, uint32_t log_n, uint64_t batch, bool use_learned = true);
// One-launch transform of a two-pass plan on an 8-CTA cluster (ntt_cluster.cu):
// 0 launched, 1 not available for this shape (run the passes), < 0 error.
int launch_cluster_transform(const omr_ntt_domain_s* d, const std::vector<PassDesc>& ps,
                             bool inverse, const void* in, void* out, uint64_t batch,
                             cudaStream_t stream);
constexpr int kClusterVariant = 3;  // PlanShape::variant of the cluster plans
constexpr int kSlabVariant = 4;     // PlanShape::variant of the slab-pass plans (ntt_pass_slab.cuh)
constexpr int kWideVariant = 5;     // 256-point passes on 128-byte-wide tiles (ntt_pass_wide.cuh)
constexpr int kTcVariant = 6;       // the wide pass with its first round on tcgen05 (ntt_pass_tc.cuh)
// Host-buffer batches: chunk size in transforms (0: run unpipelined), and the
// pipelined loop that applies `op(device_buf, transforms, stream)` to every
// chunk between its copy in and copy out.  Caller holds d->host_mu.
uint64_t host_chunk(const omr_ntt_domain_s* d, uint64_t batch);
int host_pipelined(omr_ntt_domain_s* d, char* host, uint64_t batch, uint64_t chunk,
                   const std::function<int(void*, uint64_t, cudaStream_t)>& op);
// The planner's partial strategy (1 if the database or the learned selector has one).
int planned_partial(int field, uint32_t log_n, int pattern, uint64_t count, int* strategy,
                    int* param);

// ------------------------------------------------------------------ device tables
// Per-field in-line roots omega_4096^k, k < 4096 (forward and inverse),
// stored as F::Tw, built once per device.
struct RootTables {
  const void* fwd = nullptr;
  const void* inv = nullptr;
};
int get_root_tables(int field, RootTables* out);

struct Scratch {
  void* ptr = nullptr;
  size_t bytes = 0;
};

}  // namespace omr

// The opaque domain object behind omr_ntt_domain_t.
struct omr_ntt_domain_s {
  int field;
  uint32_t log_n;
  uint64_t n;
  uint64_t omega, omega_inv, n_inv;
  int device;
  // four-step twiddle tables (device): lo = omega^i (i < 4096, twiddle-Montgomery form),
  // hi = omega^(4096 i) as F::Tw; forward and inverse
  void* tw_lo_f = nullptr;
  void* tw_hi_f = nullptr;
  void* tw_lo_i = nullptr;
  void* tw_hi_i = nullptr;
  int* err = nullptr;  // device error word raised by bounded waits (OMR_NTT_ERR_TIMEOUT)
  std::mutex mu;       // guards `scratch`
  std::mutex host_mu;  // serialises the synchronous host-buffer calls
  cudaStream_t host_streams[3] = {nullptr, nullptr, nullptr};  // copy-in, compute, copy-out
  std::map<std::pair<void*, int>, omr::Scratch> scratch;  // keyed by (stream, slot)
  std::vector<omr::PlanShape> plans;
  std::map<uint32_t, omr_ntt_domain_s*> subs;  // smaller domains (same field) for partial paths
  // [line][k] four-step twiddle tables of 256-point column passes (device),
  // keyed by (inverse, tw_scale, lines); built on first use
  std::mutex line_tw_mu;
  std::map<std::tuple<int, uint64_t, uint32_t>, void*> line_tw;
};

namespace omr {
// Scratch of at least `bytes` for (`stream`, `slot`) (grows; owned by the domain).
// Slot 0 is the transform passes' intermediate, slot 1 the partial-output
// staging, slot 2 host-call staging.
int domain_scratch(omr_ntt_domain_s* d, void* stream, size_t bytes, void** out, int slot = 0);

// Number of SMs of device `dev` (cached).
int device_sm_count(int dev);

// The domain of size 2^log_m (same field), created on first use and owned by d.
int sub_domain(omr_ntt_domain_s* d, uint32_t log_m, omr_ntt_domain_s** out);

// Run one full forward/inverse transform plan (device pointers).
int run_transform(omr_ntt_domain_s* d, int plan, bool inverse, const void* in, void* out,
                  uint64_t batch, cudaStream_t stream);

// Field dispatch: calls fn(F{}) for the field's type.
template <class Fn>
int with_field(int field, Fn&& fn) {
  switch (field) {
    case BABYBEAR: return fn(BabyBear{});
    case GOLDILOCKS: return fn(Goldilocks{});
    case KOALABEAR: return fn(KoalaBear{});
    case TEDDYBEAR: return fn(TeddyBear{});
  }
  return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "unknown field id");
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

// Typed launch of one pass.  may_alloc = false: use only device tables that
// already exist (the allocation-free entry point).
template <class F>
int launch_pass(const omr_ntt_domain_s* d, const PassDesc& p, bool inverse, const void* in,
                void* out, bool last, cudaStream_t stream, bool may_alloc = true);
}  // namespace omr
