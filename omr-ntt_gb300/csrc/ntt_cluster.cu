// ntt_cluster.cu -- one-launch four-step transforms for 2^13 <= N <= 2^16 on
// a thread-block cluster (8 CTAs up to 2^14, 16 CTAs -- a non-portable
// cluster size GB300 allows -- at 2^15 and 2^16).
//
// A two-pass plan for a small N is latency bound: two launches, each a short
// wave of tiles.  Here one cluster of CL CTAs owns one transform
// (N = N1 x N2; the grid holds one cluster per transform of the
// batch):
//   1. CTA r runs the N1-point column transforms of columns
//      [r W, (r + 1) W), W = N2 / CL, with the tile-pass rounds (first round
//      straight from global memory) and leaves the four-step-twiddled results
//      in its shared memory;
//   2. after a cluster barrier, CTA r gathers rows [r H, (r + 1) H),
//      H = N1 / CL, of all N2 columns from the CL tiles through
//      distributed shared memory (the peers' tiles mapped into its address
//      space) into a second shared-memory tile;
//   3. it runs the N2-point row transforms and writes X[k1 + N1 k2] straight
//      to global memory; a final cluster barrier keeps every tile alive until
//      its peers have read it.
// The arithmetic is the tile pass's (same rounds, twiddles and scale), so the
// words are those of the two-pass plan.  The cluster barriers are hardware
// barriers of co-scheduled CTAs: nothing spins.
#include <cooperative_groups.h>

#include "launch_pass.cuh"

namespace omr {

namespace cg = cooperative_groups;

constexpr int kClusterThreads = 256;
constexpr int cluster_ctas(int log_n) { return log_n <= 14 ? 8 : 16; }

template <class F, int LOG1, int W, bool INV, int I>
OMR_D void cluster_columns(const PassArgs<F>& a, typename F::E* s, const typename F::E* gin,
                           uint32_t llo0) {
  using RP = RoundPlan<LOG1, max_radix_log<F>()>;
  if constexpr (I < RP::ROUNDS) {
    constexpr int SRC = I == 0 ? SRC_GLOBAL : SRC_SMEM;
    constexpr int DST = I + 1 == RP::ROUNDS ? DST_STAGE : DST_SMEM;
    do_round<F, LOG1, W, kClusterThreads, RP::logr(I), RP::logns(I), INV, SRC, DST, false, true>(
        a, s, gin, nullptr, W, llo0, 0);
    cluster_columns<F, LOG1, W, INV, I + 1>(a, s, gin, llo0);
  }
}

template <class F, int LOG1, int LOG2, bool INV>
__global__ void __launch_bounds__(kClusterThreads)
    ntt_cluster_kernel(const PassArgs<F> a, const PassArgs<F> b) {
  using E = typename F::E;
  constexpr int CL = cluster_ctas(LOG1 + LOG2);
  constexpr int N1 = 1 << LOG1, N2 = 1 << LOG2;
  constexpr int W = N2 / CL;  // pass-1 columns per CTA
  constexpr int H = N1 / CL;  // pass-2 rows per CTA
  extern __shared__ __align__(16) unsigned char smem_raw[];
  E* ta = reinterpret_cast<E*>(smem_raw);  // [N1][W], tile_idx<F, W>
  E* tb = ta + N1 * W;                     // [N2][H], tile_idx<F, H>
  cg::cluster_group cluster = cg::this_cluster();
  const uint32_t r = cluster.block_rank();
  const uint64_t t = blockIdx.x / CL;  // transform of the batch

  cluster_columns<F, LOG1, W, INV, 0>(a, ta, a.in + t * a.is_b + r * W, r * W);
  cluster.sync();  // every pass-1 tile complete and visible to the cluster

  // all of a thread's remote loads are issued before its local stores: the
  // two tiles are reached through generic pointers the compiler cannot tell
  // apart, so a load-store loop would wait out each remote load in turn
  constexpr int G = H * N2 / kClusterThreads;
  static_assert(H * N2 % kClusterThreads == 0, "whole gather rounds");
  E g[G];
#pragma unroll
  for (int k = 0; k < G; k++) {
    const int idx = threadIdx.x + k * kClusterThreads;
    const int rl = idx / N2, n2 = idx % N2;  // local row, column
    const E* peer = cluster.map_shared_rank(ta, (int)(n2 / W));
    g[k] = peer[tile_idx<F, W>((int)(r * H) + rl, n2 % W)];
  }
#pragma unroll
  for (int k = 0; k < G; k++) {
    const int idx = threadIdx.x + k * kClusterThreads;
    tb[tile_idx<F, H>(idx % N2, idx / N2)] = g[k];
  }
  __syncthreads();
  all_rounds<F, LOG2, H, kClusterThreads, MODE_ROW, INV, 0>(b, tb, nullptr,
                                                            b.out + t * b.os_b + r * H, H, 0, 0);
  cluster.sync();  // no CTA exits while a peer may still read its tile
}

template <class F, int LOG1, int LOG2, bool INV>
static int launch_cluster_t(const PassArgs<F>& a, const PassArgs<F>& b, uint64_t batch,
                            cudaStream_t stream) {
  constexpr int CL = cluster_ctas(LOG1 + LOG2);
  constexpr size_t smem = (size_t)2 * ((size_t)1 << (LOG1 + LOG2)) / CL * F::WORD;
  auto kern = ntt_cluster_kernel<F, LOG1, LOG2, INV>;
  static std::atomic<int> attr_set[64];  // per device: 1 attributes set, -1 not launchable
  int dev = 0;
  OMR_CUDA_TRY(cudaGetDevice(&dev));
  int st = attr_set[dev & 63].load();
  if (st < 0) return 1;
  if (st == 0) {
    bool ok = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ==
              cudaSuccess;
    if (ok && CL > 8)
      ok = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
    if (ok) {
      // the cluster must fit on the device at all
      cudaLaunchConfig_t qc = {};
      cudaLaunchAttribute qa[1];
      qa[0].id = cudaLaunchAttributeClusterDimension;
      qa[0].val.clusterDim.x = CL;
      qa[0].val.clusterDim.y = 1;
      qa[0].val.clusterDim.z = 1;
      qc.gridDim = dim3(CL);
      qc.blockDim = dim3(kClusterThreads);
      qc.dynamicSmemBytes = smem;
      qc.attrs = qa;
      qc.numAttrs = 1;
      int clusters = 0;
      ok = cudaOccupancyMaxActiveClusters(&clusters, kern, &qc) == cudaSuccess && clusters > 0;
    }
    cudaGetLastError();  // a refused attribute or query is not an error of this call
    attr_set[dev & 63] = ok ? 1 : -1;
    if (!ok) return 1;
  }
  if (batch * CL > 0x7fffffffull) return 1;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)(batch * CL));
  cfg.blockDim = dim3(kClusterThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, kern, a, b) != cudaSuccess) {
    cudaGetLastError();
    return 1;  // not launchable here: the caller runs the passes
  }
  return OMR_NTT_OK;
}

template <class F, bool INV>
static int launch_cluster_dir(int log1, int log2, const PassArgs<F>& a, const PassArgs<F>& b,
                              uint64_t batch, cudaStream_t stream) {
  switch (log1 * 16 + log2) {
    case 7 * 16 + 6: return launch_cluster_t<F, 7, 6, INV>(a, b, batch, stream);
    case 7 * 16 + 7: return launch_cluster_t<F, 7, 7, INV>(a, b, batch, stream);
    case 8 * 16 + 7: return launch_cluster_t<F, 8, 7, INV>(a, b, batch, stream);
    case 8 * 16 + 8: return launch_cluster_t<F, 8, 8, INV>(a, b, batch, stream);
  }
  return 1;
}

// 0: launched; 1: this shape has no cluster kernel or could not be launched
// (the caller then runs the plan's passes); < 0: error.
int launch_cluster_transform(const omr_ntt_domain_s* d, const std::vector<PassDesc>& ps,
                             bool inverse, const void* in, void* out, uint64_t batch,
                             cudaStream_t stream) {
  if (ps.size() != 2) return 1;
  return with_field(d->field, [&](auto f) -> int {
    using F = decltype(f);
    PassArgs<F> a, b;
    int rc = make_pass_args<F>(d, ps[0], inverse, in, nullptr, false, &a);
    if (rc) return rc;
    rc = make_pass_args<F>(d, ps[1], inverse, nullptr, out, true, &b);
    if (rc) return rc;
    return inverse ? launch_cluster_dir<F, true>(ps[0].logT, ps[1].logT, a, b, batch, stream)
                   : launch_cluster_dir<F, false>(ps[0].logT, ps[1].logT, a, b, batch, stream);
  });
}

}  // namespace omr
