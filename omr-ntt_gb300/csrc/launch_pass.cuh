// launch_pass.cuh -- typed launch of one tile pass; instantiated per field in
// pass_<field>.cu so the four fields compile in parallel.
#pragma once
#include <atomic>

#include "engine.cuh"

namespace omr {

template <class F, int LOGT, bool INV>
static int launch_pass_t(const PassArgs<F>& a, uint64_t blocks, cudaStream_t stream) {
  constexpr int C = 32 / F::WORD;
  constexpr int NT = pass_threads<F, LOGT>();
  constexpr size_t smem = (size_t)(1 << LOGT) * C * F::WORD;
  static std::atomic<uint64_t> attr_set{0};
  int dev = 0;
  cudaGetDevice(&dev);
  uint64_t bit = 1ull << (dev & 63);
  if (smem > 48 * 1024 && !(attr_set.load() & bit)) {
    OMR_CUDA_TRY(cudaFuncSetAttribute(ntt_tile_pass<F, LOGT, INV>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set.fetch_or(bit);
  }
  if (blocks == 0) return OMR_NTT_OK;
  if (blocks > 0x7fffffffull) return fail(OMR_NTT_ERR_SIZE, "pass grid too large");
  ntt_tile_pass<F, LOGT, INV><<<(unsigned)blocks, NT, smem, stream>>>(a);
  OMR_CUDA_TRY(cudaGetLastError());
  return OMR_NTT_OK;
}

template <class F, bool INV>
static int launch_pass_logt(int logT, const PassArgs<F>& a, uint64_t blocks, cudaStream_t s) {
  switch (logT) {
    case 1: return launch_pass_t<F, 1, INV>(a, blocks, s);
    case 2: return launch_pass_t<F, 2, INV>(a, blocks, s);
    case 3: return launch_pass_t<F, 3, INV>(a, blocks, s);
    case 4: return launch_pass_t<F, 4, INV>(a, blocks, s);
    case 5: return launch_pass_t<F, 5, INV>(a, blocks, s);
    case 6: return launch_pass_t<F, 6, INV>(a, blocks, s);
    case 7: return launch_pass_t<F, 7, INV>(a, blocks, s);
    case 8: return launch_pass_t<F, 8, INV>(a, blocks, s);
    case 9: return launch_pass_t<F, 9, INV>(a, blocks, s);
    case 10: return launch_pass_t<F, 10, INV>(a, blocks, s);
    case 11: return launch_pass_t<F, 11, INV>(a, blocks, s);
    case 12: return launch_pass_t<F, 12, INV>(a, blocks, s);
    default: return fail(OMR_NTT_ERR_SIZE, "pass line length out of range");
  }
}

template <class F>
int launch_pass(const omr_ntt_domain_s* d, const PassDesc& p, bool inverse, const void* in,
                void* out, bool last, cudaStream_t stream) {
  using E = typename F::E;
  using Tw = typename F::Tw;
  RootTables rt;
  int rc = get_root_tables(F::ID, &rt);
  if (rc) return rc;
  PassArgs<F> a{};
  a.in = static_cast<const E*>(in);
  a.out = static_cast<E*>(out);
  a.L_lo = p.L_lo;
  a.L_m = p.L_m;
  a.is_lo = p.is_lo;
  a.is_m = p.is_m;
  a.is_b = p.is_b;
  a.os_lo = p.os_lo;
  a.os_m = p.os_m;
  a.os_b = p.os_b;
  a.es_in = p.es_in;
  a.es_out = p.es_out;
  a.roots = static_cast<const Tw*>(inverse ? rt.inv : rt.fwd);
  a.roots_stride = (uint32_t)(1u << (kMaxLogT - p.logT));
  if (p.twiddle) {
    a.tw_lo = static_cast<const E*>(inverse ? d->tw_lo_i : d->tw_lo_f);
    a.tw_hi = static_cast<const Tw*>(inverse ? d->tw_hi_i : d->tw_hi_f);
  } else {
    a.tw_lo = nullptr;
    a.tw_hi = nullptr;
  }
  a.tw_scale = p.tw_scale;
  a.tw_mask = d->n - 1;
  a.tw_line_mul_m = p.tw_line_mul_m;
  a.has_scale = (inverse && last) ? 1 : 0;
  a.scale = F::make_tw(d->n_inv);
  constexpr int C = 32 / F::WORD;
  uint64_t blocks = p.L_b * (uint64_t)p.L_m * (uint64_t)((p.L_lo + C - 1) / C);
  return inverse ? launch_pass_logt<F, true>(p.logT, a, blocks, stream)
                 : launch_pass_logt<F, false>(p.logT, a, blocks, stream);
}

}  // namespace omr
