// launch_pass.cuh -- typed launch of one tile pass.  Instantiated per
// (field, mode) in pass_<field>_<mode>.cu so the instances compile in parallel.
#pragma once
#include <cudaTypedefs.h>

#include <atomic>

#include "engine.cuh"
#include "ntt_pass_tma.cuh"

namespace omr {

template <class F, int LOGT, int V, int MODE, bool INV>
int launch_pass_t(const PassArgs<F>& a, uint64_t blocks, cudaStream_t stream) {
  constexpr int C = tile_cols<F, V>();
  constexpr int NT = tile_threads<F, LOGT, V>();
  constexpr size_t smem = (size_t)(1 << LOGT) * C * F::WORD;
  static std::atomic<uint64_t> attr_set{0};
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t bit = 1ull << (dev & 63);
  if (smem > 48 * 1024 && !(attr_set.load() & bit)) {
    OMR_CUDA_TRY(cudaFuncSetAttribute(ntt_tile_pass<F, LOGT, V, MODE, INV>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set.fetch_or(bit);
  }
  if (blocks == 0) return OMR_NTT_OK;
  if (blocks > 0x7fffffffull) return fail(OMR_NTT_ERR_SIZE, "pass grid too large");
  ntt_tile_pass<F, LOGT, V, MODE, INV><<<(unsigned)blocks, NT, smem, stream>>>(a);
  OMR_CUDA_TRY(cudaGetLastError());
  return OMR_NTT_OK;
}

template <class F, int MODE, bool INV, int V>
int launch_pass_logt(int logT, const PassArgs<F>& a, uint64_t blocks, cudaStream_t s) {
  switch (logT) {
    case 1: return launch_pass_t<F, 1, V, MODE, INV>(a, blocks, s);
    case 2: return launch_pass_t<F, 2, V, MODE, INV>(a, blocks, s);
    case 3: return launch_pass_t<F, 3, V, MODE, INV>(a, blocks, s);
    case 4: return launch_pass_t<F, 4, V, MODE, INV>(a, blocks, s);
    case 5: return launch_pass_t<F, 5, V, MODE, INV>(a, blocks, s);
    case 6: return launch_pass_t<F, 6, V, MODE, INV>(a, blocks, s);
    case 7: return launch_pass_t<F, 7, V, MODE, INV>(a, blocks, s);
    case 8: return launch_pass_t<F, 8, V, MODE, INV>(a, blocks, s);
    case 9: return launch_pass_t<F, 9, V, MODE, INV>(a, blocks, s);
    case 10: return launch_pass_t<F, 10, V, MODE, INV>(a, blocks, s);
    case 11: return launch_pass_t<F, 11, V, MODE, INV>(a, blocks, s);
    case 12: return launch_pass_t<F, 12, V, MODE, INV>(a, blocks, s);
    default: return fail(OMR_NTT_ERR_SIZE, "pass line length out of range");
  }
}

// Plan variants: 0 = ntt_tile_pass (32-byte line groups, one tile per CTA);
// 1, 2 = ntt_tile_pass_tma (persistent, TMA-fed, two thread counts), compiled
// for the headline fields at 256..4096-point lines.
template <class F>
constexpr bool has_tma_pass() {
  return F::ID == BABYBEAR || F::ID == GOLDILOCKS;
}
inline int effective_variant(int field, int mode, int logT, int variant) {
  if (variant <= 0 || mode == MODE_LINE || logT < 8) return 0;
  if (field != BABYBEAR && field != GOLDILOCKS) return 0;
  return variant > 2 ? 2 : variant;
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();
int device_sm_count(int dev);

template <class F, int LOGT, int NTV, int MODE, bool INV>
int launch_tma_t(const PassArgs<F>& a, int* err, cudaStream_t stream) {
  constexpr int C = tma_cols<F>();
  constexpr int NT = tma_threads<F, LOGT, NTV>();
  constexpr int T = 1 << LOGT;
  constexpr size_t smem = tma_smem_bytes<F, LOGT, C>();
  auto kern = ntt_tile_pass_tma<F, LOGT, C, NT, MODE, INV>;
  static std::atomic<uint64_t> attr_set{0};
  static std::atomic<int> occ_cache[64];
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t bit = 1ull << (dev & 63);
  if (!(attr_set.load() & bit)) {
    OMR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0;
    OMR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, NT, smem));
    occ_cache[dev & 63] = occ < 1 ? 1 : occ;
    attr_set.fetch_or(bit);
  }
  const uint64_t groups = (a.L_lo + C - 1) / C;
  const uint64_t ntiles = a.L_b * (uint64_t)a.L_m * groups;
  if (ntiles == 0) return OMR_NTT_OK;
  CUtensorMap map;
  memset(&map, 0, sizeof(map));
  if constexpr (MODE == MODE_COL) {
    auto enc = tensor_map_encoder();
    if (!enc) return fail(OMR_NTT_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[2] = {a.L_lo, (cuuint64_t)T * a.L_m * a.L_b};
    cuuint64_t strides[1] = {(cuuint64_t)a.L_lo * F::WORD};
    cuuint32_t box[2] = {(cuuint32_t)C, (cuuint32_t)(T < 256 ? T : 256)};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(&map, F::WORD == 8 ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32,
                     2, const_cast<void*>(static_cast<const void*>(a.in)), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(OMR_NTT_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  }
  const uint64_t slots = (uint64_t)device_sm_count(dev) * occ_cache[dev & 63].load();
  const unsigned grid = (unsigned)(ntiles < slots ? ntiles : slots);
  kern<<<grid, NT, smem, stream>>>(map, a, err);
  OMR_CUDA_TRY(cudaGetLastError());
  return OMR_NTT_OK;
}

// Defined here, instantiated once per (field, mode, direction) in
// pass_<field>_<mode>_<dir>.cu; the extern declarations below stop every
// other translation unit from instantiating the kernels again.
template <class F, int MODE, bool INV>
int launch_pass_dir(int logT, int variant, const PassArgs<F>& a, uint64_t blocks, int* err,
                    cudaStream_t s) {
  if constexpr (MODE != MODE_LINE && has_tma_pass<F>()) {
    if (variant == 1 || variant == 2) {
      switch (logT * 4 + variant) {
        case 8 * 4 + 1: return launch_tma_t<F, 8, 0, MODE, INV>(a, err, s);
        case 9 * 4 + 1: return launch_tma_t<F, 9, 0, MODE, INV>(a, err, s);
        case 10 * 4 + 1: return launch_tma_t<F, 10, 0, MODE, INV>(a, err, s);
        case 11 * 4 + 1: return launch_tma_t<F, 11, 0, MODE, INV>(a, err, s);
        case 12 * 4 + 1: return launch_tma_t<F, 12, 0, MODE, INV>(a, err, s);
        case 8 * 4 + 2: return launch_tma_t<F, 8, 1, MODE, INV>(a, err, s);
        case 9 * 4 + 2: return launch_tma_t<F, 9, 1, MODE, INV>(a, err, s);
        case 10 * 4 + 2: return launch_tma_t<F, 10, 1, MODE, INV>(a, err, s);
        case 11 * 4 + 2: return launch_tma_t<F, 11, 1, MODE, INV>(a, err, s);
        case 12 * 4 + 2: return launch_tma_t<F, 12, 1, MODE, INV>(a, err, s);
        default: break;
      }
    }
  }
  return launch_pass_logt<F, MODE, INV, 0>(logT, a, blocks, s);
}

#define OMR_EXTERN_PASS_DIR(F, MODE, INV)                                                       \
  extern template int launch_pass_dir<F, MODE, INV>(int, int, const PassArgs<F>&, uint64_t,    \
                                                    int*, cudaStream_t);
#define OMR_EXTERN_PASS_MODES(F)        \
  OMR_EXTERN_PASS_DIR(F, MODE_COL, false)  \
  OMR_EXTERN_PASS_DIR(F, MODE_COL, true)   \
  OMR_EXTERN_PASS_DIR(F, MODE_ROW, false)  \
  OMR_EXTERN_PASS_DIR(F, MODE_ROW, true)   \
  OMR_EXTERN_PASS_DIR(F, MODE_LINE, false) \
  OMR_EXTERN_PASS_DIR(F, MODE_LINE, true)
OMR_EXTERN_PASS_MODES(BabyBear)
OMR_EXTERN_PASS_MODES(Goldilocks)
OMR_EXTERN_PASS_MODES(KoalaBear)
OMR_EXTERN_PASS_MODES(TeddyBear)


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
  a.es_in = (uint32_t)p.es_in;
  a.es_out = (uint32_t)p.es_out;
  a.roots = static_cast<const Tw*>(inverse ? rt.inv : rt.fwd);
  a.roots_stride = (uint32_t)(1u << (kMaxLogT - p.logT));
  if (p.twiddle) {
    a.tw_lo = static_cast<const E*>(inverse ? d->tw_lo_i : d->tw_lo_f);
    a.tw_hi = static_cast<const Tw*>(inverse ? d->tw_hi_i : d->tw_hi_f);
  } else {
    a.tw_lo = nullptr;
    a.tw_hi = nullptr;
  }
  a.tw_scale = (uint32_t)p.tw_scale;
  a.tw_mask = (uint32_t)(d->n - 1);
  a.tw_line_mul_m = p.tw_line_mul_m;
  a.has_scale = (inverse && last) ? 1 : 0;
  a.scale = F::make_tw(d->n_inv);
  int variant = effective_variant(F::ID, p.mode, p.logT, p.variant);
  if (variant && ((reinterpret_cast<uintptr_t>(in) & 15) || (p.mode == MODE_COL && p.es_in != p.L_lo)))
    variant = 0;  // TMA needs 16-byte aligned sources and a dense row pitch
  a.L_b = p.L_b;
  const int C = tile_cols<F, 0>();
  const uint64_t blocks = p.L_b * (uint64_t)p.L_m * (uint64_t)((p.L_lo + C - 1) / C);
  switch (p.mode) {
    case MODE_COL:
      return inverse ? launch_pass_dir<F, MODE_COL, true>(p.logT, variant, a, blocks, d->err, stream)
                     : launch_pass_dir<F, MODE_COL, false>(p.logT, variant, a, blocks, d->err, stream);
    case MODE_ROW:
      return inverse ? launch_pass_dir<F, MODE_ROW, true>(p.logT, variant, a, blocks, d->err, stream)
                     : launch_pass_dir<F, MODE_ROW, false>(p.logT, variant, a, blocks, d->err, stream);
    case MODE_LINE:
      return inverse ? launch_pass_dir<F, MODE_LINE, true>(p.logT, 0, a, blocks, d->err, stream)
                     : launch_pass_dir<F, MODE_LINE, false>(p.logT, 0, a, blocks, d->err, stream);
  }
  return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "unknown pass mode");
}

}  // namespace omr
