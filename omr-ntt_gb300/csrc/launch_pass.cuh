// launch_pass.cuh -- typed launch of one tile pass.  Instantiated per
// (field, mode) in pass_<field>_<mode>.cu so the instances compile in parallel.
#pragma once
#include <cudaTypedefs.h>

#include <atomic>
#include <cstring>
#include <map>
#include <mutex>

#include "engine.cuh"
#include "ntt_pass_slab.cuh"
#include "ntt_pass_tma.cuh"
#include "ntt_pass_tc.cuh"
#include "ntt_pass_wide.cuh"

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
  OMR_CUDA_TRY(launch_pdl(ntt_tile_pass<F, LOGT, V, MODE, INV>, dim3((unsigned)blocks), dim3(NT), smem, stream, a));
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
// 1, 2 = ntt_tile_pass_tma at 256..4096-point lines, 1 double-buffered (one
// CTA per SM), 2 two CTAs per SM.  BabyBear and Goldilocks compile both; to
// keep the build short KoalaBear and TeddyBear compile variant 2 only, the
// faster one for both (TeddyBear on GB300: 2^24 0.197 ms against 0.210,
// 64 x 2^20 0.553 against 0.614); the other variant maps onto it.
constexpr int tma_variant_mask(int field) {  // bit v-1 set: variant v compiled
  return (field == BABYBEAR || field == GOLDILOCKS) ? 3 : 2;
}
template <class F>
constexpr bool has_tma_pass() {
  return true;
}
inline int effective_variant(int field, int mode, int logT, int variant) {
  if (variant <= 0 || mode == MODE_LINE || logT < 8) return 0;
  if (variant == kSlabVariant || variant == kWideVariant || variant == kTcVariant) return variant;
  int v = variant > 2 ? 2 : variant;
  if (!((tma_variant_mask(field) >> (v - 1)) & 1)) v = 3 - v;
  return v;
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();

constexpr size_t kMaxDynSmem = 227 * 1024 - 1024;  // leaves room for the static mbarriers

static inline CUresult encode_2d(CUtensorMap* map, int word, const void* base, uint64_t dim0,
                                 uint64_t dim1, uint64_t pitch_words, uint32_t box0, uint32_t box1,
                                 CUtensorMapSwizzle swizzle = CU_TENSOR_MAP_SWIZZLE_NONE) {
  auto enc = tensor_map_encoder();
  if (!enc) return CUDA_ERROR_NOT_SUPPORTED;
  cuuint64_t dims[2] = {dim0, dim1};
  cuuint64_t strides[1] = {pitch_words * (cuuint64_t)word};
  cuuint32_t box[2] = {box0, box1};
  cuuint32_t estr[2] = {1, 1};
  return enc(map, word == 8 ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32, 2,
             const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
}

static inline CUresult encode_4d(CUtensorMap* map, int word, const void* base, const uint64_t (&dims)[4],
                                 const uint64_t (&stride_words)[3], const uint32_t (&box)[4]) {
  auto enc = tensor_map_encoder();
  if (!enc) return CUDA_ERROR_NOT_SUPPORTED;
  cuuint64_t d[4] = {dims[0], dims[1], dims[2], dims[3]};
  cuuint64_t st[3] = {stride_words[0] * (cuuint64_t)word, stride_words[1] * (cuuint64_t)word,
                      stride_words[2] * (cuuint64_t)word};
  cuuint32_t bx[4] = {box[0], box[1], box[2], box[3]};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  return enc(map, word == 8 ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32, 4,
             const_cast<void*>(base), d, st, bx, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
}

// Whether the pass geometry is dense enough for the 2-D TMA tensors of the
// TMA pass (see issue_load / issue_store in ntt_pass_tma.cuh).
template <class F>
bool tma_geometry_ok(const PassArgs<F>& a, int logT, int mode) {
  const uint64_t T = 1ull << logT, C = tma_cols<F>();
  if ((reinterpret_cast<uintptr_t>(a.in) & 15) || (reinterpret_cast<uintptr_t>(a.out) & 15)) return false;
  if (a.L_lo % C) return false;
  if (mode == MODE_COL) {
    const uint64_t rows = T * a.L_m * a.L_b;
    return a.is_lo == 1 && a.os_lo == 1 && a.es_in == a.L_lo && a.es_out == a.L_lo &&
           (a.L_m == 1 || (a.is_m == T * a.L_lo && a.os_m == T * a.L_lo)) &&
           a.is_b == T * a.L_lo * a.L_m && a.os_b == a.is_b && rows < (1ull << 31);
  }
  if (mode == MODE_ROW) {
    const uint64_t w = (uint64_t)a.L_lo * a.L_m;
    return a.es_in == 1 && a.os_lo == 1 && (a.L_m == 1 || a.os_m == a.L_lo) && a.es_out == w &&
           a.os_b == T * w && ((a.is_lo | a.is_m | a.is_b) * F::WORD) % 16 == 0 &&
           T * a.L_b < (1ull << 31);
  }
  return false;
}

template <class F, int LOGT, int MODE, bool INV, bool TW, int NBUF>
int launch_tma_k(const PassArgs<F>& a, int* err, cudaStream_t stream) {
  constexpr int C = tma_cols<F>();
  constexpr int NT = tma_threads<F, LOGT, NBUF>();
  constexpr int T = 1 << LOGT;
  constexpr uint32_t BOX = T < 256 ? T : 256;
  constexpr size_t smem = tma_smem_total<F, LOGT, C, NBUF>();
  static_assert(smem <= kMaxDynSmem, "TMA pass tile does not fit in shared memory");
  auto kern = ntt_tile_pass_tma<F, LOGT, C, NT, MODE, INV, TW, NBUF>;
  // per device: attribute set and occupancy queried once (both cost host time)
  static std::atomic<int> occ_cache[64];
  int dev = 0;
  cudaGetDevice(&dev);
  int occ = occ_cache[dev & 63].load();
  if (occ == 0) {
    OMR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxDynSmem));
    OMR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, NT, smem));
    if (occ < 1) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "TMA pass does not fit on an SM");
    occ_cache[dev & 63] = occ;
  }
  const uint64_t ntiles = a.L_b * (uint64_t)a.L_m * (a.L_lo / C);
  if (ntiles == 0) return OMR_NTT_OK;
  CUtensorMap in_map, out_map;
  memset(&in_map, 0, sizeof(in_map));
  CUresult r;
  if constexpr (MODE == MODE_COL) {
    r = encode_2d(&in_map, F::WORD, a.in, a.L_lo, (uint64_t)T * a.L_m * a.L_b, a.L_lo, C, BOX);
    if (r != CUDA_SUCCESS) return fail(OMR_NTT_ERR_CUDA, "cuTensorMapEncodeTiled (load) failed");
    r = encode_2d(&out_map, F::WORD, a.out, a.L_lo, (uint64_t)T * a.L_m * a.L_b, a.L_lo, C, BOX);
  } else {
    const uint64_t w = (uint64_t)a.L_lo * a.L_m;
    r = encode_2d(&out_map, F::WORD, a.out, w, (uint64_t)T * a.L_b, w, C, BOX);
  }
  if (r != CUDA_SUCCESS) return fail(OMR_NTT_ERR_CUDA, "cuTensorMapEncodeTiled (store) failed");
  const uint64_t slots = (uint64_t)device_sm_count(dev) * occ;
  const unsigned grid = (unsigned)(ntiles < slots ? ntiles : slots);
  OMR_CUDA_TRY(launch_pdl(kern, dim3(grid), dim3(NT), smem, stream, in_map, out_map, a, err));
  return OMR_NTT_OK;
}

// Returns 1 ("not taken") when the geometry or the shared-memory budget does
// not suit the TMA pass; the caller then runs variant 0.
template <class F, int LOGT, int MODE, bool INV, int NBUF>
int launch_tma_t(const PassArgs<F>& a, int* err, cudaStream_t stream) {
  if (!tma_geometry_ok<F>(a, LOGT, MODE)) return 1;
  if (a.tw_lo != nullptr) return launch_tma_k<F, LOGT, MODE, INV, true, NBUF>(a, err, stream);
  return launch_tma_k<F, LOGT, MODE, INV, false, NBUF>(a, err, stream);
}

// The slab pass (ntt_pass_slab.cuh) at 256..4096-point lines.  Returns 1
// ("not taken") when the geometry does not suit it; the caller then runs
// variant 0.  Column passes always apply the four-step twiddle, row passes
// never do.
template <class F, int LOGT, int MODE, bool INV>
int launch_slab_t(const PassArgs<F>& a, int* err, cudaStream_t stream) {
  constexpr bool TW = MODE == MODE_COL;
  if (!tma_geometry_ok<F>(a, LOGT, MODE) || (a.tw_lo != nullptr) != TW) return 1;
  constexpr int C = slab_cols<F>();
  constexpr int NT = slab_threads<LOGT>();
  constexpr uint64_t T = 1ull << LOGT, R0 = T / 256;
  constexpr size_t smem = slab_smem_bytes<F, LOGT>();
  static_assert(smem <= kMaxDynSmem, "slab pass tile does not fit in shared memory");
  auto kern = ntt_slab_pass<F, LOGT, MODE, INV, TW>;
  static std::atomic<int> occ_cache[64];
  int dev = 0;
  cudaGetDevice(&dev);
  int occ = occ_cache[dev & 63].load();
  if (occ == 0) {
    OMR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    OMR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, NT, smem));
    if (occ < 1) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "slab pass does not fit on an SM");
    occ_cache[dev & 63] = occ;
  }
  const uint64_t ntiles = a.L_b * (uint64_t)a.L_m * (a.L_lo / C);
  if (ntiles == 0) return OMR_NTT_OK;
  CUtensorMap in_map, out_map;
  memset(&in_map, 0, sizeof(in_map));
  CUresult r = CUDA_SUCCESS;
  const uint32_t box[4] = {(uint32_t)C, 256u, 1u, 1u};  // one slab per store
  if constexpr (MODE == MODE_COL) {
    const uint64_t L = a.L_lo, outer = (uint64_t)a.L_m * a.L_b;
    r = encode_2d(&in_map, F::WORD, a.in, L, T * outer, L, C, 256);
    if (r != CUDA_SUCCESS) return fail(OMR_NTT_ERR_CUDA, "cuTensorMapEncodeTiled (slab load) failed");
    const uint64_t dims[4] = {L, 256, R0, outer};
    const uint64_t strides[3] = {R0 * L, L, T * L};  // output row kk = k1 + R0 (a + 16 b)
    r = encode_4d(&out_map, F::WORD, a.out, dims, strides, box);
  } else {
    const uint64_t w = (uint64_t)a.L_lo * a.L_m;
    const uint64_t dims[4] = {w, 256, R0, a.L_b};
    const uint64_t strides[3] = {R0 * w, w, T * w};
    r = encode_4d(&out_map, F::WORD, a.out, dims, strides, box);
  }
  if (r != CUDA_SUCCESS) return fail(OMR_NTT_ERR_CUDA, "cuTensorMapEncodeTiled (slab store) failed");
  const uint64_t slots = (uint64_t)device_sm_count(dev) * occ;
  const unsigned grid = (unsigned)(ntiles < slots ? ntiles : slots);
  OMR_CUDA_TRY(launch_pdl(kern, dim3(grid), dim3(NT), smem, stream, in_map, out_map, a, err));
  return OMR_NTT_OK;
}

// The wide pass (ntt_pass_wide.cuh) at 256-point lines, 128 bytes of lines
// per tile.  Returns 1 ("not taken") when the geometry does not suit it.
template <class F, int MODE, bool INV>
int launch_wide_t(const PassArgs<F>& a, int* err, cudaStream_t stream) {
  constexpr bool TW = MODE == MODE_COL;
  constexpr int C = wide_cols<F>();
  if (a.L_lo % C || !tma_geometry_ok<F>(a, 8, MODE) || (a.tw_lo != nullptr) != TW) return 1;
  const uint64_t ntiles = a.L_b * (uint64_t)a.L_m * (a.L_lo / C);
  if (ntiles == 0) return OMR_NTT_OK;
  int dev = 0;
  cudaGetDevice(&dev);
  CUtensorMap in_map, out_map;
  memset(&in_map, 0, sizeof(in_map));
  CUresult r;
  const CUtensorMapSwizzle sw = CU_TENSOR_MAP_SWIZZLE_128B;
  if constexpr (MODE == MODE_COL) {
    const uint64_t rows = 256ull * a.L_m * a.L_b;
    r = encode_2d(&in_map, F::WORD, a.in, a.L_lo, rows, a.L_lo, C, 256, sw);
    if (r != CUDA_SUCCESS) return fail(OMR_NTT_ERR_CUDA, "cuTensorMapEncodeTiled (wide load) failed");
    r = encode_2d(&out_map, F::WORD, a.out, a.L_lo, rows, a.L_lo, C, 256, sw);
  } else {
    const uint64_t w = (uint64_t)a.L_lo * a.L_m;
    r = encode_2d(&out_map, F::WORD, a.out, w, 256ull * a.L_b, w, C, 256, sw);
  }
  if (r != CUDA_SUCCESS) return fail(OMR_NTT_ERR_CUDA, "cuTensorMapEncodeTiled (wide store) failed");
  if constexpr (F::WORD == 8) {
    // Goldilocks: the warp-specialised form (one CTA per SM, no CTA barrier)
    // is 4-7% faster on GB300 (2^24 0.378 against 0.400 ms, 64 x 2^20 1.33
    // against 1.41 ms); for the 32-bit fields it is 8-10% slower at 2^24
    constexpr size_t smem = wide_ws_smem_bytes<F>();
    static_assert(smem <= kMaxDynSmem, "warp-specialised wide pass does not fit in shared memory");
    auto kern = ntt_wide_ws_pass<F, MODE, INV, TW>;
    static std::atomic<int> ready[64];
    if (!ready[dev & 63].load()) {
      OMR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      int occ = 0;
      OMR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, wide_ws_threads<F>(), smem));
      if (occ < 1) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "wide pass does not fit on an SM");
      ready[dev & 63] = 1;
    }
    const uint64_t sms = (uint64_t)device_sm_count(dev);
    OMR_CUDA_TRY(launch_pdl(kern, dim3((unsigned)(ntiles < sms ? ntiles : sms)), dim3(wide_ws_threads<F>()), smem,
                            stream, in_map, out_map, a, err));
  } else {
    constexpr size_t smem = wide_smem_bytes<F>();
    static_assert(smem <= kMaxDynSmem, "wide pass does not fit in shared memory");
    auto kern = ntt_wide_pass<F, MODE, INV, TW>;
    static std::atomic<int> occ_cache[64];
    int occ = occ_cache[dev & 63].load();
    if (occ == 0) {
      OMR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      OMR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kWideThreads, smem));
      if (occ < 1) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "wide pass does not fit on an SM");
      occ_cache[dev & 63] = occ;
    }
    const uint64_t slots = (uint64_t)device_sm_count(dev) * occ;
    OMR_CUDA_TRY(launch_pdl(kern, dim3((unsigned)(ntiles < slots ? ntiles : slots)), dim3(kWideThreads), smem,
                            stream, in_map, out_map, a, err));
  }
  return OMR_NTT_OK;
}

// The tensor-core operand of the wide pass's first round (ntt_pass_tc.cuh):
// B[(j, a)][(i, m)] = bf16(limb_j((256^i omega_16^(m a)) mod p)) in the
// canonical K-major image, 8 KB per (device, field, direction), built once.
template <class F>
int tc_operand(bool inverse, const uint16_t** out) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, void*> cache;
  int dev = 0;
  OMR_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(dev, inverse ? 1 : 0);
  auto it = cache.find(key);
  if (it != cache.end()) {
    *out = static_cast<const uint16_t*>(it->second);
    return OMR_NTT_OK;
  }
  const uint64_t p = F::p64();
  uint64_t w = root_of_unity_host<F>(4);
  if (inverse) w = hpowmod(w, p - 2, p);
  std::vector<uint16_t> img(kTcBBytes / 2, 0);
  for (int i = 0; i < 4; i++)
    for (int m = 0; m < 16; m++)
      for (int aa = 0; aa < 16; aa++) {
        const uint64_t val = hmulmod(hpowmod(256, i, p), hpowmod(w, (uint64_t)m * aa, p), p);
        for (int j = 0; j < 4; j++) {
          const float f = (float)((val >> (8 * j)) & 255u);  // exact in bf16
          uint32_t bits;
          std::memcpy(&bits, &f, 4);
          img[tc_canon(16 * j + aa, 16 * i + m) / 2] = (uint16_t)(bits >> 16);
        }
      }
  void* d = nullptr;
  OMR_CUDA_TRY(cudaMalloc(&d, kTcBBytes));
  OMR_CUDA_TRY(cudaMemcpy(d, img.data(), kTcBBytes, cudaMemcpyHostToDevice));
  cache[key] = d;
  *out = static_cast<const uint16_t*>(d);
  return OMR_NTT_OK;
}

// The wide pass with its first round on the tensor cores (BabyBear, 256-point
// lines).  Returns 1 ("not taken") when the geometry does not suit it.
template <class F, int MODE, bool INV>
int launch_tc_t(const PassArgs<F>& a, int* err, cudaStream_t stream) {
  constexpr bool TW = MODE == MODE_COL;
  constexpr int C = wide_cols<F>();
  if (a.L_lo % C || !tma_geometry_ok<F>(a, 8, MODE) || (a.tw_lo != nullptr) != TW) return 1;
  constexpr size_t smem = tc_smem_bytes<F>();
  static_assert(smem <= kMaxDynSmem, "tensor-core pass does not fit in shared memory");
  auto kern = ntt_wide_tc_pass<F, MODE, INV, TW>;
  static std::atomic<int> occ_cache[64];
  int dev = 0;
  cudaGetDevice(&dev);
  int occ = occ_cache[dev & 63].load();
  if (occ == 0) {
    OMR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // two CTAs of 112 KB share an SM only with the whole carve-out as shared memory
    OMR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    OMR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kTcThreads, smem));
    if (occ < 1) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "tensor-core pass does not fit on an SM");
    // the query can under-count against the shared-memory carve-out: size the
    // grid for two CTAs when two fit the SM's shared memory (CTAs beyond the
    // resident ones only start later; none waits on another)
    int per_sm = 0;
    OMR_CUDA_TRY(cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    if (occ < 2 && 2 * (smem + 2048) <= (size_t)per_sm) occ = 2;
    occ_cache[dev & 63] = occ;
  }
  const uint16_t* bmat = nullptr;
  int rc = tc_operand<F>(INV, &bmat);
  if (rc) return rc;
  const uint64_t ntiles = a.L_b * (uint64_t)a.L_m * (a.L_lo / C);
  if (ntiles == 0) return OMR_NTT_OK;
  CUtensorMap in_map, out_map;
  memset(&in_map, 0, sizeof(in_map));
  CUresult r;
  const CUtensorMapSwizzle sw = CU_TENSOR_MAP_SWIZZLE_128B;
  if constexpr (MODE == MODE_COL) {
    const uint64_t rows = 256ull * a.L_m * a.L_b;
    r = encode_2d(&in_map, F::WORD, a.in, a.L_lo, rows, a.L_lo, C, 256, sw);
    if (r != CUDA_SUCCESS) return fail(OMR_NTT_ERR_CUDA, "cuTensorMapEncodeTiled (tensor-core load) failed");
    r = encode_2d(&out_map, F::WORD, a.out, a.L_lo, rows, a.L_lo, C, 256, sw);
  } else {
    const uint64_t w = (uint64_t)a.L_lo * a.L_m;
    r = encode_2d(&out_map, F::WORD, a.out, w, 256ull * a.L_b, w, C, 256, sw);
  }
  if (r != CUDA_SUCCESS) return fail(OMR_NTT_ERR_CUDA, "cuTensorMapEncodeTiled (tensor-core store) failed");
  const uint64_t slots = (uint64_t)device_sm_count(dev) * occ;
  const unsigned grid = (unsigned)(ntiles < slots ? ntiles : slots);
  const typename F::Tw one_tw = F::make_tw(1), r32_tw = F::make_tw((1ull << 32) % F::p64());
  OMR_CUDA_TRY(launch_pdl(kern, dim3(grid), dim3(kTcThreads), smem, stream, in_map, out_map, a, bmat, one_tw, r32_tw, err));
  return OMR_NTT_OK;
}

// Defined here, instantiated once per (field, mode, direction) in
// pass_<field>_<mode>_<dir>.cu; the extern declarations below stop every
// other translation unit from instantiating the kernels again.
template <class F, int LOGT, int MODE, bool INV, int NBUF>
int launch_tma_compiled(const PassArgs<F>& a, int* err, cudaStream_t s) {
  if constexpr ((tma_variant_mask(F::ID) >> (NBUF == 2 ? 0 : 1)) & 1)
    return launch_tma_t<F, LOGT, MODE, INV, NBUF>(a, err, s);
  else
    return 1;  // not compiled for this field: plain tile pass
}

template <class F, int MODE, bool INV>
int launch_pass_dir(int logT, int variant, const PassArgs<F>& a, uint64_t blocks, int* err,
                    cudaStream_t s) {
  if constexpr (MODE != MODE_LINE && has_tma_pass<F>()) {
    if (variant == kTcVariant) {
      // 256-point BabyBear passes on the tensor-core variant; everything else
      // of the plan takes the wide pass
      int rc = 1;
      if constexpr (F::ID == BABYBEAR)
        if (logT == 8) rc = launch_tc_t<F, MODE, INV>(a, err, s);
      if (rc != 1) return rc;
      variant = kWideVariant;
    }
    if (variant == kWideVariant) {
      // 256-point passes on the wide tiles; other line lengths of the plan
      // take the slab pass
      int rc = logT == 8 ? launch_wide_t<F, MODE, INV>(a, err, s) : 1;
      if (rc != 1) return rc;
      variant = kSlabVariant;
    }
    if (variant == kSlabVariant) {
      int rc = 1;
      switch (logT) {
        case 8: rc = launch_slab_t<F, 8, MODE, INV>(a, err, s); break;
        case 9: rc = launch_slab_t<F, 9, MODE, INV>(a, err, s); break;
        case 10: rc = launch_slab_t<F, 10, MODE, INV>(a, err, s); break;
        case 11: rc = launch_slab_t<F, 11, MODE, INV>(a, err, s); break;
        case 12: rc = launch_slab_t<F, 12, MODE, INV>(a, err, s); break;
        default: break;
      }
      if (rc != 1) return rc;
    } else if (variant >= 1) {
      int rc = 1;
      switch (logT * 4 + variant) {
        case 8 * 4 + 1: rc = launch_tma_compiled<F, 8, MODE, INV, 2>(a, err, s); break;
        case 9 * 4 + 1: rc = launch_tma_compiled<F, 9, MODE, INV, 2>(a, err, s); break;
        case 10 * 4 + 1: rc = launch_tma_compiled<F, 10, MODE, INV, 2>(a, err, s); break;
        case 11 * 4 + 1: rc = launch_tma_compiled<F, 11, MODE, INV, 2>(a, err, s); break;
        case 12 * 4 + 1: rc = launch_tma_compiled<F, 12, MODE, INV, 2>(a, err, s); break;
        case 8 * 4 + 2: rc = launch_tma_compiled<F, 8, MODE, INV, 1>(a, err, s); break;
        case 9 * 4 + 2: rc = launch_tma_compiled<F, 9, MODE, INV, 1>(a, err, s); break;
        case 10 * 4 + 2: rc = launch_tma_compiled<F, 10, MODE, INV, 1>(a, err, s); break;
        case 11 * 4 + 2: rc = launch_tma_compiled<F, 11, MODE, INV, 1>(a, err, s); break;
        case 12 * 4 + 2: rc = launch_tma_compiled<F, 12, MODE, INV, 1>(a, err, s); break;
        default: break;
      }
      if (rc != 1) return rc;
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


// Kernel arguments of one pass descriptor.
template <class F>
int make_pass_args(const omr_ntt_domain_s* d, const PassDesc& p, bool inverse, const void* in,
                   void* out, bool last, PassArgs<F>* out_args) {
  using E = typename F::E;
  using Tw = typename F::Tw;
  RootTables rt;
  int rc = get_root_tables(F::ID, &rt);
  if (rc) return rc;
  PassArgs<F>& a = *out_args;
  a = PassArgs<F>{};
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
  a.L_b = p.L_b;
  return OMR_NTT_OK;
}

// The [line][k] four-step twiddle table of a 256-point column pass: entry
// (line, k) = omega^((line * tw_scale * k) mod N) as F::Tw, line < lines.
// Built on the host once per (domain, direction, tw_scale, lines) and kept
// by the domain; with may_alloc = false only an existing table is returned.
constexpr uint32_t kLineTwMaxLines = 8192;  // 16 MB of 8-byte operands at most

template <class F>
int line_twiddles(omr_ntt_domain_s* d, bool inverse, uint64_t tw_scale, uint32_t lines, bool may_alloc,
                  const typename F::Tw** out) {
  using Tw = typename F::Tw;
  *out = nullptr;
  const auto key = std::make_tuple(inverse ? 1 : 0, tw_scale, lines);
  std::lock_guard<std::mutex> lk(d->line_tw_mu);
  auto it = d->line_tw.find(key);
  if (it != d->line_tw.end()) {
    *out = static_cast<const Tw*>(it->second);
    return OMR_NTT_OK;
  }
  if (!may_alloc) return OMR_NTT_OK;
  const uint64_t p = F::p64(), w = inverse ? d->omega_inv : d->omega;
  std::vector<Tw> host((size_t)lines * 256);
  for (uint32_t line = 0; line < lines; line++) {
    const uint64_t step = hpowmod(w, ((uint64_t)line * tw_scale) & (d->n - 1), p);
    uint64_t t = 1;
    for (int k = 0; k < 256; k++) {
      host[(size_t)line * 256 + k] = F::make_tw(t);
      t = hmulmod(t, step, p);
    }
  }
  void* dev = nullptr;
  const size_t bytes = host.size() * sizeof(Tw);
  if (cudaMalloc(&dev, bytes) != cudaSuccess) return fail(OMR_NTT_ERR_ALLOC, "line twiddle table allocation failed");
  if (cudaMemcpy(dev, host.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(dev);
    return fail(OMR_NTT_ERR_CUDA, "line twiddle table copy failed");
  }
  d->line_tw[key] = dev;
  *out = static_cast<const Tw*>(dev);
  return OMR_NTT_OK;
}

template <class F>
int launch_pass(const omr_ntt_domain_s* d, const PassDesc& p, bool inverse, const void* in,
                void* out, bool last, cudaStream_t stream, bool may_alloc) {
  PassArgs<F> a;
  int rc = make_pass_args<F>(d, p, inverse, in, out, last, &a);
  if (rc) return rc;
  const int variant = effective_variant(F::ID, p.mode, p.logT, p.variant);
  if (p.twiddle && p.mode == MODE_COL && p.logT == 8 && variant == kWideVariant &&
      (p.L_m == 1 || p.tw_line_mul_m == 0) && p.L_lo <= kLineTwMaxLines) {
    // a 256-point wide column pass with few lines: its twiddles as one table
    rc = line_twiddles<F>(const_cast<omr_ntt_domain_s*>(d), inverse, p.tw_scale, p.L_lo, may_alloc, &a.tw_tab);
    if (rc) return rc;
  }
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
