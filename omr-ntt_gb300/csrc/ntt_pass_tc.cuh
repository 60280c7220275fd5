// ntt_pass_tc.cuh -- the wide pass with its first radix-16 round on the
// tensor cores (tcgen05.mma, kind::f16 with bf16 operands), for 32-bit fields.
//
// The wide pass (ntt_pass_wide.cuh) runs every 256-point line of its tile as
// 16 x 16: round 1 is, for each line c and each l < 16, the 16-point DFT
//   V[l][a] = sum_m x[l + 16 m] omega_16^(m a),
// i.e. one 16 x 16 matrix times the tile's 16 x 512 matrix of stride-16
// subsequences.  Exact over the integers it becomes a GEMM on 8-bit limbs:
// with x = sum_i 256^i x_i (x_i < 256) and G_ij = limb_j((256^i omega_16^(m a)) mod p),
//   sum_j 256^j * sum_{i,m} x_i[m] G_ij[m][a]  ==  V[a]   (mod p),
// so D[v][(j, a)] = sum_{(i, m)} A[v][(i, m)] B[(j, a)][(i, m)] with
//   A: 512 subsequence vectors x 64 (limb i, m) bf16 (limbs are exact in bf16),
//   B: 64 (limb j, a) x 64 (limb i, m) bf16, the folded DFT matrix,
//   D: 512 x 64 fp32 in tensor memory, every entry a sum of 64 products of
//      two values < 256, so < 2^22 and exact in fp32.
// Four M = 128 GEMMs (one per 8 lines) of N = 64, K = 64 (four K = 16
// instructions each), issued by one thread from operands in shared memory
// (canonical K-major layout without swizzle: 8-row x 16-byte core matrices,
// K-adjacent cores 128 bytes apart, row groups 1024 bytes apart), completion
// through tcgen05.commit on an mbarrier.  The epilogue reads each vector's 64
// accumulators from tensor memory (tcgen05.ld, one TMEM lane per vector),
// folds sum_j 256^j D_j mod p with two Shoup products, applies omega_256^(l a)
// and writes the exchange layout of the wide pass; round 2, the four-step
// twiddle, the stores and the row-pass re-lay are the wide pass's.
//
// Only the first of the two radix-16 rounds moves to the tensor cores; the
// limb split (about 10 integer instructions per element) and the fold (about
// 25 per output) replace a butterfly network of about 15 per element, so the
// CUDA cores, which bound the pass, get more work, not less.  The plan exists
// to measure that trade on the hardware.
//
// One tile buffer (the next tile lands after the store has read it; two CTAs
// per SM cover that gap), 256 TMEM columns per CTA (two CTAs use all 512),
// every wait bounded as in the other passes; TMEM is freed on every exit path.
#pragma once
#include <cuda.h>

#include "ntt_pass_wide.cuh"

namespace omr {

constexpr int kTcThreads = 256;
constexpr int kTcAVecBytes = 128 * 64 * 2;  // one M-tile of A: 128 vectors x 64 bf16
constexpr int kTcBBytes = 64 * 64 * 2;      // B: 64 x 64 bf16
constexpr int kTcTmemCols = 256;            // four M-tiles x 64 fp32 columns

// Byte offset of element (row, k) in a canonical K-major, no-swizzle operand.
OMR_HD int tc_canon(int row, int k) { return (row >> 3) * 1024 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2; }

template <class F>
constexpr size_t tc_smem_bytes() {
  return (size_t)wide_buf_bytes<F>() + 4 * kTcAVecBytes + kTcBBytes + 15 * 16 * sizeof(typename F::Tw) + 1024;
}

OMR_D uint64_t tc_desc(uint32_t saddr) {
  // start >> 4 | LBO 128 >> 4 at bit 16 | SBO 1024 >> 4 at bit 32 | fixed 0b001 at bit 46
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46);
}

// float(limb) for a byte of x: the byte placed under the exponent of 2^23
// (0x4B000000 | byte) minus 2^23; exact, and its top 16 bits are the bf16 value.
OMR_D float tc_limb(uint32_t x, int i) {
  const uint32_t sel = (uint32_t)i | 0x7440u;  // byte0 = x.byte i, bytes 1-2 = 0, byte3 = 0x4B
  return __uint_as_float(__byte_perm(x, 0x4B000000u, sel)) - 8388608.0f;
}
OMR_D uint32_t tc_pack(float lo, float hi) { return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632); }

// exact integer value of an fp32 accumulator < 2^23
OMR_D uint32_t tc_int(uint32_t bits) { return __float_as_uint(__uint_as_float(bits) + 8388608.0f) - 0x4B000000u; }

template <class F, int MODE, bool INV, bool TW>
__global__ void __launch_bounds__(kTcThreads, 2)
    ntt_wide_tc_pass(const __grid_constant__ CUtensorMap in_map,
                     const __grid_constant__ CUtensorMap out_map, const PassArgs<F> a,
                     const uint16_t* __restrict__ bmat, typename F::Tw one_tw, typename F::Tw r32_tw,
                     int* err) {
  pdl_entry();
  static_assert(F::WORD == 4, "32-bit fields only");
  using E = typename F::E;
  using Tw = typename F::Tw;
  constexpr int C = wide_cols<F>(), VPU = slab_vpu<F>();
  constexpr bool ROWS = MODE == MODE_COL;
  constexpr int BB = wide_buf_bytes<F>();
  extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
  __shared__ __align__(8) uint64_t bars[2];  // [0] tile landed, [1] MMA group done
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag, mma_stuck;
  unsigned char* base = tc_smem_raw + ((1024u - (smem_u32(tc_smem_raw) & 1023u)) & 1023u);
  unsigned char* s = base;             // the tile
  unsigned char* sA = base + BB;       // four M-tiles of A
  unsigned char* sB = sA + 4 * kTcAVecBytes;
  Tw* tab1 = reinterpret_cast<Tw*>(sB + kTcBBytes);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  const uint64_t ntiles = a.L_b * (uint64_t)a.L_m * (a.L_lo / C);
  uint64_t tile = blockIdx.x;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(kTcTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
    fence_proxy_async();
    abort_flag = 0;
    mma_stuck = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  bool outstanding = false;
  if (threadIdx.x == 0 && tile < ntiles) {
    wide_issue_load<F, MODE>(&in_map, a, tile, s, &bars[0]);
    outstanding = true;
  }
  for (int i = threadIdx.x; i < kTcBBytes / 16; i += kTcThreads)
    reinterpret_cast<uint4*>(sB)[i] = reinterpret_cast<const uint4*>(bmat)[i];
  for (int i = threadIdx.x; i < 15 * 16; i += kTcThreads) {
    const int aa = i / 16 + 1, l = i % 16;
    tab1[i] = a.roots[(uint32_t)(l * aa) * a.roots_stride];  // omega_256^(l a)
  }
  fence_proxy_async();  // B is read by the tensor cores (async proxy)
  __syncthreads();

  // instruction descriptor: D fp32, A and B bf16, both K-major, N = 64, M = 128
  constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);
  uint32_t lphase = 0, mphase = 0;
  for (; tile < ntiles; tile += gridDim.x) {
    if (mbar_wait_bounded(&bars[0], lphase)) {
      lphase ^= 1u;
      outstanding = false;
    } else {
      atomicExch(err, OMR_NTT_ERR_TIMEOUT);
      abort_flag = 1;
    }
    uint32_t g, lm;
    uint64_t lb;
    tile_coords<F, C>(a, tile, g, lm, lb);
    // ---- A: lane (l, u) of warp w builds the vectors (line c, l) of its two lines
    {
      const int l = lane & 15, u = lane >> 4;
      E x[VPU][16];
#pragma unroll
      for (int m = 0; m < 16; m++) {
        E t[VPU];
        wide_load_unit<F, ROWS>(s, l + 16 * m, warp, u, t);
#pragma unroll
        for (int c = 0; c < VPU; c++) x[c][m] = t[c];
      }
#pragma unroll
      for (int c = 0; c < VPU; c++) {
        const int line = warp * (16 / F::WORD) + u * VPU + c;  // 0 .. 31
        const int q = line >> 3, row = (line & 7) * 16 + l;     // M-tile, row in it
        unsigned char* dst = sA + q * kTcAVecBytes;
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int h = 0; h < 2; h++) {  // k = 16 i + 8 h .. + 7: one 16-byte core row
            uint4 w;
            w.x = tc_pack(tc_limb(x[c][8 * h + 0], i), tc_limb(x[c][8 * h + 1], i));
            w.y = tc_pack(tc_limb(x[c][8 * h + 2], i), tc_limb(x[c][8 * h + 3], i));
            w.z = tc_pack(tc_limb(x[c][8 * h + 4], i), tc_limb(x[c][8 * h + 5], i));
            w.w = tc_pack(tc_limb(x[c][8 * h + 6], i), tc_limb(x[c][8 * h + 7], i));
            *reinterpret_cast<uint4*>(dst + tc_canon(row, 16 * i + 8 * h)) = w;
          }
      }
    }
    fence_proxy_async();  // A is read by the tensor cores
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (abort_flag) break;
    if (threadIdx.x == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
      for (int q = 0; q < 4; q++)
#pragma unroll 1
        for (int ks = 0; ks < 4; ks++) {
          const uint64_t ad = tc_desc(smem_u32(sA + q * kTcAVecBytes) + ks * 256);
          const uint64_t bd = tc_desc(smem_u32(sB) + ks * 256);
          asm volatile(
              "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem + (uint32_t)(64 * q)),
              "l"(ad), "l"(bd), "r"(kIdesc), "r"((uint32_t)ks)
              : "memory");
        }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&bars[1]))
                   : "memory");
    }
    if (mbar_wait_bounded(&bars[1], mphase)) {
      mphase ^= 1u;
    } else {  // the group may still run: drained before TMEM is freed
      atomicExch(err, OMR_NTT_ERR_TIMEOUT);
      abort_flag = 1;
      mma_stuck = 1;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // ---- epilogue: warpgroup wg reads M-tiles 2 wg, 2 wg + 1; TMEM lane = vector row
    {
      const int wg = warp >> 2, quad = warp & 3;
#pragma unroll 1
      for (int qq = 0; qq < 2; qq++) {
        const int q = 2 * wg + qq;
        const int row = 32 * quad + lane;
        const int line = 8 * q + (row >> 4), l = row & 15;
        uint32_t dv[64];
#pragma unroll
        for (int c0 = 0; c0 < 64; c0 += 16) {
          const uint32_t taddr = tmem + ((uint32_t)(32 * quad) << 16) + (uint32_t)(64 * q + c0);
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
              : "=r"(dv[c0 + 0]), "=r"(dv[c0 + 1]), "=r"(dv[c0 + 2]), "=r"(dv[c0 + 3]), "=r"(dv[c0 + 4]),
                "=r"(dv[c0 + 5]), "=r"(dv[c0 + 6]), "=r"(dv[c0 + 7]), "=r"(dv[c0 + 8]), "=r"(dv[c0 + 9]),
                "=r"(dv[c0 + 10]), "=r"(dv[c0 + 11]), "=r"(dv[c0 + 12]), "=r"(dv[c0 + 13]), "=r"(dv[c0 + 14]),
                "=r"(dv[c0 + 15])
              : "r"(taddr)
              : "memory");
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int aa = 0; aa < 16; aa++) {
          // sum_j 256^j D[16 j + a]: < 2^47, folded mod p as lo + hi 2^32
          const uint64_t v = (uint64_t)tc_int(dv[aa]) + ((uint64_t)tc_int(dv[16 + aa]) << 8) +
                             ((uint64_t)tc_int(dv[32 + aa]) << 16) + ((uint64_t)tc_int(dv[48 + aa]) << 24);
          E y = F::add(F::mul_tw((uint32_t)v, one_tw), F::mul_tw((uint32_t)(v >> 32), r32_tw));
          if (aa > 0) y = F::mul_tw(y, tab1[(aa - 1) * 16 + l]);
          // exchange: V[l][a] to row 16 a + (l ^ a) of the line
          const int r = 16 * aa + (l ^ aa);
          if constexpr (ROWS)
            *reinterpret_cast<E*>(s + wide_sw(r, line >> 2, (line & 3) * 4)) = y;
          else
            *reinterpret_cast<E*>(s + line * wide_line_bytes<F>() + r * 4) = y;
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();  // the exchange is complete (and TMEM is read)
    if (abort_flag) break;
    // ---- round 2 and the rest: the wide pass's second half
    E v[VPU][16];
    {
      const int l = lane & 15, u = lane >> 4;
      const int am = l;
#pragma unroll
      for (int ll = 0; ll < 16; ll++) {
        E t[VPU];
        wide_load_unit<F, ROWS>(s, 16 * am + (ll ^ am), warp, u, t);
#pragma unroll
        for (int c = 0; c < VPU; c++) v[c][ll] = t[c];
      }
      __syncwarp();
#pragma unroll
      for (int c = 0; c < VPU; c++) dft_reg<F, 4, INV>(v[c]);
      if constexpr (TW) {
#pragma unroll
        for (int c = 0; c < VPU; c++) {
          const uint32_t line = g * C + (uint32_t)(warp * (16 / F::WORD) + u * VPU + c) + lm * a.tw_line_mul_m;
          const uint32_t ls = line * a.tw_scale;
          const uint32_t e0 = (ls * (uint32_t)am) & a.tw_mask;
          const uint32_t es = (ls * 16u) & a.tw_mask;
          E t = F::mul_tw(__ldg(&a.tw_lo[e0 & ((1u << kTwLoBits) - 1)]), a.tw_hi[e0 >> kTwLoBits]);
          const E step = F::mul_tw(__ldg(&a.tw_lo[es & ((1u << kTwLoBits) - 1)]), a.tw_hi[es >> kTwLoBits]);
#pragma unroll
          for (int b = 0; b < 16; b++) {
            v[c][b] = mul_m<F>(v[c][b], t);
            if (b + 1 < 16) t = F::mont_mul(t, step);
          }
        }
      }
      if (a.has_scale) {
#pragma unroll
        for (int c = 0; c < VPU; c++)
#pragma unroll
          for (int b = 0; b < 16; b++) v[c][b] = F::mul_tw(v[c][b], a.scale);
      }
      if constexpr (ROWS) {
#pragma unroll
        for (int b = 0; b < 16; b++) {
          E t[VPU];
#pragma unroll
          for (int c = 0; c < VPU; c++) t[c] = v[c][b];
          wide_store_unit<F, true>(s, am + 16 * b, warp, u, t);
        }
      }
    }
    if constexpr (!ROWS) {
      __syncthreads();  // every warp has read its lines: re-lay the results as rows
#pragma unroll
      for (int bb = 0; bb < 16; bb++) {
        E t[VPU];
#pragma unroll
        for (int c = 0; c < VPU; c++) t[c] = v[c][bb];
        wide_store_unit<F, true>(s, (lane & 15) + 16 * bb, warp, lane >> 4, t);
      }
    }
    fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      wide_issue_store<F, MODE>(&out_map, a, tile, s);
      if (tile + gridDim.x < ntiles) {
        bulk_wait_read_all();
        fence_proxy_async();
        wide_issue_load<F, MODE>(&in_map, a, tile + gridDim.x, s, &bars[0]);
        outstanding = true;
      }
    }
  }
  if (threadIdx.x == 0) {
    bulk_wait_all();
    if (outstanding) mbar_wait_bounded(&bars[0], lphase);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (mma_stuck && threadIdx.x == 0) mbar_wait_bounded(&bars[1], mphase);  // bounded drain
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTmemCols) : "memory");
}

}  // namespace omr
