// ntt_pass_slab.cuh -- persistent tile pass with warp-private 256-point slabs.
//
// A pass runs independent T-point line transforms, T = R0 * 256 with
// R0 = T / 256 in {1, 2, 4, 8, 16} (256 <= T <= 4096), on tiles of 16 bytes
// of adjacent lines (C = 16 / word lines: 4 for the 32-bit fields, 2 for
// Goldilocks).  With t = j + 256 q (j < 256, q < R0) and k = k1 + R0 k2:
//
//   X[k1 + R0 k2] = sum_j omega_256^(j k2) * [omega_T^(j k1) * DFT_R0(x[j + 256 .])[k1]]
//
// so a line splits into one R0-point round across the whole line and, for
// each k1, a 256-point transform of the 256 values that round leaves in
// "slab" k1.  The tile's shared memory is R0 slabs, one per warp:
//
//   * loads: slab q receives rows 256 q .. 256 q + 255 of the tile's lines
//     (column passes: one 2-D TMA box of [C lines x 256 rows], interleaved
//     16-byte rows; row passes: C 1-D bulk copies of 256 words, one
//     line-major run per line);
//   * round 0 (every thread): R0-point DFTs over the slabs (stride-256 rows),
//     twiddled by omega_T^(j k1).  A thread writes its results back to the
//     words it read, so the round runs in place with no barrier;
//   * one CTA barrier: every slab is complete;
//   * rounds 1 and 2 (warp k1 on slab k1, 16 lanes per 8-byte column unit):
//     the slab's 256-point transform as 16 x 16, exchanged through the slab
//     with __syncwarp only; an XOR swizzle keeps both exchange directions
//     free of bank conflicts.  The results land in the slab as [a + 16 b]
//     [column] rows;
//   * the warp then stores its slab with a 4-D TMA store (dims: column,
//     a + 16 b, k1, tile row) to output rows k1 + R0 (a + 16 b) -- the copy
//     engine undoes the permutation -- waits until the store has read the
//     slab and loads its slab of the CTA's next tile into it.
// So each warp's store and next load overlap the other warps' work, and a
// column or row pass costs one CTA barrier per tile (the Stockham tile pass
// of ntt_pass_tma.cuh needs two per radix-16 round).  The next tile's load
// is tracked by one mbarrier with one arrival (expect-tx) per warp; every
// wait is bounded (timeout -> the domain's error word, as in the other
// passes).
//
// Shared-memory accesses are 8 bytes per lane (column passes) or one word
// per lane (row passes) and conflict-free.  Twiddles: omega_T^(j k1) and
// omega_256^(l a) come from tables staged in shared memory once per
// persistent CTA; the four-step twiddle of column passes is the chain
// base * step^b of the other passes.
//
// This is the reference's four-step decomposition
// (src/encoders/winterfell_four_step.rs:31-81) applied inside one line:
// row transforms, twiddle, column transforms, with the transposes folded
// into shared-memory addressing and the TMA store.
#pragma once
#include <cuda.h>

#include "ntt_pass_tma.cuh"

namespace omr {

template <class F>
constexpr int slab_cols() {
  return 16 / F::WORD;  // lines per tile
}
template <class F>
constexpr int slab_vpu() {
  return 8 / F::WORD;  // lines per 8-byte column unit
}
template <int LOGT>
constexpr int slab_r0_log() {
  return LOGT - 8;
}
template <int LOGT>
constexpr int slab_threads() {
  return 32 << (LOGT - 8);  // one warp per slab
}
// Row-pass slab layout: line c of the slab at byte c * LINEB (256 words + 32
// bytes of padding: conflict-free for both lane mappings).  A slab occupies
// SLABB bytes (a 128-byte multiple) in either mode.
template <class F>
constexpr int slab_line_bytes() {
  return 256 * F::WORD + 32;
}
template <class F>
constexpr int slab_bytes() {
  return (slab_cols<F>() * slab_line_bytes<F>() + 127) / 128 * 128;
}
template <class F, int LOGT>
constexpr size_t slab_buf_bytes() {
  return (size_t)(1 << slab_r0_log<LOGT>()) * slab_bytes<F>();
}
template <class F, int LOGT>
constexpr size_t slab_tab_entries() {
  return (size_t)(((1 << slab_r0_log<LOGT>()) - 1) * 256 + 15 * 16);
}
template <class F, int LOGT>
constexpr size_t slab_smem_bytes() {
  return slab_buf_bytes<F, LOGT>() + slab_tab_entries<F, LOGT>() * sizeof(typename F::Tw) + 128;
}

// Word of line c, slab row r, in slab memory `s` (column passes: interleaved
// 16-byte rows; row passes before the final staging: line-major runs).
template <class F, int MODE>
OMR_D typename F::E* slab_word(unsigned char* s, int r, int c) {
  if constexpr (MODE == MODE_COL)
    return reinterpret_cast<typename F::E*>(s + r * 16 + c * F::WORD);
  else
    return reinterpret_cast<typename F::E*>(s + c * slab_line_bytes<F>() + r * F::WORD);
}
// The column unit u (lines VPU u .. VPU u + VPU - 1) of slab row r.
template <class F, int MODE>
OMR_D void slab_load_unit(unsigned char* s, int r, int u, typename F::E* dst) {
  constexpr int VPU = slab_vpu<F>();
  if constexpr (MODE == MODE_COL && F::WORD == 4) {
    const uint2 w = *reinterpret_cast<const uint2*>(s + r * 16 + u * 8);
    dst[0] = w.x;
    dst[1] = w.y;
  } else {
#pragma unroll
    for (int c = 0; c < VPU; c++) dst[c] = *slab_word<F, MODE>(s, r, VPU * u + c);
  }
}
template <class F, int MODE>
OMR_D void slab_store_unit(unsigned char* s, int r, int u, const typename F::E* src) {
  constexpr int VPU = slab_vpu<F>();
  if constexpr (MODE == MODE_COL && F::WORD == 4) {
    *reinterpret_cast<uint2*>(s + r * 16 + u * 8) = make_uint2(src[0], src[1]);
  } else {
#pragma unroll
    for (int c = 0; c < VPU; c++) *slab_word<F, MODE>(s, r, VPU * u + c) = src[c];
  }
}

// Issue the load of slab q of tile `tile` into `slab` (one lane of warp q).
template <class F, int LOGT, int MODE>
OMR_D void slab_issue_load(const CUtensorMap* map, const PassArgs<F>& a, uint64_t tile, int q,
                           unsigned char* slab, uint64_t* bar) {
  using E = typename F::E;
  constexpr int T = 1 << LOGT, C = slab_cols<F>();
  uint32_t g, lm;
  uint64_t lb;
  tile_coords<F, C>(a, tile, g, lm, lb);
  mbar_arrive_expect_tx(bar, (uint32_t)(256 * C * F::WORD));
  if constexpr (MODE == MODE_COL) {
    const int y0 = (int)((lb * a.L_m + lm) * (uint64_t)T) + 256 * q;
    tma_load_2d(slab, map, (int)(g * C), y0, bar);
  } else {
    const E* src = a.in + (lb * a.is_b + lm * a.is_m + (uint64_t)(g * C) * a.is_lo) + 256 * q;
#pragma unroll 1
    for (int c = 0; c < C; c++)
      bulk_load(slab + c * slab_line_bytes<F>(), src + (uint64_t)c * a.is_lo, 256 * F::WORD, bar);
  }
}

OMR_D void tma_store_4d(const CUtensorMap* map, int x, int y, int z, int w, const void* src) {
  asm volatile(
      "cp.async.bulk.tensor.4d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3, %4}], [%5];" ::"l"(
          map),
      "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(src))
      : "memory");
}

// Store slab k1 of tile `tile` (one lane of warp k1).
template <class F, int MODE>
OMR_D void slab_issue_store(const CUtensorMap* map, const PassArgs<F>& a, uint64_t tile, int k1,
                            const unsigned char* slab) {
  constexpr int C = slab_cols<F>();
  uint32_t g, lm;
  uint64_t lb;
  tile_coords<F, C>(a, tile, g, lm, lb);
  if constexpr (MODE == MODE_COL)
    tma_store_4d(map, (int)(g * C), 0, k1, (int)(lb * a.L_m + lm), slab);
  else
    tma_store_4d(map, (int)(g * C + lm * (uint32_t)a.os_m), 0, k1, (int)lb, slab);
  bulk_commit();
}

// Round 0 of one thread: R0-point DFTs of line c over rows j of every slab
// (t = j + 256 q), twiddled by omega_T^(j k1), written back in place (slab
// k1, row j).  Column passes take a column unit (two 32-bit lines) per load.
template <class F, int LOGT, int MODE, bool INV>
OMR_D void slab_round0(unsigned char* buf, const typename F::Tw* tab0) {
  using E = typename F::E;
  constexpr int LR = slab_r0_log<LOGT>(), R0 = 1 << LR, VPU = slab_vpu<F>();
  constexpr int NT = 32 << LR;
  constexpr int SB = slab_bytes<F>();
  // groups: (j, unit) for column passes, (j, line) for row passes
  constexpr int CPG = MODE == MODE_COL ? VPU : 1;  // lines per group
  constexpr int GROUPS = 256 * slab_cols<F>() / CPG;
  constexpr int PER = GROUPS / NT;
#pragma unroll 1
  for (int i = 0; i < PER; i++) {
    const int gi = threadIdx.x + i * NT;
    int j, c0;
    if constexpr (MODE == MODE_COL) {
      c0 = (gi & 1) * VPU;
      j = gi >> 1;
    } else {
      c0 = gi % slab_cols<F>();
      j = gi / slab_cols<F>();
    }
    E v[CPG][R0];
#pragma unroll
    for (int q = 0; q < R0; q++) {
      if constexpr (MODE == MODE_COL) {
        E w[VPU];
        slab_load_unit<F, MODE>(buf + q * SB, j, c0 / VPU, w);
#pragma unroll
        for (int c = 0; c < CPG; c++) v[c][q] = w[c];
      } else {
        v[0][q] = *slab_word<F, MODE>(buf + q * SB, j, c0);
      }
    }
#pragma unroll
    for (int c = 0; c < CPG; c++) dft_reg<F, LR, INV>(v[c]);
#pragma unroll
    for (int k1 = 1; k1 < R0; k1++) {
      const typename F::Tw t = tab0[(k1 - 1) * 256 + j];
#pragma unroll
      for (int c = 0; c < CPG; c++) v[c][k1] = F::mul_tw(v[c][k1], t);
    }
#pragma unroll
    for (int k1 = 0; k1 < R0; k1++) {
      if constexpr (MODE == MODE_COL) {
        E w[VPU];
#pragma unroll
        for (int c = 0; c < VPU; c++) w[c] = v[c][k1];
        slab_store_unit<F, MODE>(buf + k1 * SB, j, c0 / VPU, w);
      } else {
        *slab_word<F, MODE>(buf + k1 * SB, j, c0) = v[0][k1];
      }
    }
  }
}

// Rounds 1 and 2 of one warp on its slab; the results end in the slab as
// interleaved [a + 16 b][column] rows (the store layout).
template <class F, int LOGT, int MODE, bool INV, bool TW>
OMR_D void slab_rounds12(const PassArgs<F>& a, unsigned char* s, const typename F::Tw* tab1,
                         int k1, uint32_t llo0, uint32_t lm) {
  using E = typename F::E;
  constexpr int R0 = 1 << slab_r0_log<LOGT>(), VPU = slab_vpu<F>();
  const int lane = threadIdx.x & 31;
  // 16-byte rows (r * 16 + 8 u: column passes, and every pass's final
  // staging) take 8-byte accesses a half-warp at a time, so each half-warp
  // holds the eight values of l mod 8 and both units (l = lane bits 0-2 and 4,
  // u = bit 3): every access of the rounds below (rows l + 16 m, 16 a + (l ^ a),
  // 16 l + (k ^ l), a + 16 b) lands on 16 distinct 8-byte slots.  The
  // line-major rounds of row passes are conflict-free with it for 4-byte
  // words; for 8-byte (Goldilocks) words there l = lane & 15, u = lane >> 4
  // is, so those row passes keep that assignment.
  constexpr bool kHalfWarp = MODE == MODE_COL || F::WORD == 4;
  const int l = kHalfWarp ? ((lane & 7) | ((lane >> 1) & 8)) : (lane & 15);
  const int u = kHalfWarp ? ((lane >> 3) & 1) : (lane >> 4);
  E v[VPU][16];
  // round 1: lane l transforms rows l + 16 m (m < 16) of its column unit
#pragma unroll
  for (int m = 0; m < 16; m++) {
    E w[VPU];
    slab_load_unit<F, MODE>(s, l + 16 * m, u, w);
#pragma unroll
    for (int c = 0; c < VPU; c++) v[c][m] = w[c];
  }
  __syncwarp();
#pragma unroll
  for (int c = 0; c < VPU; c++) dft_reg<F, 4, INV>(v[c]);
#pragma unroll
  for (int aa = 1; aa < 16; aa++) {
    const typename F::Tw t = tab1[(aa - 1) * 16 + l];
#pragma unroll
    for (int c = 0; c < VPU; c++) v[c][aa] = F::mul_tw(v[c][aa], t);
  }
  // exchange: V[l][a] to row 16 a + (l ^ a)
#pragma unroll
  for (int aa = 0; aa < 16; aa++) {
    E w[VPU];
#pragma unroll
    for (int c = 0; c < VPU; c++) w[c] = v[c][aa];
    slab_store_unit<F, MODE>(s, 16 * aa + (l ^ aa), u, w);
  }
  __syncwarp();
  // round 2: lane a (= l) transforms V[.][a]
  const int am = l;
#pragma unroll
  for (int ll = 0; ll < 16; ll++) {
    E w[VPU];
    slab_load_unit<F, MODE>(s, 16 * am + (ll ^ am), u, w);
#pragma unroll
    for (int c = 0; c < VPU; c++) v[c][ll] = w[c];
  }
  __syncwarp();
#pragma unroll
  for (int c = 0; c < VPU; c++) dft_reg<F, 4, INV>(v[c]);
  // outputs b = 0..15 are line entries kk = k1 + R0 (am + 16 b)
  if constexpr (TW) {
#pragma unroll
    for (int c = 0; c < VPU; c++) {
      const uint32_t line = llo0 + (uint32_t)(u * VPU + c) + lm * a.tw_line_mul_m;
      const uint32_t ls = line * a.tw_scale;
      const uint32_t e0 = (ls * (uint32_t)(k1 + R0 * am)) & a.tw_mask;
      const uint32_t es = (ls * (uint32_t)(16 * R0)) & a.tw_mask;
      E w = F::mul_tw(__ldg(&a.tw_lo[e0 & ((1u << kTwLoBits) - 1)]), a.tw_hi[e0 >> kTwLoBits]);
      const E step = F::mul_tw(__ldg(&a.tw_lo[es & ((1u << kTwLoBits) - 1)]), a.tw_hi[es >> kTwLoBits]);
#pragma unroll
      for (int b = 0; b < 16; b++) {
        v[c][b] = mul_m<F>(v[c][b], w);
        if (b + 1 < 16) w = F::mont_mul(w, step);
      }
    }
  }
  if (a.has_scale) {
#pragma unroll
    for (int c = 0; c < VPU; c++)
#pragma unroll
      for (int b = 0; b < 16; b++) v[c][b] = F::mul_tw(v[c][b], a.scale);
  }
  // staging rows a + 16 b, interleaved columns (both modes)
#pragma unroll
  for (int b = 0; b < 16; b++) {
    E w[VPU];
#pragma unroll
    for (int c = 0; c < VPU; c++) w[c] = v[c][b];
    slab_store_unit<F, MODE_COL>(s, am + 16 * b, u, w);
  }
}

template <class F, int LOGT>
constexpr int slab_min_blocks() {
  // 32-bit fields: 64 registers a thread (1024 threads an SM); Goldilocks:
  // 128 (512 threads an SM)
  return (F::WORD == 4 ? 1024 : 512) / slab_threads<LOGT>();
}

template <class F, int LOGT, int MODE, bool INV, bool TW>
__global__ void __launch_bounds__(slab_threads<LOGT>(), (slab_min_blocks<F, LOGT>()))
    ntt_slab_pass(const __grid_constant__ CUtensorMap in_map,
                  const __grid_constant__ CUtensorMap out_map, const PassArgs<F> a, int* err) {
  pdl_entry();
  using Tw = typename F::Tw;
  constexpr int R0 = 1 << slab_r0_log<LOGT>(), C = slab_cols<F>();
  constexpr int NT = slab_threads<LOGT>();
  constexpr int SB = slab_bytes<F>();
  extern __shared__ __align__(128) unsigned char slab_smem_raw[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ int abort_flag;
  unsigned char* buf = slab_smem_raw + ((128u - (smem_u32(slab_smem_raw) & 127u)) & 127u);
  Tw* tab0 = reinterpret_cast<Tw*>(buf + slab_buf_bytes<F, LOGT>());
  Tw* tab1 = tab0 + (R0 - 1) * 256;
  const int warp = threadIdx.x >> 5;
  const bool leader = (threadIdx.x & 31) == 0;
  unsigned char* my_slab = buf + warp * SB;

  const uint32_t groups = a.L_lo / C;
  const uint64_t ntiles = a.L_b * (uint64_t)a.L_m * groups;
  uint64_t tile = blockIdx.x;
  if (threadIdx.x == 0) {
    mbar_init(&bar, R0);  // one arrival (with its bytes) per warp and tile
    fence_mbar_init();
    fence_proxy_async();
    abort_flag = 0;
  }
  __syncthreads();
  bool outstanding = false;  // this warp's load into its slab has not been waited for
  if (leader && tile < ntiles) {
    slab_issue_load<F, LOGT, MODE>(&in_map, a, tile, warp, my_slab, &bar);
    outstanding = true;
  }
  // in-line twiddle tables: tab0[(k1 - 1) 256 + j] = omega_T^(j k1),
  // tab1[(a - 1) 16 + l] = omega_256^(l a) = omega_T^(l a R0)
  for (int i = threadIdx.x; i < (R0 - 1) * 256; i += NT) {
    const int k1 = i / 256 + 1, j = i % 256;
    tab0[i] = a.roots[(uint32_t)(j * k1) * a.roots_stride];
  }
  for (int i = threadIdx.x; i < 15 * 16; i += NT) {
    const int aa = i / 16 + 1, l = i % 16;
    tab1[i] = a.roots[(uint32_t)(l * aa * R0) * a.roots_stride];
  }
  __syncthreads();

  uint32_t phase = 0;
  for (; tile < ntiles; tile += gridDim.x) {
    // every thread waits for the tile's slabs (bounded); a timeout raises the
    // error word and the flag, read by all after the barrier below
    if (mbar_wait_bounded(&bar, phase)) {
      phase ^= 1u;
      outstanding = false;
    } else {
      atomicExch(err, OMR_NTT_ERR_TIMEOUT);
      abort_flag = 1;
    }
    uint32_t g, lm;
    uint64_t lb;
    tile_coords<F, C>(a, tile, g, lm, lb);
    if constexpr (R0 > 1) slab_round0<F, LOGT, MODE, INV>(buf, tab0);
    __syncthreads();  // every slab complete (and the waits' verdicts published)
    if (abort_flag) break;
    slab_rounds12<F, LOGT, MODE, INV, TW>(a, my_slab, tab1, warp, g * C, lm);
    fence_proxy_async();  // this lane's slab writes become visible to the TMA store
    __syncwarp();
    if (leader) {
      slab_issue_store<F, MODE>(&out_map, a, tile, warp, my_slab);
      if (tile + gridDim.x < ntiles) {
        bulk_wait_read_all();  // the store has read the slab
        fence_proxy_async();
        slab_issue_load<F, LOGT, MODE>(&in_map, a, tile + gridDim.x, warp, my_slab, &bar);
        outstanding = true;
      }
    }
  }
  if (leader) {
    bulk_wait_all();  // every store of this warp has landed
    if (outstanding) mbar_wait_bounded(&bar, phase);  // drain a load still in flight
  }
}

}  // namespace omr
