// ntt_pass_wide.cuh -- persistent, double-buffered pass of 256-point lines on
// 128-byte-wide tiles.
//
// How fast a four-step pass can move its data depends on the width of its
// tile rows: on GB300 a copy in the pattern of a column pass (rows 16 KB
// apart) moves 2 x 64 MB in 43 us with 16-byte rows, 32 us with 32-byte rows,
// 27 us with 64-byte rows and 23 us -- the speed of a contiguous copy -- with
// 128-byte rows.  A 4096-point line fills 64 KB of shared memory with only 16
// bytes of lines per row; a 256-point line allows 128 bytes of lines per row
// in 32 KB.  So this pass takes C = 128 / word lines (32 for the 32-bit
// fields, 16 for Goldilocks) of 256 points per tile:
//
//   * column passes: one 2-D TMA box [C lines x 256 rows] per tile, landed
//     with the 128-byte swizzle (16-byte chunk ch of row r at chunk
//     ch ^ (r mod 8)), so that with the lane mapping of wide_lane_l /
//     wide_lane_u every access below is conflict-free;
//     row passes: one 1-D bulk copy per line into a padded line-major layout;
//   * warp w owns the 16-byte column group w (4 or 2 lines); its lanes run
//     the 256-point transforms of those lines as 16 x 16 (radix-16 round,
//     twiddle omega_256^(l a), exchange through the warp's own column group
//     with an XOR swizzle and __syncwarp, radix-16 round), then the four-step
//     twiddle (column passes: one operand per output from the domain's
//     [line][k] table when the pass has at most 8192 lines, else a
//     base * step^q chain) and the inverse scale;
//   * the results go back as 128-byte rows k = a + 16 b (natural order; a
//     256-point line needs no output permutation) and one 2-D TMA store
//     writes the tile;
//   * two tile buffers: the next tile lands while this one computes.
// Per tile that is one CTA barrier for column passes (every warp's results
// in the buffer before the store) and two for row passes (the lines are
// re-laid as rows in place).  Waits are bounded as in the other passes.
// Thread 0 waits on the previous kernel of the stream (programmatic
// dependent launch) before the first load.  Goldilocks runs the
// warp-specialised form at the end of this file.
//
// The 256-point line transform is the same 16 x 16 split as the slab pass
// (ntt_pass_slab.cuh), i.e. the reference's four-step decomposition
// (src/encoders/winterfell_four_step.rs:31-81) within a line.
#pragma once
#include <cuda.h>

#include "ntt_pass_slab.cuh"

namespace omr {

template <class F>
constexpr int wide_cols() {
  return 128 / F::WORD;  // lines per tile
}
constexpr int kWideThreads = 256;  // 8 warps: one per 16-byte column group
template <class F>
constexpr int wide_line_bytes() {
  // row-pass line-major layout, padded so that the lines of a unit sit on
  // other banks: lines 2u + c of the 32-bit fields 8 banks apart (4-byte
  // accesses, a whole warp at a time), Goldilocks lines 2w + u 16 banks apart
  // (8-byte accesses, a half-warp of eight l and two u at a time)
  return 256 * F::WORD + (F::WORD == 8 ? 64 : 32);
}
template <class F>
constexpr int wide_buf_bytes() {  // a 1024-byte multiple (128-byte swizzle atoms)
  constexpr int a = 256 * 128, b = wide_cols<F>() * wide_line_bytes<F>();
  return ((a > b ? a : b) + 1023) / 1024 * 1024;
}
template <class F>
constexpr size_t wide_smem_bytes() {
  return 2 * (size_t)wide_buf_bytes<F>() + 15 * 16 * sizeof(typename F::Tw) + 1024;
}

// 128-byte-swizzled row layout: byte of (row r, 16-byte chunk ch, offset o)
OMR_D int wide_sw(int r, int ch, int o) { return r * 128 + ((ch ^ (r & 7)) << 4) + o; }

// Lane -> (l, u) of the line transforms: l = lane bits 0-2 and 4, u = bit 3.
// The shared-memory pipe serves 8-byte accesses a half-warp at a time, so
// each half-warp (lanes 0-15, 16-31) holds the eight values of l mod 8 --
// eight distinct chunk positions of the swizzle, as rows r = l + 16 m,
// 16 a + (l ^ a) and a + 16 b all have r mod 8 = l mod 8 (^ a) -- and both
// units u: 16 distinct 8-byte slots, one wavefront per half-warp.  (l = lane
// & 15, u = lane >> 4 put rows r and r + 8 of one unit into the same
// half-warp: a two-way conflict on every access.)
OMR_D int wide_lane_l(int lane) { return (lane & 7) | ((lane >> 1) & 8); }
OMR_D int wide_lane_u(int lane) { return (lane >> 3) & 1; }

// The column unit u (8 bytes) of column group w, row r.
template <class F, bool ROWS_LAYOUT>
OMR_D void wide_load_unit(const unsigned char* s, int r, int w, int u, typename F::E* dst) {
  constexpr int VPU = slab_vpu<F>();
  if constexpr (ROWS_LAYOUT) {
    const unsigned char* p = s + wide_sw(r, w, u * 8);
    if constexpr (F::WORD == 4) {
      const uint2 x = *reinterpret_cast<const uint2*>(p);
      dst[0] = x.x;
      dst[1] = x.y;
    } else {
      dst[0] = *reinterpret_cast<const uint64_t*>(p);
    }
  } else {  // line-major: line (w * 16 + u * 8) / word + c
#pragma unroll
    for (int c = 0; c < VPU; c++)
      dst[c] = *reinterpret_cast<const typename F::E*>(
          s + (w * (16 / F::WORD) + u * VPU + c) * wide_line_bytes<F>() + r * F::WORD);
  }
}
template <class F, bool ROWS_LAYOUT>
OMR_D void wide_store_unit(unsigned char* s, int r, int w, int u, const typename F::E* src) {
  constexpr int VPU = slab_vpu<F>();
  if constexpr (ROWS_LAYOUT) {
    unsigned char* p = s + wide_sw(r, w, u * 8);
    if constexpr (F::WORD == 4)
      *reinterpret_cast<uint2*>(p) = make_uint2(src[0], src[1]);
    else
      *reinterpret_cast<uint64_t*>(p) = src[0];
  } else {
#pragma unroll
    for (int c = 0; c < VPU; c++)
      *reinterpret_cast<typename F::E*>(s + (w * (16 / F::WORD) + u * VPU + c) * wide_line_bytes<F>() +
                                        r * F::WORD) = src[c];
  }
}

template <class F, int MODE>
OMR_D void wide_issue_load(const CUtensorMap* map, const PassArgs<F>& a, uint64_t tile,
                           unsigned char* buf, uint64_t* bar) {
  using E = typename F::E;
  constexpr int C = wide_cols<F>();
  uint32_t g, lm;
  uint64_t lb;
  tile_coords<F, C>(a, tile, g, lm, lb);
  mbar_arrive_expect_tx(bar, (uint32_t)(256 * C * F::WORD));
  if constexpr (MODE == MODE_COL) {
    tma_load_2d(buf, map, (int)(g * C), (int)((lb * a.L_m + lm) * 256ull), bar);
  } else {
    const E* src = a.in + (lb * a.is_b + lm * a.is_m + (uint64_t)(g * C) * a.is_lo);
#pragma unroll 1
    for (int c = 0; c < C; c++)
      bulk_load(buf + c * wide_line_bytes<F>(), src + (uint64_t)c * a.is_lo, 256 * F::WORD, bar);
  }
}

template <class F, int MODE>
OMR_D void wide_issue_store(const CUtensorMap* map, const PassArgs<F>& a, uint64_t tile,
                            const unsigned char* buf) {
  constexpr int C = wide_cols<F>();
  uint32_t g, lm;
  uint64_t lb;
  tile_coords<F, C>(a, tile, g, lm, lb);
  if constexpr (MODE == MODE_COL)
    tma_store_2d(map, (int)(g * C), (int)((lb * a.L_m + lm) * 256ull), buf);
  else
    tma_store_2d(map, (int)(g * C + lm * (uint32_t)a.os_m), (int)(lb * 256ull), buf);
  bulk_commit();
}

// wide_issue_load by a whole warp: the row passes' C line copies go out
// from C lanes at once (one thread issues a bulk copy in ~70 ns, so C = 32
// copies from one thread take longer than the tile's compute).  The
// expect-tx arrive (lane 0) comes first; column passes are one TMA load.
template <class F, int MODE>
OMR_D void wide_issue_load_warp(const CUtensorMap* map, const PassArgs<F>& a, uint64_t tile,
                                unsigned char* buf, uint64_t* bar, int lane) {
  using E = typename F::E;
  constexpr int C = wide_cols<F>();
  if constexpr (MODE == MODE_COL) {
    if (lane == 0) wide_issue_load<F, MODE>(map, a, tile, buf, bar);
  } else {
    uint32_t g, lm;
    uint64_t lb;
    tile_coords<F, C>(a, tile, g, lm, lb);
    if (lane == 0) mbar_arrive_expect_tx(bar, (uint32_t)(256 * C * F::WORD));
    __syncwarp();
    const E* src = a.in + (lb * a.is_b + lm * a.is_m + (uint64_t)(g * C) * a.is_lo);
    if (lane < C)
      bulk_load(buf + lane * wide_line_bytes<F>(), src + (uint64_t)lane * a.is_lo, 256 * F::WORD, bar);
  }
}

// One warp: the 256-point transforms of column group w.  The results are
// left in registers, v[c][b] = line entry a + 16 b (a = wide_lane_l(lane)); column
// passes also write them to the swizzled rows in place, row passes re-lay
// them as rows after a CTA barrier (their lines span every column group).
template <class F, int MODE, bool INV, bool TW>
OMR_D void wide_lines(const PassArgs<F>& a, unsigned char* s, const typename F::Tw* tab1, int w,
                      uint32_t llo0, uint32_t lm, typename F::E (&v)[slab_vpu<F>()][16]) {
  using E = typename F::E;
  constexpr int VPU = slab_vpu<F>();
  constexpr bool ROWS = MODE == MODE_COL;
  const int lane = threadIdx.x & 31;
  const int l = wide_lane_l(lane), u = wide_lane_u(lane);
#pragma unroll
  for (int m = 0; m < 16; m++) {
    E x[VPU];
    wide_load_unit<F, ROWS>(s, l + 16 * m, w, u, x);
#pragma unroll
    for (int c = 0; c < VPU; c++) v[c][m] = x[c];
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
#pragma unroll
  for (int aa = 0; aa < 16; aa++) {
    E x[VPU];
#pragma unroll
    for (int c = 0; c < VPU; c++) x[c] = v[c][aa];
    wide_store_unit<F, ROWS>(s, 16 * aa + (l ^ aa), w, u, x);
  }
  __syncwarp();
  const int am = l;
#pragma unroll
  for (int ll = 0; ll < 16; ll++) {
    E x[VPU];
    wide_load_unit<F, ROWS>(s, 16 * am + (ll ^ am), w, u, x);
#pragma unroll
    for (int c = 0; c < VPU; c++) v[c][ll] = x[c];
  }
  __syncwarp();
#pragma unroll
  for (int c = 0; c < VPU; c++) dft_reg<F, 4, INV>(v[c]);
  // outputs b = 0..15 are line entries am + 16 b
  if (TW && a.tw_tab != nullptr) {
    // twiddle table [line][k]: one operand per output (tw_line_mul_m == 0)
#pragma unroll
    for (int c = 0; c < VPU; c++) {
      const uint32_t line = llo0 + (uint32_t)(w * (16 / F::WORD) + u * VPU + c);
      const typename F::Tw* row = a.tw_tab + (size_t)line * 256u + am;
#pragma unroll
      for (int b = 0; b < 16; b++) v[c][b] = F::mul_tw(v[c][b], row[16 * b]);
    }
  } else if constexpr (TW) {
#pragma unroll
    for (int c = 0; c < VPU; c++) {
      const uint32_t line = llo0 + (uint32_t)(w * (16 / F::WORD) + u * VPU + c) + lm * a.tw_line_mul_m;
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
      E x[VPU];
#pragma unroll
      for (int c = 0; c < VPU; c++) x[c] = v[c][b];
      wide_store_unit<F, true>(s, am + 16 * b, w, u, x);
    }
  }
}

template <class F, int MODE, bool INV, bool TW>
__global__ void __launch_bounds__(kWideThreads, 3)  // shared memory holds three CTAs an SM
    ntt_wide_pass(const __grid_constant__ CUtensorMap in_map,
                  const __grid_constant__ CUtensorMap out_map, const PassArgs<F> a, int* err) {
  using E = typename F::E;
  using Tw = typename F::Tw;
  constexpr int C = wide_cols<F>(), VPU = slab_vpu<F>();
  constexpr int BB = wide_buf_bytes<F>();
  extern __shared__ __align__(1024) unsigned char wide_smem_raw[];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ int abort_flag;
  unsigned char* base = wide_smem_raw + ((1024u - (smem_u32(wide_smem_raw) & 1023u)) & 1023u);
  Tw* tab1 = reinterpret_cast<Tw*>(base + 2 * BB);
  const int warp = threadIdx.x >> 5;

  const uint64_t ntiles = a.L_b * (uint64_t)a.L_m * (a.L_lo / C);
  uint64_t tile = blockIdx.x;
  if (threadIdx.x == 0) {
    prefetch_tmap(&in_map);
    prefetch_tmap(&out_map);
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
    fence_proxy_async();
    abort_flag = 0;
  }
  __syncthreads();
  uint32_t outstanding = 0;  // bit b: a load into buffer b has not been waited for
  if (threadIdx.x == 0) {
    // the previous pass's output is this one's input (and its input may be
    // this one's output): every global access of the pass follows this wait
    grid_dep_wait();
    if (tile < ntiles) {
      wide_issue_load<F, MODE>(&in_map, a, tile, base, &bars[0]);
      outstanding |= 1u;
    }
    if (tile + gridDim.x < ntiles) {
      wide_issue_load<F, MODE>(&in_map, a, tile + gridDim.x, base + BB, &bars[1]);
      outstanding |= 2u;
    }
  }
  grid_dep_launch();
  for (int i = threadIdx.x; i < 15 * 16; i += kWideThreads) {
    const int aa = i / 16 + 1, l = i % 16;
    tab1[i] = a.roots[(uint32_t)(l * aa) * a.roots_stride];  // omega_256^(l a)
  }
  __syncthreads();

  uint32_t phase = 0;
  for (int it = 0; tile < ntiles; tile += gridDim.x, it++) {
    const int b = it & 1;
    unsigned char* s = base + b * BB;
    if (mbar_wait_bounded(&bars[b], (phase >> b) & 1)) {
      phase ^= 1u << b;
      outstanding &= ~(1u << b);
    } else {
      atomicExch(err, OMR_NTT_ERR_TIMEOUT);
      abort_flag = 1;
    }
    uint32_t g, lm;
    uint64_t lb;
    tile_coords<F, C>(a, tile, g, lm, lb);
    E v[VPU][16];
    wide_lines<F, MODE, INV, TW>(a, s, tab1, warp, g * C, lm, v);
    if constexpr (MODE != MODE_COL) {
      // every warp has read its lines: re-lay the results as swizzled rows
      __syncthreads();
      const int lane = threadIdx.x & 31;
#pragma unroll
      for (int bb = 0; bb < 16; bb++) {
        E x[VPU];
#pragma unroll
        for (int c = 0; c < VPU; c++) x[c] = v[c][bb];
        wide_store_unit<F, true>(s, wide_lane_l(lane) + 16 * bb, warp, wide_lane_u(lane), x);
      }
    }
    fence_proxy_async();  // this thread's writes become visible to the TMA store
    __syncthreads();
    if (abort_flag) break;
    if (threadIdx.x == 0) {
      wide_issue_store<F, MODE>(&out_map, a, tile, s);
      if (tile + 2ull * gridDim.x < ntiles) {
        bulk_wait_read_all();  // the store has read the buffer
        fence_proxy_async();
        wide_issue_load<F, MODE>(&in_map, a, tile + 2ull * gridDim.x, s, &bars[b]);
        outstanding |= 1u << b;
      }
    }
  }
  if (threadIdx.x == 0) {
    bulk_wait_all();
    for (int bb = 0; bb < 2; bb++)
      if ((outstanding >> bb) & 1) mbar_wait_bounded(&bars[bb], (phase >> bb) & 1);
  }
}

// ---------------------------------------------------------------------------
// The same pass as one warp-specialised CTA per SM.  kWideSlots tile buffers
// cycle through load -> compute -> store: a loader warp issues the TMA loads,
// 24 consumer warps claim units (tile j, column group w) in order from a
// shared counter, so the eight column groups of a tile run on eight warps at
// once and every warp stays busy until the CTA's last unit, and a storer warp
// issues each tile's TMA store and hands the buffer back.  No CTA barrier:
// per buffer slot, `full` completes when the tile has landed, `done` when its
// eight units are written back, `empty` when its store has read it, and for
// row passes `rd` when its eight units have read their lines (the lines are
// re-laid as rows in place).
//
// Units are claimed in order but finish in any order, so a consumer can be
// more than one use of its slot ahead of the loads (a slow warp holding a
// unit of tile j - kWideSlots keeps that slot from being refilled while
// others run on).  A parity wait alone would then see an old phase as done:
// the producer publishes which tile each slot holds (`slot_tile`) before it
// issues the load, and a consumer waits for its tile to be the slot's before
// it waits on `full`.  `rd` and `done` are safe without that check, because
// a unit reaches them only after its tile's load, i.e. after every unit of
// the slot's previous tile has passed both.
// 24 consumer warps (72 registers at 832 threads).  For the 32-bit fields
// the form measured slower than the three-CTA pass with 24 consumers at 72
// registers and with 22 at 80, so only Goldilocks launches it.
template <class F>
constexpr int wide_consumers() {
  return 24;
}
template <class F>
constexpr int wide_ws_threads() {
  return 32 * (wide_consumers<F>() + 2);  // + loader and storer warps
}
constexpr int kWideSlots = 6;

template <class F>
constexpr size_t wide_ws_smem_bytes() {
  return kWideSlots * (size_t)wide_buf_bytes<F>() + 15 * 16 * sizeof(typename F::Tw) + 1024;
}

template <class F, int MODE, bool INV, bool TW>
__global__ void __launch_bounds__(wide_ws_threads<F>(), 1)
    ntt_wide_ws_pass(const __grid_constant__ CUtensorMap in_map,
                     const __grid_constant__ CUtensorMap out_map, const PassArgs<F> a, int* err) {
  using E = typename F::E;
  using Tw = typename F::Tw;
  constexpr int C = wide_cols<F>(), VPU = slab_vpu<F>(), S = kWideSlots;
  constexpr int BB = wide_buf_bytes<F>();
  extern __shared__ __align__(1024) unsigned char wide_ws_smem_raw[];
  __shared__ __align__(8) uint64_t full[S], done[S], rd[S], empty[S];
  __shared__ uint32_t unit_next;
  __shared__ volatile uint32_t slot_tile[S];  // j of the load last issued into each slot
  __shared__ volatile int abort_flag;
  unsigned char* base = wide_ws_smem_raw + ((1024u - (smem_u32(wide_ws_smem_raw) & 1023u)) & 1023u);
  Tw* tab1 = reinterpret_cast<Tw*>(base + S * BB);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // this CTA's tiles: blockIdx.x + j * gridDim.x, j < njobs
  const uint64_t ntiles = a.L_b * (uint64_t)a.L_m * (a.L_lo / C);
  const uint32_t njobs =
      ntiles > blockIdx.x ? (uint32_t)((ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x) : 0u;
  auto tile_of = [&](uint32_t j) { return blockIdx.x + (uint64_t)j * gridDim.x; };

  // The loader warp sets up the barriers and sends the first loads before
  // anything else, so the copies overlap the table setup.
  constexpr int NC = wide_consumers<F>();
  const bool loader = warp == NC;
  uint32_t j_load = 0;
  auto issue_next = [&]() -> bool {  // loader warp: tile j_load into its slot
    const int s = (int)(j_load % S);
    int go = 1;
    if (lane == 0) {
      if (j_load >= (uint32_t)S && !mbar_wait_bounded(&empty[s], ((j_load / S) - 1) & 1)) {
        atomicExch(err, OMR_NTT_ERR_TIMEOUT);
        abort_flag = 1;
      }
      go = !abort_flag;
      if (go) slot_tile[s] = j_load;
    }
    go = __shfl_sync(0xffffffffu, go, 0);
    if (!go) return false;
    wide_issue_load_warp<F, MODE>(&in_map, a, tile_of(j_load), base + s * BB, &full[s], lane);
    j_load++;
    return true;
  };
  if (loader) {
    if (lane == 0) {
      for (int s = 0; s < S; s++) {
        mbar_init(&full[s], 1);
        mbar_init(&done[s], 8);
        mbar_init(&rd[s], 8);
        mbar_init(&empty[s], 1);
        slot_tile[s] = 0xffffffffu;
      }
      fence_mbar_init();
      unit_next = 0;
      abort_flag = 0;
    }
    __syncwarp();
    // the previous pass's output is this one's input (and its input may be
    // this one's output): every global access of the pass follows the
    // loader's wait (the storer writes only tiles that were loaded after it)
    if (lane == 0) {
      prefetch_tmap(&in_map);
      prefetch_tmap(&out_map);
    }
    grid_dep_wait();
    while (j_load < njobs && j_load < (uint32_t)S && issue_next()) {
    }
  }
  grid_dep_launch();
  for (int i = threadIdx.x; i < 15 * 16; i += wide_ws_threads<F>()) {
    const int aa = i / 16 + 1, l = i % 16;
    tab1[i] = a.roots[(uint32_t)(l * aa) * a.roots_stride];  // omega_256^(l a)
  }
  __syncthreads();

  if (loader) {
    // slot s takes tile j once the store of tile j - S has read it
    while (j_load < njobs && issue_next()) {
    }
    // every issued load has landed before the CTA exits (all of them have
    // been consumed unless a wait gave up)
    if (lane == 0)
      for (uint32_t k = j_load > (uint32_t)S ? j_load - S : 0u; k < j_load; k++)
        mbar_wait_bounded(&full[k % S], (k / S) & 1);
    return;
  }
  if (warp == NC + 1) {
    // storer: one lane; tiles in order
    if (lane != 0) return;
    for (uint32_t j = 0; j < njobs; j++) {
      const int s = (int)(j % S);
      if (!mbar_wait_bounded(&done[s], (j / S) & 1)) {
        atomicExch(err, OMR_NTT_ERR_TIMEOUT);
        abort_flag = 1;
      }
      if (abort_flag) break;
      wide_issue_store<F, MODE>(&out_map, a, tile_of(j), base + s * BB);
      if (j + S < njobs) {
        bulk_wait_read_all();
        mbar_arrive(&empty[s]);
      }
    }
    bulk_wait_all();
    return;
  }

  // consumers
  for (;;) {
    uint32_t u = 0;
    if (lane == 0) u = atomicAdd(&unit_next, 1u);
    u = __shfl_sync(0xffffffffu, u, 0);
    const uint32_t j = u >> 3;
    const int w = (int)(u & 7u);
    if (j >= njobs || abort_flag) break;
    const int s = (int)(j % S);
    const uint32_t par = (j / S) & 1;
    unsigned char* buf = base + s * BB;
    bool mine = false;
    for (unsigned long long i = 0; i < kSpinLimit && !(mine = slot_tile[s] == j); i++) __nanosleep(20);
    if (!mine || !mbar_wait_bounded(&full[s], par)) {
      if (lane == 0) {
        atomicExch(err, OMR_NTT_ERR_TIMEOUT);
        abort_flag = 1;
      }
      break;
    }
    uint32_t g, lm;
    uint64_t lb;
    tile_coords<F, C>(a, tile_of(j), g, lm, lb);
    E v[VPU][16];
    wide_lines<F, MODE, INV, TW>(a, buf, tab1, w, g * C, lm, v);
    if constexpr (MODE != MODE_COL) {
      // the rows of the output span every column group's lines: re-lay after
      // all eight units have read theirs
      __syncwarp();
      if (lane == 0) mbar_arrive(&rd[s]);
      if (!mbar_wait_bounded(&rd[s], par)) {
        if (lane == 0) {
          atomicExch(err, OMR_NTT_ERR_TIMEOUT);
          abort_flag = 1;
        }
        break;
      }
#pragma unroll
      for (int bb = 0; bb < 16; bb++) {
        E x[VPU];
#pragma unroll
        for (int c = 0; c < VPU; c++) x[c] = v[c][bb];
        wide_store_unit<F, true>(buf, wide_lane_l(lane) + 16 * bb, w, wide_lane_u(lane), x);
      }
    }
    fence_proxy_async();  // this thread's writes become visible to the TMA store
    __syncwarp();
    if (lane == 0) mbar_arrive(&done[s]);
  }
}

}  // namespace omr
