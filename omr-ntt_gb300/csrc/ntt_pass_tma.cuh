// ntt_pass_tma.cuh -- persistent, double-buffered tile pass: TMA in, TMA out.
//
// Same arithmetic as ntt_tile_pass (ntt_pass.cuh), GB300 data movement:
//   * persistent CTAs walk the tiles of a pass (tile += gridDim.x);
//   * one elected thread lands the NEXT tile in the second shared-memory
//     buffer while the whole CTA computes the current one:
//       - column passes (adjacent lines adjacent in memory): 2-D TMA tiled
//         loads (cp.async.bulk.tensor.2d) of [C columns x 256 rows] boxes;
//       - row passes (a line is a contiguous run): one 1-D bulk copy
//         (cp.async.bulk) per line;
//     completion is tracked by one mbarrier per buffer (expect-tx bytes);
//   * the radix-2^r Stockham rounds exchange through the landed buffer; the
//     last round writes the results, four-step twiddle applied, into the same
//     buffer in the [k][c] box layout and one thread stores the tile with 2-D
//     TMA stores (cp.async.bulk.tensor ... global.shared::cta, bulk groups);
//   * per-round in-line twiddles and the four-step twiddle tables are staged in shared
//     memory once per CTA; the four-step twiddles of one butterfly are a
//     Montgomery chain base * step^q, so each output costs two products;
//   * every wait is bounded: on timeout the CTA raises the domain's error word
//     (read back as OMR_NTT_ERR_TIMEOUT), drains its own copies and exits.
// Shared-memory layouts (c-fast warp mapping; bank-conflict free except a
// 2-way conflict on the first exchange write):
//   landing, column pass: [t][c]           word t*C + c          (TMA box)
//   landing, row pass:    line c            word c*(T + PAD) + t, PAD = 128/(C*w)
//   exchange:             [t][c] + padding  word t*C + c + (t >> 3)*XPAD, XPAD = 16/w
//   staging (store):      [k][c]            word k*C + c          (TMA box)
#pragma once
#include <cuda.h>

#include "ntt_pass.cuh"

namespace omr {

constexpr unsigned long long kSpinLimit = 1ull << 24;  // bounded waits (well under a minute)

OMR_D uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

OMR_D void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
OMR_D void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
OMR_D void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
OMR_D void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
OMR_D void prefetch_tmap(const CUtensorMap* m) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(m)) : "memory");
}
OMR_D void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
OMR_D bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait; false on timeout
OMR_D bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (unsigned long long i = 0; i < kSpinLimit; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
OMR_D void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
OMR_D void tma_store_2d(const CUtensorMap* map, int x, int y, const void* src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                   map),
               "r"(x), "r"(y), "r"(smem_u32(src))
               : "memory");
}
OMR_D void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
OMR_D void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
OMR_D void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
OMR_D void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

template <class F>
constexpr int tma_cols() {
  return 16 / F::WORD;  // 16-byte line groups: conflict-free layouts, two buffers fit
}
template <class F, int C>
constexpr int land_pad() {
  return 128 / (C * F::WORD);  // words
}
template <class F>
constexpr int xchg_pad() {
  return 16 / F::WORD;  // words per padding period
}
template <class F, int LOGT>
constexpr int xchg_shift() {  // padding period: twice the first round's radix (rows)
  return RoundPlan<LOGT, max_radix_log<F>()>::logr(0) + 1;
}
template <class F, int LOGT, int C>
constexpr size_t tma_buf_words() {
  constexpr size_t T = (size_t)1 << LOGT;
  constexpr size_t a = T * C + (T >> xchg_shift<F, LOGT>()) * xchg_pad<F>();
  constexpr size_t b = (size_t)C * (T + land_pad<F, C>());
  return ((a > b ? a : b) * F::WORD + 127) / 128 * 128 / F::WORD;  // 128-byte aligned buffers
}
template <class F, int LOGT, int C, int NBUF>
constexpr size_t tma_smem_bytes() {
  return NBUF * tma_buf_words<F, LOGT, C>() * F::WORD + 128;  // + alignment slack
}


enum { LAND_COL = 0, LAND_ROW = 1, XCHG = 2, STAGE = 3 };

template <class F, int LOGT, int C, int LAYOUT>
OMR_D int sidx(int t, int c) {
  constexpr int T = 1 << LOGT;
  if constexpr (LAYOUT == LAND_COL || LAYOUT == STAGE) {
    return t * C + c;
  } else if constexpr (LAYOUT == LAND_ROW) {
    return c * (T + land_pad<F, C>()) + t;
  } else {
    return t * C + c + (t >> xchg_shift<F, LOGT>()) * xchg_pad<F>();
  }
}

// Twiddle tables of the pass.
//   rtw: the in-line twiddles of every round r > 0, staged in shared memory
//        once per persistent CTA and laid out [q][jm] so that consecutive
//        butterflies read consecutive words (round r starts at rtw_off(r);
//        entry q*NS + jm = omega_T^(q jm T/(NS R)));
//   lo/hi: the two-level four-step table in global memory (two lookups per
//        16 outputs: the chain base and step).
template <class F>
struct SmemTw {
  const typename F::Tw* rtw;
  const typename F::E* __restrict__ lo;   // four-step table, low part (twiddle-Montgomery form)
  const typename F::Tw* __restrict__ hi;  // four-step table, high part
};

template <int LOGT, int MAXR>
constexpr int rtw_off(int r) {  // offset of round r's table (r >= 1)
  int off = 0;
  for (int k = 1; k < r; k++) off += (1 << RoundPlan<LOGT, MAXR>::logr(k)) << RoundPlan<LOGT, MAXR>::logns(k);
  return off;
}
template <int LOGT, int MAXR>
constexpr int rtw_size() {
  return rtw_off<LOGT, MAXR>(RoundPlan<LOGT, MAXR>::ROUNDS);
}
// plus the staged per-round in-line twiddles (see SmemTw)
template <class F, int LOGT, int C, int NBUF>
constexpr size_t tma_smem_total() {
  return tma_smem_bytes<F, LOGT, C, NBUF>() +
         (size_t)rtw_size<LOGT, max_radix_log<F>()>() * sizeof(typename F::Tw);
}

template <class F, int LOGT, int RI>
OMR_D void build_rtw(typename F::Tw* dst, const typename F::Tw* __restrict__ roots,
                     uint32_t roots_stride, int nt) {
  using RP = RoundPlan<LOGT, max_radix_log<F>()>;
  if constexpr (RI < RP::ROUNDS) {
    if constexpr (RI >= 1) {
      constexpr int R = 1 << RP::logr(RI), NS = 1 << RP::logns(RI);
      constexpr int SCALE = (1 << LOGT) / (NS * R);
      constexpr int OFF = rtw_off<LOGT, max_radix_log<F>()>(RI);
      for (int k = threadIdx.x; k < R * NS; k += nt)
        dst[OFF + k] = roots[(uint32_t)((k / NS) * (k % NS) * SCALE) * roots_stride];
    }
    build_rtw<F, LOGT, RI + 1>(dst, roots, roots_stride, nt);
  }
}

// omega_N^e in twiddle-Montgomery form from the two-level table
template <class F>
OMR_D typename F::E tw_lookup(const SmemTw<F>& st, uint32_t e) {
  return F::mul_tw(__ldg(&st.lo[e & ((1u << kTwLoBits) - 1)]), st.hi[e >> kTwLoBits]);
}

template <class F, int LOGT, int C, int NT, int RI, int LOGR, int LOGNS, bool INV, int SRC,
          bool LAST, bool TW>
OMR_D void tma_round(const PassArgs<F>& a, const SmemTw<F>& st, typename F::E* s, uint32_t llo0,
                     uint32_t lm) {
  using E = typename F::E;
  constexpr int T = 1 << LOGT, R = 1 << LOGR, NS = 1 << LOGNS;
  constexpr int TR = T / R;
  constexpr int NB = TR * C;
  constexpr int PER = (NB + NT - 1) / NT;
  E v[PER][R];
  // Goldilocks, 4096-point columns: the four-step twiddle operands of the
  // last round (see below) are loaded before the round's shared-memory reads
  // and barrier, so that the loads' latency overlaps them; the products are
  // formed after the barrier.  NT is a multiple of C, so all groups of a
  // thread lie on one line and share its step.  Measured on GB300: the
  // Goldilocks 2^24 column pass 0.244 -> 0.234 ms.  The 32-bit fields'
  // 64-register kernels got slower with the nine extra live registers, and
  // the 1024-point Goldilocks column pass got slower too, so those look the
  // operands up after the DFT.
  constexpr bool PF = LAST && TW && F::WORD == 8 && LOGT >= 12;
  static_assert(NT % C == 0, "a thread's groups share one line");
  [[maybe_unused]] E base_lo[PF ? PER : 1];
  [[maybe_unused]] typename F::Tw base_hi[PF ? PER : 1];
  [[maybe_unused]] E step_lo{};
  [[maybe_unused]] typename F::Tw step_hi{};
  if constexpr (PF) {
    const uint32_t ls =
        (llo0 + (uint32_t)(threadIdx.x % C) + lm * a.tw_line_mul_m) * a.tw_scale;
    const uint32_t es = (ls * (uint32_t)NS) & a.tw_mask;
    step_lo = __ldg(&st.lo[es & ((1u << kTwLoBits) - 1)]);
    step_hi = st.hi[es >> kTwLoBits];
#pragma unroll
    for (int i = 0; i < PER; i++) {
      const int b = threadIdx.x + i * NT;
      if (NB % NT == 0 || b < NB) {
        const int j = b / C;
        const int d = ((j >> LOGNS) << (LOGNS + LOGR)) | (j & (NS - 1));
        const uint32_t e = (ls * (uint32_t)d) & a.tw_mask;
        base_lo[i] = __ldg(&st.lo[e & ((1u << kTwLoBits) - 1)]);
        base_hi[i] = st.hi[e >> kTwLoBits];
      }
    }
  }
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const int b = threadIdx.x + i * NT;
    if (NB % NT == 0 || b < NB) {
      const int c = b % C, j = b / C;
#pragma unroll
      for (int q = 0; q < R; q++) v[i][q] = s[sidx<F, LOGT, C, SRC>(j + q * TR, c)];
    }
  }
  __syncthreads();  // every read of the buffer precedes its overwrite
  [[maybe_unused]] E step{};
  if constexpr (PF) step = F::mul_tw(step_lo, step_hi);
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const int b = threadIdx.x + i * NT;
    if (NB % NT == 0 || b < NB) {
      const int c = b % C, j = b / C;
      const int jm = j & (NS - 1);
      if constexpr (LOGNS > 0) {
        const typename F::Tw* tw = st.rtw + rtw_off<LOGT, max_radix_log<F>()>(RI) + jm;
#pragma unroll
        for (int q = 1; q < R; q++) v[i][q] = F::mul_tw(v[i][q], tw[q * NS]);
      }
      dft_reg<F, LOGR, INV>(v[i]);
      const int d = ((j >> LOGNS) << (LOGNS + LOGR)) | jm;
      if constexpr (!LAST) {
#pragma unroll
        for (int q = 0; q < R; q++) s[sidx<F, LOGT, C, XCHG>(d + q * NS, c)] = v[i][q];
      } else {
        // outputs k = d + q * NS; four-step twiddle omega_N^(line k scale)
        // = base * step^q, base = omega_N^(line d scale), step = omega_N^(line NS scale)
        if constexpr (TW) {
          E w;
          if constexpr (PF) {
            w = F::mul_tw(base_lo[i], base_hi[i]);
          } else {
            const uint32_t ls = (llo0 + (uint32_t)c + lm * a.tw_line_mul_m) * a.tw_scale;
            w = tw_lookup<F>(st, (ls * (uint32_t)d) & a.tw_mask);
            step = tw_lookup<F>(st, (ls * (uint32_t)NS) & a.tw_mask);
          }
#pragma unroll
          for (int q = 0; q < R; q++) {
            v[i][q] = mul_m<F>(v[i][q], w);
            if (q + 1 < R) w = F::mont_mul(w, step);
          }
        }
        if (a.has_scale) {
#pragma unroll
          for (int q = 0; q < R; q++) v[i][q] = F::mul_tw(v[i][q], a.scale);
        }
#pragma unroll
        for (int q = 0; q < R; q++) s[sidx<F, LOGT, C, STAGE>(d + q * NS, c)] = v[i][q];
      }
    }
  }
  if constexpr (!LAST) __syncthreads();
}

// `between` runs (on every thread) after the barrier that ends the
// second-to-last round: the producer uses it to refill the other buffer.
template <class F, int LOGT, int C, int NT, int MODE, bool INV, bool TW, int I, class Between>
OMR_D void tma_rounds(const PassArgs<F>& a, const SmemTw<F>& st, typename F::E* s, uint32_t llo0,
                      uint32_t lm, Between&& between) {
  using RP = RoundPlan<LOGT, max_radix_log<F>()>;
  if constexpr (I < RP::ROUNDS) {
    constexpr int SRC = I == 0 ? (MODE == MODE_COL ? LAND_COL : LAND_ROW) : XCHG;
    constexpr bool LAST = I + 1 == RP::ROUNDS;
    tma_round<F, LOGT, C, NT, I, RP::logr(I), RP::logns(I), INV, SRC, LAST, TW>(a, st, s, llo0, lm);
    if constexpr (I + 2 == RP::ROUNDS) between();
    tma_rounds<F, LOGT, C, NT, MODE, INV, TW, I + 1>(a, st, s, llo0, lm, between);
  }
}

template <class F, int C>
OMR_D void tile_coords(const PassArgs<F>& a, uint64_t tile, uint32_t& g, uint32_t& lm,
                       uint64_t& lb) {
  const uint32_t groups = (a.L_lo + C - 1) / C;
  if (tile >> 32 == 0) {  // 32-bit divisions (a fraction of the 64-bit ones' cost)
    const uint32_t t = (uint32_t)tile, rest = t / groups;
    g = t - rest * groups;
    lm = rest % a.L_m;
    lb = rest / a.L_m;
    return;
  }
  g = (uint32_t)(tile % groups);
  const uint64_t rest = tile / groups;
  lm = (uint32_t)(rest % a.L_m);
  lb = rest / a.L_m;
}

template <class F, int LOGT, int C, int MODE>
OMR_D void issue_load(const CUtensorMap* map, const PassArgs<F>& a, uint64_t tile,
                      typename F::E* buf, uint64_t* bar) {
  using E = typename F::E;
  constexpr int T = 1 << LOGT;
  uint32_t g, lm;
  uint64_t lb;
  tile_coords<F, C>(a, tile, g, lm, lb);
  if constexpr (MODE == MODE_COL) {
    constexpr int BOX = T < 256 ? T : 256;
    mbar_arrive_expect_tx(bar, (uint32_t)(T * C * F::WORD));
    const int y0 = (int)((lb * a.L_m + lm) * (uint64_t)T);
#pragma unroll 1
    for (int t0 = 0; t0 < T; t0 += BOX) tma_load_2d(buf + t0 * C, map, (int)(g * C), y0 + t0, bar);
  } else {
    const uint32_t llo0 = g * C;
    const E* src = a.in + (lb * a.is_b + lm * a.is_m + (uint64_t)llo0 * a.is_lo);
    mbar_arrive_expect_tx(bar, (uint32_t)(C * T * F::WORD));
#pragma unroll 1
    for (int c = 0; c < C; c++)
      bulk_load(buf + c * (T + land_pad<F, C>()), src + (uint64_t)c * a.is_lo, T * F::WORD, bar);
  }
}

template <class F, int LOGT, int C, int MODE>
OMR_D void issue_store(const CUtensorMap* map, const PassArgs<F>& a, uint64_t tile,
                       const typename F::E* buf) {
  constexpr int T = 1 << LOGT;
  constexpr int BOX = T < 256 ? T : 256;
  uint32_t g, lm;
  uint64_t lb;
  tile_coords<F, C>(a, tile, g, lm, lb);
  int x, y0;
  if constexpr (MODE == MODE_COL) {
    x = (int)(g * C);
    y0 = (int)((lb * a.L_m + lm) * (uint64_t)T);
  } else {
    x = (int)(g * C + lm * (uint32_t)a.os_m);
    y0 = (int)(lb * (uint64_t)T);
  }
#pragma unroll 1
  for (int t0 = 0; t0 < T; t0 += BOX) tma_store_2d(map, x, y0 + t0, buf + t0 * C);
  bulk_commit();
}

// TW: the pass applies the four-step twiddle (column passes).
// NBUF = 2: one CTA per SM, the next tile lands while this one computes.
// NBUF = 1: two CTAs per SM, each loads its next tile after storing the last;
//           the other CTA keeps the SM busy meanwhile.
// Resident CTAs the register budget is sized for: NBUF = 2 one, NBUF = 1 two,
// or -- for the 16-elements-per-thread tiles of 32-bit fields -- as many
// 64-register CTAs as make 1024 threads (four at 2048-point lines).
template <class F, int LOGT, int NT, int NBUF>
constexpr int tma_min_blocks() {
  return (NBUF == 1 && F::WORD == 4 && LOGT >= 11 && NT < 512) ? 1024 / NT : 3 - NBUF;
}

template <class F, int LOGT, int C, int NT, int MODE, bool INV, bool TW, int NBUF>
__global__ void __launch_bounds__(NT, (tma_min_blocks<F, LOGT, NT, NBUF>()))
    ntt_tile_pass_tma(const __grid_constant__ CUtensorMap in_map,
                      const __grid_constant__ CUtensorMap out_map, const PassArgs<F> a, int* err) {
  pdl_entry();
  using E = typename F::E;
  using Tw = typename F::Tw;
  constexpr size_t BW = tma_buf_words<F, LOGT, C>();
  // the dynamic shared memory under its own name (every extern __shared__
  // array starts at the same address) so that its 128-byte alignment does not
  // conflict with the 16-byte declarations of the other kernels in a unit
  extern __shared__ __align__(128) unsigned char tma_smem_raw[];
  unsigned char* smem_raw = tma_smem_raw;
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ int abort_flag;
  // align by pointer arithmetic on the shared array (keeps the state space)
  E* base = reinterpret_cast<E*>(smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u));
  E* bufs[2] = {base, base + (NBUF - 1) * BW};
  Tw* srtw = reinterpret_cast<Tw*>(base + NBUF * BW);

  const uint32_t groups = (a.L_lo + C - 1) / C;
  const uint64_t ntiles = a.L_b * (uint64_t)a.L_m * groups;
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
    fence_proxy_async();
    abort_flag = 0;
  }
  __syncthreads();
  uint64_t tile = blockIdx.x;
  bool outstanding[2] = {false, false};  // a load into the buffer has not been waited for
  if (threadIdx.x == 0) {
    if (tile < ntiles) {
      issue_load<F, LOGT, C, MODE>(&in_map, a, tile, bufs[0], &bars[0]);
      outstanding[0] = true;
    }
    if (NBUF == 2 && tile + gridDim.x < ntiles) {
      issue_load<F, LOGT, C, MODE>(&in_map, a, tile + gridDim.x, bufs[1], &bars[1]);
      outstanding[1] = true;
    }
  }
  build_rtw<F, LOGT, 1>(srtw, a.roots, a.roots_stride, NT);
  const SmemTw<F> st{srtw, a.tw_lo, a.tw_hi};
  // (the first loop iteration's barrier publishes the staged tables)

  uint32_t phase = 0;
  int it = 0;
  for (; tile < ntiles; tile += gridDim.x, it++) {
    const int b = NBUF == 2 ? (it & 1) : 0;
    if (threadIdx.x == 0) {
      if (mbar_wait_bounded(&bars[b], (phase >> b) & 1)) {
        outstanding[b] = false;
      } else {
        atomicExch(err, OMR_NTT_ERR_TIMEOUT);
        abort_flag = 1;
      }
    }
    __syncthreads();
    if (abort_flag) break;
    phase ^= 1u << b;
    uint32_t g, lm;
    uint64_t lb;
    tile_coords<F, C>(a, tile, g, lm, lb);
    // buffer 1 - b held the previous tile: refill it with the next tile once
    // that tile's TMA store has finished reading it (by the second-to-last
    // round it has, so the producer thread does not hold up the barriers)
    auto refill = [&]() {
      if (NBUF == 2 && threadIdx.x == 0 && it > 0 && tile + gridDim.x < ntiles) {
        bulk_wait_read_all();
        fence_proxy_async();
        issue_load<F, LOGT, C, MODE>(&in_map, a, tile + gridDim.x, bufs[1 - b], &bars[1 - b]);
        outstanding[1 - b] = true;
      }
    };
    tma_rounds<F, LOGT, C, NT, MODE, INV, TW, 0>(a, st, bufs[b], g * C, lm, refill);
    fence_proxy_async();  // this thread's staging writes become visible to the TMA store
    __syncthreads();
    if (threadIdx.x == 0) {
      issue_store<F, LOGT, C, MODE>(&out_map, a, tile, bufs[b]);
      if (NBUF == 1 && tile + gridDim.x < ntiles) {
        bulk_wait_read_all();
        fence_proxy_async();
        issue_load<F, LOGT, C, MODE>(&in_map, a, tile + gridDim.x, bufs[0], &bars[0]);
        outstanding[0] = true;
      }
    }
  }
  if (threadIdx.x == 0) {
    bulk_wait_all();  // every store of this CTA has landed in global memory
    // drain this CTA's loads still in flight (bounded) before exiting
    for (int bb = 0; bb < 2; bb++)
      if (outstanding[bb]) mbar_wait_bounded(&bars[bb], (phase >> bb) & 1);
  }
}

// Thread count of the TMA pass: EPT elements per thread.  For 32-bit fields
// at 2048- and 4096-point lines, 16 keeps a thread at <= 64 registers, so a
// tile runs as two 512-thread CTAs per SM (NBUF = 1) whose barriers
// interleave; measured on GB300 that beats 32 elements per thread (16 warps
// per SM) by ~11% at n = 2^24.  Shorter lines keep 32 (their CTAs are small
// already; 16 was ~20% slower on the 1024-point column pass).
template <class F, int LOGT>
constexpr int tma_ept() {
  return F::WORD == 8 ? 16 : (LOGT >= 11 ? 16 : 32);
}
template <class F, int LOGT, int NBUF>
constexpr int tma_threads() {
  constexpr int TC = (1 << LOGT) * tma_cols<F>();
  constexpr int nt = TC / (tma_ept<F, LOGT>() * (3 - NBUF));
  return nt < 128 ? 128 : (nt > 1024 ? 1024 : nt);
}

}  // namespace omr
