// ntt_pass_tma.cuh -- persistent, double-buffered tile pass fed by TMA.
//
// Same arithmetic as ntt_tile_pass (ntt_pass.cuh), different data movement:
//   * persistent CTAs walk the tiles of the pass (tile += gridDim.x);
//   * one elected thread lands the NEXT tile in the second shared-memory
//     buffer while the whole CTA computes the current one:
//       - column passes (adjacent lines adjacent in memory): 2-D TMA tiled
//         loads (cp.async.bulk.tensor.2d) of [C columns x 256 rows] boxes;
//       - row passes (a line is a contiguous run): one 1-D bulk copy
//         (cp.async.bulk) per line;
//     completion is tracked by an mbarrier per buffer (expect-tx bytes);
//   * every wait is bounded: on timeout the CTA raises the domain's error
//     word (read back as OMR_NTT_ERR_TIMEOUT), drains its own copies (again
//     bounded) and exits;
//   * rounds exchange through the landed buffer itself; the last round
//     stores straight from registers (c-fast, one DRAM sector per 2 rows).
// Shared-memory layouts (bank-conflict free for the c-fast warp mapping):
//   landing, column pass: [t][c], row t at t*C words (TMA box layout);
//   landing, row pass:    line c at c*(T + PAD) words, PAD = 128/(C*w) words;
//   exchange:             [t'][c], t' = t ^ ((t >> logr0) & (RPB - 1)),
//                         RPB = rows per 128-byte bank line.
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
OMR_D void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

template <class F, int C>
constexpr int land_pad() {
  return 128 / (C * F::WORD);  // words
}
template <class F, int LOGT, int C>
constexpr size_t tma_buf_words() {
  constexpr size_t a = (size_t)(1 << LOGT) * C;
  constexpr size_t b = (size_t)C * ((1 << LOGT) + land_pad<F, C>());
  return ((a > b ? a : b) * F::WORD + 1023) / 1024 * 1024 / F::WORD;  // 1 KiB aligned buffers
}
template <class F, int LOGT, int C>
constexpr size_t tma_smem_bytes() {
  return 2 * tma_buf_words<F, LOGT, C>() * F::WORD + 1024;  // + alignment slack
}

enum { LAND_COL = 0, LAND_ROW = 1, XCHG = 2 };

template <class F, int LOGT, int C, int LAYOUT>
OMR_D int sidx(int t, int c) {
  constexpr int T = 1 << LOGT;
  if constexpr (LAYOUT == LAND_COL) {
    return t * C + c;
  } else if constexpr (LAYOUT == LAND_ROW) {
    return c * (T + land_pad<F, C>()) + t;
  } else {
    constexpr int ROWB = C * F::WORD;
    constexpr int RPB = ROWB >= 128 ? 1 : 128 / ROWB;
    constexpr int LOGR0 = RoundPlan<LOGT, max_radix_log<F>()>::logr(0);
    return (t ^ ((t >> LOGR0) & (RPB - 1))) * C + c;
  }
}

template <class F, int LOGT, int C, int NT, int LOGR, int LOGNS, bool INV, int SRC, bool LAST,
          bool TW>
OMR_D void tma_round(const PassArgs<F>& a, typename F::E* s, typename F::E* __restrict__ gout,
                     int nvalid, uint32_t llo0, uint32_t lm) {
  using E = typename F::E;
  constexpr int T = 1 << LOGT, R = 1 << LOGR, NS = 1 << LOGNS;
  constexpr int TR = T / R;
  constexpr int NB = TR * C;
  constexpr int PER = (NB + NT - 1) / NT;
  E v[PER][R];
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const int b = threadIdx.x + i * NT;
    if (NB % NT == 0 || b < NB) {
      const int c = b % C, j = b / C;
#pragma unroll
      for (int q = 0; q < R; q++) v[i][q] = s[sidx<F, LOGT, C, SRC>(j + q * TR, c)];
    }
  }
  if constexpr (!LAST) __syncthreads();  // every read of the buffer precedes its overwrite
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const int b = threadIdx.x + i * NT;
    if (NB % NT == 0 || b < NB) {
      const int c = b % C, j = b / C;
      const int jm = j & (NS - 1);
      if constexpr (LOGNS > 0) {
        constexpr int SCALE = T / (NS * R);
#pragma unroll
        for (int q = 1; q < R; q++)
          v[i][q] = F::mul_tw(v[i][q], a.roots[(uint32_t)(q * jm * SCALE) * a.roots_stride]);
      }
      dft_reg<F, LOGR, INV>(v[i]);
      const int d = ((j >> LOGNS) << (LOGNS + LOGR)) | jm;
#pragma unroll
      for (int q = 0; q < R; q++) {
        const int k = d + q * NS;
        if constexpr (!LAST) {
          s[sidx<F, LOGT, C, XCHG>(k, c)] = v[i][q];
        } else {
          if (c < nvalid) {
            E y = v[i][q];
            if constexpr (TW) {
              if (a.tw_lo != nullptr) {
                const uint32_t line = llo0 + (uint32_t)c + lm * a.tw_line_mul_m;
                const uint32_t e = (line * (uint32_t)k * a.tw_scale) & a.tw_mask;
                const E tm = F::mul_tw(a.tw_lo[e & ((1u << kTwLoBits) - 1)], a.tw_hi[e >> kTwLoBits]);
                y = mul_m<F>(y, tm);
              }
            }
            if (a.has_scale) y = F::mul_tw(y, a.scale);
            gout[(uint32_t)c + (uint32_t)k * a.es_out] = y;
          }
        }
      }
    }
  }
  if constexpr (!LAST) __syncthreads();
}

template <class F, int LOGT, int C, int NT, int MODE, bool INV, int I>
OMR_D void tma_rounds(const PassArgs<F>& a, typename F::E* s, typename F::E* gout, int nvalid,
                      uint32_t llo0, uint32_t lm) {
  using RP = RoundPlan<LOGT, max_radix_log<F>()>;
  if constexpr (I < RP::ROUNDS) {
    constexpr int SRC = I == 0 ? (MODE == MODE_COL ? LAND_COL : LAND_ROW) : XCHG;
    constexpr bool LAST = I + 1 == RP::ROUNDS;
    tma_round<F, LOGT, C, NT, RP::logr(I), RP::logns(I), INV, SRC, LAST, MODE == MODE_COL>(
        a, s, gout, nvalid, llo0, lm);
    tma_rounds<F, LOGT, C, NT, MODE, INV, I + 1>(a, s, gout, nvalid, llo0, lm);
  }
}

template <class F, int LOGT, int C, int MODE>
OMR_D void issue_tile(const CUtensorMap* map, const PassArgs<F>& a, uint64_t tile,
                      typename F::E* buf, uint64_t* bar) {
  using E = typename F::E;
  constexpr int T = 1 << LOGT;
  const uint32_t groups = (a.L_lo + C - 1) / C;
  const uint32_t g = (uint32_t)(tile % groups);
  const uint64_t rest = tile / groups;
  const uint32_t lm = (uint32_t)(rest % a.L_m);
  const uint64_t lb = rest / a.L_m;
  if constexpr (MODE == MODE_COL) {
    constexpr int BOX = T < 256 ? T : 256;
    mbar_arrive_expect_tx(bar, (uint32_t)(T * C * F::WORD));
    const int y0 = (int)((lb * a.L_m + lm) * (uint64_t)T);
#pragma unroll 1
    for (int t0 = 0; t0 < T; t0 += BOX) tma_load_2d(buf + t0 * C, map, (int)(g * C), y0 + t0, bar);
  } else {
    const uint32_t llo0 = g * C;
    const int nv = (int)min((uint32_t)C, a.L_lo - llo0);
    const E* src = a.in + (lb * a.is_b + lm * a.is_m + (uint64_t)llo0 * a.is_lo);
    mbar_arrive_expect_tx(bar, (uint32_t)(nv * T * F::WORD));
#pragma unroll 1
    for (int c = 0; c < nv; c++)
      bulk_load(buf + c * (T + land_pad<F, C>()), src + (uint64_t)c * a.is_lo, T * F::WORD, bar);
  }
}

template <class F, int LOGT, int C, int NT, int MODE, bool INV>
__global__ void __launch_bounds__(NT, 1)
    ntt_tile_pass_tma(const __grid_constant__ CUtensorMap map, const PassArgs<F> a, int* err) {
  using E = typename F::E;
  constexpr size_t BW = tma_buf_words<F, LOGT, C>();
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ int abort_flag;
  E* base = reinterpret_cast<E*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  E* bufs[2] = {base, base + BW};

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
  if (threadIdx.x == 0) {
    if (tile < ntiles) issue_tile<F, LOGT, C, MODE>(&map, a, tile, bufs[0], &bars[0]);
    if (tile + gridDim.x < ntiles)
      issue_tile<F, LOGT, C, MODE>(&map, a, tile + gridDim.x, bufs[1], &bars[1]);
  }
  uint32_t phase = 0;
  int it = 0;
  for (; tile < ntiles; tile += gridDim.x, it++) {
    const int b = it & 1;
    if (threadIdx.x == 0) {
      if (!mbar_wait_bounded(&bars[b], (phase >> b) & 1)) {
        atomicExch(err, OMR_NTT_ERR_TIMEOUT);
        abort_flag = 1;
      }
    }
    __syncthreads();
    if (abort_flag) break;
    phase ^= 1u << b;
    const uint32_t g = (uint32_t)(tile % groups);
    const uint64_t rest = tile / groups;
    const uint32_t lm = (uint32_t)(rest % a.L_m);
    const uint64_t lb = rest / a.L_m;
    const uint32_t llo0 = g * C;
    const int nvalid = (int)min((uint32_t)C, a.L_lo - llo0);
    E* gout = a.out + (lb * a.os_b + lm * a.os_m + (uint64_t)llo0 * a.os_lo);
    tma_rounds<F, LOGT, C, NT, MODE, INV, 0>(a, bufs[b], gout, nvalid, llo0, lm);
    __syncthreads();  // buffer b fully consumed
    if (threadIdx.x == 0 && tile + 2ull * gridDim.x < ntiles) {
      fence_proxy_async();
      issue_tile<F, LOGT, C, MODE>(&map, a, tile + 2ull * gridDim.x, bufs[b], &bars[b]);
    }
  }
  if (abort_flag && threadIdx.x == 0) {
    // drain this CTA's copies still in flight (bounded) before exiting
    for (int k = 0; k < 2; k++) {
      const uint64_t t = tile + (uint64_t)k * gridDim.x;
      if (t < ntiles) mbar_wait_bounded(&bars[(it + k) & 1], (phase >> ((it + k) & 1)) & 1);
    }
  }
}

// Thread-count variants of the TMA pass: EPT elements per thread.
template <class F, int NTV>
constexpr int tma_ept() {
  return F::WORD == 8 ? (NTV == 0 ? 16 : 8) : (NTV == 0 ? 32 : 16);
}
template <class F>
constexpr int tma_cols() {
  return 16 / F::WORD;  // 16-byte line groups: conflict-free layouts, two buffers fit
}
template <class F, int LOGT, int NTV>
constexpr int tma_threads() {
  constexpr int TC = (1 << LOGT) * tma_cols<F>();
  constexpr int nt = TC / tma_ept<F, NTV>();
  return nt < 32 ? 32 : (nt > 1024 ? 1024 : nt);
}

}  // namespace omr
