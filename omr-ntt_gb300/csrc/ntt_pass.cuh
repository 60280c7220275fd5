// ntt_pass.cuh -- the tile pass: batched small NTTs staged in shared memory.
//
// Every full transform in this engine is a sequence of passes.  A pass runs
// a batch of independent T-point NTTs ("lines", T = 2^LOGT <= 4096).  One CTA
// owns C adjacent lines (C * word = 32 bytes, one DRAM sector per row of the
// tile), loads the T x C tile into shared memory with coalesced accesses,
// runs the T-point transform as radix-2^r Stockham rounds (each round: every
// thread pulls R = 2^r words per butterfly into registers, applies the
// round's twiddles, runs an R-point DFT with compile-time roots, and writes
// the R results back in autosorted order), then stores the tile, optionally
// multiplying each output by the four-step twiddle omega_N^(line * k * scale)
// and/or the inverse-transform scale N^-1.
//
// The pass is the GB300 counterpart of the reference's sub-NTT building
// blocks (inplace_radix2_dit / inplace_radix2_dif_no_derange,
// src/encoders/utils.rs:26-83), its transposes (transpose_par,
// src/encoders/transpose_out_of_place.rs:340-366; here folded into the
// strided tile loads/stores) and the four-step twiddle scaling
// (src/encoders/winterfell_four_step.rs:63-78).
#pragma once
#include <cstdint>

#include "fields.cuh"

namespace omr {

constexpr int kMaxLogT = 12;  // largest line handled by one pass (4096 points)
constexpr int kTwLoBits = 12; // two-level four-step twiddle split

template <class F>
struct PassArgs {
  using E = typename F::E;
  using Tw = typename F::Tw;
  const E* in;
  E* out;
  // line geometry: line index = (lb, lm, llo); llo is the fast (adjacent) index
  uint32_t L_lo, L_m;
  uint64_t is_lo, is_m, is_b;  // input strides of the line index components
  uint64_t os_lo, os_m, os_b;  // output strides
  uint64_t es_in, es_out;      // element strides along a line
  // in-line roots: roots[k * roots_stride] = omega_T^k (forward or inverse)
  const Tw* roots;
  uint32_t roots_stride;
  // four-step twiddle on outputs: exponent e = (tw_line(llo, lm) * k * tw_scale) mod N
  const E* tw_lo;   // omega^i (i < 2^12), "twiddle-Montgomery" form; null = no twiddle
  const Tw* tw_hi;  // omega^(2^12 i)
  uint64_t tw_scale;
  uint64_t tw_mask;  // N - 1
  uint32_t tw_line_mul_m;  // tw_line = llo + lm * tw_line_mul_m
  int has_scale;
  Tw scale;  // N^-1 for inverse transforms
};

// --------------------------------------------------------------- helpers
template <class F>
OMR_D typename F::E sub_lazy(typename F::E a, typename F::E b) {
  if constexpr (F::SMALL) {
    return a - b + F::P;  // in (0, 2p): Shoup's multiply accepts any u32
  } else {
    return F::sub(a, b);
  }
}

// multiply by a runtime value in "twiddle-Montgomery" form (32-bit: x*2^32 mod p)
template <class F>
OMR_D typename F::E mul_m(typename F::E a, typename F::E bm) {
  if constexpr (F::ID == GOLDILOCKS) {
    return F::mul(a, bm);
  } else {
    return F::mont(a, bm);
  }
}

// omega_R^k as a compile-time twiddle operand
template <class F, int LOGR, int K>
struct RootConst {
  static constexpr uint64_t value = hpowmod(root_of_unity_host<F>(LOGR), K, F::p64());
  static constexpr typename F::Tw tw = F::make_tw(value);
};

template <class F, int LOGR, int K, bool INV>
OMR_D typename F::E mul_root(typename F::E x) {
  constexpr int R = 1 << LOGR;
  constexpr int KK = INV ? ((R - K) % R) : K;
  if constexpr (KK == 0) {
    return x;
  } else {
    constexpr typename F::Tw t = RootConst<F, LOGR, KK>::tw;
    return F::mul_tw(x, t);
  }
}

// In-register R-point DFT (R = 2^LOGR), natural order in and out.
// Radix-2 decimation in frequency: (u + v, (u - v) * omega_len^j), outputs in
// bit-reversed register order, undone by compile-time renaming.
template <class F, int LOGR, bool INV, int LEN_LOG, int BLK, int J>
OMR_D void dif_stage_bf(typename F::E* v) {
  constexpr int HALF = 1 << (LEN_LOG - 1);
  using E = typename F::E;
  E u = v[BLK + J], w = v[BLK + J + HALF];
  v[BLK + J] = F::add(u, w);
  if constexpr (J == 0) {
    v[BLK + J + HALF] = F::sub(u, w);
  } else {
    // omega_len^J with len = 2^LEN_LOG
    constexpr int K = J << (LOGR - LEN_LOG);
    constexpr int R = 1 << LOGR;
    constexpr int KK = INV ? ((R - K) % R) : K;
    constexpr typename F::Tw t = RootConst<F, LOGR, KK>::tw;
    v[BLK + J + HALF] = F::mul_tw(sub_lazy<F>(u, w), t);
  }
}

template <class F, int LOGR, bool INV, int LEN_LOG, int I>
OMR_D void dif_stage_iter(typename F::E* v) {
  constexpr int R = 1 << LOGR;
  constexpr int HALF = 1 << (LEN_LOG - 1);
  if constexpr (I < R / 2) {
    constexpr int BLK = (I / HALF) * (2 * HALF);
    constexpr int J = I % HALF;
    dif_stage_bf<F, LOGR, INV, LEN_LOG, BLK, J>(v);
    dif_stage_iter<F, LOGR, INV, LEN_LOG, I + 1>(v);
  }
}

template <class F, int LOGR, bool INV, int LEN_LOG>
OMR_D void dif_stages(typename F::E* v) {
  if constexpr (LEN_LOG >= 1) {
    dif_stage_iter<F, LOGR, INV, LEN_LOG, 0>(v);
    dif_stages<F, LOGR, INV, LEN_LOG - 1>(v);
  }
}

constexpr int bitrev_c(int x, int bits) {
  int r = 0;
  for (int i = 0; i < bits; i++) r |= ((x >> i) & 1) << (bits - 1 - i);
  return r;
}

template <class F, int LOGR, bool INV>
OMR_D void dft_reg(typename F::E (&v)[1 << LOGR]) {
  constexpr int R = 1 << LOGR;
  using E = typename F::E;
  dif_stages<F, LOGR, INV, LOGR>(v);
  E t[R];
#pragma unroll
  for (int k = 0; k < R; k++) t[k] = v[k];
#pragma unroll
  for (int k = 0; k < R; k++) v[k] = t[bitrev_c(k, LOGR)];
}

// Shared-memory tile [T rows][C cols] with an XOR swizzle so that both a
// column walk (32 consecutive rows, one column) and a row walk (consecutive
// columns, a few consecutive rows) are free of bank conflicts.
template <class F, int C>
OMR_D int tile_idx(int t, int c) {
  constexpr int ROWB = C * F::WORD;                  // bytes per tile row
  constexpr int SW = ROWB >= 128 ? 1 : 128 / ROWB;   // rows per 128-byte bank line
  return t * C + (c ^ ((t / SW) & (C - 1)));
}

// Radix of round `i` of a LOGT-point transform split into rounds of <= MAXR bits
template <int LOGT, int MAXR>
struct RoundPlan {
  static constexpr int ROUNDS = (LOGT + MAXR - 1) / MAXR;
  static constexpr int logr(int i) { return LOGT / ROUNDS + (i < LOGT % ROUNDS ? 1 : 0); }
  static constexpr int logns(int i) {
    int s = 0;
    for (int k = 0; k < i; k++) s += logr(k);
    return s;
  }
};

// One Stockham round in shared memory (in place: all reads, barrier, writes).
template <class F, int LOGT, int C, int NT, int LOGR, int LOGNS, bool INV>
OMR_D void stockham_round(typename F::E* s, const typename F::Tw* __restrict__ roots,
                          uint32_t roots_stride) {
  using E = typename F::E;
  constexpr int T = 1 << LOGT, R = 1 << LOGR, NS = 1 << LOGNS;
  constexpr int NB = (T / R) * C;
  constexpr int PER = (NB + NT - 1) / NT;
  E v[PER][R];
#pragma unroll
  for (int i = 0; i < PER; i++) {
    int b = threadIdx.x + i * NT;
    if (NB % NT == 0 || b < NB) {
      int c = b % C, j = b / C;
#pragma unroll
      for (int q = 0; q < R; q++) v[i][q] = s[tile_idx<F, C>(j + q * (T / R), c)];
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < PER; i++) {
    int b = threadIdx.x + i * NT;
    if (NB % NT == 0 || b < NB) {
      int c = b % C, j = b / C;
      int jm = j & (NS - 1);
      if constexpr (LOGNS > 0) {
        // a_q *= omega_{NS*R}^{q*jm} = omega_T^{q*jm*T/(NS*R)}
        constexpr int SCALE = T / (NS * R);
#pragma unroll
        for (int q = 1; q < R; q++)
          v[i][q] = F::mul_tw(v[i][q], roots[(uint32_t)(q * jm * SCALE) * roots_stride]);
      }
      dft_reg<F, LOGR, INV>(v[i]);
      int d = ((j >> LOGNS) << (LOGNS + LOGR)) | jm;
#pragma unroll
      for (int q = 0; q < R; q++) s[tile_idx<F, C>(d + q * NS, c)] = v[i][q];
    }
  }
  __syncthreads();
}

template <class F, int LOGT, int C, int NT, int MAXR, bool INV, int I>
OMR_D void all_rounds(typename F::E* s, const typename F::Tw* roots, uint32_t roots_stride) {
  using RP = RoundPlan<LOGT, MAXR>;
  if constexpr (I < RP::ROUNDS) {
    stockham_round<F, LOGT, C, NT, RP::logr(I), RP::logns(I), INV>(s, roots, roots_stride);
    all_rounds<F, LOGT, C, NT, MAXR, INV, I + 1>(s, roots, roots_stride);
  }
}

template <class F>
constexpr int max_radix_log() {
  return F::WORD == 8 ? 3 : 4;
}

template <class F, int LOGT>
constexpr int pass_threads() {
  constexpr int C = 32 / F::WORD;
  constexpr int TC = (1 << LOGT) * C;
  constexpr int nt = TC / 16;
  return nt < 32 ? 32 : (nt > 512 ? 512 : nt);
}

// ------------------------------------------------------------------ kernel
template <class F, int LOGT, bool INV>
__global__ void __launch_bounds__(pass_threads<F, LOGT>())
    ntt_tile_pass(const PassArgs<F> a) {
  using E = typename F::E;
  constexpr int T = 1 << LOGT;
  constexpr int C = 32 / F::WORD;
  constexpr int NT = pass_threads<F, LOGT>();
  constexpr int TC = T * C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  E* s = reinterpret_cast<E*>(smem_raw);

  const uint32_t groups = (a.L_lo + C - 1) / C;
  uint64_t blk = blockIdx.x;
  const uint32_t g = (uint32_t)(blk % groups);
  blk /= groups;
  const uint32_t lm = (uint32_t)(blk % a.L_m);
  const uint64_t lb = blk / a.L_m;
  const uint32_t llo0 = g * C;
  const uint64_t in_base = lb * a.is_b + lm * a.is_m + llo0 * a.is_lo;
  const uint64_t out_base = lb * a.os_b + lm * a.os_m + llo0 * a.os_lo;

  // ---- load tile: c-fastest when adjacent lines are adjacent in memory
  const bool in_cfast = (a.is_lo == 1);
  for (int i = threadIdx.x; i < TC; i += NT) {
    int t, c;
    if (in_cfast) {
      c = i % C;
      t = i / C;
    } else {
      t = i % T;
      c = i / T;
    }
    E x = 0;
    if (llo0 + c < a.L_lo) x = a.in[in_base + (uint64_t)c * a.is_lo + (uint64_t)t * a.es_in];
    s[tile_idx<F, C>(t, c)] = x;
  }
  __syncthreads();

  all_rounds<F, LOGT, C, NT, max_radix_log<F>(), INV, 0>(s, a.roots, a.roots_stride);

  // ---- store tile (+ four-step twiddle, + inverse scale)
  const bool out_cfast = (a.os_lo == 1);
  for (int i = threadIdx.x; i < TC; i += NT) {
    int k, c;
    if (out_cfast) {
      c = i % C;
      k = i / C;
    } else {
      k = i % T;
      c = i / T;
    }
    if (llo0 + c >= a.L_lo) continue;
    E y = s[tile_idx<F, C>(k, c)];
    if (a.tw_lo != nullptr) {
      uint64_t line = (uint64_t)(llo0 + c) + (uint64_t)lm * a.tw_line_mul_m;
      uint64_t e = (line * (uint64_t)k * a.tw_scale) & a.tw_mask;
      if (e != 0) {
        E tm = F::mul_tw(a.tw_lo[e & ((1u << kTwLoBits) - 1)], a.tw_hi[e >> kTwLoBits]);
        y = mul_m<F>(y, tm);
      }
    }
    if (a.has_scale) y = F::mul_tw(y, a.scale);
    a.out[out_base + (uint64_t)c * a.os_lo + (uint64_t)k * a.es_out] = y;
  }
}

}  // namespace omr
