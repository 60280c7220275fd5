// ntt_pass.cuh -- the tile pass: batched small NTTs staged in shared memory.
//
// Every full transform in this engine is a sequence of passes.  A pass runs
// a batch of independent T-point NTTs ("lines", T = 2^LOGT <= 4096).  One CTA
// owns C adjacent lines and runs their T-point transforms as radix-2^r
// Stockham rounds: each thread pulls R = 2^r words per butterfly into
// registers, applies the round's twiddles, runs an R-point DFT with
// compile-time roots, and writes the R results in autosorted order.
//
//   * The first round reads global memory straight into registers when
//     adjacent lines are adjacent words (column passes): every load of the
//     thread is issued before the first use, so a CTA keeps T*C/NT loads in
//     flight.  Row passes (a line is a contiguous run) stage the tile through
//     shared memory with the same all-loads-first pattern.
//   * Middle rounds exchange through a swizzled shared-memory tile.
//   * The last round writes global memory straight from registers, applying
//     the four-step twiddle omega_N^(line * k * scale) and the inverse scale.
//
// The pass is the GB300 counterpart of the reference's sub-NTT building
// blocks (inplace_radix2_dit / inplace_radix2_dif_no_derange,
// src/encoders/utils.rs:26-83), its transposes (transpose_par,
// src/encoders/transpose_out_of_place.rs:340-366; here folded into the
// tile loads/stores) and the four-step twiddle scaling
// (src/encoders/winterfell_four_step.rs:63-78).
#pragma once
#include <cstdint>

#include "fields.cuh"

namespace omr {

// Programmatic dependent launch.  Every kernel of the engine is launched with
// the programmatic stream-serialisation attribute (launch_pdl, engine.cuh), so
// its CTAs may start while the previous kernel of the stream finishes.
// griddepcontrol.wait blocks until that kernel has completed and its writes
// are visible; launch_dependents lets the next kernel start.  A kernel calls
// grid_dep_wait() before its first global access (its input may be the
// previous kernel's output, its output that kernel's input).
OMR_D void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
OMR_D void grid_dep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
OMR_D void pdl_entry() {
  grid_dep_wait();
  grid_dep_launch();
}

constexpr int kMaxLogT = 12;   // largest line handled by one pass (4096 points)
constexpr int kTwLoBits = 12;  // two-level four-step twiddle split

// Pass modes (how lines sit in memory).
enum PassMode : int {
  MODE_COL = 0,   // adjacent lines are adjacent words on both sides (is_lo = os_lo = 1)
  MODE_ROW = 1,   // a line is a contiguous run on input (es_in = 1), adjacent on output (os_lo = 1)
  MODE_LINE = 2,  // a line is a contiguous run on both sides (es_in = es_out = 1)
};

template <class F>
struct PassArgs {
  using E = typename F::E;
  using Tw = typename F::Tw;
  const E* in;
  E* out;
  // line geometry: line index = (lb, lm, llo); llo is the fast (adjacent) index
  uint32_t L_lo, L_m;
  uint64_t L_b;
  uint64_t is_lo, is_m, is_b;  // input strides of the line index components
  uint64_t os_lo, os_m, os_b;  // output strides
  uint32_t es_in, es_out;      // element strides along a line (within a transform: < 2^31)
  // in-line roots: roots[k * roots_stride] = omega_T^k (forward or inverse)
  const Tw* roots;
  uint32_t roots_stride;
  // four-step twiddle on outputs: exponent e = (tw_line * k * tw_scale) mod N,
  // tw_line = llo + lm * tw_line_mul_m; tw_lo == nullptr disables it
  const E* tw_lo;   // omega^i (i < 2^12), "twiddle-Montgomery" form
  const Tw* tw_hi;  // omega^(2^12 i)
  uint32_t tw_scale;
  uint32_t tw_mask;  // N - 1
  uint32_t tw_line_mul_m;
  int has_scale;
  Tw scale;  // N^-1 for inverse transforms
  // optional: the four-step twiddles of the 256-point column passes as one
  // table [line][k] (tw_line < 2^13, tw_line_mul_m == 0), replacing the
  // base * step^q chain with one table operand per output
  const Tw* tw_tab;
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

// Goldilocks: 2 has order 192 (2^96 = -1), and omega_64 = 7^((p-1)/64) = 2^39,
// so omega_R^k = 2^(39 (64/R) k mod 192) for R <= 64.
constexpr int gl_root_exp(int logr, int k) { return (39 * (64 >> logr) * k) % 192; }

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
    constexpr int K = J << (LOGR - LEN_LOG);
    constexpr int R = 1 << LOGR;
    constexpr int KK = INV ? ((R - K) % R) : K;
    if constexpr (F::ID == GOLDILOCKS && LOGR <= 6) {
      // omega_R^KK = 2^E: a shift-and-fold multiply; 2^(E - 96) = -2^E swaps the difference
      constexpr int E = gl_root_exp(LOGR, KK);
      static_assert(hpowmod(2, E, F::p64()) == RootConst<F, LOGR, KK>::value, "root as a power of 2");
      if constexpr (E >= 96)
        v[BLK + J + HALF] = F::template mul_pow2<E - 96>(F::sub(w, u));
      else
        v[BLK + J + HALF] = F::template mul_pow2<E>(F::sub(u, w));
    } else {
      constexpr typename F::Tw t = RootConst<F, LOGR, KK>::tw;
      v[BLK + J + HALF] = F::mul_tw(sub_lazy<F>(u, w), t);
    }
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
// column walk (consecutive rows, one column) and a row walk (consecutive
// columns, a few consecutive rows) are free of bank conflicts.
template <class F, int C>
OMR_D int tile_idx(int t, int c) {
  constexpr int ROWB = C * F::WORD;                 // bytes per tile row
  constexpr int SW = ROWB >= 128 ? 1 : 128 / ROWB;  // rows per 128-byte bank line
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

// Radix 16 for every field.  For Goldilocks omega_16 = -2^60, so all of a
// round's in-register twiddles are shift-and-fold multiplies; 3 rounds of a
// 4096-point line (instead of 4 of radix 8) drop a twiddle boundary and an
// exchange, and 16 u64 words per thread still fit without spills.
template <class F>
constexpr int max_radix_log() {
  return 4;
}

// Tile variants: V = 0 -> C = 32 bytes of lines (one DRAM sector per tile
// row), V = 1 -> C = 16 bytes (half the shared memory: two CTAs per SM at
// 4096-point lines).  Threads give each thread EPT elements.
template <class F, int V>
constexpr int tile_cols() {
  return (V == 0 ? 32 : 16) / F::WORD;
}
template <class F>
constexpr int tile_ept() {
  return F::WORD == 8 ? 32 : 64;
}
template <class F, int LOGT, int V>
constexpr int tile_threads() {
  constexpr int TC = (1 << LOGT) * tile_cols<F, V>();
  constexpr int nt = TC / tile_ept<F>();
  return nt < 32 ? 32 : (nt > 1024 ? 1024 : nt);
}
template <class F, int LOGT, int V>
constexpr int tile_min_blocks() {
  // keep <= 128 registers per thread for the 64-element tiles
  return tile_threads<F, LOGT, V>() >= 512 ? 1 : (65536 / 128) / tile_threads<F, LOGT, V>();
}

enum { SRC_GLOBAL = 0, SRC_SMEM = 1 };
enum { DST_SMEM = 0, DST_GLOBAL = 1, DST_STAGE = 2 };  // STAGE: smem tile, four-step twiddle applied

// One Stockham round.  SRC_GLOBAL reads the column-pass input directly (c-fast
// mapping: 8 lines x 4 rows per warp, one sector per row); DST_GLOBAL writes
// the output directly (c-fast, or j-fast for MODE_LINE so a warp writes 32
// consecutive words of one line).
template <class F, int LOGT, int C, int NT, int LOGR, int LOGNS, bool INV, int SRC, int DST,
          bool JF, bool TW>
OMR_D void do_round(const PassArgs<F>& a, typename F::E* s, const typename F::E* __restrict__ gin,
                    typename F::E* __restrict__ gout, int nvalid, uint32_t llo0, uint32_t lm) {
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
      const int c = JF ? b / TR : b % C;
      const int j = JF ? b % TR : b / C;
#pragma unroll
      for (int q = 0; q < R; q++) {
        const int t = j + q * TR;
        if constexpr (SRC == SRC_GLOBAL) {
          v[i][q] = c < nvalid ? gin[(uint32_t)c + (uint32_t)t * a.es_in] : (E)0;
        } else {
          v[i][q] = s[tile_idx<F, C>(t, c)];
        }
      }
    }
  }
  if constexpr (SRC == SRC_SMEM && DST != DST_GLOBAL) __syncthreads();
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const int b = threadIdx.x + i * NT;
    if (NB % NT == 0 || b < NB) {
      const int c = JF ? b / TR : b % C;
      const int j = JF ? b % TR : b / C;
      const int jm = j & (NS - 1);
      if constexpr (LOGNS > 0) {
        // a_q *= omega_{NS*R}^{q*jm} = omega_T^{q*jm*T/(NS*R)}
        constexpr int SCALE = T / (NS * R);
#pragma unroll
        for (int q = 1; q < R; q++)
          v[i][q] = F::mul_tw(v[i][q], a.roots[(uint32_t)(q * jm * SCALE) * a.roots_stride]);
      }
      dft_reg<F, LOGR, INV>(v[i]);
      const int d = ((j >> LOGNS) << (LOGNS + LOGR)) | jm;
      // four-step twiddle of output k = d + q NS: omega_N^(line k scale) =
      // base * step^q, base = omega_N^(line d scale), step = omega_N^(line NS
      // scale); two table lookups per group, one product per output
      [[maybe_unused]] E tw_cur{}, tw_step{};
      [[maybe_unused]] bool has_tw = false;
      if constexpr (TW && DST != DST_SMEM) {
        has_tw = (DST == DST_STAGE || a.tw_lo != nullptr) && c < nvalid;
        if (has_tw) {
          const uint32_t ls = (llo0 + (uint32_t)c + lm * a.tw_line_mul_m) * a.tw_scale;
          const uint32_t eb = (ls * (uint32_t)d) & a.tw_mask, es = (ls * (uint32_t)NS) & a.tw_mask;
          tw_cur = F::mul_tw(a.tw_lo[eb & ((1u << kTwLoBits) - 1)], a.tw_hi[eb >> kTwLoBits]);
          tw_step = F::mul_tw(a.tw_lo[es & ((1u << kTwLoBits) - 1)], a.tw_hi[es >> kTwLoBits]);
        }
      }
#pragma unroll
      for (int q = 0; q < R; q++) {
        const int k = d + q * NS;
        if constexpr (DST == DST_SMEM) {
          s[tile_idx<F, C>(k, c)] = v[i][q];
        } else if constexpr (DST == DST_STAGE) {
          E y = (E)0;
          if (c < nvalid) {
            y = v[i][q];
            if constexpr (TW) {
              y = mul_m<F>(y, tw_cur);
              if (q + 1 < R) tw_cur = F::mont_mul(tw_cur, tw_step);
            }
          }
          s[tile_idx<F, C>(k, c)] = y;
        } else {
          if (c < nvalid) {
            E y = v[i][q];
            if constexpr (TW) {
              if (has_tw) {
                y = mul_m<F>(y, tw_cur);
                if (q + 1 < R) tw_cur = F::mont_mul(tw_cur, tw_step);
              }
            }
            if (a.has_scale) y = F::mul_tw(y, a.scale);
            if constexpr (JF)
              gout[(uint64_t)c * a.os_lo + (uint32_t)k] = y;
            else
              gout[(uint32_t)c + (uint32_t)k * a.es_out] = y;
          }
        }
      }
    }
  }
  if constexpr (DST != DST_GLOBAL) __syncthreads();
}

template <class F, int LOGT, int C, int NT, int MODE, bool INV, int I>
OMR_D void all_rounds(const PassArgs<F>& a, typename F::E* s, const typename F::E* gin,
                      typename F::E* gout, int nvalid, uint32_t llo0, uint32_t lm) {
  using RP = RoundPlan<LOGT, max_radix_log<F>()>;
  if constexpr (I < RP::ROUNDS) {
    constexpr bool first = I == 0, last = I + 1 == RP::ROUNDS;
    constexpr int SRC = (first && MODE == MODE_COL) ? SRC_GLOBAL : SRC_SMEM;
    constexpr int DST = last ? DST_GLOBAL : DST_SMEM;
    constexpr bool JF = last && MODE == MODE_LINE;
    constexpr bool TW = MODE == MODE_COL;
    do_round<F, LOGT, C, NT, RP::logr(I), RP::logns(I), INV, SRC, DST, JF, TW>(a, s, gin, gout,
                                                                              nvalid, llo0, lm);
    all_rounds<F, LOGT, C, NT, MODE, INV, I + 1>(a, s, gin, gout, nvalid, llo0, lm);
  }
}

// ------------------------------------------------------------------ kernel
template <class F, int LOGT, int V, int MODE, bool INV>
__global__ void __launch_bounds__(tile_threads<F, LOGT, V>(), tile_min_blocks<F, LOGT, V>())
    ntt_tile_pass(const PassArgs<F> a) {
  pdl_entry();
  using E = typename F::E;
  constexpr int T = 1 << LOGT;
  constexpr int C = tile_cols<F, V>();
  constexpr int NT = tile_threads<F, LOGT, V>();
  constexpr int TC = T * C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  E* s = reinterpret_cast<E*>(smem_raw);

  const uint32_t groups = (a.L_lo + C - 1) / C;
  uint32_t blk = blockIdx.x;
  const uint32_t g = blk % groups;
  blk /= groups;
  const uint32_t lm = blk % a.L_m;
  const uint64_t lb = blk / a.L_m;
  const uint32_t llo0 = g * C;
  const E* gin = a.in + (lb * a.is_b + lm * a.is_m + llo0 * a.is_lo);
  E* gout = a.out + (lb * a.os_b + lm * a.os_m + llo0 * a.os_lo);
  const int nvalid = (int)min((uint32_t)C, a.L_lo - llo0);

  if constexpr (MODE != MODE_COL) {
    // stage the tile: consecutive threads read consecutive words of one line
    constexpr int PER = (TC + NT - 1) / NT;
    E r[PER];
#pragma unroll
    for (int i = 0; i < PER; i++) {
      const int idx = threadIdx.x + i * NT;
      const int t = idx % T, c = idx / T;
      r[i] = (TC % NT == 0 || idx < TC) && c < nvalid ? gin[(uint64_t)c * a.is_lo + (uint32_t)t] : (E)0;
    }
#pragma unroll
    for (int i = 0; i < PER; i++) {
      const int idx = threadIdx.x + i * NT;
      if (TC % NT == 0 || idx < TC) s[tile_idx<F, C>(idx % T, idx / T)] = r[i];
    }
    __syncthreads();
  }
  all_rounds<F, LOGT, C, NT, MODE, INV, 0>(a, s, gin, gout, nvalid, llo0, lm);
}

}  // namespace omr
