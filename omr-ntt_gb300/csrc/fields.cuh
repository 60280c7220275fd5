// fields.cuh -- prime-field arithmetic for the GB300 NTT engine (host + device).
//
// The four fields of the reference crate (src/fields.rs:4-17):
//   BabyBear   p = 2^31 - 2^27 + 1, generator 31, 2-adicity 27
//   KoalaBear  p = 2^31 - 2^24 + 1, generator 3,  2-adicity 24
//   TeddyBear  p = 2^32 - 2^30 + 1, generator 5,  2-adicity 30
//   Goldilocks p = 2^64 - 2^32 + 1, generator 7,  2-adicity 32
//
// Elements cross every boundary in canonical form ([0, p)), one u32 word (the
// 32-bit fields) or one u64 word (Goldilocks).  Inside the kernels:
//   * 31-bit fields (BabyBear, KoalaBear): data stays canonical; a multiply by
//     a precomputed twiddle is Shoup's method (w, w' = floor(w 2^32 / p)), three
//     integer multiplies plus one conditional subtract; a product of two
//     runtime values uses Montgomery reduction with one operand in Montgomery
//     form (x*2^32 mod p).
//   * TeddyBear (p > 2^31): Montgomery only (no 1-bit headroom for Shoup's
//     [0, 2p) intermediate), with carry checks on add/sub.
//   * Goldilocks: 64x64->128 product and the 2^64 = 2^32 - 1, 2^96 = -1 (mod p)
//     folding; twiddles are plain canonical words.
// Roots of unity follow ark-ff's convention used by NttDomain::new
// (src/encoder.rs:53): omega_N = GEN^((p - 1) / N) for N a power of two.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define OMR_HD __host__ __device__ __forceinline__
#define OMR_D __device__ __forceinline__
#else
#define OMR_HD inline
#define OMR_D inline
#endif

namespace omr {

enum FieldId : int { BABYBEAR = 0, GOLDILOCKS = 1, KOALABEAR = 2, TEDDYBEAR = 3 };

// ---------------------------------------------------------------- host helpers
// Exact modular arithmetic for table construction (host side, constexpr).
constexpr uint64_t hmulmod(uint64_t a, uint64_t b, uint64_t p) {
  return (uint64_t)(((unsigned __int128)a * b) % p);
}
constexpr uint64_t hpowmod(uint64_t b, uint64_t e, uint64_t p) {
  uint64_t r = 1 % p;
  b %= p;
  while (e) {
    if (e & 1) r = hmulmod(r, b, p);
    b = hmulmod(b, b, p);
    e >>= 1;
  }
  return r;
}
constexpr uint32_t inv_mod_2_32(uint32_t p) {  // p odd; Newton iteration
  uint32_t x = p;                              // correct to 3 bits
  for (int i = 0; i < 5; i++) x *= 2u - p * x;
  return x;
}

// ---------------------------------------------------------------- 32-bit fields
template <uint32_t P_, uint32_t GEN_, int TA_, int ID_>
struct Field32 {
  using E = uint32_t;
  static constexpr int ID = ID_;
  static constexpr uint32_t P = P_;
  static constexpr uint32_t GEN = GEN_;
  static constexpr int TWO_ADICITY = TA_;
  static constexpr bool SMALL = P_ < 0x80000000u;  // 1 bit of headroom: Shoup + min tricks
  static constexpr uint32_t PINV = inv_mod_2_32(P_);  // p^-1 mod 2^32
  static constexpr int WORD = 4;

  // Twiddle operand as stored in device tables.
  struct Tw {
    uint32_t w;   // SMALL: canonical w ; otherwise w * 2^32 mod p (Montgomery form)
    uint32_t wq;  // SMALL: floor(w * 2^32 / p) ; otherwise unused
  };

  static constexpr uint64_t p64() { return P_; }

  // host: build the twiddle operand for a canonical constant
  static constexpr Tw make_tw(uint64_t w) {
    return SMALL ? Tw{(uint32_t)w, (uint32_t)((w << 32) / P_)}
                 : Tw{(uint32_t)((w << 32) % P_), 0u};
  }
  static constexpr uint32_t to_mont_host(uint64_t w) { return (uint32_t)((w << 32) % P_); }

#if defined(__CUDACC__)
  OMR_D static E add(E a, E b) {
    if constexpr (SMALL) {
      E s = a + b;
      return min(s, s - P);
    } else {
      E s = a + b;
      return (s < a || s >= P) ? s - P : s;
    }
  }
  OMR_D static E sub(E a, E b) {
    if constexpr (SMALL) {
      E d = a - b + P;
      return min(d, d - P);
    } else {
      E d = a - b;
      return a < b ? d + P : d;
    }
  }
  OMR_D static E neg(E a) { return a ? P - a : 0u; }
  // a (canonical or any u32 for Montgomery) times b in Montgomery form -> canonical a*b
  OMR_D static E mont(E a, E bm) {
    uint32_t lo = a * bm;
    uint32_t hi = __umulhi(a, bm);
    uint32_t m = lo * PINV;
    uint32_t mh = __umulhi(m, P);
    uint32_t r = hi - mh;
    return hi < mh ? r + P : r;
  }
  // a * twiddle -> canonical
  OMR_D static E mul_tw(E a, Tw t) {
    if constexpr (SMALL) {
      uint32_t q = __umulhi(a, t.wq);
      uint32_t r = a * t.w - q * P;  // in [0, 2p)
      return min(r, r - P);
    } else {
      return mont(a, t.w);
    }
  }
  // runtime twiddle product: both operands in "twiddle-Montgomery" form, result too.
  // (used for on-the-fly twiddle generation; for SMALL fields the Montgomery
  //  form is kept in Tw.w only by the generator helpers below)
  OMR_D static E mont_mul(E am, E bm) { return mont(am, bm); }
#endif
};

using BabyBear = Field32<0x78000001u, 31u, 27, BABYBEAR>;
using KoalaBear = Field32<0x7f000001u, 3u, 24, KOALABEAR>;
using TeddyBear = Field32<0xc0000001u, 5u, 30, TEDDYBEAR>;

// ---------------------------------------------------------------- Goldilocks
struct Goldilocks {
  using E = uint64_t;
  static constexpr int ID = GOLDILOCKS;
  static constexpr uint64_t P = 0xffffffff00000001ull;
  static constexpr uint64_t EPS = 0xffffffffull;  // 2^64 mod p
  static constexpr uint64_t GEN = 7;
  static constexpr int TWO_ADICITY = 32;
  static constexpr bool SMALL = false;
  static constexpr int WORD = 8;
  struct Tw {
    uint64_t w;
  };
  static constexpr uint64_t p64() { return P; }
  static constexpr Tw make_tw(uint64_t w) { return Tw{w}; }

#if defined(__CUDACC__)
  OMR_D static E add(E a, E b) {
    E s = a + b;
    E t = s + EPS;  // s - p (mod 2^64)
    return (s < a || s >= P) ? t : s;
  }
  OMR_D static E sub(E a, E b) {
    E d = a - b;
    return a < b ? d - EPS : d;  // d + p (mod 2^64)
  }
  OMR_D static E neg(E a) { return a ? P - a : 0ull; }
  OMR_D static E reduce128(uint64_t lo, uint64_t hi) {
    uint64_t hh = hi >> 32, hl = hi & EPS;
    uint64_t t0 = lo - hh;
    if (lo < hh) t0 -= EPS;
    uint64_t t1 = (hl << 32) - hl;  // hl * (2^32 - 1)
    uint64_t t2 = t0 + t1;
    if (t2 < t1) t2 += EPS;
    return t2 >= P ? t2 - P : t2;
  }
  OMR_D static E mul(E a, E b) { return reduce128(a * b, __umul64hi(a, b)); }
  OMR_D static E mul_tw(E a, Tw t) { return mul(a, t.w); }
  OMR_D static E mont_mul(E a, E b) { return mul(a, b); }
#endif
};

// Host-side root of unity (ark convention): omega_N = GEN^((p-1)/N).
template <class F>
constexpr uint64_t root_of_unity_host(int log_n) {
  return hpowmod(F::GEN, (F::p64() - 1) >> log_n, F::p64());
}

}  // namespace omr
