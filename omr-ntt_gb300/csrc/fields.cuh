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
// (src/encoder.rs:34): omega_N = GEN^((p - 1) / N) for N a power of two.
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
  // Canonical in, canonical out.  The carry chains are written in PTX so that
  // a borrow or carry becomes a 0 / 0xffffffff mask that is exactly
  // EPS = 2^64 - p in the low word (2^64 = EPS mod p).
  OMR_D static uint64_t pack(uint32_t lo, uint32_t hi) { return ((uint64_t)hi << 32) | lo; }
  // a - b (mod p); also valid for any a < 2^64 (result congruent, < 2^64)
  OMR_D static E sub(E a, E b) {
    uint32_t r0, r1;
    asm("{.reg .u32 m;\n\t"
        "sub.cc.u32 %0, %2, %4;\n\t"
        "subc.cc.u32 %1, %3, %5;\n\t"
        "subc.u32 m, 0, 0;\n\t"       // borrow mask
        "sub.cc.u32 %0, %0, m;\n\t"   // - EPS on borrow (= + p)
        "subc.u32 %1, %1, 0;}"
        : "=&r"(r0), "=&r"(r1)
        : "r"((uint32_t)a), "r"((uint32_t)(a >> 32)), "r"((uint32_t)b), "r"((uint32_t)(b >> 32)));
    return pack(r0, r1);
  }
  // a + b = a - (p - b): one borrow-corrected subtraction
  OMR_D static E add(E a, E b) { return sub(a, P - b); }
  OMR_D static E neg(E a) { return a ? P - a : 0ull; }
  // a + b (2^32 - 1) - c (mod p), canonical; a, c < 2^64, b < 2^32, and
  // a - c + 2^64 > EPS whenever a < c (true for every caller: c < 2^32, or a = 0)
  //
  // w = t + b (2^32 - 1) is one 32x32 -> 64 multiply-add (mad.lo/hi with
  // carry), and each conditional + EPS is a multiply-add of the 0 / 1 carry by
  // 0xffffffff: that work runs on the multiply pipe and leaves the integer ALU
  // pipe -- the bound of the Goldilocks passes -- to the carry chains.  A flag
  // is read only by the instruction family that set it (addc after additions,
  // subc after subtractions): a subtraction's borrow and an addition's carry
  // are not interchangeable in the compiled code.
  OMR_D static E reduce3(uint64_t a, uint32_t b, uint64_t c) {
    uint32_t r0, r1;
    asm("{.reg .u32 t0, t1, x, m;\n\t"
        "sub.cc.u32 t0, %2, %5;\n\t"    // t = a - c
        "subc.cc.u32 t1, %3, %6;\n\t"
        "subc.u32 m, 0, 0;\n\t"         // borrow mask
        "sub.cc.u32 t0, t0, m;\n\t"     // borrow: - EPS
        "subc.u32 t1, t1, 0;\n\t"
        "mad.lo.cc.u32 t0, %4, 0xffffffff, t0;\n\t"   // w = t + b (2^32 - 1)
        "madc.hi.cc.u32 t1, %4, 0xffffffff, t1;\n\t"
        "addc.u32 m, 0, 0;\n\t"         // carry (0 / 1)
        "mad.lo.cc.u32 t0, m, 0xffffffff, t0;\n\t"    // carry: + EPS (cannot carry again)
        "addc.u32 t1, t1, 0;\n\t"
        "add.cc.u32 x, t0, 0xffffffff;\n\t"   // w + EPS carries  <=>  w >= p
        "addc.cc.u32 x, t1, 0;\n\t"
        "addc.u32 m, 0, 0;\n\t"
        "mad.lo.cc.u32 %0, m, 0xffffffff, t0;\n\t"    // w >= p: w + EPS = w - p
        "addc.u32 %1, t1, 0;}"
        : "=&r"(r0), "=&r"(r1)
        : "r"((uint32_t)a), "r"((uint32_t)(a >> 32)), "r"(b), "r"((uint32_t)c),
          "r"((uint32_t)(c >> 32)));
    return pack(r0, r1);
  }
  // a + b (2^32 - 1) (mod p), canonical; reduce3 with c = 0
  OMR_D static E reduce2(uint64_t a, uint32_t b) {
    uint32_t r0, r1;
    asm("{.reg .u32 t0, t1, x, m;\n\t"
        "mad.lo.cc.u32 t0, %4, 0xffffffff, %2;\n\t"
        "madc.hi.cc.u32 t1, %4, 0xffffffff, %3;\n\t"
        "addc.u32 m, 0, 0;\n\t"
        "mad.lo.cc.u32 t0, m, 0xffffffff, t0;\n\t"
        "addc.u32 t1, t1, 0;\n\t"
        "add.cc.u32 x, t0, 0xffffffff;\n\t"
        "addc.cc.u32 x, t1, 0;\n\t"
        "addc.u32 m, 0, 0;\n\t"
        "mad.lo.cc.u32 %0, m, 0xffffffff, t0;\n\t"
        "addc.u32 %1, t1, 0;}"
        : "=&r"(r0), "=&r"(r1)
        : "r"((uint32_t)a), "r"((uint32_t)(a >> 32)), "r"(b));
    return pack(r0, r1);
  }
  // reduce a 128-bit value hi 2^64 + lo:  2^64 = 2^32 - 1, 2^96 = -1
  OMR_D static E reduce128(uint64_t lo, uint64_t hi) {
    return reduce3(lo, (uint32_t)hi, hi >> 32);
  }
  OMR_D static E mul(E a, E b) {
    uint32_t r0, r1, r2, r3;
    const uint32_t a0 = (uint32_t)a, a1 = (uint32_t)(a >> 32), b0 = (uint32_t)b,
                   b1 = (uint32_t)(b >> 32);
    asm("mul.lo.u32 %0, %4, %6;\n\t"
        "mul.hi.u32 %1, %4, %6;\n\t"
        "mad.lo.cc.u32 %1, %4, %7, %1;\n\t"
        "madc.hi.u32 %2, %4, %7, 0;\n\t"
        "mad.lo.cc.u32 %1, %5, %6, %1;\n\t"
        "madc.hi.cc.u32 %2, %5, %6, %2;\n\t"
        "madc.hi.u32 %3, %5, %7, 0;\n\t"
        "mad.lo.cc.u32 %2, %5, %7, %2;\n\t"
        "addc.u32 %3, %3, 0;"
        : "=&r"(r0), "=&r"(r1), "=&r"(r2), "=&r"(r3)
        : "r"(a0), "r"(a1), "r"(b0), "r"(b1));
    return reduce3(pack(r0, r1), r2, r3);
  }
  // x * 2^S for a compile-time 0 <= S < 96, from shifts: x 2^S = a + b 2^64 + c 2^96
  template <int S>
  OMR_D static E mul_pow2(E x) {
    static_assert(S >= 0 && S < 96, "shift out of range");
    if constexpr (S == 0) {
      return x;
    } else if constexpr (S < 32) {
      return reduce2(x << S, (uint32_t)(x >> (64 - S)));
    } else if constexpr (S < 64) {
      return reduce3(x << S, (uint32_t)(x >> (64 - S)), x >> (96 - S));
    } else if constexpr (S == 64) {
      return reduce3(0ull, (uint32_t)x, x >> 32);
    } else {
      return reduce3(0ull, (uint32_t)x << (S - 64), x >> (96 - S));
    }
  }
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
