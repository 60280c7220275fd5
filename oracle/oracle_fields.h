/*
 * oracle_fields.h -- scalar prime-field arithmetic for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY: this header belongs to the CPU oracle that checks the
 * GPU engine.  Nothing in the product library includes it.
 *
 * The four fields are the ones declared in the reference crate
 * (src/fields.rs:4-17, via ark-ff's `define_field!`):
 *   BabyBear   p = 2^31 - 2^27 + 1 = 0x78000001, generator 31, 2-adicity 27
 *   KoalaBear  p = 2^31 - 2^24 + 1 = 0x7f000001, generator 3,  2-adicity 24
 *   TeddyBear  p = 2^32 - 2^30 + 1 = 0xc0000001, generator 5,  2-adicity 30
 *   Goldilocks p = 2^64 - 2^32 + 1,              generator 7,  2-adicity 32
 * ark-ff keeps elements in Montgomery form internally; the oracle keeps them
 * canonical ([0, p)), which is the representation compared at every boundary.
 * Exact modular arithmetic is representation independent, so the canonical
 * results are the ones ark-ff would print.
 */
#ifndef OMR_NTT_ORACLE_FIELDS_H
#define OMR_NTT_ORACLE_FIELDS_H

#include <stdint.h>

/* ---- 32-bit fields: products and sums in 64-bit, reduction by % ---- */
#define ORACLE_DEFINE_FIELD32(pref, PVAL)                                         \
  static inline uint32_t pref##_add(uint32_t a, uint32_t b) {                     \
    uint64_t s = (uint64_t)a + b;                                                 \
    return (uint32_t)(s >= (PVAL) ? s - (PVAL) : s);                              \
  }                                                                               \
  static inline uint32_t pref##_sub(uint32_t a, uint32_t b) {                     \
    return a >= b ? a - b : (uint32_t)((uint64_t)a + (PVAL) - b);                 \
  }                                                                               \
  static inline uint32_t pref##_neg(uint32_t a) { return a ? (PVAL) - a : 0; }   \
  static inline uint32_t pref##_mul(uint32_t a, uint32_t b) {                     \
    return (uint32_t)(((uint64_t)a * b) % (PVAL));                                \
  }

ORACLE_DEFINE_FIELD32(bb, 2013265921u)
ORACLE_DEFINE_FIELD32(kb, 2130706433u)
ORACLE_DEFINE_FIELD32(tb, 3221225473u)

/* ---- Goldilocks: 64-bit elements, 128-bit products with the
 *      2^64 = 2^32 - 1, 2^96 = -1 (mod p) folding ---- */
#define GL_P 0xffffffff00000001ull
#define GL_EPS 0xffffffffull /* 2^64 mod p */

static inline uint64_t gl_add(uint64_t a, uint64_t b) {
  uint64_t s = a + b;
  /* a,b < p: a carry out of 64 bits means the true sum is s + 2^64 = s + EPS (mod p) */
  if (s < a) s += GL_EPS;
  if (s >= GL_P) s -= GL_P;
  return s;
}
static inline uint64_t gl_sub(uint64_t a, uint64_t b) {
  return a >= b ? a - b : a + (GL_P - b);
}
static inline uint64_t gl_neg(uint64_t a) { return a ? GL_P - a : 0; }
static inline uint64_t gl_reduce128(unsigned __int128 x) {
  uint64_t lo = (uint64_t)x;
  uint64_t hi = (uint64_t)(x >> 64);
  uint64_t hh = hi >> 32, hl = hi & GL_EPS;
  /* x = lo + hl*2^64 + hh*2^96 = lo + hl*(2^32-1) - hh (mod p) */
  uint64_t t0 = lo - hh;
  if (lo < hh) t0 -= GL_EPS; /* borrow: t0 gained 2^64 = EPS (mod p) */
  uint64_t t1 = hl * GL_EPS;
  uint64_t t2 = t0 + t1;
  if (t2 < t1) t2 += GL_EPS; /* carry: t2 lost 2^64 = EPS (mod p) */
  if (t2 >= GL_P) t2 -= GL_P;
  return t2;
}
static inline uint64_t gl_mul(uint64_t a, uint64_t b) {
  return gl_reduce128((unsigned __int128)a * b);
}

#endif
