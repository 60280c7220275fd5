/*
 * ntt_oracle.c -- CPU oracle for the GB300 NTT engine.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark load it; the
 * product library never links it and never falls back to it.
 *
 * It restates, in plain C with OpenMP where the reference uses rayon, every
 * encoder of the reference crate benbencik/omr-ntt (the files under src/encoders/) over
 * the four fields of src/fields.rs, plus an inverse transform (which the
 * reference lacks).  The per-field code is oracle_encoders.inc, included once
 * per field below.
 *
 * PARITY PINNING.  The reference is Rust and cannot be built in this
 * environment, and its own tests hold no golden vectors: they only require
 * every encoder to agree with ArkRadix2 (src/lib.rs:34-54, 114-139), Dft to
 * agree with ArkRadix2 (:85-88), linearity (:90-112) and partial prefixes
 * (:141-180).  The oracle reproduces that agreement matrix and is pinned to an
 * independent big-integer evaluation of the DFT definition (the golden
 * fixtures under tests/golden/).  The absolute choice of omega follows
 * ark-ff's documented convention (GENERATOR^((p-1) >> TWO_ADICITY), squared
 * down to order N); no output of the reference itself pins it, so absolute
 * parity with the reference is "parity unpinned" beyond that convention.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle_fields.h"

enum {
  ORACLE_OK = 0,
  ORACLE_ERR_ARG = -1,
  ORACLE_ERR_SIZE = -2,
  ORACLE_ERR_PRECONDITION = -3,
  ORACLE_ERR_ALLOC = -4,
};

/* Encoder ids: the reference's encoder set (src/encoders/mod.rs:17-25). */
enum {
  ORACLE_ENC_ARK_RADIX2 = 0,
  ORACLE_ENC_DFT = 1,
  ORACLE_ENC_DFT_PARTIAL = 2,
  ORACLE_ENC_BOWERS = 3,
  ORACLE_ENC_RADIX4 = 4,
  ORACLE_ENC_LAYER_SPLIT = 5,
  ORACLE_ENC_STOCKHAM_R8 = 6,
  ORACLE_ENC_TD = 7,
  ORACLE_ENC_TD_V2 = 8,
  ORACLE_ENC_FOUR_STEP = 9,
};

/* Field ids, identical to the product ABI's (include/omr_ntt.h). */
enum { ORACLE_BABYBEAR = 0, ORACLE_GOLDILOCKS = 1, ORACLE_KOALABEAR = 2, ORACLE_TEDDYBEAR = 3 };

/* bitrev (src/encoders/utils.rs:117-119): reverse the low log_len bits. */
static inline uint64_t oracle_bitrev(uint64_t a, uint32_t log_len) {
  if (log_len == 0) return 0;
  uint64_t r = 0;
  for (uint32_t i = 0; i < log_len; i++) r |= ((a >> i) & 1ull) << (log_len - 1 - i);
  return r;
}

static inline size_t oracle_next_pow2(size_t x) {
  size_t p = 1;
  while (p < x) p <<= 1;
  return p;
}

static inline uint32_t oracle_ilog2(size_t x) {
  uint32_t l = 0;
  while (((size_t)1 << (l + 1)) <= x) l++;
  return l;
}

static int g_threads = 0;
static int oracle_threads(void) {
#ifdef _OPENMP
  return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---- instantiate per field ---- */
#define E uint32_t
#define FP(x) bb_##x
#define PMOD 2013265921u
#define GEN 31u
#define TWO_ADICITY 27u
#include "oracle_encoders.inc"
#undef E
#undef FP
#undef PMOD
#undef GEN
#undef TWO_ADICITY

#define E uint32_t
#define FP(x) kb_##x
#define PMOD 2130706433u
#define GEN 3u
#define TWO_ADICITY 24u
#include "oracle_encoders.inc"
#undef E
#undef FP
#undef PMOD
#undef GEN
#undef TWO_ADICITY

#define E uint32_t
#define FP(x) tb_##x
#define PMOD 3221225473u
#define GEN 5u
#define TWO_ADICITY 30u
#include "oracle_encoders.inc"
#undef E
#undef FP
#undef PMOD
#undef GEN
#undef TWO_ADICITY

#define E uint64_t
#define FP(x) gl_##x
#define PMOD GL_P
#define GEN 7ull
#define TWO_ADICITY 32u
#include "oracle_encoders.inc"
#undef E
#undef FP
#undef PMOD
#undef GEN
#undef TWO_ADICITY

/* ---- exported C API (loaded with ctypes by oracle/oracle.py) ---- */

int oracle_set_threads(int n) {
  g_threads = n;
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#endif
  return oracle_threads();
}

int oracle_get_threads(void) { return oracle_threads(); }

/* Run reference encoder `enc` in place on `buf` (N = 2^log_n canonical words). */
int oracle_ntt(int field, int enc, void *buf, uint32_t log_n, uint64_t s) {
  switch (field) {
    case ORACLE_BABYBEAR: return bb_encode(enc, (uint32_t *)buf, log_n, s);
    case ORACLE_KOALABEAR: return kb_encode(enc, (uint32_t *)buf, log_n, s);
    case ORACLE_TEDDYBEAR: return tb_encode(enc, (uint32_t *)buf, log_n, s);
    case ORACLE_GOLDILOCKS: return gl_encode(enc, (uint64_t *)buf, log_n, s);
    default: return ORACLE_ERR_ARG;
  }
}

/* Batched form: `count` independent transforms stored back to back. */
int oracle_ntt_batch(int field, int enc, void *buf, uint32_t log_n, uint64_t s, uint64_t count) {
  size_t w = field == ORACLE_GOLDILOCKS ? 8 : 4;
  for (uint64_t b = 0; b < count; b++) {
    int rc = oracle_ntt(field, enc, (char *)buf + (size_t)b * w * ((size_t)1 << log_n), log_n, s);
    if (rc) return rc;
  }
  return 0;
}

int oracle_inverse(int field, void *buf, uint32_t log_n) {
  switch (field) {
    case ORACLE_BABYBEAR: return bb_inverse((uint32_t *)buf, log_n);
    case ORACLE_KOALABEAR: return kb_inverse((uint32_t *)buf, log_n);
    case ORACLE_TEDDYBEAR: return tb_inverse((uint32_t *)buf, log_n);
    case ORACLE_GOLDILOCKS: return gl_inverse((uint64_t *)buf, log_n);
    default: return ORACLE_ERR_ARG;
  }
}

uint64_t oracle_root_of_unity(int field, uint32_t log_n) {
  switch (field) {
    case ORACLE_BABYBEAR: return bb_root_of_unity(log_n);
    case ORACLE_KOALABEAR: return kb_root_of_unity(log_n);
    case ORACLE_TEDDYBEAR: return tb_root_of_unity(log_n);
    case ORACLE_GOLDILOCKS: return gl_root_of_unity(log_n);
    default: return 0;
  }
}

/* Scalar field ops, exposed so host-side tests can check the arithmetic. */
uint64_t oracle_mul(int field, uint64_t a, uint64_t b) {
  switch (field) {
    case ORACLE_BABYBEAR: return bb_mul((uint32_t)a, (uint32_t)b);
    case ORACLE_KOALABEAR: return kb_mul((uint32_t)a, (uint32_t)b);
    case ORACLE_TEDDYBEAR: return tb_mul((uint32_t)a, (uint32_t)b);
    case ORACLE_GOLDILOCKS: return gl_mul(a, b);
    default: return 0;
  }
}
