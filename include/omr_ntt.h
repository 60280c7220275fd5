/*
 * omr_ntt.h -- C ABI of the GB300 NTT engine (drop-in for the hot path of
 * benbencik/omr-ntt).
 *
 * The reference crate's interface (Rust) is
 *
 *   pub struct NttDomain<F> { N, log_N, omega, twiddles, bitrev_twiddles }
 *                                                   (src/encoder.rs:9-19)
 *   NttDomain::<F>::new(N)                          (src/encoder.rs:23-51)
 *   pub trait NttEncoder<F>: Send + Sync {
 *       fn ntt(&self, buf: &mut [F], domain: &NttDomain<F>);
 *       fn name(&self) -> &str;                     (src/encoder.rs:70-74)
 *   }
 *   encoders::all(log_n) / encoders::all_partial(s) (src/encoders/mod.rs:32-54)
 *
 * over the fields of src/fields.rs.  Each function below names the reference
 * item it replaces.  Elements cross the ABI as canonical words: uint32_t for
 * BabyBear, KoalaBear and TeddyBear, uint64_t for Goldilocks (a Rust shim
 * converts ark-ff's Montgomery-form Fp to and from canonical integers).
 *
 * Errors: the reference panics through assert! (src/encoder.rs:24-32,
 * src/encoders/lambdaworks_radix4.rs:17-21, tfhe_stockham_radix8.rs:17-21,
 * transform_decomposition.rs:28); every function here returns an
 * omr_ntt_status instead and leaves the caller's buffers untouched on a
 * host-detected error.  omr_ntt_last_error() gives a one-line message.
 *
 * Device functions take device pointers and a cudaStream_t passed as void*
 * (NULL = legacy default stream) and are asynchronous.  *_host functions take
 * host pointers, copy through device memory owned by the domain, and are
 * synchronous.  Domains are thread-safe; scratch memory is owned by the domain
 * and kept per stream.
 */
#ifndef OMR_NTT_H
#define OMR_NTT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Fields (src/fields.rs:4-19). */
typedef enum {
  OMR_NTT_BABYBEAR = 0,   /* p = 2^31 - 2^27 + 1, generator 31, 2-adicity 27 (DefaultField) */
  OMR_NTT_GOLDILOCKS = 1, /* p = 2^64 - 2^32 + 1, generator 7,  2-adicity 32 */
  OMR_NTT_KOALABEAR = 2,  /* p = 2^31 - 2^24 + 1, generator 3,  2-adicity 24 */
  OMR_NTT_TEDDYBEAR = 3   /* p = 2^32 - 2^30 + 1, generator 5,  2-adicity 30 */
} omr_ntt_field;

typedef enum {
  OMR_NTT_OK = 0,
  OMR_NTT_ERR_INVALID_ARGUMENT = -1, /* null handle/pointer, unknown id, bad count */
  OMR_NTT_ERR_SIZE = -2,             /* N not a power of two, or log2 N > 2-adicity */
  OMR_NTT_ERR_PRECONDITION = -3,     /* encoder precondition (radix-4: log N even; radix-8: log N % 3 == 0) */
  OMR_NTT_ERR_CUDA = -4,             /* a CUDA runtime call failed */
  OMR_NTT_ERR_ALLOC = -5,            /* device or host allocation failed */
  OMR_NTT_ERR_TIMEOUT = -6,          /* a bounded device-side wait gave up */
  OMR_NTT_ERR_NONCANONICAL = -7,     /* an input word is >= p (checked entry points only) */
  OMR_NTT_ERR_DUPLICATE = -8,        /* an index set repeats an index */
  OMR_NTT_ERR_CAPACITY = -9          /* a batch/queue capacity was exceeded */
} omr_ntt_status;

/* Encoders: the reference's registry (src/encoders/mod.rs:17-25).  Every
 * encoder computes the same natural-order transform; on the GPU the id
 * selects the plan family, and OMR_NTT_AUTO lets the planner choose. */
typedef enum {
  OMR_NTT_AUTO = -1,
  OMR_NTT_ARK_RADIX2 = 0,               /* src/encoders/ark_radix2.rs:12-19 */
  OMR_NTT_DFT = 1,                      /* src/encoders/dft.rs:9-22 */
  OMR_NTT_DFT_PARTIAL = 2,              /* src/encoders/dft.rs:30-89 */
  OMR_NTT_LAMBDA_BOWERS = 3,            /* src/encoders/lambdaworks_bowers.rs:13-173 */
  OMR_NTT_LAMBDA_RADIX4 = 4,            /* src/encoders/lambdaworks_radix4.rs:14-75 */
  OMR_NTT_PLONKY3_LAYER_SPLIT = 5,      /* src/encoders/plonky3_radix2_layer_split.rs:18-97 */
  OMR_NTT_TFHE_STOCKHAM_R8 = 6,         /* src/encoders/tfhe_stockham_radix8.rs:15-140 */
  OMR_NTT_TRANSFORM_DECOMPOSITION = 7,  /* src/encoders/transform_decomposition.rs:10-97 */
  OMR_NTT_TRANSFORM_DECOMPOSITION_V2 = 8, /* src/encoders/transform_decomposition_v2.rs:8-100 */
  OMR_NTT_WINTERFELL_FOUR_STEP = 9      /* src/encoders/winterfell_four_step.rs:19-130 */
} omr_ntt_encoder;

/* Output index patterns for partial transforms.  PREFIX is the reference's
 * semantics (the first m outputs, src/encoders/transform_decomposition.rs:30);
 * STRIDED and INDICES have no reference path. */
typedef enum {
  OMR_NTT_PATTERN_PREFIX = 0,  /* outputs X[0..count) */
  OMR_NTT_PATTERN_STRIDED = 1, /* outputs X[j * (N / count)], j < count; count a power of two */
  OMR_NTT_PATTERN_INDICES = 2  /* outputs X[idx[j]], j < count, idx distinct and < N */
} omr_ntt_pattern;

typedef struct omr_ntt_domain_s *omr_ntt_domain_t;

/* ---------------------------------------------------------------- domain */

/* NttDomain::<F>::new(N) (src/encoder.rs:23-51) with N = 2^log_n.  Builds the
 * device twiddle tables on the current CUDA device (setup, untimed in the
 * reference's benches: benches/ntt_bench_n.rs:10). */
int omr_ntt_domain_create(int field, uint32_t log_n, omr_ntt_domain_t *out);

/* Drop of NttDomain: frees device tables and every per-stream scratch buffer. */
int omr_ntt_domain_destroy(omr_ntt_domain_t d);

/* Synchronise `stream` and report whether any kernel of this domain hit a
 * bounded device-side wait limit since the last check (OMR_NTT_ERR_TIMEOUT;
 * the word is then cleared).  Host-buffer calls check it themselves. */
int omr_ntt_domain_check(omr_ntt_domain_t d, void *stream);

/* NttDomain fields N, log_N, omega (src/encoder.rs:11-14); omega canonical. */
int omr_ntt_domain_info(omr_ntt_domain_t d, int *field, uint64_t *n, uint32_t *log_n,
                        uint64_t *omega);

/* NttDomain::twiddles (bitrev == 0: omega^k, k < N) or bitrev_twiddles
 * (bitrev != 0: omega^bitrev(i, log_N - 1), i < N/2) (src/encoder.rs:15-18,
 * :37-43), copied to host memory `out` of N (resp. N/2) words. */
int omr_ntt_domain_twiddles(omr_ntt_domain_t d, int bitrev, void *out);

/* ---------------------------------------------------------------- encoders */

/* NttEncoder::name (src/encoder.rs:73): the reference encoder's name, or NULL. */
const char *omr_ntt_encoder_name(int encoder);

/* Whether `encoder` accepts log_n (radix-4: even; radix-8: divisible by 3),
 * mirroring the reference's registry filter (src/encoders/mod.rs:39-44). */
int omr_ntt_encoder_supports(int encoder, uint32_t log_n);

/* The plan a full encoder runs for a 2^log_n transform of `field`: each of the
 * reference's algorithms (the files under src/encoders/) maps to the engine plan family
 * with its structure -- WinterfellFourStep the balanced two-pass slab plan,
 * Plonky3Radix2LayerSplit the shorter-pass-first split at log2(N) / 2,
 * LambdaBowers the 256-point wide passes, LambdaRadix4 even-length passes,
 * TfheStockhamRadix8 passes of a multiple of 3 bits on the Stockham tile
 * pass, ArkRadix2 / Dft the planner's choice (also every family's fallback).
 * All plans give the same words.  Returns the plan id, or a negative status
 * (partial encoders, unsupported sizes).  No GPU needed. */
int omr_ntt_encoder_plan(int encoder, int field, uint32_t log_n);

/* NttEncoder::ntt(&self, buf, domain) (src/encoder.rs:71) on a device buffer:
 * in place on `batch` transforms of N words stored back to back.  Partial
 * encoders (DftPartial, TransformDecomposition, TransformDecompositionV2) use
 * `s` and write only buf[..min(2s, N)] of each transform, as the reference
 * does; full encoders ignore `s`. */
int omr_ntt_encode(omr_ntt_domain_t d, int encoder, uint64_t s, void *buf, uint64_t batch,
                   void *stream);

/* Same as omr_ntt_encode on a host buffer (host -> device -> host inside). */
int omr_ntt_encode_host(omr_ntt_domain_t d, int encoder, uint64_t s, void *host_buf,
                        uint64_t batch);

/* ---------------------------------------------------------------- transforms */

/* Forward NTT X[k] = sum_i x[i] omega^(ik), natural order in and out.
 * `in` may equal `out` (in place).  `plan` is a plan id from
 * omr_ntt_plan_* or -1 for the planner's choice.  Replaces the hot call
 * encoder.ntt(&mut buf, &domain) of benches/ntt_bench_n.rs:18-24. */
int omr_ntt_forward(omr_ntt_domain_t d, int plan, const void *in, void *out, uint64_t batch,
                    void *stream);

/* Inverse NTT x[i] = N^-1 sum_k X[k] omega^(-ik) (no reference counterpart). */
int omr_ntt_inverse(omr_ntt_domain_t d, int plan, const void *in, void *out, uint64_t batch,
                    void *stream);

/* Forward NTT like omr_ntt_forward (default plan), for callers that must not
 * allocate device memory during the call (for example a framework that has
 * reserved all device memory for its own allocator, or a latency-bound loop
 * that cannot afford the device-wide synchronisation a cudaMalloc/cudaFree
 * can cause).  It calls no allocator: the multi-pass intermediate lives in a
 * fixed 16 MiB array in device memory that the library declares statically
 * (held by every GPU that loads the library until the process exits).
 * N * batch * word_bytes above 16 MiB fails with OMR_NTT_ERR_CAPACITY.  All
 * calls share that array: calls that overlap on the GPU race on it, so order
 * them (one stream, or events).  The first call on each device looks up the
 * array's device address; under CUDA's lazy module loading that is also when
 * the driver loads the code and reserves the 16 MiB there, and the first
 * launch of each kernel loads it.  So make one warm-up call per device and
 * shape before the region that must not allocate (and before any stream
 * capture).  The plan is the planner database's entry, else the built-in
 * rule (the learned selector allocates on its first use and is skipped).
 * The domain is created beforehand (omr_ntt_domain_create allocates its
 * tables).  No counterpart in the reference. */
int omr_ntt_forward_noalloc(omr_ntt_domain_t d, const void *in, void *out, uint64_t batch,
                            void *stream);

/* Host-buffer forms of the two calls above (synchronous). */
int omr_ntt_forward_host(omr_ntt_domain_t d, int plan, void *host_buf, uint64_t batch);
int omr_ntt_inverse_host(omr_ntt_domain_t d, int plan, void *host_buf, uint64_t batch);

/* Partial-output forward NTT: out[j] = X[sel(j)] for j < count, where sel is
 * the pattern (PREFIX / STRIDED / INDICES).  `indices` (device, uint32_t) is
 * read only for INDICES.  `in` is not modified.  The reference's partial
 * encoders (TransformDecomposition(s), src/encoders/transform_decomposition.rs)
 * are PREFIX with count = min(2s, N). */
int omr_ntt_partial(omr_ntt_domain_t d, int pattern, uint64_t count, const uint32_t *indices,
                    const void *in, void *out, void *stream);

/* Host-buffer form of omr_ntt_partial (indices in host memory). */
int omr_ntt_partial_host(omr_ntt_domain_t d, int pattern, uint64_t count,
                         const uint32_t *indices, const void *in, void *out);

/* Checked entry: returns OMR_NTT_ERR_NONCANONICAL if any input word >= p
 * (device-side scan, one extra read of the input). */
int omr_ntt_check_canonical(omr_ntt_domain_t d, const void *buf, uint64_t words, void *stream);

/* ---------------------------------------------------------------- plans */

/* Plans depend only on (field, log_n); these need no GPU.  A plan is a split
 * of the transform into at most three tile passes (line lengths <= 4096).
 * omr_ntt_plan_count returns the number of plans (or a negative status);
 * omr_ntt_plan_describe writes a short name into `buf` (cap bytes). */
int omr_ntt_plan_count(int field, uint32_t log_n);
int omr_ntt_plan_describe(int field, uint32_t log_n, int plan, char *buf, size_t cap);

/* Pass geometry of `plan` (-1: default) for `batch` transforms, for host-side
 * checking: writes up to `cap` records of 16 uint64 words each and returns the
 * pass count (or a negative status).  Layout of one record:
 * [logT, L_lo, L_m, L_b, is_lo, is_m, is_b, os_lo, os_m, os_b, es_in, es_out,
 *  twiddle(0/1), tw_scale, tw_line_mul_m, (in_buf | out_buf << 8)], with
 * buffers 0 = source, 1 = scratch, 2 = destination. */
int omr_ntt_plan_passes(int field, uint32_t log_n, int plan, uint64_t batch, uint64_t *records,
                        int cap);

/* Run pass `pass` (0-based) of `plan` alone, asynchronously on `stream`, with
 * the pass's buffer roles bound to `src` (source), `scratch` (N * batch words,
 * caller-owned) and `dst` (destination).  Running every pass in order equals
 * omr_ntt_forward / omr_ntt_inverse; used to time and tune passes one at a
 * time.  No reference counterpart (the reference has no pass structure). */
int omr_ntt_plan_run_pass(omr_ntt_domain_t d, int plan, int pass, int inverse, const void *src,
                          void *scratch, void *dst, uint64_t batch, void *stream);

/* ---------------------------------------------------------------- batches */

/* A mixed batch: many requests of different sizes (2^10 <= N <= 2^20),
 * fields (BabyBear, Goldilocks), directions and output sets, executed by one
 * persistent kernel that drains a device-side queue of tile tasks, launched
 * through a CUDA graph captured on the first run.  No reference counterpart
 * (the reference runs one encoder call at a time). */
typedef struct omr_ntt_batch_s *omr_ntt_batch_t;

int omr_ntt_batch_create(omr_ntt_batch_t *out);
int omr_ntt_batch_destroy(omr_ntt_batch_t b);

/* Add one request.  Its N words of input sit at byte offset `in_offset` of
 * the input arena, its output at `out_offset` of the output arena: N words for
 * a full transform (pattern < 0, or count >= N), else `count` words selected
 * by the host index set `host_indices` (pattern OMR_NTT_PATTERN_INDICES).
 * Returns the request's index (>= 0) or a negative status. */
int omr_ntt_batch_add(omr_ntt_batch_t b, int field, uint32_t log_n, int inverse, int pattern,
                      uint64_t count, const uint32_t *host_indices, uint64_t in_offset,
                      uint64_t out_offset);

/* Freeze the batch: plan every request, order the tile tasks, upload the
 * queue, allocate the scratch arena. */
int omr_ntt_batch_build(omr_ntt_batch_t b);
int omr_ntt_batch_info(omr_ntt_batch_t b, uint64_t *requests, uint64_t *tasks,
                       uint64_t *scratch_bytes);

/* Run the whole batch: one graph launch (counter reset + persistent kernel).
 * The graph is re-captured when the arena pointers change. */
int omr_ntt_batch_run(omr_ntt_batch_t b, const void *in, void *out, void *stream);

/* Synchronise and report a bounded dependency wait that gave up. */
int omr_ntt_batch_check(omr_ntt_batch_t b, void *stream);

/* Test-only fault injection (host side): request `req`'s row-pass tasks wait
 * for one column tile more than exist, so their bounded waits (about a
 * second) run out and omr_ntt_batch_check reports OMR_NTT_ERR_TIMEOUT; the
 * CUDA context stays usable.  Use on a throw-away batch. */
int omr_ntt_batch_inject_stall(omr_ntt_batch_t b, uint32_t req);

/* Baseline: the same requests through the plain kernels, one request after
 * another (what a caller of omr_ntt_forward / omr_ntt_inverse would do). */
int omr_ntt_batch_run_per_request(omr_ntt_batch_t b, const void *in, void *out, void *stream);

/* ---------------------------------------------------------------- planner */

/* Candidate plans of a planning point (field, log2 N, output pattern, count;
 * count == N or 0 means the full transform).  Each candidate is a strategy
 * and a parameter: 0 full transform with plan `param`; 1 pruned prefix
 * decomposition with line length 2^param; 2 strided fold then plan `param` of
 * the count-point transform; 3 full plan `param` then gather.  Writes up to
 * `cap` entries and returns the candidate count.  No GPU needed. */
int omr_ntt_candidates(int field, uint32_t log_n, int pattern, uint64_t count, int *strategies,
                       int *params, int cap);

/* Run one candidate on device buffers: `batch` transforms of N words in
 * `in`; full transforms write N words each, partial ones `count` words. */
int omr_ntt_run_candidate(omr_ntt_domain_t d, int strategy, int param, int pattern,
                          uint64_t count, const uint32_t *indices, const void *in, void *out,
                          uint64_t batch, void *stream);

/* Exhaustive autotuner: times every candidate of the planning point on
 * buffers it allocates (seeded random canonical inputs, L2 flushed before each
 * timed run, CUDA events); ms_out[i] = median ms of candidate i over `reps`.
 * Returns the candidate count.  Setup-time tool: it allocates. */
int omr_ntt_tune_point(int field, uint32_t log_n, uint64_t batch, int pattern, uint64_t count,
                       int reps, uint64_t seed, float *ms_out, int cap);

/* Planner database (process-wide): the chosen candidate per planning point
 * (batch and count bucketed to powers of two).  plan = -1 and the partial
 * entry points consult it before the built-in heuristic.  get returns 1 if
 * the point is known; load returns the number of entries read. */
int omr_ntt_planner_set(int field, uint32_t log_n, uint64_t batch, int pattern, uint64_t count,
                        int strategy, int param);
int omr_ntt_planner_get(int field, uint32_t log_n, uint64_t batch, int pattern, uint64_t count,
                        int *strategy, int *param);
int omr_ntt_planner_clear(void);
int omr_ntt_planner_save(const char *path);
int omr_ntt_planner_load(const char *path);

/* ---------------------------------------------------------------- learned planner */

/* Plan classes: a fixed vocabulary of 64 plans independent of N (20 full
 * transform classes: 5 pass kernels x 4 split kinds, class 3 standing for the
 * one-launch cluster plan; 4 decomposition line lengths for prefixes and
 * index sets; 20 strided-fold sub-plan classes; 20 full-then-gather classes).
 * omr_ntt_plan_class_candidate maps class `cls` of a planning point to its
 * concrete candidate (returns 1) or reports it not applicable (0). */
int omr_ntt_plan_class_count(void);
int omr_ntt_plan_class_candidate(int field, uint32_t log_n, int pattern, uint64_t count, int cls,
                                 int *strategy, int *param);
int omr_ntt_planner_use_mlp(int enable);

/* The learned selector: an fp32 MLP (n_in -> n_hidden -> n_hidden -> n_out,
 * ReLU) trained on the GPU by the library's own forward, backward and Adam
 * kernels on the autotuner's timings.  Input: the 10 features of
 * omr_ntt_mlp_features; output: one predicted (centred) log time per plan
 * class.  Installed with omr_ntt_mlp_install, the planner (plan = -1, partial
 * entry points) takes the applicable class with the lowest prediction when
 * its database has no entry.  No reference counterpart. */
typedef struct omr_ntt_mlp_s *omr_ntt_mlp_t;
int omr_ntt_mlp_features(int field, uint32_t log_n, uint64_t batch, int pattern, uint64_t count,
                         float *features10);
int omr_ntt_mlp_create(int n_in, int n_hidden, int n_out, uint64_t seed, omr_ntt_mlp_t *out);
int omr_ntt_mlp_destroy(omr_ntt_mlp_t m);
int omr_ntt_mlp_param_count(omr_ntt_mlp_t m);
int omr_ntt_mlp_get_params(omr_ntt_mlp_t m, float *host);
int omr_ntt_mlp_set_params(omr_ntt_mlp_t m, const float *host);
int omr_ntt_mlp_forward(omr_ntt_mlp_t m, const float *x, int batch, float *y);
int omr_ntt_mlp_gradients(omr_ntt_mlp_t m, const float *x, const float *target, const float *mask,
                          int batch, float *grad, float *loss);
int omr_ntt_mlp_fit(omr_ntt_mlp_t m, const float *x, const float *target, const float *mask, int n,
                    int epochs, int batch, float lr, uint64_t seed, float *loss_history);
int omr_ntt_mlp_install(omr_ntt_mlp_t m);
/* Load a network file ("OMRM", uint32 n_in, n_hidden, n_out, float32 params;
 * omr-ntt_gb300/data/planner_mlp.bin is the network trained on GB300). */
int omr_ntt_mlp_load(const char *path, omr_ntt_mlp_t *out);

/* ---------------------------------------------------------------- misc */

const char *omr_ntt_last_error(void);
const char *omr_ntt_version(void);

#ifdef __cplusplus
}
#endif

#endif /* OMR_NTT_H */
