// tuner.cu -- plan candidates, the exhaustive autotuner and the planner database.
//
// A planning point is (field, log2 N, batch, output pattern, output count).
// Its candidate plans are
//   * full transforms  (count == N): every pass split x kernel variant of
//     enumerate_plans (engine.cu);
//   * partial outputs: the pruned decomposition for each line length
//     T >= count (T <= 4096; prefixes and index sets), the strided fold +
//     every plan of the count-point transform, and every full plan followed
//     by a gather.
// omr_ntt_tune_point times every candidate on device buffers it owns (CUDA
// events, L2 flushed before each timed run, median of `reps`); the caller
// records the fastest in the planner database (omr_ntt_planner_*), which the
// planner (plan = -1) consults before its built-in heuristic.  All candidates
// are exact, so the choice changes speed, never a result.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "engine.cuh"
#include "partial.cuh"

namespace omr {

enum Strategy : int { STRAT_FULL = 0, STRAT_DECOMP = 1, STRAT_FOLD = 2, STRAT_GATHER = 3 };

struct Cand {
  int strategy;
  int param;  // full/gather: plan id; decomp: log2 T; fold: plan id of the count-point transform
};

static std::vector<Cand> candidates(int field, uint32_t log_n, int pattern, uint64_t count) {
  (void)field;
  std::vector<Cand> v;
  const uint64_t n = 1ull << log_n;
  const int nfull = (int)plan_table(log_n).size();
  if (count >= n || count == 0) {
    for (int p = 0; p < nfull; p++) v.push_back({STRAT_FULL, p});
    return v;
  }
  if (pattern == OMR_NTT_PATTERN_PREFIX || pattern == OMR_NTT_PATTERN_INDICES) {
    int lt = 0;
    while ((1ull << lt) < count) lt++;
    if (lt == 0) lt = 1;
    for (int t = lt; t <= kMaxLogT && (uint32_t)t < log_n; t++) v.push_back({STRAT_DECOMP, t});
  }
  if (pattern == OMR_NTT_PATTERN_STRIDED && (count & (count - 1)) == 0) {
    uint32_t ls = 0;
    while ((1ull << ls) < count) ls++;
    const int nsub = (int)plan_table(ls).size();
    for (int p = 0; p < nsub; p++) v.push_back({STRAT_FOLD, p});
  }
  for (int p = 0; p < nfull; p++) v.push_back({STRAT_GATHER, p});
  return v;
}

// ------------------------------------------------------------------ plan classes
// A fixed, size-independent plan vocabulary for the learned planner:
//   0..19   full transform: split kind x pass-kernel variant (class = 4 v + kind);
//           v: 0 plain tile pass, 1 TMA double-buffered, 2 TMA two CTAs an SM,
//           3 slab pass, 4 wide pass (256-point passes on 128-byte tiles);
//           kind 0: balanced split with the fewest passes, 1: its reverse,
//           2: balanced with one more pass, 3: large-first (4096, ..., 4096, remainder);
//           class 3 itself (plain tile pass, large-first: never the fastest
//           on GB300) stands for the one-launch cluster plan of 2^13..2^16
//   20..23  decomposition (prefix or index set) with line length next_pow2(count) << j, j = 0..3
//   24..43  strided fold, then the count-point transform with full class (c - 24)
//   44..63  full transform with full class (c - 44), then gather
constexpr int kFullClasses = 20;
constexpr int kDecompClass = kFullClasses, kFoldClass = kDecompClass + 4,
              kGatherClass = kFoldClass + kFullClasses;
constexpr int kNumClasses = kGatherClass + kFullClasses;
constexpr int kClassVariant[5] = {0, 1, 2, kSlabVariant, kWideVariant};

// plan id of full class fc (0..19) for a 2^log_n transform, or -1
static int full_class_plan(uint32_t log_n, int fc) {
  const auto& plans = plan_table(log_n);
  if (log_n == 0) return fc == 0 ? 0 : -1;
  if (fc < 0 || fc >= kFullClasses) return -1;
  if (fc == 3) {
    for (int i = 0; i < (int)plans.size(); i++)
      if (plans[i].variant == kClusterVariant) return i;
    return -1;
  }
  const int variant = kClassVariant[fc / 4], kind = fc % 4;
  const int pmin = std::max<int>(1, (int)((log_n + kMaxLogT - 1) / kMaxLogT));
  const int P = pmin + (kind == 2 ? 1 : 0);
  if ((uint32_t)P > log_n || P > 3) return -1;
  std::vector<int> bal(P);
  for (int i = 0; i < P; i++) bal[i] = (int)(log_n / P) + (i < (int)(log_n % P) ? 1 : 0);
  if (bal[0] > kMaxLogT) return -1;
  std::vector<int> want = bal;
  if (kind == 1) {
    std::reverse(want.begin(), want.end());
    if (want == bal) return -1;  // same as the balanced class
  } else if (kind == 3) {
    if (P < 2) return -1;
    std::fill(want.begin(), want.end(), kMaxLogT);
    want[P - 1] = (int)log_n - kMaxLogT * (P - 1);
    std::vector<int> rev(bal.rbegin(), bal.rend());
    if (want[P - 1] < 1 || want == bal || want == rev) return -1;  // same as another class
  }
  if (P == 1 && variant > 0) return -1;  // single-pass plans have one kernel
  for (int i = 0; i < (int)plans.size(); i++)
    if (plans[i].split == want && plans[i].variant == variant) return i;
  return -1;
}

static bool class_candidate(int field, uint32_t log_n, int pattern, uint64_t count, int cls,
                            Cand* out) {
  (void)field;
  const uint64_t n = 1ull << log_n;
  const bool full = count >= n || count == 0;
  if (cls < 0 || cls >= kNumClasses) return false;
  if (cls < kFullClasses) {
    if (!full) return false;
    int p = full_class_plan(log_n, cls);
    if (p < 0) return false;
    *out = Cand{STRAT_FULL, p};
    return true;
  }
  if (full) return false;
  if (cls < kFoldClass) {
    if ((pattern != OMR_NTT_PATTERN_PREFIX && pattern != OMR_NTT_PATTERN_INDICES) || count > 4096)
      return false;
    int lt = 0;
    while ((1ull << lt) < count) lt++;
    if (lt == 0) lt = 1;
    lt += cls - kDecompClass;
    if (lt > kMaxLogT || (uint32_t)lt >= log_n) return false;
    *out = Cand{STRAT_DECOMP, lt};
    return true;
  }
  if (cls < kGatherClass) {
    if (pattern != OMR_NTT_PATTERN_STRIDED || (count & (count - 1))) return false;
    uint32_t ls = 0;
    while ((1ull << ls) < count) ls++;
    int p = full_class_plan(ls, cls - kFoldClass);
    if (p < 0) return false;
    *out = Cand{STRAT_FOLD, p};
    return true;
  }
  int p = full_class_plan(log_n, cls - kGatherClass);
  if (p < 0) return false;
  *out = Cand{STRAT_GATHER, p};
  return true;
}

// The learned selector installed in the planner (mlp.cu); returns the class
// with the lowest predicted cost among the applicable ones, or -1.
int mlp_select_class(int field, uint32_t log_n, uint64_t batch, int pattern, uint64_t count,
                     const bool* applicable, int n_classes);

static bool g_use_mlp = false;

// The network is trusted only inside the domain it was trained on: BabyBear
// or Goldilocks, log2 n in [10, 24], batch <= 512, batch * n <= 2^26 words.
// Outside it the planner falls back to the built-in rule (a 2^27 transform,
// or a KoalaBear one, is not extrapolated).
constexpr uint32_t kMlpMinLogN = 10, kMlpMaxLogN = 24;
constexpr uint64_t kMlpMaxBatch = 512, kMlpMaxWords = 1ull << 26;

static bool mlp_choice(int field, uint32_t log_n, uint64_t batch, int pattern, uint64_t count,
                       Cand* out) {
  if (!g_use_mlp) return false;
  if ((field != BABYBEAR && field != GOLDILOCKS) || log_n < kMlpMinLogN || log_n > kMlpMaxLogN ||
      batch > kMlpMaxBatch ||
      (batch << log_n) > kMlpMaxWords)
    return false;
  bool app[kNumClasses];
  Cand cands[kNumClasses];
  bool any = false;
  for (int c = 0; c < kNumClasses; c++) {
    app[c] = class_candidate(field, log_n, pattern, count, c, &cands[c]);
    any |= app[c];
  }
  if (!any) return false;
  int c = mlp_select_class(field, log_n, batch, pattern, count, app, kNumClasses);
  if (c < 0 || !app[c]) return false;
  *out = cands[c];
  return true;
}

// Learned choice, remembered in the planner database so that later calls for
// the same point skip the network.
static void db_store(int field, uint32_t log_n, uint64_t batch, int pattern, uint64_t count,
                     const Cand& c);
static bool mlp_choice_cached(int field, uint32_t log_n, uint64_t batch, int pattern,
                              uint64_t count, Cand* out) {
  if (!mlp_choice(field, log_n, batch, pattern, count, out)) return false;
  db_store(field, log_n, batch, pattern, count, *out);
  return true;
}

// ------------------------------------------------------------------ planner DB
struct Key {
  int field, log_n, batch_log, pattern, count_log;
  bool operator<(const Key& o) const {
    return std::tie(field, log_n, batch_log, pattern, count_log) <
           std::tie(o.field, o.log_n, o.batch_log, o.pattern, o.count_log);
  }
};
static std::mutex g_db_mu;
static std::map<Key, Cand> g_db;

static int ilog2_ceil(uint64_t x) {
  int l = 0;
  while ((1ull << l) < x) l++;
  return l;
}

static Key make_key(int field, uint32_t log_n, uint64_t batch, int pattern, uint64_t count) {
  const uint64_t n = 1ull << log_n;
  if (count >= n || count == 0) pattern = -1;  // full transform
  return Key{field, (int)log_n, ilog2_ceil(batch ? batch : 1), pattern,
             pattern < 0 ? (int)log_n : ilog2_ceil(count)};
}

static void db_store(int field, uint32_t log_n, uint64_t batch, int pattern, uint64_t count,
                     const Cand& c) {
  std::lock_guard<std::mutex> lk(g_db_mu);
  g_db[make_key(field, log_n, batch, pattern, count)] = c;
}

static bool db_lookup(int field, uint32_t log_n, uint64_t batch, int pattern, uint64_t count,
                      Cand* out) {
  std::lock_guard<std::mutex> lk(g_db_mu);
  auto it = g_db.find(make_key(field, log_n, batch, pattern, count));
  if (it == g_db.end()) return false;
  *out = it->second;
  return true;
}

// Built-in heuristic (from the exhaustive tuner's timings on GB300): two
// passes of short lines at 2^10..2^12, the wide pass where a transform splits
// into 256-point passes only (2^24 = 256^3, and batches of 2^16 = 256^2; one
// 2^16 transform is latency bound and takes the cluster plan), the one-launch
// cluster plan for small or batched 2^13..2^16 transforms, else the slab pass
// with one more pass than the fewest (Goldilocks) or the TMA two-CTA pass on
// the balanced split (32-bit fields), else plan 0.
static int heuristic_full_plan(int field, uint32_t log_n, uint64_t batch) {
  const auto& plans = plan_table(log_n);
  if (plans.size() <= 1) return 0;
  // 2^10..2^12: two passes of short lines on the two-CTA variant (class 10)
  // beat the one-CTA single pass by 20-90% on GB300 (one CTA per transform
  // leaves the GPU idle); below 2^10 the single launch stays
  if (log_n >= 10 && log_n <= 12) {
    const int p = full_class_plan(log_n, 4 * 2 + 2);
    if (p >= 0) return p;
  }
  if (plans[0].split.size() < 2) return 0;
  if (log_n == 24 || (log_n == 16 && batch >= 8))
    for (int i = 0; i < (int)plans.size(); i++)
      if (plans[i].variant == kWideVariant &&
          std::all_of(plans[i].split.begin(), plans[i].split.end(), [](int t) { return t == 8; }))
        return i;
  // the one-launch cluster plan wins where latency dominates: up to 2^14, or
  // batches of 8 and more (one cluster per transform)
  if (log_n <= 14 || batch >= 8)
    for (int i = 0; i < (int)plans.size(); i++)
      if (plans[i].variant == kClusterVariant) return i;
  // Goldilocks 2^15..2^23: the slab pass on the balanced split with one more
  // pass (class 14)
  if (field == GOLDILOCKS) {
    const int p = full_class_plan(log_n, 4 * 3 + 2);
    if (p >= 0) return p;
  }
  size_t nsplit = 0;
  for (auto& p : plans)
    if (p.variant == 0) nsplit++;
  // 32-bit fields: variant 2 (two CTAs per SM at <= 64 registers);
  // Goldilocks: variant 1 (double-buffered)
  const bool narrow = field != GOLDILOCKS;
  const int cand = (int)nsplit * (narrow ? 2 : 1);  // first (balanced) split
  return cand < (int)plans.size() ? cand : 0;
}

int planned_full_plan(int field, uint32_t log_n, uint64_t batch, bool use_learned) {
  Cand c;
  const int n = (int)plan_table(log_n).size();
  if (db_lookup(field, log_n, batch, -1, 0, &c) && c.strategy == STRAT_FULL && c.param < n)
    return c.param;
  if (use_learned && mlp_choice_cached(field, log_n, batch, -1, 0, &c) && c.strategy == STRAT_FULL &&
      c.param < n)
    return c.param;
  return heuristic_full_plan(field, log_n, batch);
}

// Planner choice for a partial request: database, learned selector, else 0
// (the caller's built-in heuristic).
int planned_partial(int field, uint32_t log_n, int pattern, uint64_t count, int* strategy,
                    int* param) {
  Cand c;
  if (db_lookup(field, log_n, 1, pattern, count, &c) ||
      mlp_choice_cached(field, log_n, 1, pattern, count, &c)) {
    *strategy = c.strategy;
    *param = c.param;
    return 1;
  }
  return 0;
}

// ------------------------------------------------------------------ executors
int run_partial_strategy(omr_ntt_domain_s* d, int strategy, int param, int pattern,
                         uint64_t count, const uint32_t* indices, const void* in, void* out,
                         cudaStream_t stream);

static int run_candidate(omr_ntt_domain_s* d, const Cand& c, int pattern, uint64_t count,
                         const uint32_t* indices, const void* in, void* out, uint64_t batch,
                         cudaStream_t stream) {
  if (c.strategy == STRAT_FULL) return run_transform(d, c.param, false, in, out, batch, stream);
  const size_t w = word_bytes(d->field);
  for (uint64_t b = 0; b < batch; b++) {
    int rc = run_partial_strategy(d, c.strategy, c.param, pattern, count, indices,
                                  static_cast<const char*>(in) + b * d->n * w,
                                  static_cast<char*>(out) + b * count * w, stream);
    if (rc) return rc;
  }
  return OMR_NTT_OK;
}

template <class F>
__global__ void fill_random_kernel(typename F::E* x, uint64_t n, uint64_t seed) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    x[i] = (typename F::E)(z % F::p64());
  }
}

}  // namespace omr

using namespace omr;

extern "C" {

// Planner database -----------------------------------------------------------

int omr_ntt_planner_set(int field, uint32_t log_n, uint64_t batch, int pattern, uint64_t count,
                        int strategy, int param) {
  if (!valid_field(field) || (int)log_n > two_adicity(field))
    return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "bad field or size");
  std::lock_guard<std::mutex> lk(g_db_mu);
  g_db[make_key(field, log_n, batch, pattern, count)] = Cand{strategy, param};
  return OMR_NTT_OK;
}

int omr_ntt_planner_get(int field, uint32_t log_n, uint64_t batch, int pattern, uint64_t count,
                        int* strategy, int* param) {
  Cand c;
  if (!db_lookup(field, log_n, batch, pattern, count, &c)) return 0;
  if (strategy) *strategy = c.strategy;
  if (param) *param = c.param;
  return 1;
}

int omr_ntt_planner_clear(void) {
  std::lock_guard<std::mutex> lk(g_db_mu);
  g_db.clear();
  return OMR_NTT_OK;
}

int omr_ntt_planner_save(const char* path) {
  if (!path) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null path");
  std::lock_guard<std::mutex> lk(g_db_mu);
  std::ofstream f(path);
  if (!f) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, std::string("cannot write ") + path);
  f << "# omr-ntt planner db: field log_n batch_log pattern count_log strategy param\n";
  for (auto& kv : g_db)
    f << kv.first.field << ' ' << kv.first.log_n << ' ' << kv.first.batch_log << ' '
      << kv.first.pattern << ' ' << kv.first.count_log << ' ' << kv.second.strategy << ' '
      << kv.second.param << '\n';
  return OMR_NTT_OK;
}

int omr_ntt_planner_load(const char* path) {
  if (!path) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null path");
  std::ifstream f(path);
  if (!f) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, std::string("cannot read ") + path);
  std::lock_guard<std::mutex> lk(g_db_mu);
  std::string line;
  int n = 0;
  while (std::getline(f, line)) {
    if (line.empty() || line[0] == '#') continue;
    std::istringstream is(line);
    Key k;
    Cand c;
    if (is >> k.field >> k.log_n >> k.batch_log >> k.pattern >> k.count_log >> c.strategy >> c.param) {
      g_db[k] = c;
      n++;
    }
  }
  return n;
}

// Plan classes ---------------------------------------------------------------

int omr_ntt_plan_class_count(void) { return kNumClasses; }

int omr_ntt_plan_class_candidate(int field, uint32_t log_n, int pattern, uint64_t count, int cls,
                                 int* strategy, int* param) {
  if (!valid_field(field) || (int)log_n > two_adicity(field)) return 0;
  Cand c;
  if (!class_candidate(field, log_n, pattern, count, cls, &c)) return 0;
  if (strategy) *strategy = c.strategy;
  if (param) *param = c.param;
  return 1;
}

int omr_ntt_planner_use_mlp(int enable) {
  g_use_mlp = enable != 0;
  return OMR_NTT_OK;
}

// Candidates -----------------------------------------------------------------

int omr_ntt_candidates(int field, uint32_t log_n, int pattern, uint64_t count, int* strategies,
                       int* params, int cap) {
  if (!valid_field(field) || (int)log_n > two_adicity(field))
    return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "bad field or size");
  auto v = candidates(field, log_n, pattern, count);
  for (int i = 0; i < (int)v.size() && i < cap; i++) {
    if (strategies) strategies[i] = v[i].strategy;
    if (params) params[i] = v[i].param;
  }
  return (int)v.size();
}

// Run one candidate on device buffers (batch transforms; partial outputs
// are written `count` words per transform).
int omr_ntt_run_candidate(omr_ntt_domain_t d, int strategy, int param, int pattern, uint64_t count,
                          const uint32_t* indices, const void* in, void* out, uint64_t batch,
                          void* stream) {
  if (!d || !in || !out) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null argument");
  DeviceGuard g(d->device);
  return run_candidate(d, Cand{strategy, param}, pattern, count, indices, in, out, batch,
                       (cudaStream_t)stream);
}

// Time every candidate of the planning point; ms_out[i] = median ms of
// candidate i over `reps` runs (L2 flushed before each).  Returns the number
// of candidates (or a negative status).
int omr_ntt_tune_point(int field, uint32_t log_n, uint64_t batch, int pattern, uint64_t count,
                       int reps, uint64_t seed, float* ms_out, int cap) {
  if (!valid_field(field) || (int)log_n > two_adicity(field) || batch == 0 || reps < 1)
    return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "bad tuning point");
  omr_ntt_domain_t d = nullptr;
  int rc = omr_ntt_domain_create(field, log_n, &d);
  if (rc) return rc;
  const uint64_t n = 1ull << log_n;
  const bool full = count >= n || count == 0;
  const uint64_t outw = full ? n : count;
  const size_t w = word_bytes(field);
  auto cands = candidates(field, log_n, pattern, count);
  void *in = nullptr, *out = nullptr, *flush = nullptr;
  uint32_t* idx = nullptr;
  const size_t flush_bytes = 256ull << 20;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  auto cleanup = [&]() {
    cudaFree(in);
    cudaFree(out);
    cudaFree(flush);
    cudaFree(idx);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    omr_ntt_domain_destroy(d);
  };
  if (cudaMalloc(&in, n * batch * w) != cudaSuccess || cudaMalloc(&out, outw * batch * w) != cudaSuccess ||
      cudaMalloc(&flush, flush_bytes) != cudaSuccess) {
    cleanup();
    return fail(OMR_NTT_ERR_ALLOC, "tuning buffers");
  }
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    cleanup();
    return fail(OMR_NTT_ERR_CUDA, "tuning stream/events");
  }
  rc = with_field(field, [&](auto f) -> int {
    using F = decltype(f);
    fill_random_kernel<F><<<1024, 256, 0, st>>>(static_cast<typename F::E*>(in), n * batch, seed);
    return cudaGetLastError() == cudaSuccess ? OMR_NTT_OK : OMR_NTT_ERR_CUDA;
  });
  if (!rc && pattern == OMR_NTT_PATTERN_INDICES && !full) {
    // seeded distinct indices: a stride coprime to N walks a permutation
    std::vector<uint32_t> h(count);
    uint64_t stride = (seed * 2654435761ull) | 1ull, off = seed % n;
    for (uint64_t j = 0; j < count; j++) h[j] = (uint32_t)((off + j * stride) & (n - 1));
    if (cudaMalloc(&idx, count * 4) != cudaSuccess ||
        cudaMemcpy(idx, h.data(), count * 4, cudaMemcpyHostToDevice) != cudaSuccess)
      rc = fail(OMR_NTT_ERR_ALLOC, "tuning indices");
  }
  for (int i = 0; !rc && i < (int)cands.size(); i++) {
    // warm-up (also builds sub-domains and scratch outside the timed runs)
    rc = run_candidate(d, cands[i], pattern, count, idx, in, out, batch, st);
    if (rc) break;
    std::vector<float> t;
    for (int r = 0; r < reps && !rc; r++) {
      cudaMemsetAsync(flush, r & 0xff, flush_bytes, st);
      cudaEventRecord(e0, st);
      rc = run_candidate(d, cands[i], pattern, count, idx, in, out, batch, st);
      cudaEventRecord(e1, st);
      if (cudaEventSynchronize(e1) != cudaSuccess) rc = fail(OMR_NTT_ERR_CUDA, "tuning sync");
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      t.push_back(ms);
    }
    std::sort(t.begin(), t.end());
    if (i < cap && ms_out) ms_out[i] = t.empty() ? -1.f : t[t.size() / 2];
  }
  if (!rc) rc = omr_ntt_domain_check(d, st);
  cleanup();
  return rc ? rc : (int)cands.size();
}

}  // extern "C"
