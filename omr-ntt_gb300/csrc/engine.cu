// engine.cu -- domain objects, device tables, pass plans, and the C ABI of
// the full forward / inverse transforms.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "engine.cuh"
#include "launch_pass.cuh"

namespace omr {

// ------------------------------------------------------------------ errors
static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}

int two_adicity(int field) {
  switch (field) {
    case BABYBEAR: return BabyBear::TWO_ADICITY;
    case GOLDILOCKS: return Goldilocks::TWO_ADICITY;
    case KOALABEAR: return KoalaBear::TWO_ADICITY;
    case TEDDYBEAR: return TeddyBear::TWO_ADICITY;
  }
  return -1;
}

uint64_t modulus(int field) {
  switch (field) {
    case BABYBEAR: return BabyBear::P;
    case GOLDILOCKS: return Goldilocks::P;
    case KOALABEAR: return KoalaBear::P;
    case TEDDYBEAR: return TeddyBear::P;
  }
  return 0;
}

bool valid_field(int field) { return field >= 0 && field <= 3; }

static uint64_t generator(int field) {
  switch (field) {
    case BABYBEAR: return BabyBear::GEN;
    case GOLDILOCKS: return Goldilocks::GEN;
    case KOALABEAR: return KoalaBear::GEN;
    case TEDDYBEAR: return TeddyBear::GEN;
  }
  return 0;
}

// ------------------------------------------------------------------ root tables
static std::mutex g_roots_mu;
static std::map<std::pair<int, int>, RootTables> g_roots;  // (device, field)

template <class F>
static int build_root_tables(RootTables* out) {
  using Tw = typename F::Tw;
  const uint64_t p = F::p64();
  const uint64_t w = root_of_unity_host<F>(kMaxLogT);
  const uint64_t wi = hpowmod(w, p - 2, p);
  const int T = 1 << kMaxLogT;
  std::vector<Tw> f(T), iv(T);
  uint64_t a = 1, b = 1;
  for (int k = 0; k < T; k++) {
    f[k] = F::make_tw(a);
    iv[k] = F::make_tw(b);
    a = hmulmod(a, w, p);
    b = hmulmod(b, wi, p);
  }
  void *df = nullptr, *di = nullptr;
  OMR_CUDA_TRY(cudaMalloc(&df, sizeof(Tw) * T));
  OMR_CUDA_TRY(cudaMalloc(&di, sizeof(Tw) * T));
  OMR_CUDA_TRY(cudaMemcpy(df, f.data(), sizeof(Tw) * T, cudaMemcpyHostToDevice));
  OMR_CUDA_TRY(cudaMemcpy(di, iv.data(), sizeof(Tw) * T, cudaMemcpyHostToDevice));
  out->fwd = df;
  out->inv = di;
  return OMR_NTT_OK;
}

int get_root_tables(int field, RootTables* out) {
  int dev = 0;
  OMR_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_roots_mu);
  auto key = std::make_pair(dev, field);
  auto it = g_roots.find(key);
  if (it != g_roots.end()) {
    *out = it->second;
    return OMR_NTT_OK;
  }
  RootTables rt;
  int rc = with_field(field, [&](auto f) { return build_root_tables<decltype(f)>(&rt); });
  if (rc) return rc;
  g_roots[key] = rt;
  *out = rt;
  return OMR_NTT_OK;
}

// ------------------------------------------------------------------ driver helpers
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static std::atomic<PFN_cuTensorMapEncodeTiled_v12000> fn{nullptr};
  PFN_cuTensorMapEncodeTiled_v12000 f = fn.load();
  if (!f) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess) {
      f = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
      fn.store(f);
    }
  }
  return f;
}

int device_sm_count(int dev) {
  static std::atomic<int> cache[64];
  int v = cache[dev & 63].load();
  if (v <= 0) {
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    if (v <= 0) v = 1;
    cache[dev & 63] = v;
  }
  return v;
}

// ------------------------------------------------------------------ plans
std::vector<PlanShape> enumerate_plans(uint32_t log_n) {
  std::vector<PlanShape> out;
  if (log_n == 0) {
    out.push_back(PlanShape{{}, 0});
    return out;
  }
  int pmin = (int)((log_n + kMaxLogT - 1) / kMaxLogT);
  if (pmin < 1) pmin = 1;
  std::vector<std::vector<int>> splits;
  for (int P = pmin; P <= std::min(3, pmin + 1); P++) {
    if ((uint32_t)P > log_n) break;
    std::vector<int> s(P);
    for (int i = 0; i < P; i++) s[i] = (int)(log_n / P) + (i < (int)(log_n % P) ? 1 : 0);
    if (s[0] > kMaxLogT) continue;
    splits.push_back(s);
    std::vector<int> r(s.rbegin(), s.rend());
    if (r != s) splits.push_back(r);
    if (P == pmin && P >= 2) {
      // uneven splits (remainder, 4096, ..., 4096) and (4096, ..., 4096,
      // remainder): most of the work runs in the 4096-point TMA pass (e.g.
      // 4096 x 1024 at 2^22, the fastest BabyBear plan there)
      std::vector<int> g(P, kMaxLogT);
      g[0] = (int)log_n - kMaxLogT * (P - 1);
      if (g[0] >= 1 && g != s && g != r) {
        splits.push_back(g);
        std::vector<int> gr(g.rbegin(), g.rend());
        if (gr != g) splits.push_back(gr);
      }
    }
  }
  for (int v = 0; v < 3; v++)
    for (auto& s : splits) {
      if (v > 0 && s.size() == 1) continue;  // single-pass plans have one kernel
      out.push_back(PlanShape{s, v});
    }
  // 2^13..2^16: the balanced two-pass plan as one launch on an 8-CTA cluster
  // (appended, so the other plans keep their ids)
  if (log_n >= 13 && log_n <= 16) out.push_back(PlanShape{splits[0], kClusterVariant});
  // the slab pass on every multi-pass split, and the wide pass on those with
  // a 256-point pass (appended: earlier ids unchanged)
  for (auto& s : splits)
    if (s.size() > 1) out.push_back(PlanShape{s, kSlabVariant});
  for (auto& s : splits)
    if (s.size() > 1 && std::find(s.begin(), s.end(), 8) != s.end())
      out.push_back(PlanShape{s, kWideVariant});
  // the tensor-core variant of the wide pass on the splits into 256-point
  // passes only (BabyBear; other fields run these plans on the wide pass)
  for (auto& s : splits)
    if (s.size() > 1 && std::all_of(s.begin(), s.end(), [](int t) { return t == 8; }))
      out.push_back(PlanShape{s, kTcVariant});
  return out;
}

const std::vector<PlanShape>& plan_table(uint32_t log_n) {
  static const std::vector<std::vector<PlanShape>> table = [] {
    std::vector<std::vector<PlanShape>> t;
    for (uint32_t l = 0; l <= 32; l++) t.push_back(enumerate_plans(l));
    return t;
  }();
  static const std::vector<PlanShape> none;
  return log_n <= 32 ? table[log_n] : none;
}

std::vector<PassDesc> build_passes(uint32_t log_n, uint64_t batch, const PlanShape& shape) {
  std::vector<PassDesc> ps;
  const uint64_t N = 1ull << log_n;
  const int P = (int)shape.split.size();
  auto base = [&](int logT) {
    PassDesc d{};
    d.logT = logT;
    d.L_m = 1;
    d.L_b = batch;
    d.is_b = d.os_b = N;
    d.is_m = d.os_m = 0;
    d.twiddle = false;
    d.tw_scale = 1;
    d.tw_line_mul_m = 0;
    return d;
  };
  if (P == 1) {
    // lines are whole transforms
    PassDesc d = base(shape.split[0]);
    d.L_lo = (uint32_t)batch;
    d.L_b = 1;
    d.is_lo = d.os_lo = N;
    d.es_in = d.es_out = 1;
    d.in_buf = 0;
    d.out_buf = 2;
    d.mode = MODE_LINE;
    d.variant = 0;
    ps.push_back(d);
    return ps;
  }
  const uint64_t N1 = 1ull << shape.split[0];
  if (P == 2) {
    const uint64_t N2 = N / N1;
    PassDesc a = base(shape.split[0]);  // columns of length N1, stride N2
    a.L_lo = (uint32_t)N2;
    a.is_lo = a.os_lo = 1;
    a.es_in = a.es_out = N2;
    a.twiddle = true;  // omega_N^(n2 * k1)
    a.in_buf = 0;
    a.out_buf = 1;
    PassDesc b = base(shape.split[1]);  // rows k1 of length N2 -> X[k1 + N1 k2]
    b.L_lo = (uint32_t)N1;
    b.is_lo = N2;
    b.es_in = 1;
    b.os_lo = 1;
    b.es_out = N1;
    b.in_buf = 1;
    b.out_buf = 2;
    a.mode = MODE_COL;
    b.mode = MODE_ROW;
    a.variant = b.variant = shape.variant;
    ps.push_back(a);
    ps.push_back(b);
    return ps;
  }
  // P == 3: N = N1 * N2 * N3
  const uint64_t N2 = 1ull << shape.split[1];
  const uint64_t N3 = 1ull << shape.split[2];
  const uint64_t M2 = N2 * N3;
  PassDesc a = base(shape.split[0]);
  a.L_lo = (uint32_t)M2;
  a.is_lo = a.os_lo = 1;
  a.es_in = a.es_out = M2;
  a.twiddle = true;  // omega_N^(n' * k1)
  a.in_buf = 0;
  a.out_buf = 1;
  PassDesc b = base(shape.split[1]);
  b.L_lo = (uint32_t)N3;
  b.L_m = (uint32_t)N1;  // rows k1
  b.is_lo = b.os_lo = 1;
  b.is_m = b.os_m = M2;
  b.es_in = b.es_out = N3;
  b.twiddle = true;  // omega_{M2}^(n3 * k2) = omega_N^(N1 * n3 * k2)
  b.tw_scale = N1;
  b.in_buf = 1;
  b.out_buf = 1;
  PassDesc c = base(shape.split[2]);
  c.L_lo = (uint32_t)N1;  // k1
  c.L_m = (uint32_t)N2;   // k2
  c.is_lo = M2;
  c.is_m = N3;
  c.es_in = 1;
  c.os_lo = 1;
  c.os_m = N1;
  c.es_out = N1 * N2;
  c.in_buf = 1;
  c.out_buf = 2;
  a.mode = b.mode = MODE_COL;
  c.mode = MODE_ROW;
  a.variant = b.variant = c.variant = shape.variant;
  ps.push_back(a);
  ps.push_back(b);
  ps.push_back(c);
  return ps;
}

int default_plan(int field, uint32_t log_n, uint64_t batch) {
  return planned_full_plan(field, log_n, batch);
}

static std::string plan_name(int field, const PlanShape& s) {
  if (s.split.empty()) return "identity";
  const int v = s.variant == 0 ? 0 : effective_variant(field, MODE_COL, kMaxLogT, s.variant);
  std::string n = s.split.size() == 1 ? "stockham-tile " : "four-step ";
  for (size_t i = 0; i < s.split.size(); i++) {
    if (i) n += "x";
    n += std::to_string(1 << s.split[i]);
  }
  if (s.variant == kClusterVariant) return n + " cluster";
  if (s.variant == kSlabVariant) return n + " slab";
  if (s.variant == kWideVariant) return n + " wide";
  if (s.variant == kTcVariant) return n + " wide-tcgen05";
  if (s.split.size() > 1) n += v == 0 ? " tile" : (v == 1 ? " tma2buf" : " tma2cta");
  return n;
}

// ------------------------------------------------------------------ domain tables
template <class F>
static int build_domain_tables(omr_ntt_domain_s* d) {
  using E = typename F::E;
  using Tw = typename F::Tw;
  const uint64_t p = F::p64();
  const uint64_t n = d->n;
  const size_t nlo = (size_t)std::min<uint64_t>(n, 1ull << kTwLoBits);
  const size_t nhi = (size_t)std::max<uint64_t>(1, n >> kTwLoBits);
  for (int dir = 0; dir < 2; dir++) {
    const uint64_t w = dir == 0 ? d->omega : d->omega_inv;
    std::vector<E> lo(nlo);
    std::vector<Tw> hi(nhi);
    uint64_t a = 1;
    for (size_t i = 0; i < nlo; i++) {
      if constexpr (F::ID == GOLDILOCKS) {
        lo[i] = (E)a;
      } else {
        lo[i] = F::to_mont_host(a);
      }
      a = hmulmod(a, w, p);
    }
    const uint64_t step = hpowmod(w, 1ull << kTwLoBits, p);
    uint64_t b = 1;
    for (size_t i = 0; i < nhi; i++) {
      hi[i] = F::make_tw(b);
      b = hmulmod(b, step, p);
    }
    void *dlo = nullptr, *dhi = nullptr;
    OMR_CUDA_TRY(cudaMalloc(&dlo, sizeof(E) * nlo));
    OMR_CUDA_TRY(cudaMalloc(&dhi, sizeof(Tw) * nhi));
    OMR_CUDA_TRY(cudaMemcpy(dlo, lo.data(), sizeof(E) * nlo, cudaMemcpyHostToDevice));
    OMR_CUDA_TRY(cudaMemcpy(dhi, hi.data(), sizeof(Tw) * nhi, cudaMemcpyHostToDevice));
    if (dir == 0) {
      d->tw_lo_f = dlo;
      d->tw_hi_f = dhi;
    } else {
      d->tw_lo_i = dlo;
      d->tw_hi_i = dhi;
    }
  }
  return OMR_NTT_OK;
}

int domain_scratch(omr_ntt_domain_s* d, void* stream, size_t bytes, void** out, int slot) {
  std::lock_guard<std::mutex> lk(d->mu);
  Scratch& s = d->scratch[std::make_pair(stream, slot)];
  if (s.bytes < bytes) {
    if (s.ptr) {
      // the previous buffer may still be in use by work queued on this stream
      OMR_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
      OMR_CUDA_TRY(cudaFree(s.ptr));
      s.ptr = nullptr;
      s.bytes = 0;
    }
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess)
      return fail(OMR_NTT_ERR_ALLOC, std::string("scratch cudaMalloc: ") + cudaGetErrorString(e));
    s.ptr = p;
    s.bytes = bytes;
  }
  *out = s.ptr;
  return OMR_NTT_OK;
}

int sub_domain(omr_ntt_domain_s* d, uint32_t log_m, omr_ntt_domain_s** out) {
  if (log_m == d->log_n) {
    *out = d;
    return OMR_NTT_OK;
  }
  std::lock_guard<std::mutex> lk(d->mu);
  auto it = d->subs.find(log_m);
  if (it != d->subs.end()) {
    *out = it->second;
    return OMR_NTT_OK;
  }
  omr_ntt_domain_s* s = nullptr;
  int rc = omr_ntt_domain_create(d->field, log_m, &s);
  if (rc) return rc;
  d->subs[log_m] = s;
  *out = s;
  return OMR_NTT_OK;
}

int run_transform(omr_ntt_domain_s* d, int plan, bool inverse, const void* in, void* out,
                  uint64_t batch, cudaStream_t stream) {
  if (plan < 0) plan = default_plan(d->field, d->log_n, batch);
  if (plan >= (int)d->plans.size()) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "plan id out of range");
  const size_t bytes = (size_t)d->n * batch * word_bytes(d->field);
  if (d->log_n == 0) {
    if (in != out) OMR_CUDA_TRY(cudaMemcpyAsync(out, in, bytes, cudaMemcpyDeviceToDevice, stream));
    return OMR_NTT_OK;
  }
  std::vector<PassDesc> ps = build_passes(d->log_n, batch, d->plans[plan]);
  if (d->plans[plan].variant == kClusterVariant) {
    int rc = launch_cluster_transform(d, ps, inverse, in, out, batch, stream);
    if (rc <= 0) return rc;  // launched, or an error; 1: run the passes below
  }
  void* scratch = nullptr;
  if (ps.size() > 1) {
    int rc = domain_scratch(d, stream, bytes, &scratch);
    if (rc) return rc;
  }
  for (size_t i = 0; i < ps.size(); i++) {
    const PassDesc& p = ps[i];
    const void* src = p.in_buf == 0 ? in : (p.in_buf == 1 ? scratch : out);
    void* dst = p.out_buf == 1 ? scratch : out;
    bool last = i + 1 == ps.size();
    int rc = with_field(d->field, [&](auto f) {
      return launch_pass<decltype(f)>(d, p, inverse, src, dst, last, stream);
    });
    if (rc) return rc;
  }
  return OMR_NTT_OK;
}

uint64_t host_chunk(const omr_ntt_domain_s* d, uint64_t batch) {
  // chunks of >= 8 MiB, at least two of them; 0: no pipelining (one transform)
  const uint64_t per = d->n * word_bytes(d->field);
  uint64_t chunk = ((8ull << 20) + per - 1) / per;
  if (chunk > batch / 2) chunk = batch / 2;
  return batch >= 2 ? chunk : 0;
}

// Batches through host buffers: chunks of transforms flow through two device
// buffers on three streams (copy in, transform, copy out), so the copies of
// neighbouring chunks overlap each other and the transforms (the two copy
// directions overlap in part on GB300's host link).  Caller holds d->host_mu.
int host_pipelined(omr_ntt_domain_s* d, char* host, uint64_t batch, uint64_t chunk,
                   const std::function<int(void*, uint64_t, cudaStream_t)>& op) {
  const size_t per = (size_t)d->n * word_bytes(d->field);
  for (auto& s : d->host_streams)
    if (!s && cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
      return fail(OMR_NTT_ERR_CUDA, "host-pipeline stream");
  cudaStream_t sh = d->host_streams[0], sc = d->host_streams[1], sd = d->host_streams[2];
  void* buf[2] = {nullptr, nullptr};
  int rc = domain_scratch(d, sh, chunk * per, &buf[0], 2);
  if (!rc) rc = domain_scratch(d, sd, chunk * per, &buf[1], 2);
  if (rc) return rc;
  cudaEvent_t ev[3][2] = {};  // copied in / transformed / copied out, per buffer
  for (auto& row : ev)
    for (auto& e : row)
      if (!rc && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
        rc = fail(OMR_NTT_ERR_CUDA, "host-pipeline event");
  for (uint64_t off = 0, i = 0; !rc && off < batch; off += chunk, i++) {
    const int b = (int)(i & 1);
    const uint64_t cnt = batch - off < chunk ? batch - off : chunk;
    char* h = host + off * per;
    if (i >= 2) cudaStreamWaitEvent(sh, ev[2][b], 0);  // buffer b copied out
    if (cudaMemcpyAsync(buf[b], h, cnt * per, cudaMemcpyHostToDevice, sh) != cudaSuccess) {
      rc = fail(OMR_NTT_ERR_CUDA, "host-to-device copy failed");
      break;
    }
    cudaEventRecord(ev[0][b], sh);
    cudaStreamWaitEvent(sc, ev[0][b], 0);
    rc = op(buf[b], cnt, sc);
    if (rc) break;
    cudaEventRecord(ev[1][b], sc);
    cudaStreamWaitEvent(sd, ev[1][b], 0);
    if (cudaMemcpyAsync(h, buf[b], cnt * per, cudaMemcpyDeviceToHost, sd) != cudaSuccess) {
      rc = fail(OMR_NTT_ERR_CUDA, "device-to-host copy failed");
      break;
    }
    cudaEventRecord(ev[2][b], sd);
  }
  // every queued copy ends before the host buffer is handed back
  for (cudaStream_t s : {sh, sc, sd}) {
    cudaError_t se = cudaStreamSynchronize(s);
    if (!rc && se != cudaSuccess) rc = fail(OMR_NTT_ERR_CUDA, cudaGetErrorString(se));
  }
  for (auto& row : ev)
    for (auto& e : row)
      if (e) cudaEventDestroy(e);
  if (!rc) rc = omr_ntt_domain_check(d, sc);
  return rc;
}

}  // namespace omr

using namespace omr;

// ====================================================================== C ABI
extern "C" {

const char* omr_ntt_last_error(void) { return g_last_error.c_str(); }

const char* omr_ntt_version(void) { return "omr-ntt-gb300 0.1 (sm_103a)"; }

int omr_ntt_domain_create(int field, uint32_t log_n, omr_ntt_domain_t* out) {
  if (!out) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null output handle");
  *out = nullptr;
  if (!valid_field(field)) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "unknown field id");
  // NttDomain::new asserts log2 N <= TWO_ADICITY (src/encoder.rs:28-32)
  if ((int)log_n > two_adicity(field))
    return fail(OMR_NTT_ERR_SIZE, "N=2^" + std::to_string(log_n) +
                                      " requires log2(N) <= TWO_ADICITY=" +
                                      std::to_string(two_adicity(field)));
  if (log_n > 36) return fail(OMR_NTT_ERR_SIZE, "log2(N) > 36 is not supported");
  auto* d = new (std::nothrow) omr_ntt_domain_s();
  if (!d) return fail(OMR_NTT_ERR_ALLOC, "domain allocation failed");
  d->field = field;
  d->log_n = log_n;
  d->n = 1ull << log_n;
  const uint64_t p = modulus(field);
  d->omega = hpowmod(generator(field), (p - 1) >> log_n, p);
  d->omega_inv = hpowmod(d->omega, p - 2, p);
  d->n_inv = hpowmod(d->n % p, p - 2, p);
  cudaError_t e = cudaGetDevice(&d->device);
  if (e != cudaSuccess) {
    delete d;
    return fail(OMR_NTT_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  }
  d->plans = enumerate_plans(log_n);
  if (cudaMalloc(&d->err, sizeof(int)) != cudaSuccess || cudaMemset(d->err, 0, sizeof(int)) != cudaSuccess) {
    omr_ntt_domain_destroy(d);
    return fail(OMR_NTT_ERR_ALLOC, "error-word allocation failed");
  }
  int rc = with_field(field, [&](auto f) { return build_domain_tables<decltype(f)>(d); });
  if (rc == OMR_NTT_OK) {
    RootTables rt;
    rc = get_root_tables(field, &rt);
  }
  if (rc) {
    omr_ntt_domain_destroy(d);
    return rc;
  }
  *out = d;
  return OMR_NTT_OK;
}

int omr_ntt_domain_destroy(omr_ntt_domain_t d) {
  if (!d) return OMR_NTT_OK;
  DeviceGuard g(d->device);
  cudaDeviceSynchronize();
  cudaFree(d->err);
  cudaFree(d->tw_lo_f);
  cudaFree(d->tw_hi_f);
  cudaFree(d->tw_lo_i);
  cudaFree(d->tw_hi_i);
  for (auto& kv : d->scratch) cudaFree(kv.second.ptr);
  for (auto& kv : d->line_tw) cudaFree(kv.second);
  for (auto& kv : d->subs) omr_ntt_domain_destroy(kv.second);
  for (cudaStream_t s : d->host_streams)
    if (s) cudaStreamDestroy(s);
  delete d;
  return OMR_NTT_OK;
}

int omr_ntt_domain_check(omr_ntt_domain_t d, void* stream) {
  if (!d) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null domain");
  DeviceGuard g(d->device);
  int h = 0;
  OMR_CUDA_TRY(cudaMemcpyAsync(&h, d->err, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  OMR_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  if (h) {
    OMR_CUDA_TRY(cudaMemsetAsync(d->err, 0, sizeof(int), (cudaStream_t)stream));
    OMR_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    return fail(h, "a device-side bounded wait gave up (the affected outputs are invalid)");
  }
  return OMR_NTT_OK;
}

int omr_ntt_domain_info(omr_ntt_domain_t d, int* field, uint64_t* n, uint32_t* log_n,
                        uint64_t* omega) {
  if (!d) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null domain");
  if (field) *field = d->field;
  if (n) *n = d->n;
  if (log_n) *log_n = d->log_n;
  if (omega) *omega = d->omega;
  return OMR_NTT_OK;
}

int omr_ntt_domain_twiddles(omr_ntt_domain_t d, int bitrev, void* out) {
  if (!d || !out) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null argument");
  const uint64_t p = modulus(d->field);
  const uint64_t n = d->n;
  std::vector<uint64_t> tw(n);
  uint64_t a = 1;
  for (uint64_t k = 0; k < n; k++) {
    tw[k] = a;
    a = hmulmod(a, d->omega, p);
  }
  const bool wide = d->field == GOLDILOCKS;
  auto put = [&](uint64_t i, uint64_t v) {
    if (wide)
      static_cast<uint64_t*>(out)[i] = v;
    else
      static_cast<uint32_t*>(out)[i] = (uint32_t)v;
  };
  if (!bitrev) {
    for (uint64_t k = 0; k < n; k++) put(k, tw[k]);
  } else {
    const uint32_t lh = d->log_n ? d->log_n - 1 : 0;
    for (uint64_t i = 0; i < n / 2; i++) {
      uint64_t r = 0;
      for (uint32_t b = 0; b < lh; b++) r |= ((i >> b) & 1ull) << (lh - 1 - b);
      put(i, tw[r]);
    }
  }
  return OMR_NTT_OK;
}

int omr_ntt_forward(omr_ntt_domain_t d, int plan, const void* in, void* out, uint64_t batch,
                    void* stream) {
  if (!d || !in || !out) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null argument");
  if (batch == 0) return OMR_NTT_OK;
  DeviceGuard g(d->device);
  return run_transform(d, plan, false, in, out, batch, (cudaStream_t)stream);
}

int omr_ntt_inverse(omr_ntt_domain_t d, int plan, const void* in, void* out, uint64_t batch,
                    void* stream) {
  if (!d || !in || !out) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null argument");
  if (batch == 0) return OMR_NTT_OK;
  DeviceGuard g(d->device);
  return run_transform(d, plan, true, in, out, batch, (cudaStream_t)stream);
}

static int host_roundtrip(omr_ntt_domain_t d, int plan, bool inverse, void* host_buf,
                          uint64_t batch) {
  if (!d || !host_buf) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null argument");
  if (batch == 0) return OMR_NTT_OK;
  DeviceGuard g(d->device);
  std::lock_guard<std::mutex> lk(d->host_mu);
  const uint64_t chunk = host_chunk(d, batch);
  if (chunk)
    return host_pipelined(d, static_cast<char*>(host_buf), batch, chunk,
                          [&](void* buf, uint64_t cnt, cudaStream_t st) {
                            return run_transform(d, plan, inverse, buf, buf, cnt, st);
                          });
  const size_t bytes = (size_t)d->n * batch * word_bytes(d->field);
  void* dbuf = nullptr;
  cudaStream_t s = nullptr;
  int rc = domain_scratch(d, s, bytes, &dbuf, 2);
  if (rc) return rc;
  if (cudaMemcpyAsync(dbuf, host_buf, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess)
    rc = fail(OMR_NTT_ERR_CUDA, "host-to-device copy failed");
  if (!rc) rc = run_transform(d, plan, inverse, dbuf, dbuf, batch, s);
  if (!rc && cudaMemcpyAsync(host_buf, dbuf, bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    rc = fail(OMR_NTT_ERR_CUDA, "device-to-host copy failed");
  cudaError_t se = cudaStreamSynchronize(s);
  if (!rc && se != cudaSuccess) rc = fail(OMR_NTT_ERR_CUDA, cudaGetErrorString(se));
  if (!rc) rc = omr_ntt_domain_check(d, s);
  return rc;
}

int omr_ntt_forward_host(omr_ntt_domain_t d, int plan, void* host_buf, uint64_t batch) {
  return host_roundtrip(d, plan, false, host_buf, batch);
}

int omr_ntt_inverse_host(omr_ntt_domain_t d, int plan, void* host_buf, uint64_t batch) {
  return host_roundtrip(d, plan, true, host_buf, batch);
}

int omr_ntt_plan_count(int field, uint32_t log_n) {
  if (!valid_field(field)) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "unknown field id");
  if ((int)log_n > two_adicity(field)) return fail(OMR_NTT_ERR_SIZE, "log2(N) > TWO_ADICITY");
  return (int)plan_table(log_n).size();
}

int omr_ntt_plan_describe(int field, uint32_t log_n, int plan, char* buf, size_t cap) {
  int cnt = omr_ntt_plan_count(field, log_n);
  if (cnt < 0) return cnt;
  if (plan < 0) plan = default_plan(field, log_n, 1);
  if (plan >= cnt) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "plan id out of range");
  std::string n = plan_name(field, plan_table(log_n)[plan]);
  if (buf && cap) {
    std::strncpy(buf, n.c_str(), cap - 1);
    buf[cap - 1] = 0;
  }
  return OMR_NTT_OK;
}

int omr_ntt_plan_passes(int field, uint32_t log_n, int plan, uint64_t batch, uint64_t* rec,
                        int cap) {
  int cnt = omr_ntt_plan_count(field, log_n);
  if (cnt < 0) return cnt;
  if (plan < 0) plan = default_plan(field, log_n, batch);
  if (plan >= cnt) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "plan id out of range");
  std::vector<PassDesc> ps =
      log_n ? build_passes(log_n, batch, plan_table(log_n)[plan]) : std::vector<PassDesc>{};
  for (int i = 0; i < (int)ps.size() && i < cap && rec; i++) {
    const PassDesc& p = ps[i];
    uint64_t* r = rec + 16 * i;
    r[0] = p.logT;
    r[1] = p.L_lo;
    r[2] = p.L_m;
    r[3] = p.L_b;
    r[4] = p.is_lo;
    r[5] = p.is_m;
    r[6] = p.is_b;
    r[7] = p.os_lo;
    r[8] = p.os_m;
    r[9] = p.os_b;
    r[10] = p.es_in;
    r[11] = p.es_out;
    r[12] = p.twiddle ? 1 : 0;
    r[13] = p.tw_scale;
    r[14] = p.tw_line_mul_m;
    r[15] = (uint64_t)p.in_buf | ((uint64_t)p.out_buf << 8);
  }
  return (int)ps.size();
}

int omr_ntt_plan_run_pass(omr_ntt_domain_t d, int plan, int pass, int inverse, const void* src,
                          void* scratch, void* dst, uint64_t batch, void* stream) {
  if (!d || !src || !dst) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null argument");
  if (plan < 0) plan = default_plan(d->field, d->log_n, batch);
  if (plan >= (int)d->plans.size()) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "plan id out of range");
  if (batch == 0 || d->log_n == 0) return OMR_NTT_OK;
  std::vector<PassDesc> ps = build_passes(d->log_n, batch, d->plans[plan]);
  if (pass < 0 || pass >= (int)ps.size()) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "pass out of range");
  const PassDesc& p = ps[pass];
  if ((p.in_buf == 1 || p.out_buf == 1) && !scratch)
    return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "this pass needs a scratch buffer");
  DeviceGuard g(d->device);
  const void* in = p.in_buf == 0 ? src : (p.in_buf == 1 ? scratch : dst);
  void* out = p.out_buf == 1 ? scratch : dst;
  bool last = pass + 1 == (int)ps.size();
  return with_field(d->field, [&](auto f) {
    return launch_pass<decltype(f)>(d, p, inverse != 0, in, out, last, (cudaStream_t)stream);
  });
}

}  // extern "C"
