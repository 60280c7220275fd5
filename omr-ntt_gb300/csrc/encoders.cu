// encoders.cu -- the reference's encoder surface (NttEncoder::ntt / name,
// encoders::all / all_partial) and the partial-output entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "engine.cuh"
#include "partial.cuh"

namespace omr {

static const char* kEncoderNames[] = {
    "ArkRadix2",          "Dft",
    "DftPartial",         "LambdaBowers",
    "LambdaRadix4",       "Plonky3Radix2LayerSplit",
    "TfheStockhamRadix8", "TransformDecomposition",
    "TransformDecompositionV2", "WinterfellFourStep",
};
constexpr int kNumEncoders = 10;

static bool is_partial_encoder(int e) {
  return e == OMR_NTT_DFT_PARTIAL || e == OMR_NTT_TRANSFORM_DECOMPOSITION ||
         e == OMR_NTT_TRANSFORM_DECOMPOSITION_V2;
}

// The plan of the given pass split and kernel variant, or -1.
static int find_plan(uint32_t log_n, const std::vector<int>& split, int variant) {
  const auto& plans = plan_table(log_n);
  for (int i = 0; i < (int)plans.size(); i++)
    if (plans[i].variant == variant && plans[i].split == split) return i;
  return -1;
}
// The first plan of the variant whose passes all satisfy `ok`, or -1.
template <class Pred>
static int find_plan_if(uint32_t log_n, int variant, Pred ok) {
  const auto& plans = plan_table(log_n);
  for (int i = 0; i < (int)plans.size(); i++)
    if (plans[i].variant == variant && plans[i].split.size() > 1 &&
        std::all_of(plans[i].split.begin(), plans[i].split.end(), ok))
      return i;
  return -1;
}

// Plan family of each full encoder.  Every plan computes the same
// natural-order transform (so the words never depend on the encoder); the
// family gives each of the reference's algorithms the engine plan that has
// its structure:
//   WinterfellFourStep (src/encoders/winterfell_four_step.rs:31-81): two
//     factors near sqrt(N), row FFTs, twiddle, row FFTs -> the balanced
//     two-pass split on the slab pass (which splits each line four-step
//     style again: one stride-256 round, then 256-point slabs);
//   Plonky3Radix2LayerSplit (src/encoders/plonky3_radix2_layer_split.rs:30-97):
//     a DIT half and a Bowers half split at mid = log2(N) / 2 -> the split
//     with the shorter pass first (floor(log N / 2), ceil(log N / 2)) on the
//     double-buffered TMA pass;
//   LambdaBowers (src/encoders/lambdaworks_bowers.rs:42-153): one DIF
//     network with layers fused in pairs over the whole array -> the
//     shortest-line family, the wide pass (256-point passes), on a split
//     of 256-point passes only where there is one, else a split with a
//     256-point pass;
//   LambdaRadix4 (src/encoders/lambdaworks_radix4.rs:34-75): radix-4 stages
//     only (even log N) -> a split into even-length passes on the two-CTA
//     TMA pass;
//   TfheStockhamRadix8 (src/encoders/tfhe_stockham_radix8.rs:80-140):
//     radix-8 Stockham passes (log N % 3 == 0) -> a split into passes of a
//     multiple of 3 bits on the plain Stockham tile pass;
//   ArkRadix2, Dft and transforms that fit one pass (N <= 4096): the
//     planner's choice.
// A family without a plan at this size falls back to the planner's choice.
static int encoder_plan(int encoder, int field, uint32_t log_n) {
  const int dflt = default_plan(field, log_n, 1);
  if (log_n <= (uint32_t)kMaxLogT) return dflt;
  const int pmin = (int)((log_n + kMaxLogT - 1) / kMaxLogT);
  std::vector<int> bal(pmin);
  for (int i = 0; i < pmin; i++) bal[i] = (int)(log_n / pmin) + (i < (int)(log_n % pmin) ? 1 : 0);
  int p = -1;
  switch (encoder) {
    case OMR_NTT_WINTERFELL_FOUR_STEP:
      p = find_plan(log_n, bal, kSlabVariant);
      break;
    case OMR_NTT_PLONKY3_LAYER_SPLIT: {
      std::vector<int> rev(bal.rbegin(), bal.rend());
      p = find_plan(log_n, rev, 1);
      break;
    }
    case OMR_NTT_LAMBDA_BOWERS: {
      // all passes 256-point where the split allows it, else any wide plan
      p = find_plan_if(log_n, kWideVariant, [](int t) { return t == 8; });
      const auto& plans = plan_table(log_n);
      for (int i = 0; p < 0 && i < (int)plans.size(); i++)
        if (plans[i].variant == kWideVariant) p = i;
      break;
    }
    case OMR_NTT_LAMBDA_RADIX4:
      p = find_plan_if(log_n, 2, [](int t) { return t % 2 == 0; });
      break;
    case OMR_NTT_TFHE_STOCKHAM_R8:
      p = find_plan_if(log_n, 0, [](int t) { return t % 3 == 0; });
      break;
    default:
      break;
  }
  return p >= 0 ? p : dflt;
}

template <class F>
__global__ void check_canonical_kernel(const typename F::E* __restrict__ x, uint64_t n,
                                       int* flag) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  bool bad = false;
  for (; i < n; i += stride) bad |= (x[i] >= F::P);
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// Partial output of one transform (device pointers).  `out` receives count
// words; `in` is untouched.
int run_partial(omr_ntt_domain_s* d, int pattern, uint64_t count, const uint32_t* indices,
                const void* in, void* out, cudaStream_t stream) {
  if (count == 0) return OMR_NTT_OK;
  if (pattern == OMR_NTT_PATTERN_PREFIX || pattern == OMR_NTT_PATTERN_STRIDED) {
    if (count > d->n) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "count > N");
  }
  if (pattern == OMR_NTT_PATTERN_STRIDED && (count & (count - 1)))
    return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "strided pattern needs a power-of-two count");
  if (pattern == OMR_NTT_PATTERN_INDICES && !indices)
    return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null index array");
  if (pattern < 0 || pattern > 2) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "unknown pattern");
  return with_field(d->field, [&](auto f) {
    return partial_dispatch<decltype(f)>(d, pattern, count, indices, in, out, stream);
  });
}

}  // namespace omr

using namespace omr;

extern "C" {

const char* omr_ntt_encoder_name(int encoder) {
  if (encoder < 0 || encoder >= kNumEncoders) return nullptr;
  return kEncoderNames[encoder];
}

int omr_ntt_encoder_supports(int encoder, uint32_t log_n) {
  if (encoder < 0 || encoder >= kNumEncoders) return 0;
  if (encoder == OMR_NTT_LAMBDA_RADIX4) return log_n % 2 == 0;
  if (encoder == OMR_NTT_TFHE_STOCKHAM_R8) return log_n % 3 == 0;
  return 1;
}

int omr_ntt_encoder_plan(int encoder, int field, uint32_t log_n) {
  if (encoder < 0 || encoder >= kNumEncoders) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "unknown encoder id");
  if (!valid_field(field)) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "unknown field id");
  if ((int)log_n > two_adicity(field)) return fail(OMR_NTT_ERR_SIZE, "log2(N) > TWO_ADICITY");
  if (is_partial_encoder(encoder)) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "partial encoders run no full plan");
  if (!omr_ntt_encoder_supports(encoder, log_n))
    return fail(OMR_NTT_ERR_PRECONDITION, std::string(kEncoderNames[encoder]) + " does not support this size");
  return encoder_plan(encoder, field, log_n);
}

int omr_ntt_encode(omr_ntt_domain_t d, int encoder, uint64_t s, void* buf, uint64_t batch,
                   void* stream) {
  if (!d || !buf) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null argument");
  if (encoder < 0 || encoder >= kNumEncoders)
    return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "unknown encoder id");
  if (!omr_ntt_encoder_supports(encoder, d->log_n))
    return fail(OMR_NTT_ERR_PRECONDITION,
                std::string(kEncoderNames[encoder]) + " does not support log2(N)=" +
                    std::to_string(d->log_n));
  if (batch == 0) return OMR_NTT_OK;
  DeviceGuard g(d->device);
  cudaStream_t st = (cudaStream_t)stream;
  if (!is_partial_encoder(encoder))
    return run_transform(d, encoder_plan(encoder, d->field, d->log_n), false, buf, buf, batch, st);
  // partial encoders: buf[..m] = X[..m], m = min(2s, N); the rest of buf is kept
  const uint64_t m = (2 * s < d->n) ? 2 * s : d->n;
  if (m == 0) return OMR_NTT_OK;
  const size_t w = word_bytes(d->field);
  void* tmp = nullptr;
  int rc = domain_scratch(d, stream, (size_t)m * w, &tmp, 3);
  if (rc) return rc;
  for (uint64_t b = 0; b < batch; b++) {
    char* x = static_cast<char*>(buf) + (size_t)b * d->n * w;
    rc = run_partial(d, OMR_NTT_PATTERN_PREFIX, m, nullptr, x, tmp, st);
    if (rc) return rc;
    OMR_CUDA_TRY(cudaMemcpyAsync(x, tmp, (size_t)m * w, cudaMemcpyDeviceToDevice, st));
  }
  return OMR_NTT_OK;
}

int omr_ntt_encode_host(omr_ntt_domain_t d, int encoder, uint64_t s, void* host_buf,
                        uint64_t batch) {
  if (!d || !host_buf) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null argument");
  if (encoder < 0 || encoder >= kNumEncoders)
    return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "unknown encoder id");
  if (!omr_ntt_encoder_supports(encoder, d->log_n))
    return fail(OMR_NTT_ERR_PRECONDITION,
                std::string(kEncoderNames[encoder]) + " does not support log2(N)=" +
                    std::to_string(d->log_n));
  if (batch == 0) return OMR_NTT_OK;
  DeviceGuard g(d->device);
  std::lock_guard<std::mutex> lk(d->host_mu);
  const uint64_t chunk = host_chunk(d, batch);
  if (chunk)
    return host_pipelined(d, static_cast<char*>(host_buf), batch, chunk,
                          [&](void* buf, uint64_t cnt, cudaStream_t st) {
                            return omr_ntt_encode(d, encoder, s, buf, cnt, st);
                          });
  const size_t bytes = (size_t)d->n * batch * word_bytes(d->field);
  void* dbuf = nullptr;
  int rc = domain_scratch(d, nullptr, bytes, &dbuf, 2);
  if (rc) return rc;
  OMR_CUDA_TRY(cudaMemcpyAsync(dbuf, host_buf, bytes, cudaMemcpyHostToDevice, nullptr));
  rc = omr_ntt_encode(d, encoder, s, dbuf, batch, nullptr);
  if (rc) {
    cudaStreamSynchronize(nullptr);
    return rc;
  }
  OMR_CUDA_TRY(cudaMemcpyAsync(host_buf, dbuf, bytes, cudaMemcpyDeviceToHost, nullptr));
  OMR_CUDA_TRY(cudaStreamSynchronize(nullptr));
  return OMR_NTT_OK;
}

int omr_ntt_partial(omr_ntt_domain_t d, int pattern, uint64_t count, const uint32_t* indices,
                    const void* in, void* out, void* stream) {
  if (!d || !in || !out) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null argument");
  DeviceGuard g(d->device);
  return run_partial(d, pattern, count, indices, in, out, (cudaStream_t)stream);
}

int omr_ntt_partial_host(omr_ntt_domain_t d, int pattern, uint64_t count,
                         const uint32_t* indices, const void* in, void* out) {
  if (!d || !in || !out) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null argument");
  if (pattern == OMR_NTT_PATTERN_INDICES) {
    if (!indices) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null index array");
    for (uint64_t j = 0; j < count; j++)
      if (indices[j] >= d->n) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "index out of range");
  }
  if (count == 0) return OMR_NTT_OK;
  DeviceGuard g(d->device);
  std::lock_guard<std::mutex> lk(d->host_mu);
  const size_t w = word_bytes(d->field);
  const size_t in_bytes = (size_t)d->n * w, out_bytes = (size_t)count * w;
  const size_t idx_bytes = pattern == OMR_NTT_PATTERN_INDICES ? (size_t)count * 4 : 0;
  void* dbuf = nullptr;
  int rc = domain_scratch(d, nullptr, in_bytes + out_bytes + idx_bytes + 256, &dbuf, 2);
  if (rc) return rc;
  char* din = static_cast<char*>(dbuf);
  char* dout = din + in_bytes;
  uint32_t* didx = reinterpret_cast<uint32_t*>(dout + ((out_bytes + 255) / 256) * 256);
  OMR_CUDA_TRY(cudaMemcpyAsync(din, in, in_bytes, cudaMemcpyHostToDevice, nullptr));
  if (idx_bytes)
    OMR_CUDA_TRY(cudaMemcpyAsync(didx, indices, idx_bytes, cudaMemcpyHostToDevice, nullptr));
  rc = run_partial(d, pattern, count, idx_bytes ? didx : nullptr, din, dout, nullptr);
  if (rc) {
    cudaStreamSynchronize(nullptr);
    return rc;
  }
  OMR_CUDA_TRY(cudaMemcpyAsync(out, dout, out_bytes, cudaMemcpyDeviceToHost, nullptr));
  OMR_CUDA_TRY(cudaStreamSynchronize(nullptr));
  return OMR_NTT_OK;
}

int omr_ntt_check_canonical(omr_ntt_domain_t d, const void* buf, uint64_t words, void* stream) {
  if (!d || !buf) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null argument");
  if (words == 0) return OMR_NTT_OK;
  DeviceGuard g(d->device);
  cudaStream_t st = (cudaStream_t)stream;
  int* flag = nullptr;
  int rc = domain_scratch(d, stream, 256, reinterpret_cast<void**>(&flag), 4);
  if (rc) return rc;
  OMR_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), st));
  rc = with_field(d->field, [&](auto f) -> int {
    using F = decltype(f);
    check_canonical_kernel<F><<<1216, 256, 0, st>>>(static_cast<const typename F::E*>(buf), words,
                                                    flag);
    OMR_CUDA_TRY(cudaGetLastError());
    return OMR_NTT_OK;
  });
  if (rc) return rc;
  int h = 0;
  OMR_CUDA_TRY(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
  OMR_CUDA_TRY(cudaStreamSynchronize(st));
  return h ? fail(OMR_NTT_ERR_NONCANONICAL, "input word >= p") : OMR_NTT_OK;
}

}  // extern "C"
