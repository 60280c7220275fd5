// partial.cu -- partial-output transform kernels (see partial.cuh).
#include <cuda_runtime.h>

#include <atomic>

#include "partial_prefix.cuh"

namespace omr {

// out[j] = full[sel(j)]; out-of-range indices produce 0 (never an OOB read).
template <class F>
__global__ void gather_kernel(const typename F::E* __restrict__ full, uint64_t n, int pattern,
                              uint64_t count, const uint32_t* __restrict__ idx,
                              typename F::E* __restrict__ out) {
  pdl_entry();
  uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (j >= count) return;
  uint64_t k;
  if (pattern == OMR_NTT_PATTERN_PREFIX)
    k = j;
  else if (pattern == OMR_NTT_PATTERN_STRIDED)
    k = j * (n / count);
  else
    k = idx[j];
  out[j] = k < n ? full[k] : (typename F::E)0;
}

// Column sums of x viewed as rows x cols (row-major): partial[chunk][c] =
// sum over rows of this chunk.  Consecutive threads take consecutive columns.
template <class F>
__global__ void colsum_kernel(const typename F::E* __restrict__ x, uint64_t rows, uint64_t cols,
                              uint64_t rows_per_chunk, typename F::E* __restrict__ partial) {
  pdl_entry();
  using E = typename F::E;
  uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  uint64_t chunk = blockIdx.y;
  if (c >= cols) return;
  uint64_t r0 = chunk * rows_per_chunk;
  uint64_t r1 = r0 + rows_per_chunk < rows ? r0 + rows_per_chunk : rows;
  E acc = 0;
  for (uint64_t r = r0; r < r1; r++) acc = F::add(acc, x[r * cols + c]);
  partial[chunk * cols + c] = acc;
}

template <class F>
static int launch_colsum(const typename F::E* x, uint64_t rows, uint64_t cols,
                         typename F::E* partial, uint64_t max_chunks, uint64_t* nchunks_out,
                         cudaStream_t st) {
  // aim for ~2^20 threads in flight, at most max_chunks row chunks
  uint64_t col_blocks = (cols + 255) / 256;
  uint64_t want = (1ull << 20) / (col_blocks * 256) + 1;
  uint64_t nchunks = want < rows ? want : rows;
  if (nchunks > max_chunks) nchunks = max_chunks;
  uint64_t rpc = (rows + nchunks - 1) / nchunks;
  nchunks = (rows + rpc - 1) / rpc;
  dim3 grid((unsigned)col_blocks, (unsigned)nchunks);
  OMR_CUDA_TRY(launch_pdl(colsum_kernel<F>, grid, dim3(256), 0, st, x, rows, cols, rpc, partial));
  *nchunks_out = nchunks;
  return OMR_NTT_OK;
}

enum { STRAT_DECOMP_ = 1, STRAT_FOLD_ = 2, STRAT_GATHER_ = 3 };

// Strided fold for narrow outputs (count <= 4096): one grid-stride sweep over
// x with a stride that is a multiple of count, so every thread stays in one
// column; per-CTA partial column sums land in partial[rows][count].
template <class F>
__global__ void __launch_bounds__(256) fold_flat_kernel(const typename F::E* __restrict__ x,
                                                        uint64_t n, uint32_t count,
                                                        typename F::E* __restrict__ partial) {
  pdl_entry();
  using E = typename F::E;
  __shared__ E red[256];
  const uint64_t stride = (uint64_t)gridDim.x * 256;
  E acc = 0;
  for (uint64_t i = blockIdx.x * 256ull + threadIdx.x; i < n; i += stride) acc = F::add(acc, x[i]);
  if (count >= 256) {
    // this CTA covers 256 distinct columns; replica row = blockIdx / (count / 256)
    const uint32_t per = count / 256;
    partial[(uint64_t)(blockIdx.x / per) * count + (blockIdx.x % per) * 256 + threadIdx.x] = acc;
    return;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x < count) {
    E sum = 0;
    for (uint32_t j = threadIdx.x; j < 256; j += count) sum = F::add(sum, red[j]);
    partial[(uint64_t)blockIdx.x * count + threadIdx.x] = sum;
  }
}

// Strided fold with 16-byte loads.  Every thread reads VW = 16 / w adjacent
// words per load, eight loads in flight.  The grid stride is a multiple of
// count (count a power of two <= 4096; gridDim a multiple of 4 and of
// count / CH), so each of a thread's VW lanes stays in one column.  The CTA
// then sums the CH = 256 VW positions of its chunk down to columns in shared
// memory:
//   count <= CH: one row of count column sums per CTA;
//   count >  CH: the CTA's chunk is CH consecutive columns of one row
//               (row = blockIdx / (count / CH)).
constexpr int kFoldThreads = 256;
template <class F>
__global__ void __launch_bounds__(kFoldThreads) fold_vec_kernel(const typename F::E* __restrict__ x,
                                                                uint64_t n, uint32_t count,
                                                                typename F::E* __restrict__ partial) {
  pdl_entry();
  using E = typename F::E;
  constexpr int VW = 16 / F::WORD;
  constexpr int CH = kFoldThreads * VW;  // words per CTA per sweep step
  __shared__ E red[CH];
  const uint64_t stride = (uint64_t)gridDim.x * CH;
  E acc[VW];
#pragma unroll
  for (int u = 0; u < VW; u++) acc[u] = 0;
  const uint4* __restrict__ xv = reinterpret_cast<const uint4*>(x);
  uint64_t i = (uint64_t)blockIdx.x * CH + (uint64_t)threadIdx.x * VW;
  // eight predicated loads per step, all issued before the adds (a zero
  // vector past the end adds nothing)
  for (; i < n; i += 8 * stride) {
    uint4 q[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const uint64_t j = i + k * stride;
      q[k] = j < n ? xv[j / VW] : make_uint4(0u, 0u, 0u, 0u);
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const E* w = reinterpret_cast<const E*>(&q[k]);
#pragma unroll
      for (int u = 0; u < VW; u++) acc[u] = F::add(acc[u], w[u]);
    }
  }
#pragma unroll
  for (int u = 0; u < VW; u++) red[threadIdx.x * VW + u] = acc[u];
  __syncthreads();
  // position p of the chunk holds column (blockIdx * CH + p) mod count
  for (uint32_t h = CH / 2; h >= count && h >= 1; h >>= 1) {
    for (uint32_t p = threadIdx.x; p < h; p += kFoldThreads) red[p] = F::add(red[p], red[p + h]);
    __syncthreads();
  }
  if (count <= (uint32_t)CH) {
    for (uint32_t c = threadIdx.x; c < count; c += kFoldThreads)
      partial[(uint64_t)blockIdx.x * count + c] = red[c];
  } else {
    const uint32_t per = count / CH;
    E* row = partial + (uint64_t)(blockIdx.x / per) * count + (uint64_t)(blockIdx.x % per) * CH;
    for (uint32_t p = threadIdx.x; p < (uint32_t)CH; p += kFoldThreads) row[p] = red[p];
  }
}

template <class F>
static int run_fold(omr_ntt_domain_s* d, int sub_plan, uint64_t count, const void* in, void* out,
                    cudaStream_t stream) {
  using E = typename F::E;
  const size_t w = sizeof(E);
  // fold: y[n'] = sum_q x[n' + count q], then X[j N/count] = DFT_count(y)[j]
  uint32_t log_s = 0;
  while ((1ull << log_s) < count) log_s++;
  omr_ntt_domain_s* sd = nullptr;
  int rc = sub_domain(d, log_s, &sd);
  if (rc) return rc;
  const uint64_t rows = d->n / count;
  const uint64_t max_chunks = 4096;  // first-level partial sums, then y
  void* buf = nullptr;
  rc = domain_scratch(d, stream, (size_t)(max_chunks + 1) * count * w, &buf, 1);
  if (rc) return rc;
  E* part = static_cast<E*>(buf);
  uint64_t nch = 0;
  const int vw = 16 / (int)w;
  const uint64_t ch = (uint64_t)kFoldThreads * vw;
  if (count <= 4096 && d->n >= ch * 4 && !(reinterpret_cast<uintptr_t>(in) & 15)) {
    // 16-byte loads: four CTAs per SM, a multiple of 4 (and of
    // count / CH), never more than the sweep needs
    uint64_t g = (uint64_t)device_sm_count(d->device) * 4;
    const uint64_t need = d->n / ch;
    if (g > need) g = need;
    const uint64_t m = count / ch > 4 ? count / ch : 4;  // grid stride a multiple of count
    g = g < m ? m : g & ~(m - 1);
    const uint32_t grid = (uint32_t)g;
    OMR_CUDA_TRY(launch_pdl(fold_vec_kernel<F>, dim3(grid), dim3(kFoldThreads), 0, stream, static_cast<const E*>(in), d->n,
                            (uint32_t)count, part));
    nch = count > ch ? grid / (count / ch) : grid;
  } else if (count <= 4096 && d->n >= 256ull * 1216) {
    const uint32_t grid = 1216;  // 8 CTAs per SM; a multiple of count / 256 for count <= 4096
    OMR_CUDA_TRY(launch_pdl(fold_flat_kernel<F>, dim3(grid), dim3(256), 0, stream, static_cast<const E*>(in), d->n,
                            (uint32_t)count, part));
    nch = count >= 256 ? grid / (count / 256) : grid;
  } else {
    rc = launch_colsum<F>(static_cast<const E*>(in), rows, count, part, max_chunks, &nch, stream);
    if (rc) return rc;
  }
  E* y = part;
  if (nch > 1) {
    y = part + nch * count;
    rc = launch_reduce_rows<F>(part, nch, count, y, stream);
    if (rc) return rc;
  }
  return run_transform(sd, sub_plan, false, y, out, 1, stream);
}

template <class F>
static int run_gather(omr_ntt_domain_s* d, int plan, int pattern, uint64_t count,
                      const uint32_t* indices, const void* in, void* out, cudaStream_t stream) {
  using E = typename F::E;
  void* full = nullptr;
  int rc = domain_scratch(d, stream, (size_t)d->n * sizeof(E), &full, 1);
  if (rc) return rc;
  rc = run_transform(d, plan, false, in, full, 1, stream);
  if (rc) return rc;
  unsigned blocks = (unsigned)((count + 255) / 256);
  OMR_CUDA_TRY(launch_pdl(gather_kernel<F>, dim3(blocks), dim3(256), 0, stream, static_cast<const E*>(full), d->n,
                          pattern, count, indices, static_cast<E*>(out)));
  return OMR_NTT_OK;
}

template <class F>
static int run_strategy_t(omr_ntt_domain_s* d, int strategy, int param, int pattern,
                          uint64_t count, const uint32_t* indices, const void* in, void* out,
                          cudaStream_t stream) {
  const uint64_t n = d->n;
  switch (strategy) {
    case STRAT_DECOMP_:
      if ((pattern != OMR_NTT_PATTERN_PREFIX && pattern != OMR_NTT_PATTERN_INDICES) || count > 4096 ||
          count >= n)
        return fail(OMR_NTT_ERR_INVALID_ARGUMENT,
                    "decomposition serves prefixes and index sets of <= 4096 outputs");
      return launch_prefix<F>(d, (uint32_t)count, param, in, out, stream,
                              pattern == OMR_NTT_PATTERN_INDICES ? indices : nullptr);
    case STRAT_FOLD_:
      if (pattern != OMR_NTT_PATTERN_STRIDED || count >= n)
        return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "fold serves strided patterns");
      return run_fold<F>(d, param, count, in, out, stream);
    case STRAT_GATHER_:
      return run_gather<F>(d, param, pattern, count, indices, in, out, stream);
  }
  return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "unknown partial strategy");
}

int run_partial_strategy(omr_ntt_domain_s* d, int strategy, int param, int pattern,
                         uint64_t count, const uint32_t* indices, const void* in, void* out,
                         cudaStream_t stream) {
  return with_field(d->field, [&](auto f) {
    return run_strategy_t<decltype(f)>(d, strategy, param, pattern, count, indices, in, out,
                                       stream);
  });
}

template <class F>
int partial_dispatch(omr_ntt_domain_s* d, int pattern, uint64_t count, const uint32_t* indices,
                     const void* in, void* out, cudaStream_t stream) {
  const uint64_t n = d->n;
  int strategy = 0, param = 0;
  if (planned_partial(d->field, d->log_n, pattern, count, &strategy, &param) == 1 &&
      strategy >= STRAT_DECOMP_ && strategy <= STRAT_GATHER_)
    return run_strategy_t<F>(d, strategy, param, pattern, count, indices, in, out, stream);
  // built-in rule (timings of the exhaustive tuner on GB300): the fold for
  // strided sets unless they keep more than 2^16 outputs of at most 8 cosets
  // (then the full transform + gather); the pruned decomposition for <= 4096
  // outputs of transforms above 2^20, where it beats the full transform
  if (pattern == OMR_NTT_PATTERN_STRIDED && count < n && !(count > 65536 && n / count <= 8))
    return run_fold<F>(d, -1, count, in, out, stream);
  if ((pattern == OMR_NTT_PATTERN_PREFIX || pattern == OMR_NTT_PATTERN_INDICES) && count <= 4096 &&
      count < n && n / count >= 2 && d->log_n > 20)
    return launch_prefix<F>(d, (uint32_t)count, 0, in, out, stream,
                            pattern == OMR_NTT_PATTERN_INDICES ? indices : nullptr);
  return run_gather<F>(d, -1, pattern, count, indices, in, out, stream);
}

template <class F>
int launch_gather_indices(const void* full, uint64_t n, uint64_t count, const uint32_t* idx,
                          void* out, cudaStream_t stream) {
  using E = typename F::E;
  if (count == 0) return OMR_NTT_OK;
  OMR_CUDA_TRY(launch_pdl(gather_kernel<F>, dim3((unsigned)((count + 255) / 256)), dim3(256), 0, stream,
                          static_cast<const E*>(full), n, (int)OMR_NTT_PATTERN_INDICES, count, idx,
                          static_cast<E*>(out)));
  return OMR_NTT_OK;
}
template int launch_gather_indices<BabyBear>(const void*, uint64_t, uint64_t, const uint32_t*,
                                             void*, cudaStream_t);
template int launch_gather_indices<Goldilocks>(const void*, uint64_t, uint64_t, const uint32_t*,
                                               void*, cudaStream_t);
template int launch_gather_indices<KoalaBear>(const void*, uint64_t, uint64_t, const uint32_t*,
                                              void*, cudaStream_t);
template int launch_gather_indices<TeddyBear>(const void*, uint64_t, uint64_t, const uint32_t*,
                                              void*, cudaStream_t);

template int partial_dispatch<BabyBear>(omr_ntt_domain_s*, int, uint64_t, const uint32_t*,
                                        const void*, void*, cudaStream_t);
template int partial_dispatch<Goldilocks>(omr_ntt_domain_s*, int, uint64_t, const uint32_t*,
                                          const void*, void*, cudaStream_t);
template int partial_dispatch<KoalaBear>(omr_ntt_domain_s*, int, uint64_t, const uint32_t*,
                                         const void*, void*, cudaStream_t);
template int partial_dispatch<TeddyBear>(omr_ntt_domain_s*, int, uint64_t, const uint32_t*,
                                         const void*, void*, cudaStream_t);

}  // namespace omr
