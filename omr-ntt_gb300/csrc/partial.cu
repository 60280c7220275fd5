// partial.cu -- partial-output transform kernels (see partial.cuh).
#include <cuda_runtime.h>

#include "partial.cuh"

namespace omr {

// out[j] = full[sel(j)]; out-of-range indices produce 0 (never an OOB read).
template <class F>
__global__ void gather_kernel(const typename F::E* __restrict__ full, uint64_t n, int pattern,
                              uint64_t count, const uint32_t* __restrict__ idx,
                              typename F::E* __restrict__ out) {
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
  colsum_kernel<F><<<grid, 256, 0, st>>>(x, rows, cols, rpc, partial);
  OMR_CUDA_TRY(cudaGetLastError());
  *nchunks_out = nchunks;
  return OMR_NTT_OK;
}

template <class F>
int partial_dispatch(omr_ntt_domain_s* d, int pattern, uint64_t count, const uint32_t* indices,
                     const void* in, void* out, cudaStream_t stream) {
  using E = typename F::E;
  const size_t w = sizeof(E);
  const uint64_t n = d->n;
  if (pattern == OMR_NTT_PATTERN_STRIDED && count < n) {
    // fold: y[n'] = sum_q x[n' + count q], then X[j N/count] = DFT_count(y)[j]
    uint32_t log_s = 0;
    while ((1ull << log_s) < count) log_s++;
    omr_ntt_domain_s* sd = nullptr;
    int rc = sub_domain(d, log_s, &sd);
    if (rc) return rc;
    const uint64_t rows = n / count;
    // staging: first-level partial sums (<= 4096 chunks) then y
    const uint64_t max_chunks = 4096;
    void* buf = nullptr;
    rc = domain_scratch(d, stream, (size_t)(max_chunks + 1) * count * w, &buf, 1);
    if (rc) return rc;
    E* part = static_cast<E*>(buf);
    uint64_t nch = 0;
    rc = launch_colsum<F>(static_cast<const E*>(in), rows, count, part, max_chunks, &nch, stream);
    if (rc) return rc;
    E* y = part;
    if (nch > 1) {
      y = part + nch * count;
      uint64_t one = 0;
      rc = launch_colsum<F>(part, nch, count, y, 1, &one, stream);
      if (rc) return rc;
    }
    return run_transform(sd, -1, false, y, out, 1, stream);
  }
  // full transform into scratch, then gather
  void* full = nullptr;
  int rc = domain_scratch(d, stream, (size_t)n * w, &full, 1);
  if (rc) return rc;
  rc = run_transform(d, -1, false, in, full, 1, stream);
  if (rc) return rc;
  unsigned blocks = (unsigned)((count + 255) / 256);
  gather_kernel<F><<<blocks, 256, 0, stream>>>(static_cast<const E*>(full), n, pattern, count,
                                              indices, static_cast<E*>(out));
  OMR_CUDA_TRY(cudaGetLastError());
  return OMR_NTT_OK;
}

template int partial_dispatch<BabyBear>(omr_ntt_domain_s*, int, uint64_t, const uint32_t*,
                                        const void*, void*, cudaStream_t);
template int partial_dispatch<Goldilocks>(omr_ntt_domain_s*, int, uint64_t, const uint32_t*,
                                          const void*, void*, cudaStream_t);
template int partial_dispatch<KoalaBear>(omr_ntt_domain_s*, int, uint64_t, const uint32_t*,
                                         const void*, void*, cudaStream_t);
template int partial_dispatch<TeddyBear>(omr_ntt_domain_s*, int, uint64_t, const uint32_t*,
                                         const void*, void*, cudaStream_t);

}  // namespace omr
