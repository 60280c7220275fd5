// partial.cu -- partial-output transform kernels (see partial.cuh).
#include <cuda_runtime.h>

#include <atomic>

#include "partial.cuh"

namespace omr {

// ---------------------------------------------------------------- prefix
// Pruned prefix transform (the reference's TransformDecomposition,
// src/encoders/transform_decomposition.rs:25-97, with n1 = T >= m):
//   X[k] = sum_{r < N/T} omega_N^(r k) * Y_r[k],  Y_r = DFT_T(x[r + (N/T) c] over c),  k < m.
// Each CTA owns a contiguous run of groups of C adjacent columns r.  Per group
// it runs the T-point Stockham rounds of the tile pass (the first round reads
// global memory straight into registers) into a shared-memory tile, then
// folds the group into per-thread accumulators by Horner's rule over the
// columns: thread (k, slice) visits columns r_i = r_first + slice + TPK i
// (TPK column slices), acc = acc * omega_N^(-TPK k) + Y_{r_i}[k], and at the
// end multiplies by omega_N^(k r_last); so sum_i omega_N^(k r_i) Y_{r_i}[k]
// costs one constant multiply and one add per needed output and column,
// with no per-element twiddle lookups.  The slices are combined in shared
// memory, one row of m words per CTA, and a row-reduction kernel sums the
// rows.  The input is read once.
template <class F, int LOGT>
constexpr int prefix_cols() {  // ~64 KiB tile, rows of >= 16 bytes, <= 256 columns
  constexpr int lo = 16 / F::WORD;
  constexpr int c = (65536 / F::WORD) >> LOGT;
  return c < lo ? lo : (c > 256 ? 256 : c);
}
template <class F, int LOGT>
constexpr int prefix_threads() {  // <= 256 threads at <= 128 registers: two CTAs per SM
  constexpr int tc = (1 << LOGT) * prefix_cols<F, LOGT>();
  // short lines (one round) take 16 words a thread: more warps for the loads
  constexpr int nt = tc / (LOGT <= 4 ? 16 : tile_ept<F>());
  return nt < 64 ? 64 : (nt > 256 ? 256 : nt);
}

template <class F, int LOGT, int C, int NT, int I>
OMR_D void prefix_rounds(const PassArgs<F>& a, typename F::E* s, const typename F::E* gin,
                         int nvalid) {
  using RP = RoundPlan<LOGT, max_radix_log<F>()>;
  if constexpr (I < RP::ROUNDS) {
    constexpr int SRC = I == 0 ? SRC_GLOBAL : SRC_SMEM;
    do_round<F, LOGT, C, NT, RP::logr(I), RP::logns(I), false, SRC, DST_SMEM, false, false>(
        a, s, gin, nullptr, nvalid, 0, 0);
    prefix_rounds<F, LOGT, C, NT, I + 1>(a, s, gin, nvalid);
  }
}

// omega_N^e in "twiddle-Montgomery" form (what mul_m takes) from the
// two-level four-step tables.
template <class F>
OMR_D typename F::E omega_m(const PassArgs<F>& a, uint64_t e) {
  const uint32_t ee = (uint32_t)e & a.tw_mask;
  return F::mul_tw(a.tw_lo[ee & ((1u << kTwLoBits) - 1)], a.tw_hi[ee >> kTwLoBits]);
}
// omega_N^e as a twiddle operand for mul_tw.
template <class F>
OMR_D typename F::Tw omega_tw(const PassArgs<F>& a, uint64_t e) {
  const typename F::E wm = omega_m<F>(a, e);
  if constexpr (F::ID == GOLDILOCKS) {
    return F::make_tw(wm);
  } else {
    return F::make_tw(F::mont(wm, 1u));  // canonical omega^e
  }
}

template <class F, int LOGT>
__global__ void __launch_bounds__(prefix_threads<F, LOGT>(), 2)
    prefix_decomp_kernel(const PassArgs<F> a, uint32_t m, typename F::E* __restrict__ partial) {
  using E = typename F::E;
  using Tw = typename F::Tw;
  constexpr int T = 1 << LOGT;
  constexpr int C = prefix_cols<F, LOGT>();
  constexpr int NT = prefix_threads<F, LOGT>();
  constexpr int KMAX = T > NT ? T / NT : 1;  // outputs per thread when m > NT
  extern __shared__ __align__(16) unsigned char smem_raw[];
  E* s = reinterpret_cast<E*>(smem_raw);

  // thread -> KACT adjacent outputs x TPK column slices (m <= NT), or
  // outputs k = t + j NT (m > NT, one slice)
  uint32_t kact = 1;
  while (kact < m && kact < (uint32_t)NT) kact <<= 1;
  const uint32_t tpk = min((uint32_t)NT / kact, (uint32_t)C);
  const uint32_t kper = (m + NT - 1) / NT;
  const uint32_t kbase = threadIdx.x % kact;
  const uint32_t slice = threadIdx.x / kact;
  const bool active = slice < tpk;

  E acc[KMAX];
  Tw zi[KMAX];
#pragma unroll
  for (int j = 0; j < KMAX; j++) {
    acc[j] = 0;
    const uint32_t k = kbase + j * NT;
    zi[j] = omega_tw<F>(a, (uint64_t)0 - (uint64_t)tpk * k);  // omega_N^(-TPK k)
  }

  const uint32_t groups = (a.L_lo + C - 1) / C;
  const uint32_t g0 = (uint32_t)((uint64_t)blockIdx.x * groups / gridDim.x);
  const uint32_t g1 = (uint32_t)((uint64_t)(blockIdx.x + 1) * groups / gridDim.x);
  for (uint32_t g = g0; g < g1; g++) {
    const uint32_t llo0 = g * C;
    const int nvalid = (int)min((uint32_t)C, a.L_lo - llo0);
    prefix_rounds<F, LOGT, C, NT, 0>(a, s, a.in + llo0, nvalid);
    if (active) {
#pragma unroll
      for (int j = 0; j < KMAX; j++) {
        const uint32_t k = kbase + j * NT;
        if (j < (int)kper && k < m) {
          E h = acc[j];
#pragma unroll 4
          for (uint32_t c = slice; c < (uint32_t)C; c += tpk)
            h = F::add(F::mul_tw(h, zi[j]), s[tile_idx<F, C>((int)k, (int)c)]);
          acc[j] = h;
        }
      }
    }
    __syncthreads();  // the next group's first round overwrites the tile
  }
  if (g1 > g0) {
    const uint64_t r_last = (uint64_t)(g1 - 1) * C + (C - tpk) + slice;
#pragma unroll
    for (int j = 0; j < KMAX; j++) {
      const uint32_t k = kbase + j * NT;
      if (active && j < (int)kper && k < m) acc[j] = mul_m<F>(acc[j], omega_m<F>(a, r_last * k));
    }
  }
  if (tpk > 1) {
    // combine the slices of every output: s[slice * kact + k]
    if (active) s[slice * kact + kbase] = acc[0];
    __syncthreads();
    if (threadIdx.x < m) {
      E sum = 0;
      for (uint32_t sl = 0; sl < tpk; sl++) sum = F::add(sum, s[sl * kact + threadIdx.x]);
      partial[(uint64_t)blockIdx.x * m + threadIdx.x] = sum;
    }
  } else {
#pragma unroll
    for (int j = 0; j < KMAX; j++) {
      const uint32_t k = threadIdx.x + j * NT;
      if (j < (int)kper && k < m) partial[(uint64_t)blockIdx.x * m + k] = acc[j];
    }
  }
}

// out[k] = sum over rows of partial[row * cols + k].  A CTA of kReduceThreads
// covers cw adjacent columns (cw a power of two <= 32) with kReduceThreads / cw
// row slices, so each thread sums only rows / slices values (independent
// loads, no long serial chain) before a shared-memory tree over the slices.
constexpr int kReduceThreads = 1024;

template <class F>
__global__ void __launch_bounds__(kReduceThreads)
    reduce_rows_kernel(const typename F::E* __restrict__ partial, uint32_t rows, uint32_t cols,
                       uint32_t cw, typename F::E* __restrict__ out) {
  using E = typename F::E;
  __shared__ E red[kReduceThreads];
  const uint32_t slices = kReduceThreads / cw;
  const uint32_t slice = threadIdx.x / cw;
  const uint32_t c = blockIdx.x * cw + threadIdx.x % cw;
  E acc = 0;
  if (c < cols) {
    // eight predicated loads in flight per step
    for (uint32_t r = slice; r < rows; r += 8 * slices) {
      E v[8];
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const uint32_t rr = r + k * slices;
        v[k] = rr < rows ? partial[(uint64_t)rr * cols + c] : (E)0;
      }
#pragma unroll
      for (int k = 0; k < 8; k++) acc = F::add(acc, v[k]);
    }
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (uint32_t h = slices >> 1; h >= 1; h >>= 1) {
    if (slice < h) red[threadIdx.x] = F::add(red[threadIdx.x], red[threadIdx.x + h * cw]);
    __syncthreads();
  }
  if (slice == 0 && c < cols) out[c] = red[threadIdx.x];
}

template <class F>
static int launch_reduce_rows(const typename F::E* partial, uint64_t rows, uint64_t cols,
                              typename F::E* out, cudaStream_t stream) {
  uint32_t cw = 1;
  while (cw < 32 && cw < cols) cw <<= 1;
  const unsigned blocks = (unsigned)((cols + cw - 1) / cw);
  reduce_rows_kernel<F><<<blocks, kReduceThreads, 0, stream>>>(partial, (uint32_t)rows, (uint32_t)cols,
                                                               cw, out);
  OMR_CUDA_TRY(cudaGetLastError());
  return OMR_NTT_OK;
}

template <class F, int LOGT>
static int launch_prefix_t(omr_ntt_domain_s* d, uint32_t m, const void* in, void* out,
                           cudaStream_t stream) {
  using E = typename F::E;
  using Tw = typename F::Tw;
  constexpr int T = 1 << LOGT;
  constexpr int C = prefix_cols<F, LOGT>();
  constexpr int NT = prefix_threads<F, LOGT>();
  constexpr size_t smem = (size_t)T * C * sizeof(E);
  auto kern = prefix_decomp_kernel<F, LOGT>;
  static std::atomic<int> occ_cache[64];
  int dev = 0;
  OMR_CUDA_TRY(cudaGetDevice(&dev));
  int occ = occ_cache[dev & 63].load();
  if (occ == 0) {
    if (smem > 48 * 1024)
      OMR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    OMR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, NT, smem));
    occ_cache[dev & 63] = occ < 1 ? 1 : occ;
    occ = occ_cache[dev & 63];
  }
  RootTables rt;
  int rc = get_root_tables(F::ID, &rt);
  if (rc) return rc;
  PassArgs<F> a{};
  a.in = static_cast<const E*>(in);
  a.L_lo = (uint32_t)(d->n >> LOGT);  // columns r
  a.L_m = 1;
  a.L_b = 1;
  a.is_lo = 1;
  a.es_in = (uint32_t)(d->n >> LOGT);
  a.roots = static_cast<const Tw*>(rt.fwd);
  a.roots_stride = 1u << (kMaxLogT - LOGT);
  a.tw_lo = static_cast<const E*>(d->tw_lo_f);
  a.tw_hi = static_cast<const Tw*>(d->tw_hi_f);
  a.tw_scale = 1;
  a.tw_mask = (uint32_t)(d->n - 1);
  a.tw_line_mul_m = 0;
  const uint32_t groups = (a.L_lo + C - 1) / C;
  uint32_t grid = (uint32_t)device_sm_count(dev) * (uint32_t)occ;
  if (grid > groups) grid = groups;
  void* part = nullptr;
  rc = domain_scratch(d, stream, (size_t)grid * m * sizeof(E), &part, 1);
  if (rc) return rc;
  kern<<<grid, NT, smem, stream>>>(a, m, static_cast<E*>(part));
  OMR_CUDA_TRY(cudaGetLastError());
  return launch_reduce_rows<F>(static_cast<const E*>(part), grid, m, static_cast<E*>(out), stream);
}

template <class F>
static int launch_prefix(omr_ntt_domain_s* d, uint32_t m, int logt, const void* in, void* out,
                         cudaStream_t stream) {
  if (logt <= 0) {
    logt = 0;
    while ((1u << logt) < m) logt++;
    if (logt == 0) logt = 1;
  }
  if ((1u << logt) < m || (uint32_t)logt > d->log_n) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "decomposition line shorter than the prefix");
  switch (logt) {
    case 1: return launch_prefix_t<F, 1>(d, m, in, out, stream);
    case 2: return launch_prefix_t<F, 2>(d, m, in, out, stream);
    case 3: return launch_prefix_t<F, 3>(d, m, in, out, stream);
    case 4: return launch_prefix_t<F, 4>(d, m, in, out, stream);
    case 5: return launch_prefix_t<F, 5>(d, m, in, out, stream);
    case 6: return launch_prefix_t<F, 6>(d, m, in, out, stream);
    case 7: return launch_prefix_t<F, 7>(d, m, in, out, stream);
    case 8: return launch_prefix_t<F, 8>(d, m, in, out, stream);
    case 9: return launch_prefix_t<F, 9>(d, m, in, out, stream);
    case 10: return launch_prefix_t<F, 10>(d, m, in, out, stream);
    case 11: return launch_prefix_t<F, 11>(d, m, in, out, stream);
    case 12: return launch_prefix_t<F, 12>(d, m, in, out, stream);
  }
  return fail(OMR_NTT_ERR_SIZE, "prefix decomposition needs m <= 4096");
}

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

enum { STRAT_DECOMP_ = 1, STRAT_FOLD_ = 2, STRAT_GATHER_ = 3 };

// Strided fold for narrow outputs (count <= 4096): one grid-stride sweep over
// x with a stride that is a multiple of count, so every thread stays in one
// column; per-CTA partial column sums land in partial[rows][count].
template <class F>
__global__ void __launch_bounds__(256) fold_flat_kernel(const typename F::E* __restrict__ x,
                                                        uint64_t n, uint32_t count,
                                                        typename F::E* __restrict__ partial) {
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
    fold_vec_kernel<F><<<grid, kFoldThreads, 0, stream>>>(static_cast<const E*>(in), d->n, (uint32_t)count, part);
    OMR_CUDA_TRY(cudaGetLastError());
    nch = count > ch ? grid / (count / ch) : grid;
  } else if (count <= 4096 && d->n >= 256ull * 1216) {
    const uint32_t grid = 1216;  // 8 CTAs per SM; a multiple of count / 256 for count <= 4096
    fold_flat_kernel<F><<<grid, 256, 0, stream>>>(static_cast<const E*>(in), d->n, (uint32_t)count, part);
    OMR_CUDA_TRY(cudaGetLastError());
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
  gather_kernel<F><<<blocks, 256, 0, stream>>>(static_cast<const E*>(full), d->n, pattern, count,
                                              indices, static_cast<E*>(out));
  OMR_CUDA_TRY(cudaGetLastError());
  return OMR_NTT_OK;
}

template <class F>
static int run_strategy_t(omr_ntt_domain_s* d, int strategy, int param, int pattern,
                          uint64_t count, const uint32_t* indices, const void* in, void* out,
                          cudaStream_t stream) {
  const uint64_t n = d->n;
  switch (strategy) {
    case STRAT_DECOMP_:
      if (pattern != OMR_NTT_PATTERN_PREFIX || count > 4096 || count >= n)
        return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "decomposition serves prefixes of <= 4096 outputs");
      return launch_prefix<F>(d, (uint32_t)count, param, in, out, stream);
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
  if (pattern == OMR_NTT_PATTERN_STRIDED && count < n)
    return run_fold<F>(d, -1, count, in, out, stream);
  if (pattern == OMR_NTT_PATTERN_PREFIX && count <= 4096 && count < n && n / count >= 2)
    return launch_prefix<F>(d, (uint32_t)count, 0, in, out, stream);
  return run_gather<F>(d, -1, pattern, count, indices, in, out, stream);
}

template <class F>
int launch_gather_indices(const void* full, uint64_t n, uint64_t count, const uint32_t* idx,
                          void* out, cudaStream_t stream) {
  using E = typename F::E;
  if (count == 0) return OMR_NTT_OK;
  gather_kernel<F><<<(unsigned)((count + 255) / 256), 256, 0, stream>>>(
      static_cast<const E*>(full), n, OMR_NTT_PATTERN_INDICES, count, idx, static_cast<E*>(out));
  OMR_CUDA_TRY(cudaGetLastError());
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
