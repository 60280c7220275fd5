// partial_prefix.cuh -- the pruned prefix transform and the row reduction
// shared by the partial-output paths.  launch_prefix<F> is instantiated once
// per field in partial_prefix_<field>.cu (parallel compiles); every other
// translation unit sees the extern declarations below.
#pragma once
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
//
// The same sum serves any output index, not just a prefix: with M = N / T
// columns, X[j] = sum_{r < M} omega_N^(r j) * Y_r[j mod T] for every j < N.
// With an index list (idx != nullptr), output slot q < m is X[idx[q]]: its
// tile row is idx[q] mod T and its Horner factor omega_N^(-TPK idx[q]) -- an
// index-set request of m <= T outputs costs the prefix's work instead of a
// full transform and a gather.
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

// Shared-memory words of the kernel: the tile, and for lines longer than the
// CTA (more outputs than threads) one accumulator and one Horner multiplier
// per output, which would not fit in registers.
template <class F, int LOGT>
constexpr size_t prefix_smem_bytes() {
  constexpr size_t T = (size_t)1 << LOGT;
  constexpr size_t tile = T * prefix_cols<F, LOGT>() * sizeof(typename F::E);
  return T > (size_t)prefix_threads<F, LOGT>()
             ? tile + T * (sizeof(typename F::E) + sizeof(typename F::Tw))
             : tile;
}

template <class F, int LOGT>
__global__ void __launch_bounds__(prefix_threads<F, LOGT>(), 2)
    prefix_decomp_kernel(const PassArgs<F> a, uint32_t m, const uint32_t* __restrict__ idx,
                         typename F::E* __restrict__ partial) {
  pdl_entry();
  using E = typename F::E;
  using Tw = typename F::Tw;
  constexpr int T = 1 << LOGT;
  constexpr int C = prefix_cols<F, LOGT>();
  constexpr int NT = prefix_threads<F, LOGT>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  E* s = reinterpret_cast<E*>(smem_raw);
  // m > NT (only when T > NT): outputs k = t + j NT, accumulators in smem
  E* acc_s = s + (size_t)T * C;
  Tw* zi_s = reinterpret_cast<Tw*>(acc_s + T);

  // thread -> KACT adjacent outputs x TPK column slices (m <= NT), or
  // outputs k = t + j NT (m > NT, one slice)
  uint32_t kact = 1;
  while (kact < m && kact < (uint32_t)NT) kact <<= 1;
  const uint32_t tpk = min((uint32_t)NT / kact, (uint32_t)C);
  const bool many = m > (uint32_t)NT;
  const uint32_t kbase = threadIdx.x % kact;
  const uint32_t slice = threadIdx.x / kact;
  const bool active = slice < tpk && kbase < m;
  // output slot q is X[jq]: a prefix (jq = q) or an index list; its tile row
  // is jq mod T
  auto out_index = [&](uint32_t q) -> uint32_t { return idx ? idx[q] : q; };
  // an index past N yields 0, as the gather of the full transform gives it
  auto in_range = [&](uint32_t q) -> bool { return (uint64_t)out_index(q) <= (uint64_t)a.tw_mask; };
  const uint32_t jb = active ? out_index(kbase) : 0u;
  const int rowb = (int)(jb & (uint32_t)(T - 1));

  E acc = 0;
  const Tw zi = omega_tw<F>(a, (uint64_t)0 - (uint64_t)tpk * jb);  // omega_N^(-TPK j)
  if constexpr (T > NT) {
    if (many)
      for (uint32_t k = threadIdx.x; k < m; k += NT) {  // this thread's outputs only
        acc_s[k] = 0;
        zi_s[k] = omega_tw<F>(a, (uint64_t)0 - (uint64_t)out_index(k));
      }
  }

  const uint32_t groups = (a.L_lo + C - 1) / C;
  const uint32_t g0 = (uint32_t)((uint64_t)blockIdx.x * groups / gridDim.x);
  const uint32_t g1 = (uint32_t)((uint64_t)(blockIdx.x + 1) * groups / gridDim.x);
  for (uint32_t g = g0; g < g1; g++) {
    const uint32_t llo0 = g * C;
    const int nvalid = (int)min((uint32_t)C, a.L_lo - llo0);
    prefix_rounds<F, LOGT, C, NT, 0>(a, s, a.in + llo0, nvalid);
    if constexpr (T > NT) {
      if (many) {
        for (uint32_t k = threadIdx.x; k < m; k += NT) {
          E h = acc_s[k];
          const Tw z = zi_s[k];
          const int row = (int)(out_index(k) & (uint32_t)(T - 1));
#pragma unroll
          for (int c = 0; c < C; c++) h = F::add(F::mul_tw(h, z), s[tile_idx<F, C>(row, c)]);
          acc_s[k] = h;
        }
      }
    }
    if (!many && active) {
#pragma unroll 4
      for (uint32_t c = slice; c < (uint32_t)C; c += tpk)
        acc = F::add(F::mul_tw(acc, zi), s[tile_idx<F, C>(rowb, (int)c)]);
    }
    __syncthreads();  // the next group's first round overwrites the tile
  }
  if constexpr (T > NT) {
    if (many) {
      const uint64_t r_last = (uint64_t)(g1 - 1) * C + (C - 1);
      for (uint32_t k = threadIdx.x; k < m; k += NT)
        partial[(uint64_t)blockIdx.x * m + k] =
            g1 > g0 && in_range(k) ? mul_m<F>(acc_s[k], omega_m<F>(a, r_last * out_index(k))) : (E)0;
      return;
    }
  }
  if (g1 > g0 && active) {
    const uint64_t r_last = (uint64_t)(g1 - 1) * C + (C - tpk) + slice;
    acc = in_range(kbase) ? mul_m<F>(acc, omega_m<F>(a, r_last * jb)) : (E)0;
  }
  if (tpk > 1) {
    // combine the slices of every output: s[slice * kact + k]
    if (slice < tpk) s[slice * kact + kbase] = active ? acc : (E)0;
    __syncthreads();
    if (threadIdx.x < m) {
      E sum = 0;
      for (uint32_t sl = 0; sl < tpk; sl++) sum = F::add(sum, s[sl * kact + threadIdx.x]);
      partial[(uint64_t)blockIdx.x * m + threadIdx.x] = sum;
    }
  } else if (threadIdx.x < m) {
    partial[(uint64_t)blockIdx.x * m + threadIdx.x] = acc;
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
  pdl_entry();
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
inline int launch_reduce_rows(const typename F::E* partial, uint64_t rows, uint64_t cols,
                              typename F::E* out, cudaStream_t stream) {
  uint32_t cw = 1;
  while (cw < 32 && cw < cols) cw <<= 1;
  const unsigned blocks = (unsigned)((cols + cw - 1) / cw);
  OMR_CUDA_TRY(launch_pdl(reduce_rows_kernel<F>, dim3(blocks), dim3(kReduceThreads), 0, stream, partial,
                          (uint32_t)rows, (uint32_t)cols, cw, out));
  return OMR_NTT_OK;
}

template <class F, int LOGT>
inline int launch_prefix_t(omr_ntt_domain_s* d, uint32_t m, const uint32_t* idx, const void* in,
                           void* out, cudaStream_t stream) {
  using E = typename F::E;
  using Tw = typename F::Tw;
  constexpr int T = 1 << LOGT;
  constexpr int C = prefix_cols<F, LOGT>();
  constexpr int NT = prefix_threads<F, LOGT>();
  constexpr size_t smem = prefix_smem_bytes<F, LOGT>();
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
  OMR_CUDA_TRY(launch_pdl(kern, dim3(grid), dim3(NT), smem, stream, a, m, idx, static_cast<E*>(part)));
  return launch_reduce_rows<F>(static_cast<const E*>(part), grid, m, static_cast<E*>(out), stream);
}

// m outputs: X[0..m) (idx == nullptr) or X[idx[q]] (device index list, every
// idx[q] < N), line length 2^logt >= m (logt <= 0: the shortest).
template <class F>
int launch_prefix(omr_ntt_domain_s* d, uint32_t m, int logt, const void* in, void* out,
                  cudaStream_t stream, const uint32_t* idx) {
  if (logt <= 0) {
    logt = 0;
    while ((1u << logt) < m) logt++;
    if (logt == 0) logt = 1;
  }
  if ((1u << logt) < m || (uint32_t)logt > d->log_n) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "decomposition line shorter than the prefix");
  switch (logt) {
    case 1: return launch_prefix_t<F, 1>(d, m, idx, in, out, stream);
    case 2: return launch_prefix_t<F, 2>(d, m, idx, in, out, stream);
    case 3: return launch_prefix_t<F, 3>(d, m, idx, in, out, stream);
    case 4: return launch_prefix_t<F, 4>(d, m, idx, in, out, stream);
    case 5: return launch_prefix_t<F, 5>(d, m, idx, in, out, stream);
    case 6: return launch_prefix_t<F, 6>(d, m, idx, in, out, stream);
    case 7: return launch_prefix_t<F, 7>(d, m, idx, in, out, stream);
    case 8: return launch_prefix_t<F, 8>(d, m, idx, in, out, stream);
    case 9: return launch_prefix_t<F, 9>(d, m, idx, in, out, stream);
    case 10: return launch_prefix_t<F, 10>(d, m, idx, in, out, stream);
    case 11: return launch_prefix_t<F, 11>(d, m, idx, in, out, stream);
    case 12: return launch_prefix_t<F, 12>(d, m, idx, in, out, stream);
  }
  return fail(OMR_NTT_ERR_SIZE, "prefix decomposition needs m <= 4096");
}

extern template int launch_prefix<BabyBear>(omr_ntt_domain_s*, uint32_t, int, const void*, void*, cudaStream_t,
                                        const uint32_t*);
extern template int launch_prefix<Goldilocks>(omr_ntt_domain_s*, uint32_t, int, const void*, void*, cudaStream_t,
                                        const uint32_t*);
extern template int launch_prefix<KoalaBear>(omr_ntt_domain_s*, uint32_t, int, const void*, void*, cudaStream_t,
                                        const uint32_t*);
extern template int launch_prefix<TeddyBear>(omr_ntt_domain_s*, uint32_t, int, const void*, void*, cudaStream_t,
                                        const uint32_t*);

}  // namespace omr
