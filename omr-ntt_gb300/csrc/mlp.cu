// mlp.cu -- the learned plan selector: a small fp32 MLP cost model trained on
// the GPU with hand-written kernels.
//
// Network: features (10) -> 64 -> ReLU -> 64 -> ReLU -> one score per plan
// class (64, tuner.cu).  A score is the predicted log run time of the class
// relative to the mean over the point's applicable classes; the selector
// takes the applicable class with the lowest score.  Training minimises the
// masked mean squared error against the autotuner's measured (centred) log
// times with Adam.  Every kernel computes each output element in one thread
// with a fixed summation order, so training is deterministic.  All plans are
// exact: the network can change speed, never a result.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "engine.cuh"

namespace omr {

constexpr int kFeatures = 10;

// Y[r, o] = act(sum_k X[r, k] W[o, k] + b[o])
__global__ void mlp_linear_fwd(const float* __restrict__ X, const float* __restrict__ W,
                               const float* __restrict__ b, float* __restrict__ Y, int B, int in,
                               int out, int relu) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B * out) return;
  const int r = i / out, o = i % out;
  float acc = b[o];
  for (int k = 0; k < in; k++) acc = fmaf(X[r * in + k], W[o * in + k], acc);
  Y[i] = relu ? fmaxf(acc, 0.f) : acc;
}

// dY = 2 mask (Y - T) / denom ; loss partials per row
__global__ void mlp_loss_grad(const float* __restrict__ Y, const float* __restrict__ T,
                              const float* __restrict__ M, float* __restrict__ dY,
                              float* __restrict__ row_loss, int B, int out, float denom) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= B) return;
  float l = 0.f;
  for (int o = 0; o < out; o++) {
    const int i = r * out + o;
    const float d = M[i] * (Y[i] - T[i]);
    dY[i] = 2.f * d / denom;
    l += d * d;
  }
  row_loss[r] = l / denom;
}

// dX[r, k] = (sum_o dY[r, o] W[o, k]) * relu'(H[r, k])   (H = forward output of that layer)
__global__ void mlp_linear_bwd_input(const float* __restrict__ dY, const float* __restrict__ W,
                                     const float* __restrict__ H, float* __restrict__ dX, int B,
                                     int in, int out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B * in) return;
  const int r = i / in, k = i % in;
  float acc = 0.f;
  for (int o = 0; o < out; o++) acc = fmaf(dY[r * out + o], W[o * in + k], acc);
  dX[i] = H[i] > 0.f ? acc : 0.f;
}

// dW[o, k] = sum_r dY[r, o] X[r, k] ; db[o] = sum_r dY[r, o]
__global__ void mlp_linear_bwd_params(const float* __restrict__ dY, const float* __restrict__ X,
                                      float* __restrict__ dW, float* __restrict__ db, int B,
                                      int in, int out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < out * in) {
    const int o = i / in, k = i % in;
    float acc = 0.f;
    for (int r = 0; r < B; r++) acc = fmaf(dY[r * out + o], X[r * in + k], acc);
    dW[i] = acc;
  }
  if (i < out) {
    float acc = 0.f;
    for (int r = 0; r < B; r++) acc += dY[r * out + i];
    db[i] = acc;
  }
}

__global__ void mlp_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                         float* __restrict__ v, int n, float lr, float b1, float b2, float eps,
                         float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void mlp_sum_rows(const float* __restrict__ row, int B, float* __restrict__ out) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    float s = 0.f;
    for (int r = 0; r < B; r++) s += row[r];
    *out = s;
  }
}

}  // namespace omr

using namespace omr;

struct omr_ntt_mlp_s {
  int nin, nh, nout;
  int nparam;
  int device;
  float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;  // params, grads, Adam moments
  int cap = 0;                                                    // rows of the work buffers
  float *x = nullptr, *t = nullptr, *mask = nullptr;
  float *h1 = nullptr, *h2 = nullptr, *y = nullptr;
  float *dy = nullptr, *dh2 = nullptr, *dh1 = nullptr, *rowloss = nullptr, *loss = nullptr;
  int step = 0;
  std::mutex mu;
  // parameter offsets
  int oW1() const { return 0; }
  int ob1() const { return nh * nin; }
  int oW2() const { return ob1() + nh; }
  int ob2() const { return oW2() + nh * nh; }
  int oW3() const { return ob2() + nh; }
  int ob3() const { return oW3() + nout * nh; }
};

static std::mutex g_mlp_mu;
static omr_ntt_mlp_s* g_installed = nullptr;

static int mlp_reserve(omr_ntt_mlp_s* m, int B) {
  if (B <= m->cap) return OMR_NTT_OK;
  float** bufs[] = {&m->x, &m->t, &m->mask, &m->h1, &m->h2, &m->y, &m->dy, &m->dh2, &m->dh1, &m->rowloss};
  for (auto b : bufs) {
    cudaFree(*b);
    *b = nullptr;
  }
  const size_t sizes[] = {(size_t)B * m->nin, (size_t)B * m->nout, (size_t)B * m->nout,
                          (size_t)B * m->nh,  (size_t)B * m->nh,   (size_t)B * m->nout,
                          (size_t)B * m->nout, (size_t)B * m->nh,  (size_t)B * m->nh, (size_t)B};
  for (int i = 0; i < 10; i++)
    if (cudaMalloc(bufs[i], sizes[i] * sizeof(float)) != cudaSuccess)
      return fail(OMR_NTT_ERR_ALLOC, "mlp work buffers");
  m->cap = B;
  return OMR_NTT_OK;
}

static inline int nblk(int n) { return (n + 255) / 256; }

static void mlp_forward_dev(omr_ntt_mlp_s* m, int B, cudaStream_t s) {
  mlp_linear_fwd<<<nblk(B * m->nh), 256, 0, s>>>(m->x, m->p + m->oW1(), m->p + m->ob1(), m->h1, B,
                                                  m->nin, m->nh, 1);
  mlp_linear_fwd<<<nblk(B * m->nh), 256, 0, s>>>(m->h1, m->p + m->oW2(), m->p + m->ob2(), m->h2, B,
                                                  m->nh, m->nh, 1);
  mlp_linear_fwd<<<nblk(B * m->nout), 256, 0, s>>>(m->h2, m->p + m->oW3(), m->p + m->ob3(), m->y, B,
                                                    m->nh, m->nout, 0);
}

static void mlp_backward_dev(omr_ntt_mlp_s* m, int B, float denom, cudaStream_t s) {
  mlp_loss_grad<<<nblk(B), 256, 0, s>>>(m->y, m->t, m->mask, m->dy, m->rowloss, B, m->nout, denom);
  mlp_sum_rows<<<1, 32, 0, s>>>(m->rowloss, B, m->loss);
  mlp_linear_bwd_params<<<nblk(m->nout * m->nh), 256, 0, s>>>(m->dy, m->h2, m->g + m->oW3(),
                                                               m->g + m->ob3(), B, m->nh, m->nout);
  mlp_linear_bwd_input<<<nblk(B * m->nh), 256, 0, s>>>(m->dy, m->p + m->oW3(), m->h2, m->dh2, B,
                                                        m->nh, m->nout);
  mlp_linear_bwd_params<<<nblk(m->nh * m->nh), 256, 0, s>>>(m->dh2, m->h1, m->g + m->oW2(),
                                                             m->g + m->ob2(), B, m->nh, m->nh);
  mlp_linear_bwd_input<<<nblk(B * m->nh), 256, 0, s>>>(m->dh2, m->p + m->oW2(), m->h1, m->dh1, B,
                                                        m->nh, m->nh);
  mlp_linear_bwd_params<<<nblk(m->nh * m->nin), 256, 0, s>>>(m->dh1, m->x, m->g + m->oW1(),
                                                              m->g + m->ob1(), B, m->nin, m->nh);
}

static float mask_denom(const float* mask, int B, int nout) {
  double s = 0;
  for (int i = 0; i < B * nout; i++) s += mask[i];
  return s > 0 ? (float)s : 1.f;
}

namespace omr {

// Planner hook (tuner.cu): lowest predicted score among applicable classes.
int mlp_select_class(int field, uint32_t log_n, uint64_t batch, int pattern, uint64_t count,
                     const bool* applicable, int n_classes);

}  // namespace omr

extern "C" {

int omr_ntt_mlp_features(int field, uint32_t log_n, uint64_t batch, int pattern, uint64_t count,
                         float* f) {
  if (!f) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null features");
  const uint64_t n = 1ull << log_n;
  const bool full = count == 0 || count >= n;
  double ls = full ? (double)log_n : std::log2((double)count);
  double lb = std::log2((double)(batch ? batch : 1));
  f[0] = field == GOLDILOCKS ? 1.f : 0.f;
  f[1] = (float)(log_n / 24.0);
  f[2] = (float)(ls / 24.0);
  f[3] = (float)((log_n - ls) / 24.0);
  f[4] = !full && pattern == OMR_NTT_PATTERN_PREFIX ? 1.f : 0.f;
  f[5] = !full && pattern == OMR_NTT_PATTERN_STRIDED ? 1.f : 0.f;
  f[6] = !full && pattern == OMR_NTT_PATTERN_INDICES ? 1.f : 0.f;
  f[7] = (float)(lb / 9.0);
  f[8] = (float)((log_n + lb) / 33.0);
  f[9] = full ? 1.f : 0.f;
  return kFeatures;
}

int omr_ntt_mlp_create(int n_in, int n_hidden, int n_out, uint64_t seed, omr_ntt_mlp_t* out) {
  if (!out || n_in <= 0 || n_hidden <= 0 || n_out <= 0)
    return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "bad mlp shape");
  auto* m = new (std::nothrow) omr_ntt_mlp_s();
  if (!m) return fail(OMR_NTT_ERR_ALLOC, "mlp");
  m->nin = n_in;
  m->nh = n_hidden;
  m->nout = n_out;
  m->nparam = m->ob3() + n_out;
  cudaGetDevice(&m->device);
  const size_t bytes = sizeof(float) * m->nparam;
  if (cudaMalloc(&m->p, bytes) != cudaSuccess || cudaMalloc(&m->g, bytes) != cudaSuccess ||
      cudaMalloc(&m->m, bytes) != cudaSuccess || cudaMalloc(&m->v, bytes) != cudaSuccess ||
      cudaMalloc(&m->loss, sizeof(float)) != cudaSuccess) {
    omr_ntt_mlp_destroy(m);
    return fail(OMR_NTT_ERR_ALLOC, "mlp parameters");
  }
  // He-uniform initialisation from a seeded splitmix64 stream; zero biases
  std::vector<float> h(m->nparam, 0.f);
  uint64_t st = seed;
  auto uni = [&]() {
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) / 9007199254740992.0 * 2.0 - 1.0;
  };
  auto fill = [&](int off, int rows, int cols) {
    const double a = std::sqrt(6.0 / cols);
    for (int i = 0; i < rows * cols; i++) h[off + i] = (float)(a * uni());
  };
  fill(m->oW1(), n_hidden, n_in);
  fill(m->oW2(), n_hidden, n_hidden);
  fill(m->oW3(), n_out, n_hidden);
  cudaMemcpy(m->p, h.data(), bytes, cudaMemcpyHostToDevice);
  cudaMemset(m->m, 0, bytes);
  cudaMemset(m->v, 0, bytes);
  cudaMemset(m->g, 0, bytes);
  *out = m;
  return OMR_NTT_OK;
}

int omr_ntt_mlp_destroy(omr_ntt_mlp_t m) {
  if (!m) return OMR_NTT_OK;
  {
    std::lock_guard<std::mutex> lk(g_mlp_mu);
    if (g_installed == m) g_installed = nullptr;
  }
  float* bufs[] = {m->p, m->g, m->m, m->v, m->x, m->t, m->mask, m->h1, m->h2, m->y, m->dy, m->dh2, m->dh1, m->rowloss, m->loss};
  for (auto b : bufs) cudaFree(b);
  delete m;
  return OMR_NTT_OK;
}

int omr_ntt_mlp_param_count(omr_ntt_mlp_t m) { return m ? m->nparam : 0; }

int omr_ntt_mlp_get_params(omr_ntt_mlp_t m, float* host) {
  if (!m || !host) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null argument");
  OMR_CUDA_TRY(cudaMemcpy(host, m->p, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost));
  return OMR_NTT_OK;
}

int omr_ntt_mlp_set_params(omr_ntt_mlp_t m, const float* host) {
  if (!m || !host) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null argument");
  OMR_CUDA_TRY(cudaMemcpy(m->p, host, sizeof(float) * m->nparam, cudaMemcpyHostToDevice));
  return OMR_NTT_OK;
}

// y[B, n_out] = network(x[B, n_in]) (host arrays)
int omr_ntt_mlp_forward(omr_ntt_mlp_t m, const float* x, int B, float* y) {
  if (!m || !x || !y || B <= 0) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "bad forward call");
  std::lock_guard<std::mutex> lk(m->mu);
  DeviceGuard g(m->device);
  int rc = mlp_reserve(m, B);
  if (rc) return rc;
  OMR_CUDA_TRY(cudaMemcpy(m->x, x, sizeof(float) * B * m->nin, cudaMemcpyHostToDevice));
  mlp_forward_dev(m, B, nullptr);
  OMR_CUDA_TRY(cudaGetLastError());
  OMR_CUDA_TRY(cudaMemcpy(y, m->y, sizeof(float) * B * m->nout, cudaMemcpyDeviceToHost));
  return OMR_NTT_OK;
}

// Gradients of the masked MSE at the current parameters (no update):
// grad[n_param] in the parameter layout W1, b1, W2, b2, W3, b3.
int omr_ntt_mlp_gradients(omr_ntt_mlp_t m, const float* x, const float* target, const float* mask,
                          int B, float* grad, float* loss) {
  if (!m || !x || !target || !mask || B <= 0) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "bad call");
  std::lock_guard<std::mutex> lk(m->mu);
  DeviceGuard g(m->device);
  int rc = mlp_reserve(m, B);
  if (rc) return rc;
  OMR_CUDA_TRY(cudaMemcpy(m->x, x, sizeof(float) * B * m->nin, cudaMemcpyHostToDevice));
  OMR_CUDA_TRY(cudaMemcpy(m->t, target, sizeof(float) * B * m->nout, cudaMemcpyHostToDevice));
  OMR_CUDA_TRY(cudaMemcpy(m->mask, mask, sizeof(float) * B * m->nout, cudaMemcpyHostToDevice));
  mlp_forward_dev(m, B, nullptr);
  mlp_backward_dev(m, B, mask_denom(mask, B, m->nout), nullptr);
  OMR_CUDA_TRY(cudaGetLastError());
  if (grad) OMR_CUDA_TRY(cudaMemcpy(grad, m->g, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost));
  if (loss) OMR_CUDA_TRY(cudaMemcpy(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost));
  return OMR_NTT_OK;
}

// Full-batch-free training on device: `epochs` passes over n points in
// minibatches of B (order reshuffled per epoch from `seed`), Adam(lr).
// loss_hist[epoch] = mean minibatch loss (optional).
int omr_ntt_mlp_fit(omr_ntt_mlp_t m, const float* x, const float* target, const float* mask, int n,
                    int epochs, int B, float lr, uint64_t seed, float* loss_hist) {
  if (!m || !x || !target || !mask || n <= 0 || B <= 0) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "bad fit call");
  std::lock_guard<std::mutex> lk(m->mu);
  DeviceGuard g(m->device);
  int rc = mlp_reserve(m, B);
  if (rc) return rc;
  std::vector<int> order(n);
  for (int i = 0; i < n; i++) order[i] = i;
  std::vector<float> bx((size_t)B * m->nin), bt((size_t)B * m->nout), bm((size_t)B * m->nout);
  uint64_t st = seed;
  auto next = [&]() {
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int e = 0; e < epochs; e++) {
    for (int i = n - 1; i > 0; i--) std::swap(order[i], order[next() % (i + 1)]);
    double tot = 0;
    int nb = 0;
    for (int s0 = 0; s0 < n; s0 += B) {
      const int bs = std::min(B, n - s0);
      for (int r = 0; r < bs; r++) {
        const int src = order[s0 + r];
        std::memcpy(&bx[(size_t)r * m->nin], x + (size_t)src * m->nin, sizeof(float) * m->nin);
        std::memcpy(&bt[(size_t)r * m->nout], target + (size_t)src * m->nout, sizeof(float) * m->nout);
        std::memcpy(&bm[(size_t)r * m->nout], mask + (size_t)src * m->nout, sizeof(float) * m->nout);
      }
      OMR_CUDA_TRY(cudaMemcpy(m->x, bx.data(), sizeof(float) * bs * m->nin, cudaMemcpyHostToDevice));
      OMR_CUDA_TRY(cudaMemcpy(m->t, bt.data(), sizeof(float) * bs * m->nout, cudaMemcpyHostToDevice));
      OMR_CUDA_TRY(cudaMemcpy(m->mask, bm.data(), sizeof(float) * bs * m->nout, cudaMemcpyHostToDevice));
      mlp_forward_dev(m, bs, nullptr);
      mlp_backward_dev(m, bs, mask_denom(bm.data(), bs, m->nout), nullptr);
      m->step++;
      const float c1 = 1.f - std::pow(b1, (float)m->step), c2 = 1.f - std::pow(b2, (float)m->step);
      mlp_adam<<<nblk(m->nparam), 256>>>(m->p, m->g, m->m, m->v, m->nparam, lr, b1, b2, eps, c1, c2);
      float l = 0;
      OMR_CUDA_TRY(cudaMemcpy(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost));
      tot += l;
      nb++;
    }
    OMR_CUDA_TRY(cudaGetLastError());
    if (loss_hist) loss_hist[e] = (float)(tot / (nb ? nb : 1));
  }
  return OMR_NTT_OK;
}

// Load a network written as: "OMRM", uint32 n_in, n_hidden, n_out, then the
// float32 parameters (little endian, layout of omr_ntt_mlp_get_params).
int omr_ntt_mlp_load(const char* path, omr_ntt_mlp_t* out) {
  if (!path || !out) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, "null argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(OMR_NTT_ERR_INVALID_ARGUMENT, std::string("cannot read ") + path);
  char magic[4];
  uint32_t dims[3];
  bool ok = std::fread(magic, 1, 4, f) == 4 && std::memcmp(magic, "OMRM", 4) == 0 &&
            std::fread(dims, 4, 3, f) == 3 && dims[0] > 0 && dims[0] < 4096 && dims[1] > 0 &&
            dims[1] < 4096 && dims[2] > 0 && dims[2] < 4096;
  omr_ntt_mlp_t m = nullptr;
  int rc = OMR_NTT_OK;
  if (ok) rc = omr_ntt_mlp_create((int)dims[0], (int)dims[1], (int)dims[2], 0, &m);
  if (ok && !rc) {
    std::vector<float> p(m->nparam);
    ok = std::fread(p.data(), sizeof(float), p.size(), f) == p.size();
    if (ok) rc = omr_ntt_mlp_set_params(m, p.data());
  }
  std::fclose(f);
  if (!ok || rc) {
    omr_ntt_mlp_destroy(m);
    return rc ? rc : fail(OMR_NTT_ERR_INVALID_ARGUMENT, std::string("malformed network file ") + path);
  }
  *out = m;
  return OMR_NTT_OK;
}

// Make `m` (features -> kNumClasses scores) the planner's learned selector
// (m = NULL uninstalls it); the planner still prefers its database.
int omr_ntt_mlp_install(omr_ntt_mlp_t m) {
  std::lock_guard<std::mutex> lk(g_mlp_mu);
  g_installed = m;
  omr_ntt_planner_use_mlp(m != nullptr);
  return OMR_NTT_OK;
}

}  // extern "C"

namespace omr {

int mlp_select_class(int field, uint32_t log_n, uint64_t batch, int pattern, uint64_t count,
                     const bool* applicable, int n_classes) {
  omr_ntt_mlp_s* m;
  {
    std::lock_guard<std::mutex> lk(g_mlp_mu);
    m = g_installed;
  }
  if (!m || m->nin != kFeatures || m->nout != n_classes) return -1;
  float f[kFeatures];
  omr_ntt_mlp_features(field, log_n, batch, pattern, count, f);
  std::vector<float> y(m->nout);
  if (omr_ntt_mlp_forward(m, f, 1, y.data())) return -1;
  int best = -1;
  for (int c = 0; c < n_classes; c++)
    if (applicable[c] && (best < 0 || y[c] < y[best])) best = c;
  return best;
}

}  // namespace omr
