// tt_mlp.cu -- the learned variant selector's network: a 12 -> 64 -> 64 -> 64 ->
// nout multilayer perceptron (ReLU on the hidden layers) with its forward,
// masked-MSE loss, backward and Adam kernels.
//
// The reference picks kernel variants by an offline codegen sweep
// (generated_kernels/codegen.py:44-247 and the *_tune.sh scripts) and a person
// reading the timings.  Here the sweep's timings train this network, which then
// scores every variant from a tensor's features; the sweep stays available as a
// selection mode and as the yardstick of the network's picks (regret against the
// sweep's best), and the fixed heuristic is the fallback where no model applies.
//
// Parameters are one flat FP32 array, layer by layer: W_l (K_l x N_l, row-major,
// W[k * N + n]) then b_l (N_l).  Every reduction is a serial loop in a fixed
// order or a fixed tree, so training is deterministic.
#include <cuda_runtime.h>
#include "tt_internal.h"
#include "../../include/tentaco/tentaco_select.h"

namespace tt {
namespace {

constexpr int kLayers = 4;

struct Dims {
  int K[kLayers], N[kLayers];
  explicit Dims(int nout) {
    const int k[kLayers] = {TT_MLP_IN, TT_MLP_HIDDEN, TT_MLP_HIDDEN, TT_MLP_HIDDEN};
    const int n[kLayers] = {TT_MLP_HIDDEN, TT_MLP_HIDDEN, TT_MLP_HIDDEN, nout};
    for (int l = 0; l < kLayers; l++) { K[l] = k[l]; N[l] = n[l]; }
  }
  int64_t w_off(int l) const {
    int64_t o = 0;
    for (int i = 0; i < l; i++) o += (int64_t)K[i] * N[i] + N[i];
    return o;
  }
  int64_t b_off(int l) const { return w_off(l) + (int64_t)K[l] * N[l]; }
  int64_t params() const { return w_off(kLayers); }
  // scratch: the output of every layer (B x N_l), then two B x max(N) gradient buffers
  int64_t act_off(int l, int B) const {
    int64_t o = 0;
    for (int i = 0; i < l; i++) o += (int64_t)B * N[i];
    return o;
  }
  int maxn() const {
    int m = 0;
    for (int l = 0; l < kLayers; l++) m = N[l] > m ? N[l] : m;
    return m;
  }
  int64_t scratch(int B) const { return act_off(kLayers, B) + 2 * (int64_t)B * maxn(); }
};

// Y = act(X W + b): one thread per output element; consecutive threads take
// consecutive columns (coalesced W reads, X row broadcast).
__global__ void mlp_linear_kernel(const float* __restrict__ X, const float* __restrict__ W,
                                  const float* __restrict__ b, float* __restrict__ Y, int B, int K, int N,
                                  int relu) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * N) return;
  const int r = idx / N, n = idx % N;
  float acc = b[n];
  const float* x = X + (size_t)r * K;
  for (int k = 0; k < K; k++) acc = fmaf(x[k], W[(size_t)k * N + n], acc);
  Y[idx] = relu ? fmaxf(acc, 0.f) : acc;
}

// Masked mean squared error over B x N outputs: loss = sum M (O - T)^2 / sum M;
// dO = 2 M (O - T) / sum M.  One block; fixed-order partial sums and tree.
__global__ void mlp_loss_kernel(const float* __restrict__ O, const float* __restrict__ T,
                                const float* __restrict__ M, int n, float* __restrict__ dO,
                                float* __restrict__ loss) {
  __shared__ float s_sq[256], s_cnt[256];
  float sq = 0.f, cnt = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float d = M[i] != 0.f ? O[i] - T[i] : 0.f;
    sq = fmaf(d, d, sq);
    cnt += M[i] != 0.f ? 1.f : 0.f;
  }
  s_sq[threadIdx.x] = sq;
  s_cnt[threadIdx.x] = cnt;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      s_sq[threadIdx.x] += s_sq[threadIdx.x + s];
      s_cnt[threadIdx.x] += s_cnt[threadIdx.x + s];
    }
    __syncthreads();
  }
  const float total = s_cnt[0] > 0.f ? s_cnt[0] : 1.f;
  if (threadIdx.x == 0) *loss = s_sq[0] / total;
  const float scale = 2.f / total;
  for (int i = threadIdx.x; i < n; i += blockDim.x) dO[i] = M[i] != 0.f ? scale * (O[i] - T[i]) : 0.f;
}

// dZ = dY where the layer's (ReLU) output is positive, else 0 (in place).
__global__ void mlp_relu_back_kernel(float* __restrict__ dY, const float* __restrict__ Y, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && !(Y[i] > 0.f)) dY[i] = 0.f;
}

// Weight and bias gradients of one layer: thread (k, n), k == K is the bias;
// serial sum over the batch rows in order.
__global__ void mlp_wgrad_kernel(const float* __restrict__ X, const float* __restrict__ dZ,
                                 float* __restrict__ dW, float* __restrict__ db, int B, int K, int N) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (K + 1) * N) return;
  const int k = idx / N, n = idx % N;
  float acc = 0.f;
  if (k < K) {
    for (int r = 0; r < B; r++) acc = fmaf(X[(size_t)r * K + k], dZ[(size_t)r * N + n], acc);
    dW[(size_t)k * N + n] = acc;
  } else {
    for (int r = 0; r < B; r++) acc += dZ[(size_t)r * N + n];
    db[n] = acc;
  }
}

// dX = dZ W^T: thread (r, k), serial sum over the layer's outputs.
__global__ void mlp_xgrad_kernel(const float* __restrict__ dZ, const float* __restrict__ W,
                                 float* __restrict__ dX, int B, int K, int N) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * K) return;
  const int r = idx / K, k = idx % K;
  float acc = 0.f;
  const float* dz = dZ + (size_t)r * N;
  const float* w = W + (size_t)k * N;
  for (int n = 0; n < N; n++) acc = fmaf(dz[n], w[n], acc);
  dX[idx] = acc;
}

// Adam with bias correction (Kingma & Ba, 2015), decoupled weight decay wd.
__global__ void mlp_adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                                float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps,
                                float c1, float c2, float wd) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / c1, vh = vi / c2;
  p[i] -= lr * (mh / (sqrtf(vh) + eps) + wd * p[i]);
}

inline int blocks(int64_t n, int tb) { return (int)((n + tb - 1) / tb); }

tt_status check_launch(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(TT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return TT_OK;
}

tt_status forward(const Dims& d, const float* params, const float* X, int B, float* scratch, cudaStream_t st) {
  const float* in = X;
  for (int l = 0; l < kLayers; l++) {
    float* out = scratch + d.act_off(l, B);
    mlp_linear_kernel<<<blocks((int64_t)B * d.N[l], 128), 128, 0, st>>>(
        in, params + d.w_off(l), params + d.b_off(l), out, B, d.K[l], d.N[l], l + 1 < kLayers ? 1 : 0);
    in = out;
  }
  return check_launch("mlp forward");
}

}  // namespace
}  // namespace tt

using namespace tt;

TT_EXPORT int64_t tt_mlp_num_params(int32_t nout) { return nout > 0 ? Dims(nout).params() : -1; }

TT_EXPORT int64_t tt_mlp_scratch_floats(int32_t batch, int32_t nout) {
  return (batch > 0 && nout > 0) ? Dims(nout).scratch(batch) : -1;
}

TT_EXPORT tt_status tt_mlp_forward(const float* params, int32_t nout, const float* X, int32_t batch,
                                   float* scratch, float* out, void* stream) {
  clear_error();
  if (!params || !X || !scratch || !out || batch <= 0 || nout <= 0)
    return set_error(TT_ERR_INVALID_ARGUMENT, "tt_mlp_forward: null pointer or empty shape");
  const Dims d(nout);
  cudaStream_t st = (cudaStream_t)stream;
  tt_status s = forward(d, params, X, batch, scratch, st);
  if (s != TT_OK) return s;
  const cudaError_t e = cudaMemcpyAsync(out, scratch + d.act_off(kLayers - 1, batch),
                                        sizeof(float) * (size_t)batch * nout, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return set_error(TT_ERR_CUDA, "tt_mlp_forward copy: %s", cudaGetErrorString(e));
  return TT_OK;
}

TT_EXPORT tt_status tt_mlp_grad(const float* params, int32_t nout, const float* X, int32_t batch,
                                const float* T, const float* M, float* scratch, float* grads, float* loss,
                                void* stream) {
  clear_error();
  if (!params || !X || !T || !M || !scratch || !grads || !loss || batch <= 0 || nout <= 0)
    return set_error(TT_ERR_INVALID_ARGUMENT, "tt_mlp_grad: null pointer or empty shape");
  const Dims d(nout);
  cudaStream_t st = (cudaStream_t)stream;
  tt_status s = forward(d, params, X, batch, scratch, st);
  if (s != TT_OK) return s;
  const int B = batch;
  float* g0 = scratch + d.act_off(kLayers, B);
  float* g1 = g0 + (int64_t)B * d.maxn();
  mlp_loss_kernel<<<1, 256, 0, st>>>(scratch + d.act_off(kLayers - 1, B), T, M, B * nout, g0, loss);
  for (int l = kLayers - 1; l >= 0; l--) {
    const float* Y = scratch + d.act_off(l, B);
    const float* Xl = l > 0 ? scratch + d.act_off(l - 1, B) : X;
    const int K = d.K[l], N = d.N[l];
    if (l + 1 < kLayers) mlp_relu_back_kernel<<<blocks((int64_t)B * N, 256), 256, 0, st>>>(g0, Y, B * N);
    mlp_wgrad_kernel<<<blocks((int64_t)(K + 1) * N, 128), 128, 0, st>>>(Xl, g0, grads + d.w_off(l),
                                                                        grads + d.b_off(l), B, K, N);
    if (l > 0) {
      mlp_xgrad_kernel<<<blocks((int64_t)B * K, 128), 128, 0, st>>>(g0, params + d.w_off(l), g1, B, K, N);
      float* t = g0;
      g0 = g1;
      g1 = t;
    }
  }
  return check_launch("mlp backward");
}

TT_EXPORT tt_status tt_mlp_adam(float* params, const float* grads, float* m, float* v, int64_t n, float lr,
                                float beta1, float beta2, float eps, float weight_decay, int32_t step,
                                void* stream) {
  clear_error();
  if (!params || !grads || !m || !v || n <= 0 || step < 1)
    return set_error(TT_ERR_INVALID_ARGUMENT, "tt_mlp_adam: null pointer, empty array or step < 1");
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  mlp_adam_kernel<<<blocks(n, 256), 256, 0, (cudaStream_t)stream>>>(params, grads, m, v, n, lr, beta1, beta2, eps,
                                                                    c1, c2, weight_decay);
  return check_launch("mlp adam");
}
