// mlp.cu — training and inference kernels of the learned GEMM tile selector.
//
// Network: in -> hidden -> hidden -> hidden -> out, GELU (erf form) after
// the three hidden layers, FP32.  Parameters are one packed device array
// [W1 (hid x in), b1, W2 (hid x hid), b2, W3 (hid x hid), b3, W4 (out x hid),
// b4], row-major (o, i).  The loss is a masked mean squared error.  Every
// reduction (weight gradients over the batch, the loss) runs in a fixed order,
// so training is deterministic.  Sizes are tiny (in 11, hidden 64, out 40,
// a few thousand rows); one thread per output element is plenty.
#include <cmath>

#include "common.cuh"

namespace gb {

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  // d/dx [x Phi(x)] = Phi(x) + x phi(x)
  const float phi = 0.39894228040143268f * expf(-0.5f * x * x);
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * phi;
}

// Z[n][o] = b[o] + sum_i X[n][i] W[o][i];  A = GELU(Z) when act
__global__ void mlp_linear_fwd(const float* __restrict__ X, int din, const float* __restrict__ W,
                               const float* __restrict__ b, int dout, int64_t n, float* __restrict__ Z,
                               float* __restrict__ A, int act) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= n * dout) return;
  const int64_t r = e / dout;
  const int o = int(e % dout);
  float acc = b[o];
  const float* xr = X + r * din;
  const float* wr = W + int64_t(o) * din;
  for (int i = 0; i < din; ++i) acc = fmaf(xr[i], wr[i], acc);
  Z[e] = acc;
  if (A) A[e] = act ? gelu_f(acc) : acc;
}

// dY = 2 * mask * (Y - T) / valid; per-row partial losses for the fold
__global__ void mlp_mse_grad(const float* __restrict__ Y, const float* __restrict__ T,
                             const float* __restrict__ mask, int dout, int64_t n, float inv_valid,
                             float* __restrict__ dY, float* __restrict__ row_loss) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= n) return;
  float l = 0.f;
  for (int o = 0; o < dout; ++o) {
    const int64_t e = r * dout + o;
    const float d = (Y[e] - T[e]) * mask[e];
    dY[e] = 2.0f * d * inv_valid;
    l = fmaf(d, d, l);
  }
  row_loss[r] = l;
}

// loss = inv_valid * sum_r row_loss[r], one block, fixed order
__global__ void mlp_loss_fold(const float* __restrict__ row_loss, int64_t n, float inv_valid,
                              float* __restrict__ loss) {
  __shared__ double s[256];
  double acc = 0.0;
  for (int64_t r = threadIdx.x; r < n; r += blockDim.x) acc += double(row_loss[r]);
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = float(s[0] * double(inv_valid));
}

// dZ = dA * GELU'(Z)
__global__ void mlp_gelu_bwd(const float* __restrict__ Z, float* __restrict__ dA, int64_t count) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e < count) dA[e] *= gelu_grad(Z[e]);
}

// dW[o][i] = sum_r dZ[r][o] X[r][i];  db[o] = sum_r dZ[r][o]   (fixed order in r)
__global__ void mlp_linear_bwd_w(const float* __restrict__ X, int din, const float* __restrict__ dZ, int dout,
                                 int64_t n, float* __restrict__ dW, float* __restrict__ db) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= dout * (din + 1)) return;
  const int o = e / (din + 1), i = e % (din + 1);
  float acc = 0.f;
  if (i < din)
    for (int64_t r = 0; r < n; ++r) acc = fmaf(dZ[r * dout + o], X[r * din + i], acc);
  else
    for (int64_t r = 0; r < n; ++r) acc += dZ[r * dout + o];
  if (i < din) dW[o * din + i] = acc;
  else db[o] = acc;
}

// dX[r][i] = sum_o dZ[r][o] W[o][i]
__global__ void mlp_linear_bwd_x(const float* __restrict__ dZ, int dout, const float* __restrict__ W, int din,
                                 int64_t n, float* __restrict__ dX) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= n * din) return;
  const int64_t r = e / din;
  const int i = int(e % din);
  float acc = 0.f;
  for (int o = 0; o < dout; ++o) acc = fmaf(dZ[r * dout + o], W[int64_t(o) * din + i], acc);
  dX[e] = acc;
}

// Adam with decoupled weight decay (AdamW, Loshchilov & Hutter 2019)
__global__ void mlp_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                         float* __restrict__ v, int64_t count, float lr, float b1, float b2, float eps, float wd,
                         float c1, float c2) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= count) return;
  const float gi = g[e];
  const float mi = b1 * m[e] + (1.f - b1) * gi;
  const float vi = b2 * v[e] + (1.f - b2) * gi * gi;
  m[e] = mi;
  v[e] = vi;
  p[e] -= lr * ((mi / c1) / (sqrtf(vi / c2) + eps) + wd * p[e]);
}

struct MlpShape {
  int in, hid, out;
  int64_t off[8];  // W1 b1 W2 b2 W3 b3 W4 b4
  int64_t count;
  explicit MlpShape(int i, int h, int o) : in(i), hid(h), out(o) {
    int64_t p = 0;
    const int d[5] = {i, h, h, h, o};
    for (int l = 0; l < 4; ++l) {
      off[2 * l] = p;
      p += int64_t(d[l + 1]) * d[l];
      off[2 * l + 1] = p;
      p += d[l + 1];
    }
    count = p;
  }
  int din(int l) const { return l == 0 ? in : hid; }
  int dout(int l) const { return l == 3 ? out : hid; }
};

static inline unsigned nblk(int64_t n, int t = 256) { return unsigned((n + t - 1) / t); }

// Forward pass storing every layer's pre-activation Z[l] and activation A[l]
// in `act` ([4][n][hid] floats each for Z and A, last layer uses `out`).
static gbblas_status_t mlp_forward_store(gbblas_handle_t h, const MlpShape& s, const float* params, const float* x,
                                         int64_t n, float* act, float* y) {
  const int64_t L = n * std::max(s.hid, s.out);
  const float* in = x;
  for (int l = 0; l < 4; ++l) {
    float* Z = act + (2 * l) * L;
    float* A = l < 3 ? act + (2 * l + 1) * L : y;
    mlp_linear_fwd<<<nblk(n * s.dout(l)), 256, 0, h->stream>>>(in, s.din(l), params + s.off[2 * l],
                                                               params + s.off[2 * l + 1], s.dout(l), n, Z, A,
                                                               l < 3 ? 1 : 0);
    GB_TRY(after_launch("mlp_linear_fwd"));
    in = A;
  }
  return GBBLAS_STATUS_SUCCESS;
}

}  // namespace gb

using namespace gb;

extern "C" {

gbblas_status_t gbblas_mlp_param_count(int in_dim, int hidden, int out_dim, int64_t* count) {
  if (!count || in_dim <= 0 || hidden <= 0 || out_dim <= 0) return fail(GBBLAS_STATUS_INVALID_ARG, "mlp: bad shape");
  *count = MlpShape(in_dim, hidden, out_dim).count;
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_mlp_forward(gbblas_handle_t h, int in_dim, int hidden, int out_dim, const float* params,
                                   const float* x, int64_t n, float* y) {
  clear_error();
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "mlp: null handle");
  if (n <= 0) return GBBLAS_STATUS_SUCCESS;
  MlpShape s(in_dim, hidden, out_dim);
  void* tmp;
  GB_TRY(temp_acquire(h, sizeof(float) * 8 * size_t(n) * size_t(std::max(hidden, out_dim)), &tmp));
  return mlp_forward_store(h, s, params, x, n, static_cast<float*>(tmp), y);
}

gbblas_status_t gbblas_mlp_loss_grad(gbblas_handle_t h, int in_dim, int hidden, int out_dim, const float* params,
                                     const float* x, const float* target, const float* mask, int64_t n,
                                     float valid_count, float* grads, float* loss) {
  clear_error();
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "mlp: null handle");
  if (n <= 0 || valid_count <= 0.f) return fail(GBBLAS_STATUS_INVALID_ARG, "mlp: empty batch");
  MlpShape s(in_dim, hidden, out_dim);
  const int64_t L = n * std::max(hidden, out_dim);
  void* tmp;
  // Z/A per layer (8 L) + y + dY + two dX buffers + row losses
  GB_TRY(temp_acquire(h, sizeof(float) * (12 * size_t(L) + size_t(n)), &tmp));
  float* act = static_cast<float*>(tmp);
  float* y = act + 8 * L;
  float* d0 = y + L;
  float* d1 = d0 + L;
  float* rl = d1 + L;
  GB_TRY(mlp_forward_store(h, s, params, x, n, act, y));
  const float inv = 1.0f / valid_count;
  mlp_mse_grad<<<nblk(n), 256, 0, h->stream>>>(y, target, mask, out_dim, n, inv, d0, rl);
  GB_TRY(after_launch("mlp_mse_grad"));
  mlp_loss_fold<<<1, 256, 0, h->stream>>>(rl, n, inv, loss);
  GB_TRY(after_launch("mlp_loss_fold"));
  // d0 holds dZ of layer 3 (linear output)
  for (int l = 3; l >= 0; --l) {
    const float* Xin = l == 0 ? x : act + (2 * (l - 1) + 1) * L;  // A of the previous layer
    const int din = s.din(l), dout = s.dout(l);
    mlp_linear_bwd_w<<<nblk(int64_t(dout) * (din + 1)), 256, 0, h->stream>>>(
        Xin, din, d0, dout, n, grads + s.off[2 * l], grads + s.off[2 * l + 1]);
    GB_TRY(after_launch("mlp_linear_bwd_w"));
    if (l == 0) break;
    mlp_linear_bwd_x<<<nblk(n * din), 256, 0, h->stream>>>(d0, dout, params + s.off[2 * l], din, n, d1);
    GB_TRY(after_launch("mlp_linear_bwd_x"));
    mlp_gelu_bwd<<<nblk(n * din), 256, 0, h->stream>>>(act + (2 * (l - 1)) * L, d1, n * din);
    GB_TRY(after_launch("mlp_gelu_bwd"));
    std::swap(d0, d1);
  }
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_mlp_adam(gbblas_handle_t h, int64_t count, float* params, const float* grads, float* m,
                                float* v, int step, float lr, float beta1, float beta2, float eps,
                                float weight_decay) {
  clear_error();
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "mlp: null handle");
  if (step < 1) return fail(GBBLAS_STATUS_INVALID_ARG, "mlp: adam step counts from 1");
  const float c1 = 1.f - std::pow(beta1, float(step)), c2 = 1.f - std::pow(beta2, float(step));
  mlp_adam<<<nblk(count), 256, 0, h->stream>>>(params, grads, m, v, count, lr, beta1, beta2, eps, weight_decay, c1,
                                                c2);
  return after_launch("mlp_adam");
}

}  // extern "C"
