// sg_mlp.cu -- forward, backward and Adam for the learned preconditioner's
// MLP (layout and sizes in sg_mlp.h).  Every matrix product runs on the
// tensor cores through gemm_bf16 (sg_gemm.cu); the elementwise kernels here
// apply biases and ReLU, round to BF16, transpose, reduce and update.
//
// Rounding contract (the CPU oracle oracle/mlp.py follows it): weights,
// layer inputs and backward signals are rounded to BF16 (round to nearest
// even) before each product; products accumulate in FP32; biases, the loss
// and the parameters stay FP32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <random>

#include "sg_kernels.h"
#include "sg_mlp.h"

namespace sg {

namespace {

constexpr int kT = 256;

__device__ __forceinline__ uint16_t to_bf16(float f) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(f));
}
__device__ __forceinline__ float from_bf16(uint16_t b) {
  return __bfloat162float(__ushort_as_bfloat16(b));
}

__global__ void k_to_bf16(const float* in, uint16_t* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = to_bf16(in[i]);
}

// out[c][r] = in[r][c]; 32 x 32 tiles through shared memory
__global__ void k_transpose(const uint16_t* in, uint16_t* out, int rows, int cols) {
  __shared__ uint16_t tile[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[i][threadIdx.x] = in[(size_t)r * cols + c];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int c = c0 + i, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[(size_t)c * rows + r] = tile[threadIdx.x][i];
  }
}

// h = bf16(relu(acc + b)), acc [B x n]
__global__ void k_bias_relu(const float* acc, const float* b, uint16_t* h, int B, int n) {
  const long long tot = (long long)B * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot;
       i += (long long)gridDim.x * blockDim.x) {
    const float v = acc[i] + b[i % n];
    h[i] = to_bf16(v > 0.f ? v : 0.f);
  }
}

__global__ void k_bias(const float* acc, const float* b, float* y, int B, int n) {
  const long long tot = (long long)B * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = acc[i] + b[i % n];
}

// d = bf16(2 w (y - t) / (B n)); per-block partial sums of w (y - t)^2
__global__ void k_mse(const float* y, const float* t, const float* w, uint16_t* d, long long tot,
                      float scale, double* part) {
  __shared__ double sh[kT / 32];
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot;
       i += (long long)gridDim.x * blockDim.x) {
    const float e = y[i] - t[i];
    const float wi = w ? w[i] : 1.f;
    d[i] = to_bf16(2.f * wi * e * scale);
    acc += (double)wi * e * e;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kT / 32; w++) s += sh[w];
    part[blockIdx.x] = s;
  }
}

__global__ void k_loss(const double* part, int n, double scale, float* loss) {
  __shared__ double sh[kT / 32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += kT) acc += part[i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kT / 32; w++) s += sh[w];
    *loss = (float)(s * scale);
  }
}

// gb[c] = sum_r d[r][c] (BF16 signal, FP32 sum in row order)
__global__ void k_colsum(const uint16_t* d, int B, int n, float* gb) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  float s = 0.f;
  for (int r = 0; r < B; r++) s += from_bf16(d[(size_t)r * n + c]);
  gb[c] = s;
}

// d = bf16(acc * (h > 0)), acc [B x n]
__global__ void k_relu_back(const float* acc, const uint16_t* h, uint16_t* d, long long tot) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot;
       i += (long long)gridDim.x * blockDim.x)
    d[i] = to_bf16(from_bf16(h[i]) > 0.f ? acc[i] : 0.f);
}

__global__ void k_adam(float* w, const float* g, float* m, float* v, long long n, float lr,
                       float b1, float b2, float c1, float c2, float eps) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

int blocks_for(long long n) {
  const long long b = (n + kT - 1) / kT;
  return (int)(b < 2048 ? (b > 0 ? b : 1) : 2048);
}

}  // namespace

long long mlp_nparams() {
  long long n = 0;
  for (int l = 0; l < kLayers; l++) n += (long long)kLayerOut[l] * kLayerIn[l] + kLayerOut[l];
  return n;
}

long long Mlp::w_off(int l) const {
  long long o = 0;
  for (int i = 0; i < l; i++) o += (long long)kLayerOut[i] * kLayerIn[i] + kLayerOut[i];
  return o;
}
long long Mlp::b_off(int l) const { return w_off(l) + (long long)kLayerOut[l] * kLayerIn[l]; }

cudaError_t f32_to_bf16(const float* in, uint16_t* out, long long n, cudaStream_t st) {
  k_to_bf16<<<blocks_for(n), kT, 0, st>>>(in, out, n);
  return cudaGetLastError();
}

cudaError_t bf16_transpose(const uint16_t* in, uint16_t* out, int rows, int cols,
                           cudaStream_t st) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  k_transpose<<<grid, block, 0, st>>>(in, out, rows, cols);
  return cudaGetLastError();
}

void Mlp::release() {
  void* ptrs[] = {w32, m, v, g, x, xt, db, dbt, acc, y, loss, err};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (int l = 0; l < kLayers; l++) {
    if (wb[l]) cudaFree(wb[l]);
    if (wbt[l]) cudaFree(wbt[l]);
    wb[l] = wbt[l] = nullptr;
  }
  for (int l = 0; l < 3; l++) {
    if (h[l]) cudaFree(h[l]);
    if (ht[l]) cudaFree(ht[l]);
    h[l] = ht[l] = nullptr;
  }
  w32 = m = v = g = acc = y = loss = nullptr;
  x = xt = db = dbt = nullptr;
  err = nullptr;
  cap = 0;
}

cudaError_t Mlp::init(int capacity, uint64_t seed, cudaStream_t st) {
  release();
  cap = capacity;
  const long long np = mlp_nparams();
  cudaError_t e = cudaSuccess;
  auto A = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) e = cudaMemsetAsync(*p, 0, bytes, st);
  };
  A((void**)&w32, 4 * np);
  A((void**)&m, 4 * np);
  A((void**)&v, 4 * np);
  A((void**)&g, 4 * np);
  for (int l = 0; l < kLayers; l++) {
    A((void**)&wb[l], 2 * (size_t)kLayerOut[l] * kLayerIn[l]);
    A((void**)&wbt[l], 2 * (size_t)kLayerOut[l] * kLayerIn[l]);
  }
  A((void**)&x, 2 * (size_t)cap * kIn);
  A((void**)&xt, 2 * (size_t)cap * kIn);
  for (int l = 0; l < 3; l++) {
    A((void**)&h[l], 2 * (size_t)cap * kHid);
    A((void**)&ht[l], 2 * (size_t)cap * kHid);
  }
  A((void**)&db, 2 * (size_t)cap * kIn);
  A((void**)&dbt, 2 * (size_t)cap * kIn);
  A((void**)&acc, 4 * (size_t)cap * kIn);
  A((void**)&y, 4 * (size_t)cap * kIn);
  A((void**)&loss, 4096 * sizeof(double) + 16);
  A((void**)&err, sizeof(int));
  if (e == cudaSuccess) e = gemm_prepare();
  if (e != cudaSuccess) return e;
  // He-normal hidden layers; the output layer starts small so the untrained
  // correction is close to zero (the preconditioner starts as block-Jacobi)
  std::vector<float> hw(np, 0.f);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < kLayers; l++) {
    const double sd = std::sqrt(2.0 / kLayerIn[l]) * (l == kLayers - 1 ? 0.01 : 1.0);
    std::normal_distribution<double> nd(0.0, sd);
    float* w = hw.data() + w_off(l);
    for (long long i = 0; i < (long long)kLayerOut[l] * kLayerIn[l]; i++) w[i] = (float)nd(rng);
  }
  e = cudaMemcpyAsync(w32, hw.data(), 4 * np, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  step = 0;
  gemm_flops = 0;
  return e == cudaSuccess ? sync_weights(st) : e;
}

cudaError_t Mlp::sync_weights(cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  for (int l = 0; l < kLayers && e == cudaSuccess; l++) {
    const long long n = (long long)kLayerOut[l] * kLayerIn[l];
    e = f32_to_bf16(w32 + w_off(l), wb[l], n, st);
    if (e == cudaSuccess) e = bf16_transpose(wb[l], wbt[l], kLayerOut[l], kLayerIn[l], st);
  }
  return e;
}

cudaError_t Mlp::forward(int B, cudaStream_t st) {
  if (B <= 0 || B > cap || B % 128) return cudaErrorInvalidValue;
  cudaError_t e = cudaSuccess;
  const uint16_t* in = x;
  for (int l = 0; l < kLayers && e == cudaSuccess; l++) {
    const int n = kLayerOut[l], k = kLayerIn[l];
    e = gemm_bf16(in, wb[l], acc, B, n, k, 0, err, st);
    gemm_flops += 2LL * B * n * k;
    if (e != cudaSuccess) break;
    const long long tot = (long long)B * n;
    if (l < kLayers - 1) {
      k_bias_relu<<<blocks_for(tot), kT, 0, st>>>(acc, w32 + b_off(l), h[l], B, n);
      in = h[l];
    } else {
      k_bias<<<blocks_for(tot), kT, 0, st>>>(acc, w32 + b_off(l), y, B, n);
    }
    e = cudaGetLastError();
  }
  return e;
}

cudaError_t Mlp::backward(int B, const float* t, cudaStream_t st, const float* w) {
  if (B <= 0 || B > cap || B % 128) return cudaErrorInvalidValue;
  const long long tot = (long long)B * kIn;
  double* part = reinterpret_cast<double*>(loss + 4);  // after the float loss slot
  const int nb = 1024;
  k_mse<<<nb, kT, 0, st>>>(y, t, w, db, tot, 1.f / (float)tot, part);
  k_loss<<<1, kT, 0, st>>>(part, nb, 1.0 / (double)tot, loss);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? backward_core(B, st) : e;
}

cudaError_t Mlp::backward_dy(int B, const float* dy, cudaStream_t st) {
  if (B <= 0 || B > cap || B % 128) return cudaErrorInvalidValue;
  cudaError_t e = f32_to_bf16(dy, db, (long long)B * kIn, st);
  return e == cudaSuccess ? backward_core(B, st) : e;
}

cudaError_t Mlp::backward_core(int B, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  // activations transposed for the weight gradients
  if (e == cudaSuccess) e = bf16_transpose(x, xt, B, kIn, st);
  for (int l = 0; l < 3 && e == cudaSuccess; l++) e = bf16_transpose(h[l], ht[l], B, kHid, st);
  for (int l = kLayers - 1; l >= 0 && e == cudaSuccess; l--) {
    const int n = kLayerOut[l], k = kLayerIn[l];
    const uint16_t* in_t = (l == 0) ? xt : ht[l - 1];
    // dW_l [n x k] = d^T [n x B] . in [B x k]  (K = B)
    e = bf16_transpose(db, dbt, B, n, st);
    if (e == cudaSuccess) e = gemm_bf16(dbt, in_t, g + w_off(l), n, k, B, 0, err, st);
    gemm_flops += 2LL * B * n * k;
    if (e != cudaSuccess) break;
    k_colsum<<<(n + kT - 1) / kT, kT, 0, st>>>(db, B, n, g + b_off(l));
    if (l == 0) break;
    // d_in [B x k] = d [B x n] . W_l [n x k]  (B operand W_l^T stored [k x n])
    e = gemm_bf16(db, wbt[l], acc, B, k, n, 0, err, st);
    gemm_flops += 2LL * B * n * k;
    if (e != cudaSuccess) break;
    const long long tk = (long long)B * k;
    k_relu_back<<<blocks_for(tk), kT, 0, st>>>(acc, h[l - 1], db, tk);
    e = cudaGetLastError();
  }
  return e;
}

cudaError_t Mlp::adam(float lr, cudaStream_t st) {
  step++;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
  const long long np = mlp_nparams();
  k_adam<<<blocks_for(np), kT, 0, st>>>(w32, g, m, v, np, lr, b1, b2, c1, c2, eps);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? sync_weights(st) : e;
}

}  // namespace sg
