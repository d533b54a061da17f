// sg_mlp.h -- the learned preconditioner's network: a 4-layer MLP
// 768 -> 256 -> 256 -> 256 -> 768 (ReLU between layers) that maps a 3 x 256
// nested-pixel patch of the block-Jacobi-preconditioned residual (normalised
// by its RMS) to a correction of the same shape.  BF16 weights and
// activations on the tensor cores (sg_gemm.cu), FP32 accumulation, FP32
// master weights and Adam moments.  No reference counterpart.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace sg {

constexpr int kPatch = 256;             // nested pixels per patch
constexpr int kIn = 3 * kPatch;         // I, Q, U
constexpr int kHid = 256;
constexpr int kLayers = 4;
// parameters per layer l: W [out x in] then b [out]
constexpr int kLayerIn[kLayers] = {kIn, kHid, kHid, kHid};
constexpr int kLayerOut[kLayers] = {kHid, kHid, kHid, kIn};
long long mlp_nparams();

struct Mlp {
  int cap = 0;  // batch capacity (rows), multiple of 128
  // parameters: FP32 master [nparams], Adam moments, FP32 gradients
  float *w32 = nullptr, *m = nullptr, *v = nullptr, *g = nullptr;
  // BF16 weights W_l [out x in] and their transposes [in x out]
  uint16_t *wb[kLayers] = {}, *wbt[kLayers] = {};
  // activations: X [cap x 768] bf16 (+ transpose), H_l [cap x 256] bf16 (+ transposes),
  // pre-activation / output FP32 scratch, gradients
  uint16_t *x = nullptr, *xt = nullptr, *h[3] = {}, *ht[3] = {};
  uint16_t *db = nullptr, *dbt = nullptr;  // BF16 backward signal [cap x 768] and transpose
  float *acc = nullptr;                    // FP32 GEMM output [cap x 768]
  float *y = nullptr;                      // network output [cap x 768]
  float *loss = nullptr;                   // device scalar(s)
  int* err = nullptr;                      // GEMM pipeline error flag
  long long gemm_flops = 0;                // tensor-core FLOPs issued (for reporting)
  int step = 0;                            // Adam step count

  cudaError_t init(int capacity, uint64_t seed, cudaStream_t st);
  void release();
  ~Mlp() { release(); }
  long long w_off(int l) const;  // offset of W_l in the parameter vector
  long long b_off(int l) const;  // offset of b_l
  // refresh BF16 copies (and transposes) of the weights from w32
  cudaError_t sync_weights(cudaStream_t st);
  // y = f(x) for rows [0, B) (x already filled); B multiple of 128
  cudaError_t forward(int B, cudaStream_t st);
  // loss = mean w (y - t)^2 over B x 768 (t, w FP32 [B x 768]; w = 1 if null);
  // g = d loss / d params
  cudaError_t backward(int B, const float* t, cudaStream_t st, const float* w = nullptr);
  // g = parameter gradient for an externally computed d loss / d y (FP32 [B x 768])
  cudaError_t backward_dy(int B, const float* dy, cudaStream_t st);
  cudaError_t backward_core(int B, cudaStream_t st);  // from the BF16 signal in db
  cudaError_t adam(float lr, cudaStream_t st);
};

// elementwise helpers (sg_mlp.cu)
cudaError_t f32_to_bf16(const float* in, uint16_t* out, long long n, cudaStream_t st);
cudaError_t bf16_transpose(const uint16_t* in, uint16_t* out, int rows, int cols,
                           cudaStream_t st);

}  // namespace sg
