// sg_cg.cu -- FP64 conjugate-gradient vector algebra, fused into a few
// grid-stride kernels whose reductions are deterministic (fixed per-block
// trees, then every block re-reduces the per-block partials in the same
// order).  Scalars (alpha, beta, delta, ...) stay on the device so one CG
// iteration can be captured in a CUDA graph; the host only reads `var` to
// test convergence.
//
// Replaces the rank-0 vector passes of the reference's PCG
// (sanepic.cc:1336-1411 init, 1455-1481 and 1573-1610 per iteration).
// Vectors are compact maps [I | Q | U] of npix each (sanepic.cc:919-921).
#include <cuda_runtime.h>

#include "sg_kernels.h"

namespace sg {

template <int N>
__device__ __forceinline__ void block_reduce_store(double (&v)[N], double* part, int stride) {
  __shared__ double sh[N][kCgThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < N; k++) {
    double x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sh[k][wid] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; k++) {
      double s = 0.0;
      for (int w = 0; w < kCgThreads / 32; w++) s += sh[k][w];
      part[k * stride + blockIdx.x] = s;
    }
  }
}

// Every block computes the same total from the per-block partials.
__device__ __forceinline__ double reduce_partials(const double* part) {
  __shared__ double sh[kCgThreads / 32];
  __shared__ double tot;
  double x = 0.0;
  for (int i = threadIdx.x; i < kCgBlocks; i += kCgThreads) x += part[i];
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kCgThreads / 32; w++) s += sh[w];
    tot = s;
  }
  __syncthreads();
  const double r = tot;
  __syncthreads();
  return r;
}

__device__ __forceinline__ void apply_m(const CgVecs& v, long long m, double r0, double r1,
                                        double r2, double& z0, double& z1, double& z2) {
  const long long n = v.npix;
  if (v.precond == 1) {
    const double* o = v.minv;
    const double o00 = o[m], o01 = o[n + m], o02 = o[2 * n + m];
    const double o11 = o[3 * n + m], o12 = o[4 * n + m], o22 = o[5 * n + m];
    z0 = o00 * r0 + o01 * r1 + o02 * r2;
    z1 = o01 * r0 + o11 * r1 + o12 * r2;
    z2 = o02 * r0 + o12 * r1 + o22 * r2;
  } else {
    z0 = v.mdiag[m] * r0;
    z1 = v.mdiag[n + m] * r1;
    z2 = v.mdiag[2 * n + m] * r2;
  }
}

template <typename T>
__device__ __forceinline__ void store_map(T* dmap, long long m, double a, double b, double c) {
  dmap[4 * m] = (T)a;
  dmap[4 * m + 1] = (T)b;
  dmap[4 * m + 2] = (T)c;
  dmap[4 * m + 3] = (T)0;
}

// ---- init: r = b - r (r holds the masked A x0), z = M r, d = z ------------
__global__ void __launch_bounds__(kCgThreads) k_init_a(CgVecs v) {
  const long long n = v.npix;
  double acc[3] = {0.0, 0.0, 0.0};  // r.z, r.r, b.b
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
       m += (long long)gridDim.x * blockDim.x) {
    double r[3], b[3], z[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      b[c] = v.b[c * n + m];
      r[c] = b[c] - v.r[c * n + m];
    }
    if (v.precond == 2) {
      z[0] = z[1] = z[2] = 0.0;
    } else {
      apply_m(v, m, r[0], r[1], r[2], z[0], z[1], z[2]);
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
      v.r[c * n + m] = r[c];
      if (v.precond != 2) {
        v.z[c * n + m] = z[c];
        v.d[c * n + m] = z[c];
      }
      acc[0] += r[c] * z[c];
      acc[1] += r[c] * r[c];
      acc[2] += b[c] * b[c];
    }
  }
  block_reduce_store<3>(acc, v.part, kCgBlocks);
}

__global__ void __launch_bounds__(kCgThreads) k_init_b(CgVecs v) {
  const double rz = reduce_partials(v.part);
  const double rr = reduce_partials(v.part + kCgBlocks);
  const double bb = reduce_partials(v.part + 2 * kCgBlocks);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    v.sc->delta = rz;
    v.sc->delta0 = rz;
    v.sc->delta_old = rz;
    v.sc->var = rr;
    v.sc->var00 = bb;
    v.sc->alpha = 0.0;
    v.sc->beta = 0.0;
    v.sc->flag = 0;
  }
}

template <typename T>
cudaError_t cg_init(const CgVecs& v, cudaStream_t st) {
  k_init_a<<<kCgBlocks, kCgThreads, 0, st>>>(v);
  k_init_b<<<1, kCgThreads, 0, st>>>(v);
  return cudaGetLastError();
}
template cudaError_t cg_init<float>(const CgVecs&, cudaStream_t);
template cudaError_t cg_init<double>(const CgVecs&, cudaStream_t);

// ---- per iteration ---------------------------------------------------------
// (a) rtq = q . d  (q is already masked by P^T)
__global__ void __launch_bounds__(kCgThreads) k_step_a(CgVecs v) {
  const long long n3 = 3 * v.npix;
  double acc[1] = {0.0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3;
       i += (long long)gridDim.x * blockDim.x)
    acc[0] += v.q[i] * v.d[i];
  block_reduce_store<1>(acc, v.part, kCgBlocks);
}

cudaError_t cg_step_a(const CgVecs& v, cudaStream_t st) {
  k_step_a<<<kCgBlocks, kCgThreads, 0, st>>>(v);
  return cudaGetLastError();
}

// (b) alpha = delta / rtq; x += alpha d; unless refreshing: r -= alpha q,
// z = M r and the partial dots (r.z, r.r, z.rprev).
__global__ void __launch_bounds__(kCgThreads) k_step_b(CgVecs v, int refresh, int flexible) {
  const double rtq = reduce_partials(v.part);
  const double delta = v.sc->delta;
  const double alpha = delta / rtq;
  const long long n = v.npix;
  double acc[3] = {0.0, 0.0, 0.0};
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
       m += (long long)gridDim.x * blockDim.x) {
    double r[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const long long i = c * n + m;
      v.x[i] += alpha * v.d[i];
      r[c] = v.r[i];
    }
    if (refresh) continue;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const long long i = c * n + m;
      if (flexible) v.rprev[i] = r[c];
      r[c] -= alpha * v.q[i];
      v.r[i] = r[c];
    }
    if (v.precond != 2) {
      double z[3];
      apply_m(v, m, r[0], r[1], r[2], z[0], z[1], z[2]);
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const long long i = c * n + m;
        v.z[i] = z[c];
        acc[0] += r[c] * z[c];
        acc[1] += r[c] * r[c];
        if (flexible) acc[2] += z[c] * v.rprev[i];
      }
    }
  }
  __syncthreads();
  block_reduce_store<3>(acc, v.part + kCgBlocks, kCgBlocks);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    v.sc->alpha = alpha;
    v.sc->rtq = rtq;
    v.sc->delta_old = delta;
    if (!(rtq > 0.0)) v.sc->flag |= 1;
  }
}

cudaError_t cg_step_b(const CgVecs& v, int refresh, int flexible, cudaStream_t st) {
  k_step_b<<<kCgBlocks, kCgThreads, 0, st>>>(v, refresh, flexible);
  return cudaGetLastError();
}

// refresh: r = b - q (q = masked A x), or r = q (q = masked P^T N^-1 (d - P x)),
// z = M r, partial dots
__global__ void __launch_bounds__(kCgThreads) k_refresh_r(CgVecs v, int flexible, int direct) {
  const long long n = v.npix;
  double acc[3] = {0.0, 0.0, 0.0};
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
       m += (long long)gridDim.x * blockDim.x) {
    double r[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const long long i = c * n + m;
      if (flexible) v.rprev[i] = v.r[i];
      r[c] = direct ? v.q[i] : v.b[i] - v.q[i];
      v.r[i] = r[c];
    }
    if (v.precond != 2) {
      double z[3];
      apply_m(v, m, r[0], r[1], r[2], z[0], z[1], z[2]);
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const long long i = c * n + m;
        v.z[i] = z[c];
        acc[0] += r[c] * z[c];
        acc[1] += r[c] * r[c];
        if (flexible) acc[2] += z[c] * v.rprev[i];
      }
    }
  }
  block_reduce_store<3>(acc, v.part + kCgBlocks, kCgBlocks);
}

cudaError_t cg_refresh_r(const CgVecs& v, int flexible, int direct, cudaStream_t st) {
  k_refresh_r<<<kCgBlocks, kCgThreads, 0, st>>>(v, flexible, direct);
  return cudaGetLastError();
}

// chi^2 (sanepic.cc:1089-1110, 1542-1546): the filter leaves one partial per
// CTA; one block adds them in a fixed order.
__global__ void __launch_bounds__(kCgThreads) k_chi2_sum(const double* part, int n, double* out) {
  __shared__ double sh[kCgThreads / 32];
  double x = 0.0;
  for (int i = threadIdx.x; i < n; i += kCgThreads) x += part[i];
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kCgThreads / 32; w++) s += sh[w];
    *out = 2.0 * s;
  }
}

cudaError_t chi2_sum(const double* part, int n, double* out, cudaStream_t st) {
  k_chi2_sum<<<1, kCgThreads, 0, st>>>(part, n, out);
  return cudaGetLastError();
}

// dots only (z supplied by an external preconditioner)
__global__ void __launch_bounds__(kCgThreads) k_dots(CgVecs v, int flexible) {
  const long long n3 = 3 * v.npix;
  double acc[3] = {0.0, 0.0, 0.0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3;
       i += (long long)gridDim.x * blockDim.x) {
    const double r = v.r[i], z = v.z[i];
    acc[0] += r * z;
    acc[1] += r * r;
    if (flexible) acc[2] += z * v.rprev[i];
  }
  block_reduce_store<3>(acc, v.part + kCgBlocks, kCgBlocks);
}

cudaError_t cg_dots(const CgVecs& v, int flexible, cudaStream_t st) {
  k_dots<<<kCgBlocks, kCgThreads, 0, st>>>(v, flexible);
  return cudaGetLastError();
}

// (c) delta_new = r.z, var = r.r, beta, d = z + beta d, map copy of d for P.
template <typename T>
__global__ void __launch_bounds__(kCgThreads) k_step_c(CgVecs v, T* dmap, int flexible) {
  const double rz = reduce_partials(v.part + kCgBlocks);
  const double rr = reduce_partials(v.part + 2 * kCgBlocks);
  const double zrp = flexible ? reduce_partials(v.part + 3 * kCgBlocks) : 0.0;
  const double dold = v.sc->delta_old;
  double beta = flexible ? (rz - zrp) / dold : rz / dold;
  const long long n = v.npix;
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
       m += (long long)gridDim.x * blockDim.x) {
    double d[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const long long i = c * n + m;
      d[c] = v.z[i] + beta * v.d[i];
      v.d[i] = d[c];
    }
    store_map<T>(dmap, m, d[0], d[1], d[2]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    v.sc->delta = rz;
    v.sc->var = rr;
    v.sc->beta = beta;
    if (!(rz > 0.0)) v.sc->flag |= 2;
  }
}

template <typename T>
cudaError_t cg_step_c(const CgVecs& v, T* dmap, int flexible, cudaStream_t st) {
  k_step_c<T><<<kCgBlocks, kCgThreads, 0, st>>>(v, dmap, flexible);
  return cudaGetLastError();
}
template cudaError_t cg_step_c<float>(const CgVecs&, float*, int, cudaStream_t);
template cudaError_t cg_step_c<double>(const CgVecs&, double*, int, cudaStream_t);

// restart the search direction from an externally supplied z: d = z,
// delta = delta0 = r.z (partials from cg_dots)
template <typename T>
__global__ void __launch_bounds__(kCgThreads) k_reinit_d(CgVecs v, T* dmap) {
  const double rz = reduce_partials(v.part + kCgBlocks);
  const long long n = v.npix;
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
       m += (long long)gridDim.x * blockDim.x) {
    double d[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      d[c] = v.z[c * n + m];
      v.d[c * n + m] = d[c];
    }
    store_map<T>(dmap, m, d[0], d[1], d[2]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    v.sc->delta = rz;
    v.sc->delta0 = rz;
    v.sc->delta_old = rz;
    if (!(rz > 0.0)) v.sc->flag |= 2;
  }
}

template <typename T>
cudaError_t cg_reinit_d(const CgVecs& v, T* dmap, cudaStream_t st) {
  k_reinit_d<T><<<kCgBlocks, kCgThreads, 0, st>>>(v, dmap);
  return cudaGetLastError();
}
template cudaError_t cg_reinit_d<float>(const CgVecs&, float*, cudaStream_t);
template cudaError_t cg_reinit_d<double>(const CgVecs&, double*, cudaStream_t);

template <typename T>
__global__ void k_to_map4(const double* x, long long n, T* map) {
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
       m += (long long)gridDim.x * blockDim.x)
    store_map<T>(map, m, x[m], x[n + m], x[2 * n + m]);
}

template <typename T>
cudaError_t to_map4(const double* x, long long npix, T* map, cudaStream_t st) {
  k_to_map4<T><<<kCgBlocks, kCgThreads, 0, st>>>(x, npix, map);
  return cudaGetLastError();
}
template cudaError_t to_map4<float>(const double*, long long, float*, cudaStream_t);
template cudaError_t to_map4<double>(const double*, long long, double*, cudaStream_t);

__global__ void k_mask_qu(double* v, const int* hits, long long n) {
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
       m += (long long)gridDim.x * blockDim.x)
    if (hits[m] < 2) {
      v[n + m] = 0.0;
      v[2 * n + m] = 0.0;
    }
}

cudaError_t mask_qu(double* v, const int* hits_true, long long npix, cudaStream_t st) {
  k_mask_qu<<<kCgBlocks, kCgThreads, 0, st>>>(v, hits_true, npix);
  return cudaGetLastError();
}

// y = M x for an arbitrary vector (used by the learned preconditioner path)
__global__ void k_apply_precond(CgVecs v, const double* x, double* y) {
  const long long n = v.npix;
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
       m += (long long)gridDim.x * blockDim.x) {
    double z0, z1, z2;
    apply_m(v, m, x[m], x[n + m], x[2 * n + m], z0, z1, z2);
    y[m] = z0;
    y[n + m] = z1;
    y[2 * n + m] = z2;
  }
}

cudaError_t apply_precond(const CgVecs& v, const double* x, double* y, cudaStream_t st) {
  k_apply_precond<<<kCgBlocks, kCgThreads, 0, st>>>(v, x, y);
  return cudaGetLastError();
}

// ---- two-level preconditioner with a coarse space U (kc columns) ------------
// Balancing form (Mandel's balancing Neumann-Neumann; A-DEF2 in Tang et al.
// 2009), with AU = A U and E = U^T A U:
//   z = (I - U E^-1 AU^T) M (I - AU E^-1 U^T) r + U E^-1 U^T r
// computed as  c = E^-1 U^T r,  y = M (r - AU c),  z = y + U (c - E^-1 AU^T y).
// Symmetric positive definite for any SPD E and M, so plain (or flexible)
// PCG applies.  U and AU are FP32 rows [kc][ld]; their products with a vector
// run in FP32 (GB300's FP64 rate would make kc FP64 FMAs per element cost
// more than reading U), per-thread partials and the coarse solve in FP64
// with fixed-order reductions.  The rounding makes the preconditioner
// slightly inexact, which the flexible (Polak-Ribiere) PCG absorbs.

// part[k][block] = sum over the block's elements of U[k][i] v[i]
__global__ void __launch_bounds__(kCgThreads)
    k_coarse_dots(const float* __restrict__ U, long long ld, int kc, long long n3,
                  const double* __restrict__ v, double* part) {
  float acc[kCoarseMax];
#pragma unroll
  for (int k = 0; k < kCoarseMax; k++) acc[k] = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3;
       i += (long long)gridDim.x * blockDim.x) {
    const float vi = (float)v[i];
#pragma unroll
    for (int k = 0; k < kCoarseMax; k++)
      if (k < kc) acc[k] = fmaf(U[k * ld + i], vi, acc[k]);
  }
  __shared__ double sh[kCoarseMax][kCgThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kCoarseMax; k++) {
    if (k >= kc) break;
    double x = (double)acc[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sh[k][wid] = x;
  }
  __syncthreads();
  if (threadIdx.x < kc) {
    double s = 0.0;
    for (int w = 0; w < kCgThreads / 32; w++) s += sh[threadIdx.x][w];
    part[threadIdx.x * kCgBlocks + blockIdx.x] = s;
  }
}

// warp k reduces row k of the partials; then coef[k] = (E^-1 dots)[k]
// (mode 0) or coef[kCoarseMax + k] = coef[k] - (E^-1 dots)[k] (mode 1)
__global__ void __launch_bounds__(1024)
    k_coarse_solve(const double* __restrict__ part, int kc, const double* __restrict__ einv,
                   double* coef, int mode) {
  __shared__ double dots[kCoarseMax];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (w < kc) {
    double x = 0.0;
    for (int b = lane; b < kCgBlocks; b += 32) x += part[w * kCgBlocks + b];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) dots[w] = x;
  }
  __syncthreads();
  if (threadIdx.x < kc) {
    const int k = threadIdx.x;
    double c = 0.0;
    for (int j = 0; j < kc; j++) c += einv[k * kc + j] * dots[j];
    if (mode == 0)
      coef[k] = c;
    else
      coef[kCoarseMax + k] = coef[k] - c;
  }
}

// z = M (r - sum_k AU[k] coef[k])  (M: the context's block-Jacobi or diagonal)
__global__ void __launch_bounds__(kCgThreads)
    k_coarse_pre(CgVecs v, const float* __restrict__ AU, long long ld, int kc,
                 const double* __restrict__ coef) {
  __shared__ float c[kCoarseMax];
  if (threadIdx.x < kCoarseMax) c[threadIdx.x] = threadIdx.x < kc ? (float)coef[threadIdx.x] : 0.f;
  __syncthreads();
  const long long n = v.npix;
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
       m += (long long)gridDim.x * blockDim.x) {
    double t[3];
#pragma unroll
    for (int cc = 0; cc < 3; cc++) {
      const long long i = cc * n + m;
      float s = 0.f;
#pragma unroll
      for (int k = 0; k < kCoarseMax; k++)
        if (k < kc) s = fmaf(AU[k * ld + i], c[k], s);
      t[cc] = v.r[i] - (double)s;
    }
    double z0, z1, z2;
    apply_m(v, m, t[0], t[1], t[2], z0, z1, z2);
    v.z[m] = z0;
    v.z[n + m] = z1;
    v.z[2 * n + m] = z2;
  }
}

// z += sum_k U[k] coef[kCoarseMax + k]
__global__ void __launch_bounds__(kCgThreads)
    k_coarse_post(double* z, const float* __restrict__ U, long long ld, int kc, long long n3,
                  const double* __restrict__ coef) {
  __shared__ float c[kCoarseMax];
  if (threadIdx.x < kCoarseMax)
    c[threadIdx.x] = threadIdx.x < kc ? (float)coef[kCoarseMax + threadIdx.x] : 0.f;
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3;
       i += (long long)gridDim.x * blockDim.x) {
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < kCoarseMax; k++)
      if (k < kc) s = fmaf(U[k * ld + i], c[k], s);
    z[i] += (double)s;
  }
}

cudaError_t coarse_apply(const CgVecs& v, const CoarseSpace& cs, cudaStream_t st) {
  if (cs.kc < 1 || cs.kc > kCoarseMax) return cudaErrorInvalidValue;
  const long long n3 = 3 * v.npix;
  k_coarse_dots<<<kCgBlocks, kCgThreads, 0, st>>>(cs.u, cs.ld, cs.kc, n3, v.r, cs.part);
  k_coarse_solve<<<1, 1024, 0, st>>>(cs.part, cs.kc, cs.einv, cs.coef, 0);
  k_coarse_pre<<<kCgBlocks, kCgThreads, 0, st>>>(v, cs.au, cs.ld, cs.kc, cs.coef);
  k_coarse_dots<<<kCgBlocks, kCgThreads, 0, st>>>(cs.au, cs.ld, cs.kc, n3, v.z, cs.part);
  k_coarse_solve<<<1, 1024, 0, st>>>(cs.part, cs.kc, cs.einv, cs.coef, 1);
  k_coarse_post<<<kCgBlocks, kCgThreads, 0, st>>>(v.z, cs.u, cs.ld, cs.kc, n3, cs.coef);
  return cudaGetLastError();
}

// ---- building the coarse space ------------------------------------------------
// part[s][i][j] = sum over split s of X[i][:] . Y[j][:]  (16 x 16 output tile
// per block, 32-column chunks staged in shared memory)
constexpr int kGramTile = 16, kGramChunk = 32;
__global__ void __launch_bounds__(kGramTile* kGramTile)
    k_gram(const double* __restrict__ X, const double* __restrict__ Y, long long ld, int m,
           long long n, long long per_split, double* part) {
  __shared__ double xs[kGramTile][kGramChunk + 1], ys[kGramTile][kGramChunk + 1];
  const int tx = threadIdx.x % kGramTile, ty = threadIdx.x / kGramTile;
  const int i0 = blockIdx.x * kGramTile, j0 = blockIdx.y * kGramTile;
  const long long c0 = blockIdx.z * per_split;
  const long long c1 = c0 + per_split < n ? c0 + per_split : n;
  double acc = 0.0;
  for (long long c = c0; c < c1; c += kGramChunk) {
    for (int e = threadIdx.x; e < kGramTile * kGramChunk; e += kGramTile * kGramTile) {
      const int r = e / kGramChunk, k = e % kGramChunk;
      const long long col = c + k;
      const bool in = col < c1;
      xs[r][k] = (in && i0 + r < m) ? X[(i0 + r) * ld + col] : 0.0;
      ys[r][k] = (in && j0 + r < m) ? Y[(j0 + r) * ld + col] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < kGramChunk; k++) acc += xs[ty][k] * ys[tx][k];
    __syncthreads();
  }
  const int i = i0 + ty, j = j0 + tx;
  if (i < m && j < m) part[((long long)blockIdx.z * m + i) * m + j] = acc;
}

cudaError_t gram_launch(const double* X, const double* Y, long long ld, int m, long long n,
                        int nsplit, double* part, cudaStream_t st) {
  const int t = (m + kGramTile - 1) / kGramTile;
  long long per = (n + nsplit - 1) / nsplit;
  per = (per + kGramChunk - 1) / kGramChunk * kGramChunk;
  dim3 grid(t, t, nsplit);
  k_gram<<<grid, kGramTile * kGramTile, 0, st>>>(X, Y, ld, m, n, per, part);
  return cudaGetLastError();
}

// out[k][i] = (float) sum_j V[j][i] C[j][k]   (C [m][kc] FP64, m * kc <= 4096)
__global__ void __launch_bounds__(kCgThreads)
    k_combine(const double* __restrict__ V, long long ld, int m, const double* __restrict__ C,
              int kc, long long n, float* out) {
  __shared__ double cs[4096];
  for (int e = threadIdx.x; e < m * kc; e += blockDim.x) cs[e] = C[e];
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double acc[kCoarseMax];
#pragma unroll
    for (int k = 0; k < kCoarseMax; k++) acc[k] = 0.0;
    for (int j = 0; j < m; j++) {
      const double vj = V[j * ld + i];
#pragma unroll
      for (int k = 0; k < kCoarseMax; k++)
        if (k < kc) acc[k] += vj * cs[j * kc + k];
    }
#pragma unroll
    for (int k = 0; k < kCoarseMax; k++)
      if (k < kc) out[k * ld + i] = (float)acc[k];
  }
}

cudaError_t combine_launch(const double* V, long long ld, int m, const double* C, int kc,
                           long long n, float* out, cudaStream_t st) {
  if (kc < 1 || kc > kCoarseMax || m * kc > 4096) return cudaErrorInvalidValue;
  k_combine<<<kCgBlocks * 4, kCgThreads, 0, st>>>(V, ld, m, C, kc, n, out);
  return cudaGetLastError();
}

}  // namespace sg
