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
#include <cuda_bf16.h>
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

__global__ void __launch_bounds__(256) k_to_f32(const double* __restrict__ in,
                                                float* __restrict__ out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

cudaError_t to_f32_launch(const double* in, float* out, long long n, cudaStream_t st) {
  long long blocks = (n + 255) / 256;
  if (blocks > 152LL * 16) blocks = 152LL * 16;
  if (blocks < 1) return cudaSuccess;
  k_to_f32<<<(unsigned)blocks, 256, 0, st>>>(in, out, n);
  return cudaGetLastError();
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
  const long long stride = (long long)gridDim.x * blockDim.x;
  double acc[1] = {0.0};
  // four elements' loads in flight per round, added in the same order
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3; i += 4 * stride) {
    double qv[4], dv[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const long long k = i + u * stride;
      qv[u] = k < n3 ? v.q[k] : 0.0;
      dv[u] = k < n3 ? v.d[k] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (i + u * stride < n3) acc[0] += qv[u] * dv[u];
  }
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
  const long long stride = (long long)gridDim.x * blockDim.x;
  double acc[3] = {0.0, 0.0, 0.0};
  // two pixels per round: every load of both before any store
  for (long long m0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; m0 < n; m0 += 2 * stride) {
    double xv[2][3], dv[2][3], rv[2][3], qv[2][3];
#pragma unroll
    for (int p = 0; p < 2; p++) {
      const long long m = m0 + p * stride;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const long long i = c * n + m;
        const bool in = m < n;
        xv[p][c] = in ? v.x[i] : 0.0;
        dv[p][c] = in ? v.d[i] : 0.0;
        rv[p][c] = in ? v.r[i] : 0.0;
        qv[p][c] = (in && !refresh) ? v.q[i] : 0.0;
      }
    }
#pragma unroll
    for (int p = 0; p < 2; p++) {
      const long long m = m0 + p * stride;
      if (m >= n) break;
      double r[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const long long i = c * n + m;
        v.x[i] = xv[p][c] + alpha * dv[p][c];
        r[c] = rv[p][c];
      }
      if (refresh) continue;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const long long i = c * n + m;
        if (flexible) v.rprev[i] = r[c];
        r[c] -= alpha * qv[p][c];
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
          if (flexible) acc[2] += z[c] * rv[p][c];
        }
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
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long m0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; m0 < n; m0 += 2 * stride) {
    double zv[2][3], dv[2][3];
#pragma unroll
    for (int p = 0; p < 2; p++) {
      const long long m = m0 + p * stride;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        zv[p][c] = m < n ? v.z[c * n + m] : 0.0;
        dv[p][c] = m < n ? v.d[c * n + m] : 0.0;
      }
    }
#pragma unroll
    for (int p = 0; p < 2; p++) {
      const long long m = m0 + p * stride;
      if (m >= n) break;
      double d[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        d[c] = zv[p][c] + beta * dv[p][c];
        v.d[c * n + m] = d[c];
      }
      store_map<T>(dmap, m, d[0], d[1], d[2]);
    }
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

// ---- the PCG loop on the device ----------------------------------------------
// One thread decides; the WHILE node repeats its body (begin, the iteration
// under one of two IF nodes, end) while the handle is non-zero.  The limit on
// iterations is checked on the device, so the loop always ends.
__global__ void k_loop_begin(const LoopState* s, cudaGraphConditionalHandle refresh,
                             cudaGraphConditionalHandle normal) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const bool r = refresh_at(s->iter, s->refresh_every, s->skip0);
    cudaGraphSetConditional(refresh, r ? 1u : 0u);
    cudaGraphSetConditional(normal, r ? 0u : 1u);
  }
}

__global__ void k_loop_end(LoopState* s, const CgScalars* sc, double* hist,
                           cudaGraphConditionalHandle loop) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const double crit = sc->var / sc->var00;
    if (s->iter < s->maxiter) hist[s->iter] = crit;
    const int it = s->iter + 1;
    s->iter = it;
    // the host loop's test: go on while iter < maxiter and crit > stop (a NaN
    // crit stops), and stop at a breakdown flag
    int done = 0;
    if (!(crit > s->stop)) done = 1;
    else if (it >= s->maxiter) done = 2;
    else if (sc->flag) done = 3;
    s->done = done;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (it == 1) s->t_first = t;
    s->t_last = t;
    cudaGraphSetConditional(loop, done ? 0u : 1u);
  }
}

cudaError_t loop_begin_launch(const LoopState* s, cudaGraphConditionalHandle refresh,
                              cudaGraphConditionalHandle normal, cudaStream_t st) {
  k_loop_begin<<<1, 32, 0, st>>>(s, refresh, normal);
  return cudaGetLastError();
}

cudaError_t loop_end_launch(LoopState* s, const CgScalars* sc, double* hist,
                            cudaGraphConditionalHandle loop, cudaStream_t st) {
  k_loop_end<<<1, 32, 0, st>>>(s, sc, hist, loop);
  return cudaGetLastError();
}

// ---- two-level preconditioner with a coarse space U (kc columns) ------------
// Balancing form (Mandel's balancing Neumann-Neumann; A-DEF2 in Tang et al.
// 2009), with AU = A U and E = U^T A U:
//   z = (I - U E^-1 AU^T) M (I - AU E^-1 U^T) r + U E^-1 U^T r
// computed as  c = E^-1 U^T r,  y = M (r - AU c),  z = y + U (c - E^-1 AU^T y)
// in three passes (U^T r; y and AU^T y; z and the CG's dots).
// Symmetric positive definite for any SPD E and M, so plain (or flexible)
// PCG applies.  U and AU are stored element-major, [3 npix][kp] BF16 with
// kp = kc rounded up to 8 (zero columns), so one thread reads an element's
// kp values as 16-byte loads; the preconditioner stays symmetric positive
// definite whatever their rounding (the same U on both sides, E exact in
// FP64).  Their products with a vector run in FP32 (GB300's
// FP64 rate would make kc FP64 FMAs per element cost more than reading U);
// the per-thread sums are FP32, the warp sums double-FP32, the block sums
// FP64 (kept as double-FP32 pairs), their fixed-order reductions
// double-FP32 and the coarse solves FP64.  Every
// block of the kernel that needs c (or c - g) re-reduces the partials
// itself, so the coarse solve costs no launch.  The rounding makes the
// preconditioner slightly inexact, which flexible PCG absorbs.

// eight BF16 values (one 16-byte load) as floats
__device__ __forceinline__ void bf16x8(const uint4 q, float (&f)[8]) {
  const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
  for (int t = 0; t < 4; t++) {
    f[2 * t] = __uint_as_float(w[t] << 16);
    f[2 * t + 1] = __uint_as_float(w[t] & 0xffff0000u);
  }
}

// Double-FP32 addition (hi, lo) += (b, bl): Knuth's two-sum of the high
// parts, the low parts added to the error term.  ~44 bits, FP32 instructions.
__device__ __forceinline__ void df_add(float& hi, float& lo, float b, float bl) {
  const float s = hi + b;
  const float bb = s - hi;
  const float e = ((hi - (s - bb)) + (b - bb)) + (lo + bl);
  hi = s + e;
  lo = e - (hi - s);
}

// part[k][block] = the block's sum of acc[k] (FP64, stored as a double-FP32
// pair so that every block can re-reduce the partials with FP32
// instructions).  A warp first adds its
// lanes' FP32 accumulators as double-FP32 pairs through a fixed xor tree
// (FP32 instructions only), lane k takes total k and widens it to FP64, and
// KP threads add the warps in order: GB300's FP64 rate would make an FP64
// shuffle tree of KP values per warp cost more than the kernel's loop.
template <int KP>
__device__ __forceinline__ void coarse_block_store(float (&acc)[KP], float2* part) {
  __shared__ double sh[KP][kCgThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float mh = 0.f, ml = 0.f;  // this lane's total: k = lane
#pragma unroll
  for (int k = 0; k < KP; k++) {
    float hi = acc[k], lo = 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      df_add(hi, lo, __shfl_xor_sync(0xffffffffu, hi, o), __shfl_xor_sync(0xffffffffu, lo, o));
    if (lane == k) {
      mh = hi;
      ml = lo;
    }
  }
  if (lane < KP) sh[lane][wid] = (double)mh + (double)ml;
  __syncthreads();
  if (threadIdx.x < KP) {
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < kCgThreads / 32; w++) t += sh[threadIdx.x][w];
    const float hi = (float)t;
    part[threadIdx.x * kCgBlocks + blockIdx.x] = make_float2(hi, (float)(t - (double)hi));
  }
}

// elements per thread and round in the streaming coarse kernels: four rows
// in flight, two for the widest coarse space (two blocks of 256 threads per
// SM leave 128 registers a thread)
template <int KP>
constexpr int coarse_rows() { return KP > 24 ? 2 : 4; }

// part[k][block] = sum over the block's elements of U[i][k] v[i]
template <int KP>
__global__ void __launch_bounds__(kCgThreads)
    k_coarse_dots(const uint16_t* __restrict__ U, long long n3, const double* __restrict__ v,
                  float2* part) {
  float acc[KP];
#pragma unroll
  for (int k = 0; k < KP; k++) acc[k] = 0.f;
  constexpr int kCoarseRows = coarse_rows<KP>();
  const long long stride = (long long)gridDim.x * blockDim.x;
  // kCoarseRows elements' rows in flight per round (the grid is fixed at two
  // blocks per SM, so the loads in flight per thread set the bandwidth),
  // added in element order
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3;
       i += kCoarseRows * stride) {
    uint4 rows[kCoarseRows][KP / 8];
    float vi[kCoarseRows];
#pragma unroll
    for (int p = 0; p < kCoarseRows; p++) {
      const long long k = i + p * stride;
      const uint4* row = reinterpret_cast<const uint4*>(U + k * KP);
      vi[p] = k < n3 ? (float)v[k] : 0.f;
#pragma unroll
      for (int q = 0; q < KP / 8; q++) rows[p][q] = k < n3 ? row[q] : make_uint4(0, 0, 0, 0);
    }
#pragma unroll
    for (int p = 0; p < kCoarseRows; p++) {
      if (i + p * stride >= n3) break;
#pragma unroll
      for (int q = 0; q < KP / 8; q++) {
        float u[8];
        bf16x8(rows[p][q], u);
#pragma unroll
        for (int t = 0; t < 8; t++) acc[8 * q + t] = fmaf(u[t], vi[p], acc[8 * q + t]);
      }
    }
  }
  coarse_block_store<KP>(acc, part);
}

// out[k] = (E^-1 d)[k], d[k] = sum_b part[k][b] in a fixed order (identical in
// every block; double-FP32 sums, warp w reduces rows w, w + 8, ...), E^-1 d
// in FP64
template <int KP>
__device__ __forceinline__ void coarse_solve_block(const float2* __restrict__ part,
                                                   const double* __restrict__ einv, int kc,
                                                   double* d, double* out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int NB = (kCgBlocks + 31) / 32;
  for (int k = wid; k < KP; k += kCgThreads / 32) {
    float hi = 0.f, lo = 0.f;
    float2 q[NB];  // every load in flight before the dependent sums
#pragma unroll
    for (int t = 0; t < NB; t++) {
      const int b = lane + 32 * t;
      q[t] = b < kCgBlocks ? part[k * kCgBlocks + b] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int t = 0; t < NB; t++)
      if (lane + 32 * t < kCgBlocks) df_add(hi, lo, q[t].x, q[t].y);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      df_add(hi, lo, __shfl_xor_sync(0xffffffffu, hi, o), __shfl_xor_sync(0xffffffffu, lo, o));
    if (lane == 0) d[k] = (double)hi + (double)lo;
  }
  __syncthreads();
  if (threadIdx.x < KP) {
    const int k = threadIdx.x;
    double c = 0.0;
    if (k < kc)
      for (int j = 0; j < kc; j++) c += einv[k * kc + j] * d[j];
    out[k] = c;
  }
  __syncthreads();
}

// c = E^-1 U^T r (from part1); z = M (r - AU c); block 0 keeps c in coef;
// part2[k][block] = partial sums of AU[i][k] z[i] (the rows are read once for
// both: the second use hits L1).  With the FP32 blocks (FP32 operators),
// r - AU c and M_bj3 run on the FP32 pipe: GB300's FP64 pipe had bounded
// this kernel (18 FP64 instructions a pixel, 6 this way), and flexible PCG
// takes the FP32-rounded preconditioner as it is (its residual stays FP64).
template <int KP, bool M32>
__global__ void __launch_bounds__(kCgThreads, 2)
    k_coarse_pre(CgVecs v, const uint16_t* __restrict__ AU, const float2* __restrict__ part1,
                 const double* __restrict__ einv, int kc, double* coef, float2* part2) {
  __shared__ double d[KP], cd[KP];
  __shared__ float c[KP];
  coarse_solve_block<KP>(part1, einv, kc, d, cd);
  if (threadIdx.x < KP) {
    c[threadIdx.x] = (float)cd[threadIdx.x];
    if (blockIdx.x == 0) coef[threadIdx.x] = cd[threadIdx.x];
  }
  __syncthreads();
  float acc[KP];
#pragma unroll
  for (int k = 0; k < KP; k++) acc[k] = 0.f;
  const long long n = v.npix;
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
       m += (long long)gridDim.x * blockDim.x) {
    double t[3];
    float tf[3];
#pragma unroll
    for (int cc = 0; cc < 3; cc++) {
      const long long i = cc * n + m;
      const uint4* row = reinterpret_cast<const uint4*>(AU + i * KP);
      float s = 0.f;
#pragma unroll
      for (int q = 0; q < KP / 8; q++) {
        float a[8];
        bf16x8(row[q], a);
#pragma unroll
        for (int t2 = 0; t2 < 8; t2++) s = fmaf(a[t2], c[8 * q + t2], s);
      }
      if constexpr (M32)
        tf[cc] = (float)v.r[i] - s;
      else
        t[cc] = v.r[i] - (double)s;
    }
    double z[3];
    float zq[3];
    if constexpr (M32) {
      const float* o = v.minv32;  // 00 01 02 11 12 22
      const float o00 = o[m], o01 = o[n + m], o02 = o[2 * n + m];
      const float o11 = o[3 * n + m], o12 = o[4 * n + m], o22 = o[5 * n + m];
      zq[0] = fmaf(o00, tf[0], fmaf(o01, tf[1], o02 * tf[2]));
      zq[1] = fmaf(o01, tf[0], fmaf(o11, tf[1], o12 * tf[2]));
      zq[2] = fmaf(o02, tf[0], fmaf(o12, tf[1], o22 * tf[2]));
    } else {
      apply_m(v, m, t[0], t[1], t[2], z[0], z[1], z[2]);
    }
#pragma unroll
    for (int cc = 0; cc < 3; cc++) {
      const long long i = cc * n + m;
      v.z[i] = M32 ? (double)zq[cc] : z[cc];
      const float zf = M32 ? zq[cc] : (float)z[cc];
      const uint4* row = reinterpret_cast<const uint4*>(AU + i * KP);
#pragma unroll
      for (int q = 0; q < KP / 8; q++) {
        float a[8];
        bf16x8(__ldcg(row + q), a);  // again, from L2: keeps the rows out of registers
#pragma unroll
        for (int t2 = 0; t2 < 8; t2++) acc[8 * q + t2] = fmaf(a[t2], zf, acc[8 * q + t2]);
      }
    }
  }
  coarse_block_store<KP>(acc, part2);
}

// g = E^-1 AU^T y (from part2); z = y + U (c - g); the CG's partial dots
// r.z, r.r (and z.r_prev when flexible) into part + kCgBlocks..
template <int KP>
__global__ void __launch_bounds__(kCgThreads)
    k_coarse_post(CgVecs v, const uint16_t* __restrict__ U, const float2* __restrict__ part2,
                  const double* __restrict__ einv, int kc, const double* __restrict__ coef,
                  int flexible) {
  __shared__ double d[KP], gd[KP];
  __shared__ float w[KP];
  coarse_solve_block<KP>(part2, einv, kc, d, gd);
  if (threadIdx.x < KP) w[threadIdx.x] = (float)(coef[threadIdx.x] - gd[threadIdx.x]);
  __syncthreads();
  const long long n3 = 3 * v.npix;
  const long long stride = (long long)gridDim.x * blockDim.x;
  double acc[3] = {0.0, 0.0, 0.0};
  constexpr int kCoarseRows = coarse_rows<KP>();
  // kCoarseRows elements per round: every load of all before any store
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3;
       i += kCoarseRows * stride) {
    uint4 rows[kCoarseRows][KP / 8];
    double zv[kCoarseRows], rv[kCoarseRows], pv[kCoarseRows];
#pragma unroll
    for (int p = 0; p < kCoarseRows; p++) {
      const long long k = i + p * stride;
      const bool in = k < n3;
      const uint4* row = reinterpret_cast<const uint4*>(U + k * KP);
#pragma unroll
      for (int q = 0; q < KP / 8; q++) rows[p][q] = in ? row[q] : make_uint4(0, 0, 0, 0);
      zv[p] = in ? v.z[k] : 0.0;
      rv[p] = in ? v.r[k] : 0.0;
      pv[p] = (in && flexible) ? v.rprev[k] : 0.0;
    }
#pragma unroll
    for (int p = 0; p < kCoarseRows; p++) {
      const long long k = i + p * stride;
      if (k >= n3) break;
      float s = 0.f;
#pragma unroll
      for (int q = 0; q < KP / 8; q++) {
        float u[8];
        bf16x8(rows[p][q], u);
#pragma unroll
        for (int t2 = 0; t2 < 8; t2++) s = fmaf(u[t2], w[8 * q + t2], s);
      }
      const double z = zv[p] + (double)s, r = rv[p];
      v.z[k] = z;
      acc[0] += r * z;
      acc[1] += r * r;
      if (flexible) acc[2] += z * pv[p];
    }
  }
  block_reduce_store<3>(acc, v.part + kCgBlocks, kCgBlocks);
}

template <int KP>
static cudaError_t coarse_apply_kp(const CgVecs& v, const CoarseSpace& cs, int flexible,
                                   cudaStream_t st) {
  const long long n3 = 3 * v.npix;
  float2* part1 = reinterpret_cast<float2*>(cs.part);  // same 8 bytes per partial
  float2* part2 = part1 + (size_t)kCoarseMax * kCgBlocks;
  k_coarse_dots<KP><<<kCgBlocks, kCgThreads, 0, st>>>(cs.u, n3, v.r, part1);
  if (v.minv32 && v.precond == 1)
    k_coarse_pre<KP, true><<<kCgBlocks, kCgThreads, 0, st>>>(v, cs.au, part1, cs.einv, cs.kc,
                                                             cs.coef, part2);
  else
    k_coarse_pre<KP, false><<<kCgBlocks, kCgThreads, 0, st>>>(v, cs.au, part1, cs.einv, cs.kc,
                                                              cs.coef, part2);
  k_coarse_post<KP><<<kCgBlocks, kCgThreads, 0, st>>>(v, cs.u, part2, cs.einv, cs.kc, cs.coef,
                                                       flexible);
  return cudaGetLastError();
}

int coarse_pad(int kc) { return (kc + 7) / 8 * 8; }

cudaError_t coarse_apply(const CgVecs& v, const CoarseSpace& cs, int flexible, cudaStream_t st) {
  if (cs.kc < 1 || cs.kc > kCoarseMax) return cudaErrorInvalidValue;
  switch (coarse_pad(cs.kc)) {
    case 8: return coarse_apply_kp<8>(v, cs, flexible, st);
    case 16: return coarse_apply_kp<16>(v, cs, flexible, st);
    case 24: return coarse_apply_kp<24>(v, cs, flexible, st);
    default: return coarse_apply_kp<32>(v, cs, flexible, st);
  }
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

// out[i][k] = BF16(sum_j V[j][i] C[j][k]) for k < kc, 0 for kc <= k < kp
// (C [m][kc] FP64); one block per 256 elements, C staged through shared
// memory in chunks of rows
__global__ void __launch_bounds__(kCgThreads)
    k_combine(const double* __restrict__ V, long long ld, int m, const double* __restrict__ C,
              int kc, int kp, long long n, uint16_t* out) {
  constexpr int kChunk = 4096;
  __shared__ double cs[kChunk];
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double acc[kCoarseMax];
#pragma unroll
  for (int k = 0; k < kCoarseMax; k++) acc[k] = 0.0;
  const int rows = kChunk / kc;
  for (int j0 = 0; j0 < m; j0 += rows) {
    const int j1 = j0 + rows < m ? j0 + rows : m;
    __syncthreads();
    for (int e = threadIdx.x; e < (j1 - j0) * kc; e += blockDim.x) cs[e] = C[j0 * kc + e];
    __syncthreads();
    if (i < n)
      for (int j = j0; j < j1; j++) {
        const double vj = V[j * ld + i];
#pragma unroll
        for (int k = 0; k < kCoarseMax; k++)
          if (k < kc) acc[k] += vj * cs[(j - j0) * kc + k];
      }
  }
  if (i < n) {
#pragma unroll
    for (int k = 0; k < kCoarseMax; k++)
      if (k < kp) out[i * kp + k] = k < kc ? __bfloat16_as_ushort(__float2bfloat16_rn((float)acc[k])) : 0;
  }
}

cudaError_t combine_launch(const double* V, long long ld, int m, const double* C, int kc,
                           long long n, uint16_t* out, cudaStream_t st) {
  if (kc < 1 || kc > kCoarseMax || m < 1) return cudaErrorInvalidValue;
  const long long blocks = (n + kCgThreads - 1) / kCgThreads;
  k_combine<<<(unsigned)blocks, kCgThreads, 0, st>>>(V, ld, m, C, kc, coarse_pad(kc), n, out);
  return cudaGetLastError();
}

}  // namespace sg
