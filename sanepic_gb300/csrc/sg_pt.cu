// sg_pt.cu -- the two projections of the operator: P (map -> timeline) and
// P^T (timeline -> map), atomic-free and deterministic.
//
// P replaces deproject (sanepic.cc:2845-2873):
//   t_i = I[p_i] + cos(2 psi_i) Q[p_i] + sin(2 psi_i) U[p_i]
// four samples per thread with 16-byte vector loads; the map (float4 per
// observed pixel) stays in L2.
//
// P^T replaces the scatter in do_PtNd (sanepic.cc:2584-2611) and the
// MPI_Reduce of the map over ranks (sanepic.cc:1448): for every observed
// pixel m
//   q_I[m] = sum y_i,  q_Q[m] = sum cos(2psi_i) y_i,  q_U[m] = sum sin(2psi_i) y_i
// over the samples i that hit m, read through the pixel-sorted sample index
// (CSR built once at setup; the pointing never changes).  One warp per
// pixel: the lanes stride through its samples in a fixed order (several
// independent gathers in flight per lane) and the warp combines lanes with a
// fixed xor tree, so the result is bitwise identical run to run.  A block
// owns 32 consecutive pixels (warps interleaved over them); with the
// nested-order pixel numbering, neighbouring pixels along the scan share the
// block, so the 32-byte sectors of y they gather are reused from L1.  The
// block's 32 totals are converted to FP64 and stored together.  The
// degeneracy mask (sanepic.cc:1455-1459) is applied here.
//
// Precision: FP64 problems accumulate in FP64.  FP32 problems accumulate each
// lane's FP32 products with Neumaier-compensated FP32 sums and combine lanes
// as double-FP32 (hi, lo) pairs; the FP64 conversion happens once per pixel,
// 32 pixels at a time.  GB300's FP64 rate (~1/64 of FP32) could not sustain
// per-sample FP64 adds at HBM speed, while the compensated sum keeps ~48 bits
// of the running total.
#include <cuda_runtime.h>

#include "sg_kernels.h"

namespace sg {

// ---- P ------------------------------------------------------------------------
template <typename T>
struct alignas(4 * sizeof(T)) pmap4 {
  T I, Q, U, pad;
};

__global__ void __launch_bounds__(256) k_project_f32(const int4* __restrict__ pix,
                                                     const float4* __restrict__ cs,
                                                     const pmap4<float>* __restrict__ map,
                                                     long long n4, float4* __restrict__ t) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4;
       i += (long long)gridDim.x * blockDim.x) {
    const int4 p = __ldcs(pix + i);
    const float4 a = __ldcs(cs + 2 * i), b = __ldcs(cs + 2 * i + 1);
    const pmap4<float> m0 = map[p.x], m1 = map[p.y], m2 = map[p.z], m3 = map[p.w];
    float4 o;
    o.x = m0.I + a.x * m0.Q + a.y * m0.U;
    o.y = m1.I + a.z * m1.Q + a.w * m1.U;
    o.z = m2.I + b.x * m2.Q + b.y * m2.U;
    o.w = m3.I + b.z * m3.Q + b.w * m3.U;
    __stcs(t + i, o);
  }
}

__global__ void __launch_bounds__(256) k_project_f64(const int* __restrict__ pix,
                                                     const double2* __restrict__ cs,
                                                     const pmap4<double>* __restrict__ map,
                                                     long long n, double* __restrict__ t) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const pmap4<double> m = map[pix[i]];
    const double2 w = cs[i];
    t[i] = m.I + (w.x * m.Q + w.y * m.U);
  }
}

template <>
cudaError_t project_launch<float>(const int* pix, const float* cs, const float* map, long long n,
                                  float* t, cudaStream_t st) {
  const long long n4 = n / 4;  // n is a multiple of 4 (ns >= 256)
  long long blocks = (n4 + 255) / 256;
  if (blocks > 152LL * 16) blocks = 152LL * 16;
  k_project_f32<<<(unsigned)blocks, 256, 0, st>>>(
      reinterpret_cast<const int4*>(pix), reinterpret_cast<const float4*>(cs),
      reinterpret_cast<const pmap4<float>*>(map), n4, reinterpret_cast<float4*>(t));
  return cudaGetLastError();
}

template <>
cudaError_t project_launch<double>(const int* pix, const double* cs, const double* map,
                                   long long n, double* t, cudaStream_t st) {
  long long blocks = (n + 255) / 256;
  if (blocks > 152LL * 16) blocks = 152LL * 16;
  k_project_f64<<<(unsigned)blocks, 256, 0, st>>>(pix, reinterpret_cast<const double2*>(cs),
                                                  reinterpret_cast<const pmap4<double>*>(map), n,
                                                  t);
  return cudaGetLastError();
}

// ---- compensated FP32 -------------------------------------------------------------
struct ff {
  float hi, lo;
};

__device__ __forceinline__ void ff_add_f(ff& a, float x) {
  const float t = a.hi + x;
  a.lo += (fabsf(a.hi) >= fabsf(x)) ? ((a.hi - t) + x) : ((x - t) + a.hi);
  a.hi = t;
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b.hi - bb) + a.lo + b.lo;
  const float hi = s + e;
  return ff{hi, e - (hi - s)};
}

__device__ __forceinline__ ff ff_shfl_xor(ff a, int o) {
  return ff{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
}

// ---- P^T --------------------------------------------------------------------------
constexpr int kPtUnroll = 4;
constexpr int kPtPix = 32;  // pixels per block (4 per warp)

__global__ void __launch_bounds__(256) k_pt_f32(const long long* __restrict__ off,
                                                const uint32_t* __restrict__ idx,
                                                const float2* __restrict__ ccs,
                                                const float* __restrict__ y, long long npix,
                                                const int* __restrict__ hits,
                                                double* __restrict__ q) {
  __shared__ float sh[kPtPix][6];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long m0 = (long long)blockIdx.x * kPtPix;
  for (int k = w; k < kPtPix; k += 8) {
    const long long m = m0 + k;
    ff a0{0.f, 0.f}, a1{0.f, 0.f}, a2{0.f, 0.f};
    if (m < npix) {
      const long long jend = off[m + 1];
      long long j = off[m] + lane;
      for (; j + 32 * (kPtUnroll - 1) < jend; j += 32 * kPtUnroll) {
        uint32_t ii[kPtUnroll];
        float v[kPtUnroll];
        float2 wv[kPtUnroll];
#pragma unroll
        for (int u = 0; u < kPtUnroll; u++) ii[u] = __ldcs(idx + j + 32 * u);
#pragma unroll
        for (int u = 0; u < kPtUnroll; u++) {
          v[u] = __ldg(y + ii[u]);
          wv[u] = __ldcs(ccs + j + 32 * u);
        }
#pragma unroll
        for (int u = 0; u < kPtUnroll; u++) {
          ff_add_f(a0, v[u]);
          ff_add_f(a1, wv[u].x * v[u]);
          ff_add_f(a2, wv[u].y * v[u]);
        }
      }
      for (; j < jend; j += 32) {
        const float v = __ldg(y + __ldcs(idx + j));
        const float2 wv = __ldcs(ccs + j);
        ff_add_f(a0, v);
        ff_add_f(a1, wv.x * v);
        ff_add_f(a2, wv.y * v);
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      a0 = ff_add(a0, ff_shfl_xor(a0, o));
      a1 = ff_add(a1, ff_shfl_xor(a1, o));
      a2 = ff_add(a2, ff_shfl_xor(a2, o));
    }
    if (lane == 0) {
      sh[k][0] = a0.hi;
      sh[k][1] = a0.lo;
      sh[k][2] = a1.hi;
      sh[k][3] = a1.lo;
      sh[k][4] = a2.hi;
      sh[k][5] = a2.lo;
    }
  }
  __syncthreads();
  // 32 lanes convert the block's 32 totals to FP64 at once
  if (threadIdx.x < kPtPix) {
    const long long m = m0 + threadIdx.x;
    if (m < npix) {
      const float* r = sh[threadIdx.x];
      const bool pol = hits == nullptr || hits[m] >= 2;
      q[m] = (double)r[0] + (double)r[1];
      q[npix + m] = pol ? (double)r[2] + (double)r[3] : 0.0;
      q[2 * npix + m] = pol ? (double)r[4] + (double)r[5] : 0.0;
    }
  }
}

__global__ void __launch_bounds__(256) k_pt_f64(const long long* off, const uint32_t* idx,
                                                const double2* ccs, const double* y,
                                                long long npix, const int* hits, double* q) {
  const int lane = threadIdx.x & 31;
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long m = warp; m < npix; m += nwarps) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    const long long j1 = off[m + 1];
    for (long long j = off[m] + lane; j < j1; j += 32) {
      const double v = __ldg(y + idx[j]);
      const double2 w = ccs[j];
      a0 += v;
      a1 += w.x * v;
      a2 += w.y * v;
    }
    for (int o = 16; o > 0; o >>= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (lane == 0) {
      const bool pol = hits == nullptr || hits[m] >= 2;
      q[m] = a0;
      q[npix + m] = pol ? a1 : 0.0;
      q[2 * npix + m] = pol ? a2 : 0.0;
    }
  }
}

template <>
cudaError_t pt_launch<float>(const long long* csr_off, const uint32_t* csr_idx,
                             const float* csr_cs, const float* y, long long npix,
                             const int* hits_true, double* q, cudaStream_t st) {
  const long long blocks = (npix + kPtPix - 1) / kPtPix;
  k_pt_f32<<<(unsigned)blocks, 256, 0, st>>>(csr_off, csr_idx,
                                             reinterpret_cast<const float2*>(csr_cs), y, npix,
                                             hits_true, q);
  return cudaGetLastError();
}

template <>
cudaError_t pt_launch<double>(const long long* csr_off, const uint32_t* csr_idx,
                              const double* csr_cs, const double* y, long long npix,
                              const int* hits_true, double* q, cudaStream_t st) {
  long long blocks = (npix * 32 + 255) / 256;
  if (blocks > 152LL * 8 * 16) blocks = 152LL * 8 * 16;
  k_pt_f64<<<(unsigned)blocks, 256, 0, st>>>(csr_off, csr_idx,
                                             reinterpret_cast<const double2*>(csr_cs), y, npix,
                                             hits_true, q);
  return cudaGetLastError();
}

}  // namespace sg
