// sg_pt.cu -- P^T: the deterministic, atomic-free transpose projection.
//
// Replaces the scatter in do_PtNd (sanepic.cc:2584-2611) and the MPI_Reduce
// of the map over ranks (sanepic.cc:1448): for every observed pixel m
//   q_I[m] = sum y_i,  q_Q[m] = sum cos(2psi_i) y_i,  q_U[m] = sum sin(2psi_i) y_i
// over the samples i that hit m, read through the pixel-sorted sample index
// (CSR built once at setup; the pointing never changes).  One warp per pixel:
// lanes stride through the pixel's samples in a fixed order and the warp
// combines lanes with a fixed xor tree, so the result is bitwise identical
// run to run.  The degeneracy mask (sanepic.cc:1455-1459) is applied here.
//
// Precision: FP64 problems accumulate in FP64.  FP32 problems accumulate each
// lane's FP32 products with Neumaier-compensated FP32 sums and combine lanes
// as double-FP32 (hi, lo) pairs, converting to FP64 once per pixel: GB300's
// FP64 rate (~1/64 of FP32) could not sustain per-sample FP64 adds at HBM
// speed, while the compensated sum keeps ~48 bits of the running total.
#include <cuda_runtime.h>

#include "sg_kernels.h"

namespace sg {

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

__global__ void __launch_bounds__(256) k_pt_f32(const long long* off, const uint32_t* idx,
                                                const float* ccs, const float* y, long long npix,
                                                const int* hits, double* q) {
  const int lane = threadIdx.x & 31;
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long m = warp; m < npix; m += nwarps) {
    ff a0{0.f, 0.f}, a1{0.f, 0.f}, a2{0.f, 0.f};
    const long long j1 = off[m + 1];
#pragma unroll 4
    for (long long j = off[m] + lane; j < j1; j += 32) {
      const float v = __ldg(y + idx[j]);
      const float2 w = *reinterpret_cast<const float2*>(ccs + 2 * j);
      ff_add_f(a0, v);
      ff_add_f(a1, w.x * v);
      ff_add_f(a2, w.y * v);
    }
    for (int o = 16; o > 0; o >>= 1) {
      a0 = ff_add(a0, ff_shfl_xor(a0, o));
      a1 = ff_add(a1, ff_shfl_xor(a1, o));
      a2 = ff_add(a2, ff_shfl_xor(a2, o));
    }
    if (lane == 0) {
      const bool pol = hits == nullptr || hits[m] >= 2;
      q[m] = (double)a0.hi + (double)a0.lo;
      q[npix + m] = pol ? (double)a1.hi + (double)a1.lo : 0.0;
      q[2 * npix + m] = pol ? (double)a2.hi + (double)a2.lo : 0.0;
    }
  }
}

__global__ void __launch_bounds__(256) k_pt_f64(const long long* off, const uint32_t* idx,
                                                const double* ccs, const double* y,
                                                long long npix, const int* hits, double* q) {
  const int lane = threadIdx.x & 31;
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long m = warp; m < npix; m += nwarps) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    const long long j1 = off[m + 1];
    for (long long j = off[m] + lane; j < j1; j += 32) {
      const double v = __ldg(y + idx[j]);
      const double2 w = *reinterpret_cast<const double2*>(ccs + 2 * j);
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
  long long blocks = (npix * 32 + 255) / 256;
  if (blocks > 152LL * 8 * 16) blocks = 152LL * 8 * 16;
  k_pt_f32<<<(unsigned)blocks, 256, 0, st>>>(csr_off, csr_idx, csr_cs, y, npix, hits_true, q);
  return cudaGetLastError();
}

template <>
cudaError_t pt_launch<double>(const long long* csr_off, const uint32_t* csr_idx,
                              const double* csr_cs, const double* y, long long npix,
                              const int* hits_true, double* q, cudaStream_t st) {
  long long blocks = (npix * 32 + 255) / 256;
  if (blocks > 152LL * 8 * 16) blocks = 152LL * 8 * 16;
  k_pt_f64<<<(unsigned)blocks, 256, 0, st>>>(csr_off, csr_idx, csr_cs, y, npix, hits_true, q);
  return cudaGetLastError();
}

}  // namespace sg
