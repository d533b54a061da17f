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
// over the samples i that hit m.  Detectors that share a pixel stream (an
// offset group) are first summed per group sample (k_detsum, or the group
// operator's inverse FFTs), so P^T walks the group samples, read through the
// pixel-sorted index (CSR built once at setup; the pointing never changes).
// The sums (S0, S1, S2) are stored in blocks of 8 group samples,
// [i / 8][3][8]: a writer that produces one component for consecutive
// samples fills whole 32-byte sectors, and P^T's gathers of neighbouring
// samples share them.  A team of L lanes per pixel (L from
// the mean samples per pixel: about four per lane) strides through its
// samples in a fixed order (several independent gathers in flight per lane)
// and combines its lanes with a fixed xor tree, so the result is bitwise
// identical run to run.  A block owns 256 / L consecutive pixels; with the
// nested-order pixel numbering, neighbouring pixels along the scan share the
// block, so the 32-byte sectors of y they gather are reused from L1.  The
// block's totals are converted to FP64 and stored together.  The degeneracy
// mask (sanepic.cc:1455-1459) is applied here.
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

// Four group samples per thread: one pixel/angle load and one map gather per
// sample, then the P value of every detector of the group (coalesced writes).
// tsc (or null): one factor per (detector, segment) tile -- the squared gains
// of a recalibrated operator, G N^-1 G = g^2 N^-1 on a tile.
__global__ void __launch_bounds__(256) k_project_f32(const int4* __restrict__ gpix,
                                                     const float4* __restrict__ gcs,
                                                     const pmap4<float>* __restrict__ map,
                                                     long long n4, long long nsd4,
                                                     const int* __restrict__ grp_off,
                                                     const int* __restrict__ grp_det,
                                                     const float2* __restrict__ dcs,
                                                     float4* __restrict__ t,
                                                     const float* __restrict__ tsc,
                                                     long long ns4) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4;
       i += (long long)gridDim.x * blockDim.x) {
    const int g = (int)(i / nsd4);
    const long long w4 = i - (long long)g * nsd4;
    const int4 p = __ldcs(gpix + i);
    const float4 ca = __ldcs(gcs + 2 * i), cb = __ldcs(gcs + 2 * i + 1);
    const pmap4<float> m0 = map[p.x], m1 = map[p.y], m2 = map[p.z], m3 = map[p.w];
    // t_det = a + cos2d' b + sin2d' e with a = I, b = c Q + s U, e = c U - s Q
    const float4 a = make_float4(m0.I, m1.I, m2.I, m3.I);
    const float4 b = make_float4(ca.x * m0.Q + ca.y * m0.U, ca.z * m1.Q + ca.w * m1.U,
                                 cb.x * m2.Q + cb.y * m2.U, cb.z * m3.Q + cb.w * m3.U);
    const float4 e = make_float4(ca.x * m0.U - ca.y * m0.Q, ca.z * m1.U - ca.w * m1.Q,
                                 cb.x * m2.U - cb.y * m2.Q, cb.z * m3.U - cb.w * m3.Q);
    for (int k = grp_off[g]; k < grp_off[g + 1]; k++) {
      const int d = grp_det[k];
      const float2 r = dcs[d];
      float4 o;
      o.x = a.x + r.x * b.x + r.y * e.x;
      o.y = a.y + r.x * b.y + r.y * e.y;
      o.z = a.z + r.x * b.z + r.y * e.z;
      o.w = a.w + r.x * b.w + r.y * e.w;
      if (tsc) {
        const float f = tsc[(long long)d * (nsd4 / ns4) + w4 / ns4];
        o.x *= f;
        o.y *= f;
        o.z *= f;
        o.w *= f;
      }
      __stcs(t + (long long)d * nsd4 + w4, o);
    }
  }
}

__global__ void __launch_bounds__(256) k_project_f64(const int* __restrict__ gpix,
                                                     const double2* __restrict__ gcs,
                                                     const pmap4<double>* __restrict__ map,
                                                     long long n, long long nsd,
                                                     const int* __restrict__ grp_off,
                                                     const int* __restrict__ grp_det,
                                                     const double2* __restrict__ dcs,
                                                     double* __restrict__ t,
                                                     const double* __restrict__ tsc,
                                                     long long ns) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int g = (int)(i / nsd);
    const long long w = i - (long long)g * nsd;
    const pmap4<double> m = map[gpix[i]];
    const double2 c = gcs[i];
    const double b = c.x * m.Q + c.y * m.U, e = c.x * m.U - c.y * m.Q;
    for (int k = grp_off[g]; k < grp_off[g + 1]; k++) {
      const int d = grp_det[k];
      const double2 r = dcs[d];
      const double v = m.I + (r.x * b + r.y * e);
      t[(long long)d * nsd + w] = tsc ? v * tsc[(long long)d * (nsd / ns) + w / ns] : v;
    }
  }
}

template <>
cudaError_t project_launch<float>(const int* gpix, const float* gcs, const float* map,
                                  long long n, long long nsd, const int* grp_off,
                                  const int* grp_det, const float* dcs, float* t,
                                  const float* tsc, long long ns, cudaStream_t st) {
  const long long n4 = n / 4;  // nsd is a multiple of 4 (ns >= 256)
  long long blocks = (n4 + 255) / 256;
  if (blocks > 152LL * 16) blocks = 152LL * 16;
  k_project_f32<<<(unsigned)blocks, 256, 0, st>>>(
      reinterpret_cast<const int4*>(gpix), reinterpret_cast<const float4*>(gcs),
      reinterpret_cast<const pmap4<float>*>(map), n4, nsd / 4, grp_off, grp_det,
      reinterpret_cast<const float2*>(dcs), reinterpret_cast<float4*>(t), tsc, ns / 4);
  return cudaGetLastError();
}

template <>
cudaError_t project_launch<double>(const int* gpix, const double* gcs, const double* map,
                                   long long n, long long nsd, const int* grp_off,
                                   const int* grp_det, const double* dcs, double* t,
                                   const double* tsc, long long ns, cudaStream_t st) {
  long long blocks = (n + 255) / 256;
  if (blocks > 152LL * 16) blocks = 152LL * 16;
  k_project_f64<<<(unsigned)blocks, 256, 0, st>>>(
      gpix, reinterpret_cast<const double2*>(gcs), reinterpret_cast<const pmap4<double>*>(map),
      n, nsd, grp_off, grp_det, reinterpret_cast<const double2*>(dcs), t, tsc, ns);
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

// ---- detector sums ------------------------------------------------------------
// Per group sample: S0 = sum y_det, A = sum cos2d' y_det, B = sum sin2d' y_det over
// the group's detectors (Neumaier-compensated FP32, fixed detector order), so
// that P^T only visits the group's samples: cos 2(phi + d') = c C - s S and
// sin 2(phi + d') = s C + c S with (C, S) the detector rotation.
__global__ void __launch_bounds__(256) k_detsum_f32(const float4* __restrict__ y, long long n4,
                                                    long long nsd4,
                                                    const int* __restrict__ grp_off,
                                                    const int* __restrict__ grp_det,
                                                    const float2* __restrict__ dcs,
                                                    float* __restrict__ ys) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4;
       i += (long long)gridDim.x * blockDim.x) {
    const int g = (int)(i / nsd4);
    const long long w4 = i - (long long)g * nsd4;
    ff s0[4], sa[4], sb[4];
#pragma unroll
    for (int k = 0; k < 4; k++) s0[k] = sa[k] = sb[k] = ff{0.f, 0.f};
    const int k1 = grp_off[g + 1];
    int k = grp_off[g];
    // four detectors' loads in flight before their (in-order) accumulation
    for (; k + 4 <= k1; k += 4) {
      float4 v[4];
      float2 r[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int d = grp_det[k + u];
        r[u] = dcs[d];
        v[u] = __ldcs(y + (long long)d * nsd4 + w4);
      }
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const float vv[4] = {v[u].x, v[u].y, v[u].z, v[u].w};
#pragma unroll
        for (int q = 0; q < 4; q++) {
          ff_add_f(s0[q], vv[q]);
          ff_add_f(sa[q], r[u].x * vv[q]);
          ff_add_f(sb[q], r[u].y * vv[q]);
        }
      }
    }
    for (; k < k1; k++) {
      const int d = grp_det[k];
      const float2 r = dcs[d];
      const float4 v = __ldcs(y + (long long)d * nsd4 + w4);
      const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int q = 0; q < 4; q++) {
        ff_add_f(s0[q], vv[q]);
        ff_add_f(sa[q], r.x * vv[q]);
        ff_add_f(sb[q], r.y * vv[q]);
      }
    }
    // samples 4i..4i+3: half of one 8-sample block of the [block][3][8] layout
    float* blk = ys + (i >> 1) * 24 + (i & 1) * 4;
    *reinterpret_cast<float4*>(blk) = make_float4(s0[0].hi + s0[0].lo, s0[1].hi + s0[1].lo,
                                                  s0[2].hi + s0[2].lo, s0[3].hi + s0[3].lo);
    *reinterpret_cast<float4*>(blk + 8) = make_float4(sa[0].hi + sa[0].lo, sa[1].hi + sa[1].lo,
                                                      sa[2].hi + sa[2].lo, sa[3].hi + sa[3].lo);
    *reinterpret_cast<float4*>(blk + 16) = make_float4(sb[0].hi + sb[0].lo, sb[1].hi + sb[1].lo,
                                                       sb[2].hi + sb[2].lo, sb[3].hi + sb[3].lo);
  }
}

__global__ void __launch_bounds__(256) k_detsum_f64(const double* __restrict__ y, long long n,
                                                    long long nsd,
                                                    const int* __restrict__ grp_off,
                                                    const int* __restrict__ grp_det,
                                                    const double2* __restrict__ dcs,
                                                    double* __restrict__ ys) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int g = (int)(i / nsd);
    const long long w = i - (long long)g * nsd;
    double s0 = 0.0, sa = 0.0, sb = 0.0;
    for (int k = grp_off[g]; k < grp_off[g + 1]; k++) {
      const int d = grp_det[k];
      const double v = y[(long long)d * nsd + w];
      s0 += v;
      sa += dcs[d].x * v;
      sb += dcs[d].y * v;
    }
    double* blk = ys + (i >> 3) * 24 + (i & 7);
    blk[0] = s0;
    blk[8] = sa;
    blk[16] = sb;
  }
}

template <>
cudaError_t detsum_launch<float>(const float* y, long long n, long long nsd, const int* grp_off,
                                 const int* grp_det, const float* dcs, float* ys,
                                 cudaStream_t st) {
  const long long n4 = n / 4;
  long long blocks = (n4 + 255) / 256;
  if (blocks > 152LL * 16) blocks = 152LL * 16;
  k_detsum_f32<<<(unsigned)blocks, 256, 0, st>>>(reinterpret_cast<const float4*>(y), n4, nsd / 4,
                                                 grp_off, grp_det,
                                                 reinterpret_cast<const float2*>(dcs), ys);
  return cudaGetLastError();
}

template <>
cudaError_t detsum_launch<double>(const double* y, long long n, long long nsd,
                                  const int* grp_off, const int* grp_det, const double* dcs,
                                  double* ys, cudaStream_t st) {
  long long blocks = (n + 255) / 256;
  if (blocks > 152LL * 16) blocks = 152LL * 16;
  k_detsum_f64<<<(unsigned)blocks, 256, 0, st>>>(y, n, nsd, grp_off, grp_det,
                                                 reinterpret_cast<const double2*>(dcs), ys);
  return cudaGetLastError();
}

// ---- P^T --------------------------------------------------------------------------
constexpr int kPtUnroll = 4;

// (S0, S1, S2) of group sample i in the [i / 8][3][8] layout
__device__ __forceinline__ float3 ys_at(const float* __restrict__ ys, uint32_t i) {
  const float* b = ys + (size_t)(i >> 3) * 24 + (i & 7);
  return make_float3(__ldg(b), __ldg(b + 8), __ldg(b + 16));
}

// L lanes per pixel (a team; 256 / L pixels per block, consecutive): the
// lanes stride through the pixel's samples in a fixed order, four gathers in
// flight each, and the team combines its lanes with a fixed xor tree.  L is
// chosen from the mean samples per pixel, so a pixel's few samples do not
// leave most of a warp idle; for a given problem the order of every sum is
// fixed, so the result is bitwise identical run to run.
template <int L>
__global__ void __launch_bounds__(256) k_pt_f32(const long long* __restrict__ off,
                                                const uint32_t* __restrict__ idx,
                                                const float2* __restrict__ ccs,
                                                const float* __restrict__ ys, long long npix,
                                                const int* __restrict__ hits,
                                                double* __restrict__ q) {
  constexpr int T = 256 / L;  // pixels per block
  __shared__ float sh[T][6];
  const int lane = threadIdx.x % L, team = threadIdx.x / L;
  const long long m0 = (long long)blockIdx.x * T;
  const long long m = m0 + team;
  ff a0{0.f, 0.f}, a1{0.f, 0.f}, a2{0.f, 0.f};
  if (m < npix) {
    const long long jend = off[m + 1];
    // kPtUnroll samples per lane per round, the ones past the pixel's end
    // masked: a pixel's few samples (about four per lane) take one round of
    // dependent loads, not one per sample; each lane still adds its samples
    // j, j + L, j + 2L, ... in that order
    for (long long j = off[m] + lane; j < jend; j += L * kPtUnroll) {
      uint32_t ii[kPtUnroll];
      float3 v[kPtUnroll];
      float2 wv[kPtUnroll];
#pragma unroll
      for (int u = 0; u < kPtUnroll; u++) ii[u] = j + L * u < jend ? __ldcs(idx + j + L * u) : 0u;
#pragma unroll
      for (int u = 0; u < kPtUnroll; u++) {
        if (j + L * u < jend) {
          v[u] = ys_at(ys, ii[u]);
          wv[u] = __ldcs(ccs + j + L * u);
        }
      }
#pragma unroll
      for (int u = 0; u < kPtUnroll; u++) {
        if (j + L * u < jend) {
          ff_add_f(a0, v[u].x);
          ff_add_f(a1, wv[u].x * v[u].y - wv[u].y * v[u].z);
          ff_add_f(a2, wv[u].y * v[u].y + wv[u].x * v[u].z);
        }
      }
    }
  }
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) {
    a0 = ff_add(a0, ff_shfl_xor(a0, o));
    a1 = ff_add(a1, ff_shfl_xor(a1, o));
    a2 = ff_add(a2, ff_shfl_xor(a2, o));
  }
  if (lane == 0) {
    sh[team][0] = a0.hi;
    sh[team][1] = a0.lo;
    sh[team][2] = a1.hi;
    sh[team][3] = a1.lo;
    sh[team][4] = a2.hi;
    sh[team][5] = a2.lo;
  }
  __syncthreads();
  // the block's T totals converted to FP64 and stored together
  if (threadIdx.x < T) {
    const long long mm = m0 + threadIdx.x;
    if (mm < npix) {
      const float* r = sh[threadIdx.x];
      const bool pol = hits == nullptr || hits[mm] >= 2;
      q[mm] = (double)r[0] + (double)r[1];
      q[npix + mm] = pol ? (double)r[2] + (double)r[3] : 0.0;
      q[2 * npix + mm] = pol ? (double)r[4] + (double)r[5] : 0.0;
    }
  }
}

int pt_lanes(long long nsamples, long long npix) {
  const double mean = npix > 0 ? (double)nsamples / (double)npix : 1.0;
  int L = 1;
  while (L < 32 && L * 4 < mean) L *= 2;  // about four samples per lane
  return L;
}

__global__ void __launch_bounds__(256) k_pt_f64(const long long* off, const uint32_t* idx,
                                                const double2* ccs, const double* ys,
                                                long long npix, const int* hits, double* q) {
  const int lane = threadIdx.x & 31;
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long m = warp; m < npix; m += nwarps) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    const long long j1 = off[m + 1];
    for (long long j = off[m] + lane; j < j1; j += 32) {
      const uint32_t i = idx[j];
      const double* v = ys + (size_t)(i >> 3) * 24 + (i & 7);
      const double2 w = ccs[j];
      a0 += v[0];
      a1 += w.x * v[8] - w.y * v[16];
      a2 += w.y * v[8] + w.x * v[16];
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

template <int L>
static void pt_f32_launch(const long long* csr_off, const uint32_t* csr_idx, const float* csr_cs,
                          const float* ys, long long npix, const int* hits_true, double* q,
                          cudaStream_t st) {
  const long long blocks = (npix + 256 / L - 1) / (256 / L);
  k_pt_f32<L><<<(unsigned)blocks, 256, 0, st>>>(csr_off, csr_idx,
                                                reinterpret_cast<const float2*>(csr_cs),
                                                ys, npix, hits_true, q);
}

template <>
cudaError_t pt_launch<float>(const long long* csr_off, const uint32_t* csr_idx,
                             const float* csr_cs, const float* ys, long long npix,
                             const int* hits_true, double* q, int lanes, cudaStream_t st) {
  switch (lanes) {
    case 1: pt_f32_launch<1>(csr_off, csr_idx, csr_cs, ys, npix, hits_true, q, st); break;
    case 2: pt_f32_launch<2>(csr_off, csr_idx, csr_cs, ys, npix, hits_true, q, st); break;
    case 4: pt_f32_launch<4>(csr_off, csr_idx, csr_cs, ys, npix, hits_true, q, st); break;
    case 8: pt_f32_launch<8>(csr_off, csr_idx, csr_cs, ys, npix, hits_true, q, st); break;
    case 16: pt_f32_launch<16>(csr_off, csr_idx, csr_cs, ys, npix, hits_true, q, st); break;
    default: pt_f32_launch<32>(csr_off, csr_idx, csr_cs, ys, npix, hits_true, q, st); break;
  }
  return cudaGetLastError();
}

template <>
cudaError_t pt_launch<double>(const long long* csr_off, const uint32_t* csr_idx,
                              const double* csr_cs, const double* ys, long long npix,
                              const int* hits_true, double* q, int, cudaStream_t st) {
  long long blocks = (npix * 32 + 255) / 256;
  if (blocks > 152LL * 8 * 16) blocks = 152LL * 8 * 16;
  k_pt_f64<<<(unsigned)blocks, 256, 0, st>>>(csr_off, csr_idx,
                                             reinterpret_cast<const double2*>(csr_cs), ys, npix,
                                             hits_true, q);
  return cudaGetLastError();
}

}  // namespace sg
