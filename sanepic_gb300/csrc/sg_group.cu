// sg_group.cu -- the operator A = P^T N^-1 P for an offset group (detectors
// that share one pixel stream) at the cost of three timelines instead of one
// per detector.
//
// With the group's base angle phi and detector d's rotation (c_d, s_d) =
// (cos 2d', sin 2d'), detector d sees
//   y_d = a + c_d b1 + s_d b2,   a = I,  b1 = Q cos 2phi + U sin 2phi,
//                                        b2 = U cos 2phi - Q sin 2phi,
// and P^T only needs S0 = sum_d y'_d, S1 = sum_d c_d y'_d, S2 = sum_d s_d y'_d
// of the weighted timelines y'_d = N_d^-1 y_d (sg_pt.cu's k_pt).  Every N_d^-1
// is diagonal in each segment's Fourier basis (h_d[k]), so per frequency
//   (S0, S1, S2)^ = H[k] (a, b1, b2)^,   H = sum_d h_d [1 c s]^T [1 c s]
// with a real symmetric 3 x 3 H per group and frequency.  A group of D
// detectors then costs 3 forward and 3 inverse FFTs per segment instead of D
// of each.  This is the same linear map as the reference's per-detector
// deproject -> FFT -> iSpf -> inverse FFT -> scatter (sanepic.cc:2845-2873,
// 2390-2445, 2522-2611), regrouped; only the rounding differs.
#include <cuda_runtime.h>

#include "sg_kernels.h"

namespace sg {

static unsigned blocks_for(long long n, long long cap = 152LL * 16) {
  long long b = (n + 255) / 256;
  if (b > cap) b = cap;
  return (unsigned)(b < 1 ? 1 : b);
}

// Where component c of group sample w of group g goes: [G][3][nsd], or with
// ilv P^T's interleaved layout [G][nsd / 8][3][8] (the three-pass weighting of
// sg_fft3.cu works in place there)
__device__ __forceinline__ long long gtl_at(long long g, int c, long long w, long long nsd, int ilv) {
  return ilv ? 3 * g * nsd + 24 * (w >> 3) + 8 * c + (w & 7) : (3 * g + c) * nsd + w;
}

// gtl: a, b1, b2 of every group sample
template <typename T>
__global__ void __launch_bounds__(256)
    k_group_project(const int* __restrict__ gpix, const T* __restrict__ gcs,
                    const T* __restrict__ map, long long ng, long long nsd, int ilv,
                    T* __restrict__ gtl) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ng;
       i += (long long)gridDim.x * blockDim.x) {
    const long long g = i / nsd, w = i - g * nsd;
    const int m = gpix[i];
    const T c = gcs[2 * i], s = gcs[2 * i + 1];
    const T I = map[4 * (long long)m], Q = map[4 * (long long)m + 1], U = map[4 * (long long)m + 2];
    gtl[gtl_at(g, 0, w, nsd, ilv)] = I;
    gtl[gtl_at(g, 1, w, nsd, ilv)] = Q * c + U * s;
    gtl[gtl_at(g, 2, w, nsd, ilv)] = U * c - Q * s;
  }
}

// FP32 into P^T's interleaved layout, four group samples per thread (16-byte
// pixel and angle loads, one float4 map gather per sample, one float4 store
// per component: the four samples of a component are contiguous there);
// with wmix (uniform groups) the three timelines are mixed by W as below.
// ng and nsd are multiples of 8 (ns >= 1024).
__global__ void __launch_bounds__(256)
    k_group_project4(const int4* __restrict__ gpix, const float4* __restrict__ gcs,
                     const float4* __restrict__ map, const float* __restrict__ wmix,
                     long long n4, long long nsd, float* __restrict__ gtl) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4;
       i += (long long)gridDim.x * blockDim.x) {
    const long long i0 = 4 * i, g = i0 / nsd, w = i0 - g * nsd;
    const int4 p = __ldcs(gpix + i);
    const float4 ca = __ldcs(gcs + 2 * i), cb = __ldcs(gcs + 2 * i + 1);
    const float4 m0 = map[p.x], m1 = map[p.y], m2 = map[p.z], m3 = map[p.w];
    float4 a = make_float4(m0.x, m1.x, m2.x, m3.x);
    float4 b = make_float4(ca.x * m0.y + ca.y * m0.z, ca.z * m1.y + ca.w * m1.z,
                           cb.x * m2.y + cb.y * m2.z, cb.z * m3.y + cb.w * m3.z);
    float4 e = make_float4(ca.x * m0.z - ca.y * m0.y, ca.z * m1.z - ca.w * m1.y,
                           cb.x * m2.z - cb.y * m2.y, cb.z * m3.z - cb.w * m3.y);
    if (wmix) {
      const float* W = wmix + 6 * g;  // W00 W01 W02 W11 W12 W22
      const float4 a0 = a, b0 = b, e0 = e;
      a = make_float4(W[0] * a0.x + W[1] * b0.x + W[2] * e0.x, W[0] * a0.y + W[1] * b0.y + W[2] * e0.y,
                      W[0] * a0.z + W[1] * b0.z + W[2] * e0.z, W[0] * a0.w + W[1] * b0.w + W[2] * e0.w);
      b = make_float4(W[1] * a0.x + W[3] * b0.x + W[4] * e0.x, W[1] * a0.y + W[3] * b0.y + W[4] * e0.y,
                      W[1] * a0.z + W[3] * b0.z + W[4] * e0.z, W[1] * a0.w + W[3] * b0.w + W[4] * e0.w);
      e = make_float4(W[2] * a0.x + W[4] * b0.x + W[5] * e0.x, W[2] * a0.y + W[4] * b0.y + W[5] * e0.y,
                      W[2] * a0.z + W[4] * b0.z + W[5] * e0.z, W[2] * a0.w + W[4] * b0.w + W[5] * e0.w);
    }
    float* o = gtl + gtl_at(g, 0, w, nsd, 1);
    *reinterpret_cast<float4*>(o) = a;
    *reinterpret_cast<float4*>(o + 8) = b;
    *reinterpret_cast<float4*>(o + 16) = e;
  }
}

// Uniform groups (one noise spectrum h for all the group's detectors):
// H = h W with the constant W = sum_d [1 c s]^T [1 c s], so W mixes the three
// timelines before the filter instead of per frequency after it:
// gtl = W (a, b1, b2), then N^-1 on each by the fused filter kernel.
template <typename T>
__global__ void __launch_bounds__(256)
    k_group_project_w(const int* __restrict__ gpix, const T* __restrict__ gcs,
                      const T* __restrict__ map, const T* __restrict__ wmix, long long ng,
                      long long nsd, int ilv, T* __restrict__ gtl) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ng;
       i += (long long)gridDim.x * blockDim.x) {
    const long long g = i / nsd, w = i - g * nsd;
    const int m = gpix[i];
    const T c = gcs[2 * i], s = gcs[2 * i + 1];
    const T I = map[4 * (long long)m], Q = map[4 * (long long)m + 1], U = map[4 * (long long)m + 2];
    const T a = I, b1 = Q * c + U * s, b2 = U * c - Q * s;
    const T* W = wmix + 6 * g;  // W00 W01 W02 W11 W12 W22
    gtl[gtl_at(g, 0, w, nsd, ilv)] = W[0] * a + W[1] * b1 + W[2] * b2;
    gtl[gtl_at(g, 1, w, nsd, ilv)] = W[1] * a + W[3] * b1 + W[4] * b2;
    gtl[gtl_at(g, 2, w, nsd, ilv)] = W[2] * a + W[4] * b1 + W[5] * b2;
  }
}

// wmix [G][6] = sum over the group's detectors of (1, c, s, cc, cs, ss), FP64 sums
template <typename T>
__global__ void k_group_wmix(const T* __restrict__ dcs, const int* __restrict__ grp_off,
                             const int* __restrict__ grp_det, long long G, T* __restrict__ wmix) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= G) return;
  double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int e = grp_off[g]; e < grp_off[g + 1]; e++) {
    const int d = grp_det[e];
    const double c = (double)dcs[2 * d], s = (double)dcs[2 * d + 1];
    acc[0] += 1.0;
    acc[1] += c;
    acc[2] += s;
    acc[3] += c * c;
    acc[4] += c * s;
    acc[5] += s * s;
  }
  for (int j = 0; j < 6; j++) wmix[6 * g + j] = (T)acc[j];
}

template <typename T>
cudaError_t group_project_w_launch(const int* gpix, const T* gcs, const T* map, const T* wmix,
                                   long long ng, long long nsd, T* gtl, int ilv, cudaStream_t st) {
  if constexpr (sizeof(T) == 4) {
    if (ilv && nsd % 8 == 0) {
      k_group_project4<<<blocks_for(ng / 4), 256, 0, st>>>(
          reinterpret_cast<const int4*>(gpix), reinterpret_cast<const float4*>(gcs),
          reinterpret_cast<const float4*>(map), wmix, ng / 4, nsd, gtl);
      return cudaGetLastError();
    }
  }
  k_group_project_w<T><<<blocks_for(ng), 256, 0, st>>>(gpix, gcs, map, wmix, ng, nsd, ilv, gtl);
  return cudaGetLastError();
}
template <typename T>
cudaError_t group_wmix_launch(const T* dcs, const int* grp_off, const int* grp_det, long long G,
                              T* wmix, cudaStream_t st) {
  k_group_wmix<T><<<(unsigned)((G + 127) / 128), 128, 0, st>>>(dcs, grp_off, grp_det, G, wmix);
  return cudaGetLastError();
}

// in place on the half spectra [G][3][nseg][M+1]: (S0, S1, S2) = H (a, b1, b2)
template <typename T>
__global__ void __launch_bounds__(256)
    k_group_mix(cplx<T>* __restrict__ spec, const T* __restrict__ hmix, long long G,
                long long nseg, long long M1) {
  const long long n = G * nseg * M1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long k = i % M1, gs = i / M1;
    const long long seg = gs % nseg, g = gs / nseg;
    cplx<T>* x0 = spec + ((g * 3) * nseg + seg) * M1 + k;
    cplx<T>* x1 = x0 + nseg * M1;
    cplx<T>* x2 = x1 + nseg * M1;
    const T* h = hmix + (g * M1 + k) * 6;
    const T h0 = h[0], h1 = h[1], h2 = h[2], h11 = h[3], h12 = h[4], h22 = h[5];
    const cplx<T> a = *x0, b = *x1, c = *x2;
    *x0 = cplx<T>{h0 * a.x + h1 * b.x + h2 * c.x, h0 * a.y + h1 * b.y + h2 * c.y};
    *x1 = cplx<T>{h1 * a.x + h11 * b.x + h12 * c.x, h1 * a.y + h11 * b.y + h12 * c.y};
    *x2 = cplx<T>{h2 * a.x + h12 * b.x + h22 * c.x, h2 * a.y + h12 * b.y + h22 * c.y};
  }
}

// hmix [G][slot][6] = sum over the group's detectors of h_d[k] (1, c, s, cc, cs, ss),
// k = kslot[slot] (spectra are kept in the filter's slot order)
template <typename T>
__global__ void __launch_bounds__(256)
    k_group_hmix(const T* __restrict__ filt, const T* __restrict__ dcs, const int* __restrict__ grp_off,
                 const int* __restrict__ grp_det, const int* __restrict__ kslot, long long G,
                 long long M1, T* __restrict__ hmix) {
  const long long n = G * M1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long g = i / M1, k = kslot[i - g * M1];
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int e = grp_off[g]; e < grp_off[g + 1]; e++) {
      const int d = grp_det[e];
      const double h = (double)filt[d * M1 + k];
      const double c = (double)dcs[2 * d], s = (double)dcs[2 * d + 1];
      acc[0] += h;
      acc[1] += c * h;
      acc[2] += s * h;
      acc[3] += c * c * h;
      acc[4] += c * s * h;
      acc[5] += s * s * h;
    }
    for (int j = 0; j < 6; j++) hmix[i * 6 + j] = (T)acc[j];
  }
}

// right-hand side of a group from its detectors' data spectra X_d [ndet][nseg][M+1]
// (slot order; filt holds the filter rows in the same order):
// gspec (S0, S1, S2)^ = sum_d h_d X_d (1, c_d, s_d), detectors in list order;
// chi2_part[block] = sum of h_d |X_d|^2 over the block's bins (k = 0..M).
// A thread takes four consecutive slots, so a warp reads 1 KB of every
// detector's spectrum at once (the detectors' spectra lie 25 MB apart).
// Plain FP32 sums over the group's detectors in a fixed order (a
// compensated sum made the kernel issue-bound; with tens of terms of
// similar size the plain sum keeps ~1e-6 of the largest term).
template <typename T>
__global__ void __launch_bounds__(256)
    k_group_rhs(const cplx<T>* __restrict__ dspec, const T* __restrict__ filt,
                const T* __restrict__ dcs, const int* __restrict__ grp_off,
                const int* __restrict__ grp_det, long long G, long long nseg, long long M1,
                cplx<T>* __restrict__ gspec, double* chi2_part) {
  constexpr int KV = 4;
  const long long nq = (M1 + KV - 1) / KV;  // slot quads per (group, segment)
  const long long n = G * nseg * nq;
  double chi = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long k0 = (i % nq) * KV, gs = i / nq;
    const long long seg = gs % nseg, g = gs / nseg;
    const int kn = (int)(M1 - k0 < KV ? M1 - k0 : KV);
    T a[KV][6];
#pragma unroll
    for (int u = 0; u < KV; u++)
#pragma unroll
      for (int q = 0; q < 6; q++) a[u][q] = T(0);
    T cl = T(0);
#pragma unroll 4
    for (int e = grp_off[g]; e < grp_off[g + 1]; e++) {
      const int d = grp_det[e];
      const cplx<T>* x = dspec + ((long long)d * nseg + seg) * M1 + k0;
      const T* h = filt + d * M1 + k0;
      const T c = dcs[2 * d], s = dcs[2 * d + 1];
      cplx<T> xv[KV];
      T hv[KV];
#pragma unroll
      for (int u = 0; u < KV; u++) {
        xv[u] = u < kn ? x[u] : cplx<T>{T(0), T(0)};
        hv[u] = u < kn ? h[u] : T(0);
      }
#pragma unroll
      for (int u = 0; u < KV; u++) {
        const T hx = hv[u] * xv[u].x, hy = hv[u] * xv[u].y;
        a[u][0] += hx;
        a[u][1] += hy;
        a[u][2] = fma(c, hx, a[u][2]);
        a[u][3] = fma(c, hy, a[u][3]);
        a[u][4] = fma(s, hx, a[u][4]);
        a[u][5] = fma(s, hy, a[u][5]);
        cl = fma(hx, xv[u].x, fma(hy, xv[u].y, cl));
      }
    }
    chi += (double)cl;
    cplx<T>* o = gspec + ((g * 3) * nseg + seg) * M1 + k0;
#pragma unroll
    for (int u = 0; u < KV; u++) {
      if (u >= kn) break;
      o[u] = cplx<T>{a[u][0], a[u][1]};
      o[nseg * M1 + u] = cplx<T>{a[u][2], a[u][3]};
      o[2 * nseg * M1 + u] = cplx<T>{a[u][4], a[u][5]};
    }
  }
  __shared__ double red[8];
  for (int o = 16; o > 0; o >>= 1) chi += __shfl_xor_sync(0xffffffffu, chi, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = chi;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; w++) t += red[w];
    chi2_part[blockIdx.x] = t;
  }
}

// A group whose detectors all have the same noise spectrum h needs no
// per-detector FFT for its right-hand side: sum_d h X_d (1, c_d, s_d) =
// h FFT(sum_d d_d (1, c_d, s_d)), so the detectors' timelines are summed
// first (gtl [G][3][nsd], detectors in list order, FP32) ...
template <typename T>
__global__ void __launch_bounds__(256)
    k_group_tod_sums(const T* __restrict__ tod, long long nsd, const int* __restrict__ grp_off,
                     const int* __restrict__ grp_det, const T* __restrict__ dcs, long long G,
                     int ilv, T* __restrict__ gtl) {
  const long long n = G * nsd;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long g = i / nsd, w = i - g * nsd;
    T s0 = T(0), s1 = T(0), s2 = T(0);
#pragma unroll 4
    for (int e = grp_off[g]; e < grp_off[g + 1]; e++) {
      const int d = grp_det[e];
      const T x = tod[(long long)d * nsd + w];
      s0 += x;
      s1 = fma(dcs[2 * d], x, s1);
      s2 = fma(dcs[2 * d + 1], x, s2);
    }
    gtl[gtl_at(g, 0, w, nsd, ilv)] = s0;
    gtl[gtl_at(g, 1, w, nsd, ilv)] = s1;
    gtl[gtl_at(g, 2, w, nsd, ilv)] = s2;
  }
}

// ... and their half spectra [G][3][nseg][M+1] (slot order) are scaled by the
// group's one filter row (filt [ndet][M+1] in slot order; its first detector's)
template <typename T>
__global__ void __launch_bounds__(256)
    k_group_scale(cplx<T>* __restrict__ spec, const T* __restrict__ filt,
                  const int* __restrict__ grp_off, const int* __restrict__ grp_det, long long G,
                  long long nseg, long long M1) {
  const long long n = G * 3 * nseg * M1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long k = i % M1, g = i / (3 * nseg * M1);
    const T h = filt[(long long)grp_det[grp_off[g]] * M1 + k];
    spec[i] = cscale(spec[i], h);
  }
}

// same[d] = 1 if detector d's filter row equals (bitwise) the row of its
// group's first detector; one block per detector
template <typename T>
__global__ void __launch_bounds__(256)
    k_rows_match_group(const T* __restrict__ filt, long long M1, const int* __restrict__ grp_off,
                       const int* __restrict__ grp_det, long long G, int* __restrict__ same) {
  const long long e = blockIdx.x;  // position in the group lists
  int g = 0;
  while (g + 1 < G && grp_off[g + 1] <= e) g++;
  const int d = grp_det[e], d0 = grp_det[grp_off[g]];
  const T* a = filt + (long long)d * M1;
  const T* b = filt + (long long)d0 * M1;
  int diff = 0;
  for (long long k = threadIdx.x; k < M1 && !diff; k += blockDim.x) diff = a[k] != b[k];
  diff = __syncthreads_or(diff);
  if (threadIdx.x == 0) same[d] = diff ? 0 : 1;
}

template <typename T>
cudaError_t group_tod_rhs_launch(const T* tod, long long nsd, const int* grp_off,
                                 const int* grp_det, const T* dcs, long long G, T* gtl, int ilv,
                                 cudaStream_t st) {
  k_group_tod_sums<T><<<blocks_for(G * nsd), 256, 0, st>>>(tod, nsd, grp_off, grp_det, dcs, G, ilv,
                                                            gtl);
  return cudaGetLastError();
}
template <typename T>
cudaError_t group_scale_launch(cplx<T>* spec, const T* filt, const int* grp_off, const int* grp_det,
                               long long G, long long nseg, long long M1, cudaStream_t st) {
  k_group_scale<T><<<blocks_for(G * 3 * nseg * M1), 256, 0, st>>>(spec, filt, grp_off, grp_det, G,
                                                                  nseg, M1);
  return cudaGetLastError();
}
template <typename T>
cudaError_t rows_match_group_launch(const T* filt, long long M1, const int* grp_off,
                                    const int* grp_det, long long G, long long ndet_listed,
                                    int* same, cudaStream_t st) {
  k_rows_match_group<T><<<(unsigned)ndet_listed, 256, 0, st>>>(filt, M1, grp_off, grp_det, G, same);
  return cudaGetLastError();
}

template <typename T>
cudaError_t group_rhs_launch(const cplx<T>* dspec, const T* filt, const T* dcs, const int* grp_off,
                             const int* grp_det, long long G, long long nseg, long long M1,
                             cplx<T>* gspec, double* chi2_part, int nblocks, cudaStream_t st) {
  k_group_rhs<T><<<nblocks, 256, 0, st>>>(dspec, filt, dcs, grp_off, grp_det, G, nseg, M1, gspec,
                                         chi2_part);
  return cudaGetLastError();
}

template <typename T>
cudaError_t group_project_launch(const int* gpix, const T* gcs, const T* map, long long ng,
                                 long long nsd, T* gtl, int ilv, cudaStream_t st) {
  if constexpr (sizeof(T) == 4) {
    if (ilv && nsd % 8 == 0) {
      k_group_project4<<<blocks_for(ng / 4), 256, 0, st>>>(
          reinterpret_cast<const int4*>(gpix), reinterpret_cast<const float4*>(gcs),
          reinterpret_cast<const float4*>(map), nullptr, ng / 4, nsd, gtl);
      return cudaGetLastError();
    }
  }
  k_group_project<T><<<blocks_for(ng), 256, 0, st>>>(gpix, gcs, map, ng, nsd, ilv, gtl);
  return cudaGetLastError();
}
template <typename T>
cudaError_t group_mix_launch(cplx<T>* spec, const T* hmix, long long G, long long nseg,
                             long long M1, cudaStream_t st) {
  k_group_mix<T><<<blocks_for(G * nseg * M1), 256, 0, st>>>(spec, hmix, G, nseg, M1);
  return cudaGetLastError();
}
template <typename T>
cudaError_t group_hmix_launch(const T* filt, const T* dcs, const int* grp_off, const int* grp_det,
                              const int* kslot, long long G, long long M1, T* hmix,
                              cudaStream_t st) {
  k_group_hmix<T><<<blocks_for(G * M1), 256, 0, st>>>(filt, dcs, grp_off, grp_det, kslot, G, M1,
                                                     hmix);
  return cudaGetLastError();
}

// out [rows][slot] = in [rows][kslot[slot]]
template <typename T>
__global__ void __launch_bounds__(256)
    k_permute_rows(const T* __restrict__ in, const int* __restrict__ kslot, long long rows,
                   long long M1, T* __restrict__ out) {
  const long long n = rows * M1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / M1;
    out[i] = in[r * M1 + kslot[i - r * M1]];
  }
}

template <typename T>
cudaError_t permute_rows_launch(const T* in, const int* kslot, long long rows, long long M1, T* out,
                                cudaStream_t st) {
  k_permute_rows<T><<<blocks_for(rows * M1), 256, 0, st>>>(in, kslot, rows, M1, out);
  return cudaGetLastError();
}

#define SG_GROUP_INST(T)                                                                       \
  template cudaError_t group_project_launch<T>(const int*, const T*, const T*, long long,        \
                                               long long, T*, int, cudaStream_t);                \
  template cudaError_t group_mix_launch<T>(cplx<T>*, const T*, long long, long long, long long,  \
                                           cudaStream_t);                                        \
  template cudaError_t group_hmix_launch<T>(const T*, const T*, const int*, const int*,          \
                                            const int*, long long, long long, T*, cudaStream_t); \
  template cudaError_t permute_rows_launch<T>(const T*, const int*, long long, long long, T*,    \
                                              cudaStream_t);                                     \
  template cudaError_t group_rhs_launch<T>(const cplx<T>*, const T*, const T*, const int*,       \
                                           const int*, long long, long long, long long,          \
                                           cplx<T>*, double*, int, cudaStream_t);                \
  template cudaError_t group_tod_rhs_launch<T>(const T*, long long, const int*, const int*,      \
                                               const T*, long long, T*, int, cudaStream_t);      \
  template cudaError_t group_scale_launch<T>(cplx<T>*, const T*, const int*, const int*,         \
                                             long long, long long, long long, cudaStream_t);     \
  template cudaError_t rows_match_group_launch<T>(const T*, long long, const int*, const int*,   \
                                                  long long, long long, int*, cudaStream_t);     \
  template cudaError_t group_project_w_launch<T>(const int*, const T*, const T*, const T*,        \
                                                 long long, long long, T*, int, cudaStream_t);   \
  template cudaError_t group_wmix_launch<T>(const T*, const int*, const int*, long long, T*,     \
                                            cudaStream_t);
SG_GROUP_INST(float)
SG_GROUP_INST(double)

}  // namespace sg
