// sg_filter.cu -- per-(detector, segment) noise weighting N^-1 as one fused
// GB300 kernel: load (TOD, or the projection P of a map) -> real FFT ->
// multiply by the inverse-noise spectrum -> inverse real FFT -> store.
//
// Replaces the reference's write_tfAS + the first half of do_PtNd
// (sanepic.cc:2390-2445, 2522-2582): per tile of ns samples it computes
//   y = c2r( h . r2c(x) ),   h[k] = SpN_all[k] (k <= ns/2, sanepic.cc:533-537)
// with FFTW's unnormalised conventions (r2c sign -1, c2r sign +1).
//
// Algorithm.  The real tile x (N = ns samples) is packed as M = N/2 complex
// points z[m] = x[2m] + i x[2m+1].  The length-M complex FFT is a four-step
// FFT, M = R x C: column FFTs of length R, a W_M twiddle, row FFTs of length
// C.  A tile is spread over a thread-block cluster of S CTAs (one tile at a
// time per cluster): CTA j owns columns [j C/S, (j+1) C/S) for the column
// pass and a set of R/S rows for the row pass; the transposes between the
// passes go through distributed shared memory (no HBM round trip, no TMA
// multicast).  Rows are dealt out in pairs (k1, R-k1) so that every
// frequency k and its real-FFT partner M-k live in the same CTA, which lets
// the split into the real spectrum, the multiply by h and the re-packing for
// the inverse all happen in place.  Each sub-FFT (length R or C) runs as two
// in-register radix passes (sizes 2..16) through shared memory; the forward
// sub-FFT leaves its output digit-reversed and the inverse consumes it that
// way, so no reordering pass is needed.  Twiddles come from two small
// shared-memory tables (W_M^j = W_M^{64 jh} W_M^{jl}) built in FP64 on the
// host.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "sg_cplx.cuh"
#include "sg_dft.cuh"
#include "sg_kernels.h"

namespace cg = cooperative_groups;

namespace sg {

template <typename T>
struct alignas(4 * sizeof(T)) map4 {
  T I, Q, U, pad;
};

constexpr int kFilterThreads = 512;
constexpr int kTwLo = 64;

template <typename T>
struct Tw {
  const cplx<T>* lo;  // W_M^j, j < 64
  const cplx<T>* hi;  // W_M^{64 j}, j < M/64
  __device__ __forceinline__ cplx<T> operator()(int j) const {
    return cmul(hi[j >> 6], lo[j & (kTwLo - 1)]);
  }
};

// Row index list: rows 0 and R/2 first, then the pairs (p, R-p).
template <int R>
__device__ __forceinline__ int row_of(int i) {
  if (i == 0) return 0;
  if (i == 1) return R / 2;
  int p = i >> 1;
  return (i & 1) ? R - p : p;
}

template <typename T, int LOGR, int LOGC>
__global__ void __launch_bounds__(kFilterThreads, 1)
    k_noise_filter(FilterArgs<T> p) {
  constexpr int R = 1 << LOGR, C = 1 << LOGC, M = R * C;
  constexpr int R1 = 1 << ((LOGR + 1) / 2), R2 = R / R1;
  constexpr int C1 = 1 << ((LOGC + 1) / 2), C2 = C / C1;
  cg::cluster_group cl = cg::this_cluster();
  const int S = (int)cl.num_blocks();
  const int j = (int)cl.block_rank();
  const int Cs = C / S, Rs = R / S;
  const int PA = Cs + 1, PC = Rs + 1;
  const int E = M / S;
  const int tid = threadIdx.x, nth = blockDim.x;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* bufA = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* bufC = bufA + R * PA;
  cplx<T>* twlo = bufC + C * PC;
  cplx<T>* twhi = twlo + kTwLo;
  for (int i = tid; i < kTwLo; i += nth) twlo[i] = p.tw_lo[i];
  for (int i = tid; i < M / kTwLo; i += nth) twhi[i] = p.tw_hi[i];
  __syncthreads();
  const Tw<T> tw{twlo, twhi};
  const cplx<T> wn1 = p.wn1;

  const int cluster_id = blockIdx.x / S;
  const int nclusters = gridDim.x / S;
  for (long long tile = cluster_id; tile < p.ntiles; tile += nclusters) {
    const long long base = tile * (long long)(2 * M);
    const int det = (int)(tile / p.nseg);
    // ---- 1. load z for this CTA's columns -------------------------------
    for (int e = tid; e < E; e += nth) {
      const int c = e % Cs, n1 = e / Cs;
      const long long s0 = base + 2LL * (C * n1 + j * Cs + c);
      cplx<T> v;
      if (p.mode == kLoadTod) {
        v = *reinterpret_cast<const cplx<T>*>(p.tod + s0);
      } else if (p.mode == kLoadProj) {
        const int2 pp = *reinterpret_cast<const int2*>(p.pix + s0);
        const cplx<T> cs0 = *reinterpret_cast<const cplx<T>*>(p.cs + 2 * s0);
        const cplx<T> cs1 = *reinterpret_cast<const cplx<T>*>(p.cs + 2 * s0 + 2);
        const map4<T> m0 = reinterpret_cast<const map4<T>*>(p.map)[pp.x];
        const map4<T> m1 = reinterpret_cast<const map4<T>*>(p.map)[pp.y];
        v.x = m0.I + cs0.x * m0.Q + cs0.y * m0.U;
        v.y = m1.I + cs1.x * m1.Q + cs1.y * m1.U;
      } else {  // unit impulse at sample 0 of the tile
        v.x = (s0 == base) ? T(1) : T(0);
        v.y = T(0);
      }
      bufA[n1 * PA + c] = v;
    }
    __syncthreads();
    // ---- 2. forward column FFTs (length R), then the W_M twiddle ---------
    for (int u = tid; u < Cs * R2; u += nth) {
      const int c = u % Cs, n2 = u / Cs;
      cplx<T> a[R1];
#pragma unroll
      for (int i = 0; i < R1; i++) a[i] = bufA[(R2 * i + n2) * PA + c];
      SgDft<R1, false, T>::run(a);
#pragma unroll
      for (int k = 0; k < R1; k++) {
        cplx<T> w = tw((n2 * k * C) & (M - 1));
        bufA[(R2 * k + n2) * PA + c] = (k == 0 || n2 == 0) ? a[k] : cmul(a[k], w);
      }
    }
    __syncthreads();
    for (int u = tid; u < Cs * R1; u += nth) {
      const int c = u % Cs, ka = u / Cs;
      const int n2g = j * Cs + c;
      cplx<T> b[R2];
#pragma unroll
      for (int i = 0; i < R2; i++) b[i] = bufA[(R2 * ka + i) * PA + c];
      SgDft<R2, false, T>::run(b);
#pragma unroll
      for (int kb = 0; kb < R2; kb++) {
        const int k1 = ka + R1 * kb;
        bufA[(R2 * ka + kb) * PA + c] = cmul(b[kb], tw((n2g * k1) & (M - 1)));
      }
    }
    cl.sync();
    // ---- 3. transpose through DSMEM: rows of this CTA, all columns -------
    for (int e = tid; e < E; e += nth) {
      const int c = e % Cs, r = e / Cs, q = r % S, t = r / S;
      const int k1 = row_of<R>(j * Rs + t);
      const int posr = R2 * (k1 % R1) + k1 / R1;
      const cplx<T>* src = cl.map_shared_rank(bufA, q);
      bufC[(q * Cs + c) * PC + t] = src[posr * PA + c];
    }
    __syncthreads();
    // ---- 4. forward row FFTs (length C) ----------------------------------
    for (int u = tid; u < Rs * C2; u += nth) {
      const int t = u % Rs, n2 = u / Rs;
      cplx<T> a[C1];
#pragma unroll
      for (int i = 0; i < C1; i++) a[i] = bufC[(C2 * i + n2) * PC + t];
      SgDft<C1, false, T>::run(a);
#pragma unroll
      for (int k = 0; k < C1; k++) {
        cplx<T> w = tw((n2 * k * R) & (M - 1));
        bufC[(C2 * k + n2) * PC + t] = (k == 0 || n2 == 0) ? a[k] : cmul(a[k], w);
      }
    }
    __syncthreads();
    for (int u = tid; u < Rs * C1; u += nth) {
      const int t = u % Rs, ka = u / Rs;
      cplx<T> b[C2];
#pragma unroll
      for (int i = 0; i < C2; i++) b[i] = bufC[(C2 * ka + i) * PC + t];
      SgDft<C2, false, T>::run(b);
#pragma unroll
      for (int kb = 0; kb < C2; kb++) bufC[(C2 * ka + kb) * PC + t] = b[kb];
    }
    __syncthreads();
    // ---- 5. real-spectrum split, multiply by h, re-pack for c2r ----------
    {
      const T* h = p.filt + (long long)det * (M + 1);
      for (int e = tid; e < E; e += nth) {
        const int t = e % Rs, pos = e / Rs;
        const int k2 = pos / C2 + C1 * (pos % C2);
        const int k1 = row_of<R>(j * Rs + t);
        const int k = k1 + R * k2;
        if (k == 0) {
          const cplx<T> z = bufC[pos * PC + t];
          T h0 = h[0], hM = h[M];
          if (p.filt_abs) { h0 = fabs(h0); hM = fabs(hM); }
          const T y0 = h0 * (z.x + z.y), yM = hM * (z.x - z.y);
          bufC[pos * PC + t] = cplx<T>{y0 + yM, y0 - yM};
          continue;
        }
        int k2p, tp;
        if (k1 == 0) {
          k2p = C - k2;
          tp = t;
        } else {
          k2p = C - 1 - k2;
          tp = (j == 0 && t < 2) ? t : (t ^ 1);
        }
        const int kp = M - k;
        if (k > kp) continue;
        const int posp = C2 * (k2p % C1) + k2p / C1;
        const cplx<T> zk = bufC[pos * PC + t];
        const cplx<T> zm = bufC[posp * PC + tp];
        T hk = h[k], hm = h[kp];
        if (p.filt_abs) { hk = fabs(hk); hm = fabs(hm); }
        // E = (Zk + conj Zm)/2, O = -i (Zk - conj Zm)/2
        const cplx<T> Ev{T(0.5) * (zk.x + zm.x), T(0.5) * (zk.y - zm.y)};
        const cplx<T> Ov{T(0.5) * (zk.y + zm.y), T(-0.5) * (zk.x - zm.x)};
        cplx<T> w = tw(k >> 1);
        if (k & 1) w = cmul(w, wn1);
        const cplx<T> wO = cmul(w, Ov);
        const cplx<T> Xk = Ev + wO;
        const cplx<T> Xm = cconj(Ev - wO);
        const cplx<T> Yk = cscale(Xk, hk), Ym = cscale(Xm, hm);
        const cplx<T> P = Yk + cconj(Ym), Q = Yk - cconj(Ym);
        const cplx<T> cwQ = cmulc(Q, w);              // conj(w) Q
        const cplx<T> iwQ{-cwQ.y, cwQ.x};             // i conj(w) Q
        bufC[pos * PC + t] = P + iwQ;
        bufC[posp * PC + tp] = cconj(P - iwQ);
      }
    }
    __syncthreads();
    // ---- 6. inverse row FFTs (digit-reversed in, natural out), W_M^-1 ----
    for (int u = tid; u < Rs * C1; u += nth) {
      const int t = u % Rs, a1 = u / Rs;
      cplx<T> b[C2];
#pragma unroll
      for (int i = 0; i < C2; i++) b[i] = bufC[(C2 * a1 + i) * PC + t];
      SgDft<C2, true, T>::run(b);
#pragma unroll
      for (int n2 = 0; n2 < C2; n2++) {
        cplx<T> w = tw((n2 * a1 * R) & (M - 1));
        bufC[(C2 * a1 + n2) * PC + t] = (a1 == 0 || n2 == 0) ? b[n2] : cmulc(b[n2], w);
      }
    }
    __syncthreads();
    for (int u = tid; u < Rs * C2; u += nth) {
      const int t = u % Rs, n2 = u / Rs;
      const int k1 = row_of<R>(j * Rs + t);
      cplx<T> a[C1];
#pragma unroll
      for (int i = 0; i < C1; i++) a[i] = bufC[(C2 * i + n2) * PC + t];
      SgDft<C1, true, T>::run(a);
#pragma unroll
      for (int n1 = 0; n1 < C1; n1++) {
        const int n = C2 * n1 + n2;
        bufC[n * PC + t] = cmulc(a[n1], tw((n * k1) & (M - 1)));
      }
    }
    cl.sync();
    // ---- 7. transpose back through DSMEM: this CTA's columns, all rows ---
    for (int e = tid; e < E; e += nth) {
      const int t = e % Rs, r = e / Rs, c = r % Cs, q = r / Cs;
      const int k1 = row_of<R>(q * Rs + t);
      const int posr = R2 * (k1 % R1) + k1 / R1;
      const cplx<T>* src = cl.map_shared_rank(bufC, q);
      bufA[posr * PA + c] = src[(j * Cs + c) * PC + t];
    }
    __syncthreads();
    // ---- 8. inverse column FFTs ------------------------------------------
    for (int u = tid; u < Cs * R1; u += nth) {
      const int c = u % Cs, a1 = u / Cs;
      cplx<T> b[R2];
#pragma unroll
      for (int i = 0; i < R2; i++) b[i] = bufA[(R2 * a1 + i) * PA + c];
      SgDft<R2, true, T>::run(b);
#pragma unroll
      for (int n2 = 0; n2 < R2; n2++) {
        cplx<T> w = tw((n2 * a1 * C) & (M - 1));
        bufA[(R2 * a1 + n2) * PA + c] = (a1 == 0 || n2 == 0) ? b[n2] : cmulc(b[n2], w);
      }
    }
    __syncthreads();
    for (int u = tid; u < Cs * R2; u += nth) {
      const int c = u % Cs, n2 = u / Cs;
      cplx<T> a[R1];
#pragma unroll
      for (int i = 0; i < R1; i++) a[i] = bufA[(R2 * i + n2) * PA + c];
      SgDft<R1, true, T>::run(a);
#pragma unroll
      for (int n1 = 0; n1 < R1; n1++) bufA[(R2 * n1 + n2) * PA + c] = a[n1];
    }
    __syncthreads();
    // ---- 9. store ---------------------------------------------------------
    for (int e = tid; e < E; e += nth) {
      const int c = e % Cs, n1 = e / Cs;
      const long long s0 = base + 2LL * (C * n1 + j * Cs + c);
      *reinterpret_cast<cplx<T>*>(p.out + s0) = bufA[n1 * PA + c];
    }
    __syncthreads();
  }
  cl.sync();  // peers may still read this CTA's shared memory
}

// ---------------------------------------------------------------------------
template <typename T, int LOGR, int LOGC>
static cudaError_t launch_one(const FilterArgs<T>& a, int S, int nclusters,
                              cudaStream_t st) {
  constexpr int R = 1 << LOGR, C = 1 << LOGC, M = R * C;
  const size_t smem = sizeof(cplx<T>) *
                      ((size_t)R * (C / S + 1) + (size_t)C * (R / S + 1) + kTwLo + M / kTwLo);
  auto fn = k_noise_filter<T, LOGR, LOGC>;
  cudaError_t err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
  if (err != cudaSuccess) return err;
  if (S > 8) {
    err = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (err != cudaSuccess) return err;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(S * nclusters);
  cfg.blockDim = dim3(kFilterThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = S;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, fn, a);
}

template <typename T, int LOGR, int LOGC>
static int max_clusters_one(int S) {
  constexpr int R = 1 << LOGR, C = 1 << LOGC, M = R * C;
  const size_t smem = sizeof(cplx<T>) *
                      ((size_t)R * (C / S + 1) + (size_t)C * (R / S + 1) + kTwLo + M / kTwLo);
  auto fn = k_noise_filter<T, LOGR, LOGC>;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return 0;
  if (S > 8) cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(S);
  cfg.blockDim = dim3(kFilterThreads);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = S;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, fn, &cfg) != cudaSuccess) return 0;
  return n;
}

size_t filter_smem_bytes(int logm, int S, int esize) {
  const int logr = (logm + 1) / 2, logc = logm / 2;
  const size_t R = 1u << logr, C = 1u << logc, M = R * C;
  return (size_t)esize * 2 * (R * (C / S + 1) + C * (R / S + 1) + kTwLo + M / kTwLo);
}

#define SG_FILTER_CASES(X, T) \
  X(T, 4, 3) X(T, 4, 4) X(T, 5, 4) X(T, 5, 5) X(T, 6, 5) X(T, 6, 6) X(T, 7, 6) X(T, 7, 7) \
  X(T, 8, 7) X(T, 8, 8)

template <typename T>
cudaError_t filter_launch(const FilterArgs<T>& a, int logm, int S, int nclusters,
                          cudaStream_t st) {
  const int logr = (logm + 1) / 2, logc = logm / 2;
#define SG_CASE(TT, LR, LC) \
  if (logr == LR && logc == LC) return launch_one<TT, LR, LC>(a, S, nclusters, st);
  SG_FILTER_CASES(SG_CASE, T)
#undef SG_CASE
  return cudaErrorInvalidValue;
}

template <typename T>
int filter_max_clusters(int logm, int S) {
  const int logr = (logm + 1) / 2, logc = logm / 2;
#define SG_CASE(TT, LR, LC) \
  if (logr == LR && logc == LC) return max_clusters_one<TT, LR, LC>(S);
  SG_FILTER_CASES(SG_CASE, T)
#undef SG_CASE
  return 0;
}

template cudaError_t filter_launch<float>(const FilterArgs<float>&, int, int, int, cudaStream_t);
template cudaError_t filter_launch<double>(const FilterArgs<double>&, int, int, int, cudaStream_t);
template int filter_max_clusters<float>(int, int);
template int filter_max_clusters<double>(int, int);

}  // namespace sg
