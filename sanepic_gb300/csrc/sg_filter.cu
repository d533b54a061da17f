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
// frequency k and its real-FFT partner M-k live in the same warp, which lets
// the split into the real spectrum, the multiply by h and the re-packing for
// the inverse all happen in place.
//
// Scheduling.  All 512 threads of a CTA cooperate on every pass with the
// batch index (column, or row) fastest across lanes, which makes every
// shared-memory access of the radix passes conflict-free.  The transposes
// are staged through registers (coalesced DSMEM reads), so one shared buffer
// per CTA suffices (~76 KB with the twiddle tables): two CTAs of different
// clusters share an SM (32 warps), and one cluster's barrier waits overlap
// the other's arithmetic.  Each sub-FFT (length R or C) is two in-register
// radix passes (sizes 2..16); the forward sub-FFT leaves its output
// digit-reversed and the inverse consumes it that way.  Twiddles come from
// two shared-memory tables (W_M^j = W_M^{64 jh} W_M^{jl}) built in FP64 on
// the host.  The projection P runs as its own streaming kernel (sg_pt.cu);
// this kernel can also load a map projection itself (kLoadProj), which the
// library uses only for small problems.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>

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
constexpr int kFilterWarps = kFilterThreads / 32;
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
  const int p = i >> 1;
  return (i & 1) ? R - p : p;
}

__device__ __forceinline__ void cluster_arrive() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

template <int LOGR, int LOGC, int S>
struct Geo {
  static constexpr int R = 1 << LOGR, C = 1 << LOGC, M = R * C;
  static constexpr int R1 = 1 << ((LOGR + 1) / 2), R2 = R / R1;
  static constexpr int C1 = 1 << ((LOGC + 1) / 2), C2 = C / C1;
  static constexpr int Cs = C / S, Rs = R / S;   // columns / rows per CTA
  static constexpr int PA = Cs + 1, PC = Rs + 1; // padded strides
  static constexpr int E = M / S;                // complex points per CTA
  static constexpr int BUF = (R * PA > C * PC) ? R * PA : C * PC;
  static constexpr int XE = (E + kFilterThreads - 1) / kFilterThreads;  // per thread
  static_assert(Rs >= 2 && Rs % 2 == 0 && Cs >= 1, "tile too small");
};

template <typename T, int LOGR, int LOGC, int S>
__global__ void __launch_bounds__(kFilterThreads, sizeof(T) == 4 ? 2 : 1)
    k_noise_filter(FilterArgs<T> p) {
  using G = Geo<LOGR, LOGC, S>;
  constexpr int R = G::R, C = G::C, M = G::M, R1 = G::R1, R2 = G::R2, C1 = G::C1, C2 = G::C2;
  constexpr int Cs = G::Cs, Rs = G::Rs, PA = G::PA, PC = G::PC, E = G::E;
  constexpr int NT = kFilterThreads;
  cg::cluster_group cl = cg::this_cluster();
  const int j = (int)cl.block_rank();
  const int tid = threadIdx.x;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* buf = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* twlo = buf + G::BUF;
  cplx<T>* twhi = twlo + kTwLo;
  for (int i = tid; i < kTwLo; i += NT) twlo[i] = p.tw_lo[i];
  for (int i = tid; i < M / kTwLo; i += NT) twhi[i] = p.tw_hi[i];
  __syncthreads();
  const Tw<T> tw{twlo, twhi};
  const cplx<T> wn1 = p.wn1;

  const int cluster_id = blockIdx.x / S;
  const int nclusters = gridDim.x / S;
  double chi2 = 0.0;  // sum of h[k] |X[k]|^2 over this thread's bins
  for (long long tile = cluster_id; tile < p.ntiles; tile += nclusters) {
    const long long base = tile * (long long)(2 * M);
    const int det = (int)(tile / p.nseg);
    // ---- 1. load: z[C n1 + n2] = x[2n] + i x[2n+1], this CTA's columns ----
#pragma unroll 4
    for (int it = 0; it < G::XE; it++) {
      const int e = it * NT + tid;
      if (E % NT != 0 && e >= E) break;
      const int c = e % Cs, n1 = e / Cs;
      const long long s0 = base + 2LL * (C * n1 + j * Cs + c);
      cplx<T> v;
      if (p.mode == kLoadTod) {
        v = *reinterpret_cast<const cplx<T>*>(p.tod + s0);
      } else if (p.mode == kLoadTodMinus) {
        v = *reinterpret_cast<const cplx<T>*>(p.tod + s0) -
            *reinterpret_cast<const cplx<T>*>(p.sub + s0);
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
      buf[n1 * PA + c] = v;
    }
    __syncthreads();
    // ---- 2. forward column FFTs (length R) and the W_M twiddle ------------
    for (int u = tid; u < Cs * R2; u += NT) {
      const int c = u % Cs, n2 = u / Cs;
      cplx<T> a[R1];
#pragma unroll
      for (int i = 0; i < R1; i++) a[i] = buf[(R2 * i + n2) * PA + c];
      SgDft<R1, false, T>::run(a);
#pragma unroll
      for (int k = 0; k < R1; k++)
        buf[(R2 * k + n2) * PA + c] = (k == 0 || n2 == 0) ? a[k] : cmul(a[k], tw((n2 * k * C) & (M - 1)));
    }
    __syncthreads();
    for (int u = tid; u < Cs * R1; u += NT) {
      const int c = u % Cs, ka = u / Cs;
      const int n2g = j * Cs + c;
      cplx<T> b[R2];
#pragma unroll
      for (int i = 0; i < R2; i++) b[i] = buf[(R2 * ka + i) * PA + c];
      SgDft<R2, false, T>::run(b);
#pragma unroll
      for (int kb = 0; kb < R2; kb++)
        buf[(R2 * ka + kb) * PA + c] = cmul(b[kb], tw((n2g * (ka + R1 * kb)) & (M - 1)));
    }
    cluster_arrive();
    cluster_wait();
    // ---- 3. transpose A -> C through registers -----------------------------
    {
      cplx<T> v[G::XE];
#pragma unroll
      for (int it = 0; it < G::XE; it++) {
        const int e = it * NT + tid;           // over (t, q, c) with c fastest
        if (E % NT != 0 && e >= E) break;
        const int c = e % Cs, r = e / Cs, q = r % S, t = r / S;
        const int k1 = row_of<R>(j * Rs + t);
        const int posr = R2 * (k1 % R1) + k1 / R1;
        const cplx<T>* src = cl.map_shared_rank(buf, q);
        v[it] = src[posr * PA + c];
      }
      cluster_arrive();
      cluster_wait();
#pragma unroll
      for (int it = 0; it < G::XE; it++) {
        const int e = it * NT + tid;
        if (E % NT != 0 && e >= E) break;
        const int c = e % Cs, r = e / Cs, q = r % S, t = r / S;
        buf[(q * Cs + c) * PC + t] = v[it];
      }
    }
    __syncthreads();
    // ---- 4. forward row FFTs (length C) -----------------------------------
    for (int u = tid; u < Rs * C2; u += NT) {
      const int t = u % Rs, n2 = u / Rs;
      cplx<T> a[C1];
#pragma unroll
      for (int i = 0; i < C1; i++) a[i] = buf[(C2 * i + n2) * PC + t];
      SgDft<C1, false, T>::run(a);
#pragma unroll
      for (int k = 0; k < C1; k++)
        buf[(C2 * k + n2) * PC + t] = (k == 0 || n2 == 0) ? a[k] : cmul(a[k], tw((n2 * k * R) & (M - 1)));
    }
    __syncthreads();
    for (int u = tid; u < Rs * C1; u += NT) {
      const int t = u % Rs, ka = u / Rs;
      cplx<T> b[C2];
#pragma unroll
      for (int i = 0; i < C2; i++) b[i] = buf[(C2 * ka + i) * PC + t];
      SgDft<C2, false, T>::run(b);
#pragma unroll
      for (int kb = 0; kb < C2; kb++) buf[(C2 * ka + kb) * PC + t] = b[kb];
    }
    __syncthreads();
    // ---- 5. real-spectrum split, multiply by h, re-pack for c2r -----------
    {
      const T* h = p.filt + (long long)det * (M + 1);
      T c2 = T(0);
      for (int e = tid; e < E; e += NT) {
        const int t = e % Rs, pos = e / Rs;
        const int k2 = pos / C2 + C1 * (pos % C2);
        const int k1 = row_of<R>(j * Rs + t);
        const int k = k1 + R * k2;
        if (k == 0) {
          const cplx<T> z = buf[pos * PC + t];
          T h0 = h[0], hM = h[M];
          if (p.filt_abs) {
            h0 = h0 < T(0) ? -h0 : h0;
            hM = hM < T(0) ? -hM : hM;
          }
          const T x0 = z.x + z.y, xM = z.x - z.y;
          c2 += h0 * x0 * x0 + hM * xM * xM;
          const T y0 = h0 * x0, yM = hM * xM;
          buf[pos * PC + t] = cplx<T>{y0 + yM, y0 - yM};
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
        const cplx<T> zk = buf[pos * PC + t];
        const cplx<T> zm = buf[posp * PC + tp];
        T hk = h[k], hm = h[kp];
        if (p.filt_abs) {
          hk = hk < T(0) ? -hk : hk;
          hm = hm < T(0) ? -hm : hm;
        }
        const cplx<T> Ev{T(0.5) * (zk.x + zm.x), T(0.5) * (zk.y - zm.y)};
        const cplx<T> Ov{T(0.5) * (zk.y + zm.y), T(-0.5) * (zk.x - zm.x)};
        cplx<T> wk = tw(k >> 1);
        if (k & 1) wk = cmul(wk, wn1);
        const cplx<T> wO = cmul(wk, Ov);
        const cplx<T> Xk = Ev + wO;
        const cplx<T> Xm = cconj(Ev - wO);
        // bin M/2 pairs with itself: count it once
        c2 += hk * (Xk.x * Xk.x + Xk.y * Xk.y) + (k == kp ? T(0) : hm * (Xm.x * Xm.x + Xm.y * Xm.y));
        const cplx<T> Yk = cscale(Xk, hk), Ym = cscale(Xm, hm);
        const cplx<T> P = Yk + cconj(Ym), Q = Yk - cconj(Ym);
        const cplx<T> cwQ = cmulc(Q, wk);
        const cplx<T> iwQ{-cwQ.y, cwQ.x};
        buf[pos * PC + t] = P + iwQ;
        buf[posp * PC + tp] = cconj(P - iwQ);
      }
      chi2 += (double)c2;
    }
    __syncthreads();
    // ---- 6. inverse row FFTs and the W_M^-1 twiddle ------------------------
    for (int u = tid; u < Rs * C1; u += NT) {
      const int t = u % Rs, a1 = u / Rs;
      cplx<T> b[C2];
#pragma unroll
      for (int i = 0; i < C2; i++) b[i] = buf[(C2 * a1 + i) * PC + t];
      SgDft<C2, true, T>::run(b);
#pragma unroll
      for (int n2 = 0; n2 < C2; n2++)
        buf[(C2 * a1 + n2) * PC + t] = (a1 == 0 || n2 == 0) ? b[n2] : cmulc(b[n2], tw((n2 * a1 * R) & (M - 1)));
    }
    __syncthreads();
    for (int u = tid; u < Rs * C2; u += NT) {
      const int t = u % Rs, n2 = u / Rs;
      const int k1 = row_of<R>(j * Rs + t);
      cplx<T> a[C1];
#pragma unroll
      for (int i = 0; i < C1; i++) a[i] = buf[(C2 * i + n2) * PC + t];
      SgDft<C1, true, T>::run(a);
#pragma unroll
      for (int n1 = 0; n1 < C1; n1++) {
        const int n = C2 * n1 + n2;
        buf[n * PC + t] = cmulc(a[n1], tw((n * k1) & (M - 1)));
      }
    }
    cluster_arrive();
    cluster_wait();
    // ---- 7. transpose C -> A through registers -----------------------------
    {
      cplx<T> v[G::XE];
#pragma unroll
      for (int it = 0; it < G::XE; it++) {
        const int e = it * NT + tid;           // over (q, c, t) with t fastest
        if (E % NT != 0 && e >= E) break;
        const int t = e % Rs, r = e / Rs, c = r % Cs, q = r / Cs;
        const cplx<T>* src = cl.map_shared_rank(buf, q);
        v[it] = src[(j * Cs + c) * PC + t];
      }
      cluster_arrive();
      cluster_wait();
#pragma unroll
      for (int it = 0; it < G::XE; it++) {
        const int e = it * NT + tid;
        if (E % NT != 0 && e >= E) break;
        const int t = e % Rs, r = e / Rs, c = r % Cs, q = r / Cs;
        const int k1 = row_of<R>(q * Rs + t);
        const int posr = R2 * (k1 % R1) + k1 / R1;
        buf[posr * PA + c] = v[it];
      }
    }
    __syncthreads();
    // ---- 8. inverse column FFTs --------------------------------------------
    for (int u = tid; u < Cs * R1; u += NT) {
      const int c = u % Cs, a1 = u / Cs;
      cplx<T> b[R2];
#pragma unroll
      for (int i = 0; i < R2; i++) b[i] = buf[(R2 * a1 + i) * PA + c];
      SgDft<R2, true, T>::run(b);
#pragma unroll
      for (int n2 = 0; n2 < R2; n2++)
        buf[(R2 * a1 + n2) * PA + c] = (a1 == 0 || n2 == 0) ? b[n2] : cmulc(b[n2], tw((n2 * a1 * C) & (M - 1)));
    }
    __syncthreads();
    for (int u = tid; u < Cs * R2; u += NT) {
      const int c = u % Cs, n2 = u / Cs;
      cplx<T> a[R1];
#pragma unroll
      for (int i = 0; i < R1; i++) a[i] = buf[(R2 * i + n2) * PA + c];
      SgDft<R1, true, T>::run(a);
#pragma unroll
      for (int n1 = 0; n1 < R1; n1++) buf[(R2 * n1 + n2) * PA + c] = a[n1];
    }
    __syncthreads();
    // ---- 9. store ------------------------------------------------------------
#pragma unroll 4
    for (int it = 0; it < G::XE; it++) {
      const int e = it * NT + tid;
      if (E % NT != 0 && e >= E) break;
      const int c = e % Cs, n1 = e / Cs;
      const long long s0 = base + 2LL * (C * n1 + j * Cs + c);
      *reinterpret_cast<cplx<T>*>(p.out + s0) = buf[n1 * PA + c];
    }
    __syncthreads();
  }
  if (p.chi2_part) {
    __shared__ double red[kFilterWarps];
    for (int o = 16; o > 0; o >>= 1) chi2 += __shfl_xor_sync(0xffffffffu, chi2, o);
    if ((tid & 31) == 0) red[tid >> 5] = chi2;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < kFilterWarps; w++) s += red[w];
      p.chi2_part[blockIdx.x] = s;
    }
  }
  // peers may still read this CTA's shared memory: keep it alive
  cluster_arrive();
  cluster_wait();
}

// ---------------------------------------------------------------------------
template <typename T, int LOGR, int LOGC, int S>
static size_t smem_bytes() {
  using G = Geo<LOGR, LOGC, S>;
  return sizeof(cplx<T>) * ((size_t)G::BUF + kTwLo + G::M / kTwLo);
}

template <typename T, int LOGR, int LOGC, int S>
static cudaLaunchConfig_t make_cfg(cudaLaunchAttribute* attr, int nclusters, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(S * nclusters);
  cfg.blockDim = dim3(kFilterThreads);
  cfg.dynamicSmemBytes = smem_bytes<T, LOGR, LOGC, S>();
  cfg.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = S;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

template <typename T, int LOGR, int LOGC, int S>
static cudaError_t prepare() {
  auto fn = k_noise_filter<T, LOGR, LOGC, S>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem_bytes<T, LOGR, LOGC, S>());
  if (e == cudaSuccess && S > 8)
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  return e;
}

template <typename T, int LOGR, int LOGC, int S>
static cudaError_t launch_one(const FilterArgs<T>& a, int nclusters, cudaStream_t st) {
  cudaError_t e = prepare<T, LOGR, LOGC, S>();
  if (e != cudaSuccess) return e;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = make_cfg<T, LOGR, LOGC, S>(attr, nclusters, st);
  return cudaLaunchKernelEx(&cfg, k_noise_filter<T, LOGR, LOGC, S>, a);
}

template <typename T, int LOGR, int LOGC, int S>
static int max_clusters_one() {
  if (prepare<T, LOGR, LOGC, S>() != cudaSuccess) return 0;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = make_cfg<T, LOGR, LOGC, S>(attr, 1, nullptr);
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_noise_filter<T, LOGR, LOGC, S>, &cfg) != cudaSuccess)
    return 0;
  return n;
}

// (LOGR, LOGC, S) per log2(M) and precision; S keeps the per-CTA share at
// 8192 (FP32) or 4096 (FP64) complex points.
#define SG_FILTER_CASES_F32(X)                                                               \
  X(float, 4, 3, 1) X(float, 4, 4, 1) X(float, 5, 4, 1) X(float, 5, 5, 1) X(float, 6, 5, 1)  \
  X(float, 6, 6, 1) X(float, 7, 6, 1) X(float, 7, 7, 2) X(float, 8, 7, 4) X(float, 8, 8, 8)
#define SG_FILTER_CASES_F64(X)                                                                 \
  X(double, 4, 3, 1) X(double, 4, 4, 1) X(double, 5, 4, 1) X(double, 5, 5, 1)                  \
  X(double, 6, 5, 1) X(double, 6, 6, 1) X(double, 7, 6, 2) X(double, 7, 7, 4)                 \
  X(double, 8, 7, 8) X(double, 8, 8, 16)

size_t filter_smem_bytes(int logm, int S, int esize) {
  const int logr = (logm + 1) / 2, logc = logm / 2;
  const size_t R = 1u << logr, C = 1u << logc, M = R * C;
  const size_t buf = std::max(R * (C / S + 1), C * (R / S + 1));
  return (size_t)esize * 2 * (buf + kTwLo + M / kTwLo);
}

int filter_cluster_size(int logm, int esize) {
  const long M = 1L << logm;
  const long emax = esize == 4 ? 8192 : 4096;
  return (int)(M / emax > 1 ? M / emax : 1);
}

template <>
cudaError_t filter_launch<float>(const FilterArgs<float>& a, int logm, int S, int nclusters,
                                 cudaStream_t st) {
  const int logr = (logm + 1) / 2, logc = logm / 2;
#define SG_CASE(TT, LR, LC, SS) \
  if (logr == LR && logc == LC && S == SS) return launch_one<TT, LR, LC, SS>(a, nclusters, st);
  SG_FILTER_CASES_F32(SG_CASE)
#undef SG_CASE
  return cudaErrorInvalidValue;
}

template <>
cudaError_t filter_launch<double>(const FilterArgs<double>& a, int logm, int S, int nclusters,
                                  cudaStream_t st) {
  const int logr = (logm + 1) / 2, logc = logm / 2;
#define SG_CASE(TT, LR, LC, SS) \
  if (logr == LR && logc == LC && S == SS) return launch_one<TT, LR, LC, SS>(a, nclusters, st);
  SG_FILTER_CASES_F64(SG_CASE)
#undef SG_CASE
  return cudaErrorInvalidValue;
}

template <>
int filter_max_clusters<float>(int logm, int S) {
  const int logr = (logm + 1) / 2, logc = logm / 2;
#define SG_CASE(TT, LR, LC, SS) \
  if (logr == LR && logc == LC && S == SS) return max_clusters_one<TT, LR, LC, SS>();
  SG_FILTER_CASES_F32(SG_CASE)
#undef SG_CASE
  return 0;
}

template <>
int filter_max_clusters<double>(int logm, int S) {
  const int logr = (logm + 1) / 2, logc = logm / 2;
#define SG_CASE(TT, LR, LC, SS) \
  if (logr == LR && logc == LC && S == SS) return max_clusters_one<TT, LR, LC, SS>();
  SG_FILTER_CASES_F64(SG_CASE)
#undef SG_CASE
  return 0;
}

}  // namespace sg
