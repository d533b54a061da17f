#pragma once
// sg_filter.cuh -- per-(detector, segment) noise weighting N^-1 as one fused
// GB300 kernel: load (a timeline, or a timeline minus another) -> real FFT ->
// multiply by the inverse-noise spectrum -> inverse real FFT -> store,
// optionally accumulating chi^2 of the input.  Two more variants split it at
// the spectrum (forward FFT to the half spectrum X[k], k = 0..M; inverse FFT
// from such a spectrum), for weightings that mix several timelines per
// frequency (the offset-group operator, sg_group.cu).  Spectra are stored in
// the order the kernel's units hold them (slot
// ((i C1 + ka) S + j) Rs + t for element i of unit (row t of CTA j, column
// ka); row 0's slots equal their frequencies; slot M holds the Nyquist bin),
// so loads and stores are coalesced; spec_slot_freq() gives each slot's k.
//
// Replaces the reference's write_tfAS + the first half of do_PtNd
// (sanepic.cc:2390-2445, 2522-2582): per tile of ns samples it computes
//   y = c2r( h . r2c(x) ),   h[k] = SpN_all[k] (k <= ns/2, sanepic.cc:533-537)
// with FFTW's unnormalised conventions (r2c sign -1, c2r sign +1), and the
// chi^2 terms sum_k h[k] |r2c(x)[k]|^2 of sanepic.cc:1089-1110, 1528-1546.
//
// Algorithm.  The real tile x (N = ns samples) is packed as M = N/2 complex
// points z[m] = x[2m] + i x[2m+1].  The length-M complex FFT is a four-step
// FFT, M = R x C: column FFTs of length R, a W_M twiddle, row FFTs of length
// C.  A tile is spread over a thread-block cluster of S CTAs (one tile at a
// time per cluster): CTA j owns columns [j C/S, (j+1) C/S) for the column
// pass and a set of R/S rows for the row pass; the transposes between the
// passes go through distributed shared memory (no HBM round trip, no TMA
// multicast).  Rows are dealt out in pairs (k1, R-k1) so that every
// frequency k and its real-FFT partner M-k live in the same CTA.
//
// Each sub-FFT (length R or C) is two in-register radix passes (sizes
// 2..16) through shared memory; the forward sub-FFT leaves its output
// digit-reversed and the inverse consumes it that way.  Every pass works on
// "units" (one small DFT each) with the batch index fastest across lanes, so
// the shared-memory accesses are conflict-free, and in FP32 a thread carries
// two units at once for instruction-level parallelism.  256 threads per CTA
// with up to 128 registers each: two CTAs of different clusters share an SM,
// so one cluster's barrier waits overlap the other's arithmetic.
//
// The last forward row pass, the real-spectrum split, the multiply by h, the
// re-packing for the inverse and the first inverse row pass are one register
// phase: the unit holding frequencies k and the unit holding M-k sit in
// lanes l and l^17 of one warp (l^16 for row R/2) and swap their values with
// shuffles.  Only row 0, whose partners are in the same row, goes through
// shared memory.  The inverse-from-spectrum variant first stages its CTA's
// spectrum slots in shared memory where the units keep them (one coalesced
// pass), then exchanges partners the same way.
//
// Twiddles: the inner ones (W_R, W_C) come from per-length shared tables,
// the four-step ones (W_M) from two shared tables (W_M^j = W_M^{64 jh} W_M^{jl})
// built in FP64 on the host, the real-FFT split twiddle W_N^k from one table
// value per unit times a per-digit table.
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

constexpr int kFilterThreads = 256;
// kernel variants: the fused filter, forward FFT to a half spectrum, inverse
// FFT from a half spectrum
constexpr int kFused = 0, kSpecOut = 1, kSpecIn = 2;
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

// 32-bit shared-window addresses of a peer CTA's shared memory (mapa), and
// loads through them: keeps the transposes' addresses in one register each.
__device__ __forceinline__ uint32_t cluster_map(const void* local, int rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n"
               : "=r"(r)
               : "r"((uint32_t)__cvta_generic_to_shared(local)), "r"(rank));
  return r;
}
__device__ __forceinline__ cplx<float> ld_cluster(uint32_t addr, cplx<float>*) {
  cplx<float> v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];\n" : "=f"(v.x), "=f"(v.y) : "r"(addr));
  return v;
}
__device__ __forceinline__ cplx<double> ld_cluster(uint32_t addr, cplx<double>*) {
  cplx<double> v;
  asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];\n" : "=d"(v.x), "=d"(v.y) : "r"(addr));
  return v;
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
  // column-pass (A) layout: element (row, column) at row PA + row / 16 +
  // column.  The extra element per 16 rows spreads the transpose back from the
  // row passes, whose lanes write rows k1 -> R2 (k1 % R1) + k1 / R1 (16 apart
  // for consecutive k1), over all bank pairs.
  static __device__ __forceinline__ int pa(int row, int c) { return row * PA + (row >> 4) + c; }
  static constexpr int ABUF = R * PA + R / 16;
  static constexpr int BUF = (ABUF > C * PC) ? ABUF : C * PC;
  static constexpr int XE = (E + kFilterThreads - 1) / kFilterThreads;  // per thread
  // shared twiddle tables: lo, hi, W_R, W_C, W_N^{R C1 i} (i < C2)
  static constexpr int TWN = kTwLo + M / kTwLo + R + C + C2;
  static_assert(Rs >= 16 && Rs % 16 == 0, "the fused spectrum phase needs 16-row blocks");
  static_assert(C1 >= 2 && (Rs * C1) % 32 == 0, "fused phase: whole warps of units");
  static_assert(Cs >= 1, "tile too small");
};

// Runs U units through load -> DFT<P> -> store; with PAIR a thread carries
// two units at once (independent instruction streams for latency hiding).
template <typename T, int P, bool INV, int U, bool PAIR, class Ld, class St>
__device__ __forceinline__ void run_pass(int tid, Ld ld, St st) {
  constexpr int NT = kFilterThreads;
  if constexpr (PAIR) {
    for (int u0 = tid; u0 < U; u0 += 2 * NT) {
      const int u1 = u0 + NT;
      const bool two = (U % (2 * NT) == 0) || u1 < U;
      cplx<T> a[P], b[P];
      ld(u0, a);
      if (two) ld(u1, b);
      SgDft<P, INV, T>::run(a);
      if (two) SgDft<P, INV, T>::run(b);
      st(u0, a);
      if (two) st(u1, b);
    }
  } else {
    for (int u = tid; u < U; u += NT) {
      cplx<T> a[P];
      ld(u, a);
      SgDft<P, INV, T>::run(a);
      st(u, a);
    }
  }
}

template <typename T>
__device__ __forceinline__ T shfl(T v, int src) {
  return __shfl_sync(0xffffffffu, v, src);
}

// The packed spectrum value at the slot of `own` (k if own_is_k, else M-k)
// for the inverse real FFT of the half spectrum with values Yk at k and Ym at
// M-k (k < M-k, wk = W_N^k).
template <typename T>
__device__ __forceinline__ cplx<T> repack(cplx<T> Yk, cplx<T> Ym, cplx<T> wk, bool own_is_k) {
  const cplx<T> P = Yk + cconj(Ym), Q = Yk - cconj(Ym);
  const cplx<T> cwQ = cmulc(Q, wk);
  const cplx<T> iwQ{-cwQ.y, cwQ.x};
  return own_is_k ? P + iwQ : cconj(P - iwQ);
}

// One real-FFT frequency pair (k, M-k) of the packed spectrum z: split into
// the r2c values X[k], X[M-k], multiply by h, re-pack for the inverse.
// Returns the re-packed value at the slot of `own` (k if own_is_k, else M-k)
// and the r2c value X at that slot (for chi^2).  wk = W_N^k, k < M-k.
template <typename T>
__device__ __forceinline__ cplx<T> split_filter(cplx<T> zk, cplx<T> zm, T hk, T hm, cplx<T> wk,
                                                bool own_is_k, cplx<T>& xown) {
  const cplx<T> Ev{T(0.5) * (zk.x + zm.x), T(0.5) * (zk.y - zm.y)};
  const cplx<T> Ov{T(0.5) * (zk.y + zm.y), T(-0.5) * (zk.x - zm.x)};
  const cplx<T> wO = cmul(wk, Ov);
  const cplx<T> Xk = Ev + wO;
  const cplx<T> Xm = cconj(Ev - wO);
  xown = own_is_k ? Xk : Xm;
  return repack(cscale(Xk, hk), cscale(Xm, hm), wk, own_is_k);
}

template <typename T, int LOGR, int LOGC, int S, int MODE>
__global__ void __launch_bounds__(kFilterThreads, sizeof(T) == 4 ? 2 : 1)
    k_noise_filter(FilterArgs<T> p) {
  using G = Geo<LOGR, LOGC, S>;
  constexpr int R = G::R, C = G::C, M = G::M, R1 = G::R1, R2 = G::R2, C1 = G::C1, C2 = G::C2;
  constexpr int Cs = G::Cs, Rs = G::Rs, PC = G::PC, E = G::E;
  constexpr int NT = kFilterThreads;
  constexpr bool PAIR = sizeof(T) == 4;
  cg::cluster_group cl = cg::this_cluster();
  const int j = (int)cl.block_rank();
  const int tid = threadIdx.x;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* buf = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* twlo = buf + G::BUF;
  cplx<T>* twhi = twlo + kTwLo;
  cplx<T>* twr = twhi + M / kTwLo;  // W_R^i, i < R
  cplx<T>* twc = twr + R;           // W_C^i, i < C
  cplx<T>* twd = twc + C;           // W_N^{R C1 i}, i < C2
  for (int i = tid; i < kTwLo; i += NT) twlo[i] = p.tw_lo[i];
  for (int i = tid; i < M / kTwLo; i += NT) twhi[i] = p.tw_hi[i];
  __syncthreads();
  const Tw<T> tw{twlo, twhi};
  for (int i = tid; i < R; i += NT) twr[i] = tw((i * C) & (M - 1));
  for (int i = tid; i < C; i += NT) twc[i] = tw((i * R) & (M - 1));
  for (int i = tid; i < C2; i += NT) twd[i] = tw(((R * C1 / 2) * i) & (M - 1));
  __syncthreads();
  const cplx<T> wn1 = p.wn1;

  const int cluster_id = blockIdx.x / S;
  const int nclusters = gridDim.x / S;
  // 16-byte global accesses: FP32, even column count per CTA, whole pairs per
  // thread, and every timeline pointer 16-byte aligned (callers may pass
  // offset pointers; then the 8-byte path runs)
  const bool kVec = sizeof(T) == 4 && Cs % 2 == 0 && (E / 2) % NT == 0 &&
                    ((reinterpret_cast<uintptr_t>(p.tod) | reinterpret_cast<uintptr_t>(p.sub) |
                      reinterpret_cast<uintptr_t>(p.out)) & 15) == 0;
  double chi2 = 0.0;  // sum of h[k] |X[k]|^2 over this thread's bins
  for (long long L = cluster_id; L < p.ntiles; L += nclusters) {
    // the inverse into P^T's layout visits the three components of a group
    // segment side by side (L = (group * nseg + segment) * 3 + component), so
    // that their stores into the same 96-byte blocks meet in L2
    long long tile = L;
    if (MODE != kSpecOut && p.ilv3) {
      const long long q = L % (3LL * p.nseg);
      tile = (L - q) + (q % 3) * p.nseg + q / 3;
    }
    const long long base = tile * (long long)(2 * M);
    const int det = (int)(tile / p.nseg);
    const T* h = p.filt + (long long)det * (M + 1);
    // spectrum modes: spec_out stops after the forward FFT with the half
    // spectrum X[k], k = 0..M, in natural order; spec_in starts from such a
    // spectrum (already weighted) and runs the inverse FFT only
    const cplx<T>* Yin = MODE == kSpecIn ? p.spec_in + tile * (long long)(M + 1) : nullptr;
    cplx<T>* Xout = MODE == kSpecOut ? p.spec_out + tile * (long long)(M + 1) : nullptr;
    if constexpr (MODE != kSpecIn) {
    // ---- 1. load: z[C n1 + n2] = x[2n] + i x[2n+1], this CTA's columns ----
    // FP32 timelines on 16-byte aligned buffers: two columns per 16-byte load
    if (kVec && (p.mode == kLoadTod || p.mode == kLoadTodMinus)) {
#pragma unroll 8
      for (int it = 0; it < E / 2 / NT; it++) {
        const int e2 = it * NT + tid;
        const int c = 2 * (e2 % (Cs / 2)), n1 = e2 / (Cs / 2);
        const long long s0 = base + 2LL * (C * n1 + j * Cs + c);
        float4 v = *reinterpret_cast<const float4*>(p.tod + s0);
        if (p.mode == kLoadTodMinus) {
          const float4 w = *reinterpret_cast<const float4*>(p.sub + s0);
          v.x -= w.x;
          v.y -= w.y;
          v.z -= w.z;
          v.w -= w.w;
        }
        buf[G::pa(n1, c)] = cplx<T>{(T)v.x, (T)v.y};
        buf[G::pa(n1, c + 1)] = cplx<T>{(T)v.z, (T)v.w};
      }
    } else
#pragma unroll 16
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
      } else {  // unit impulse at sample 0 of the tile
        v.x = (s0 == base) ? T(1) : T(0);
        v.y = T(0);
      }
      buf[G::pa(n1, c)] = v;
    }
    __syncthreads();
    // ---- 2. forward column pass 1: DFT_R1 over n1, twiddle W_R^{n2 k} ------
    run_pass<T, R1, false, Cs * R2, PAIR>(
        tid,
        [&](int u, auto& a) {
          const int c = u % Cs, n2 = u / Cs;
#pragma unroll
          for (int i = 0; i < R1; i++) a[i] = buf[G::pa(R2 * i + n2, c)];
        },
        [&](int u, auto& a) {
          const int c = u % Cs, n2 = u / Cs;
#pragma unroll
          for (int k = 0; k < R1; k++)
            buf[G::pa(R2 * k + n2, c)] =
                (k == 0 || n2 == 0) ? a[k] : cmul(a[k], twr[(n2 * k) & (R - 1)]);
        });
    __syncthreads();
    // ---- 3. forward column pass 2: DFT_R2, four-step twiddle W_M ------------
    run_pass<T, R2, false, Cs * R1, PAIR>(
        tid,
        [&](int u, auto& b) {
          const int c = u % Cs, ka = u / Cs;
#pragma unroll
          for (int i = 0; i < R2; i++) b[i] = buf[G::pa(R2 * ka + i, c)];
        },
        [&](int u, auto& b) {
          const int c = u % Cs, ka = u / Cs;
          const int n2g = j * Cs + c;
#pragma unroll
          for (int kb = 0; kb < R2; kb++)
            buf[G::pa(R2 * ka + kb, c)] = cmul(b[kb], tw((n2g * (ka + R1 * kb)) & (M - 1)));
        });
    cluster_arrive();
    cluster_wait();
    // ---- 4. transpose A -> C through registers -----------------------------
    {
      cplx<T> v[G::XE];
#pragma unroll
      for (int it = 0; it < G::XE; it++) {
        const int e = it * NT + tid;  // over (t, q, c) with c fastest
        if (E % NT != 0 && e >= E) break;
        const int c = e % Cs, r = e / Cs, q = r % S, t = r / S;
        const int k1 = row_of<R>(j * Rs + t);
        const int posr = R2 * (k1 % R1) + k1 / R1;
        v[it] = ld_cluster(cluster_map(buf + G::pa(posr, c), q), (cplx<T>*)nullptr);
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
    // ---- 5. forward row pass 1: DFT_C1 over n1, twiddle W_C^{n2 k} ---------
    run_pass<T, C1, false, Rs * C2, PAIR>(
        tid,
        [&](int u, auto& a) {
          const int t = u % Rs, n2 = u / Rs;
#pragma unroll
          for (int i = 0; i < C1; i++) a[i] = buf[(C2 * i + n2) * PC + t];
        },
        [&](int u, auto& a) {
          const int t = u % Rs, n2 = u / Rs;
#pragma unroll
          for (int k = 0; k < C1; k++)
            buf[(C2 * k + n2) * PC + t] =
                (k == 0 || n2 == 0) ? a[k] : cmul(a[k], twc[(n2 * k) & (C - 1)]);
        });
    __syncthreads();
    }  // MODE != kSpecIn
    if constexpr (MODE == kSpecIn) {
      // stage this CTA's spectrum slots, coalesced: slot ((i C1 + ka) S + j)
      // Rs + t (a run of Rs per (i, ka)) goes where unit (t, ka) keeps its
      // element i, (C2 ka + i) PC + t
#pragma unroll 16
      for (int it = 0; it < G::XE; it++) {
        const int e = it * NT + tid;
        if (E % NT != 0 && e >= E) break;
        const int t = e % Rs, r = e / Rs;  // r = i C1 + ka
        buf[(C2 * (r % C1) + r / C1) * PC + t] = Yin[((long long)r * S + j) * Rs + t];
      }
      __syncthreads();
    }
    // ---- 6. forward row pass 2 + spectrum + inverse row pass 1, in registers --
    // unit (t, ka): lanes l < 16 take ka = q, lanes l >= 16 take C1-1-q, so
    // the partner unit (t^1, C1-1-ka) is lane l^17 (row R/2: (t, C1-1-ka),
    // lane l^16); its element C2-1-i holds frequency M - k_i.
    {
      T c2 = T(0);
      constexpr int TB = Rs / 16;
      for (int u = tid; u < Rs * C1; u += NT) {
        const int l = u & 31, g = u >> 5;
        const int t = 16 * (g % TB) + (l & 15);
        const int q = g / TB;
        const int ka = (l < 16) ? q : C1 - 1 - q;
        const int k1 = row_of<R>(j * Rs + t);
        if constexpr (MODE == kSpecIn) {
          // re-pack the staged spectrum: own slots from shared memory, the
          // partner's (frequencies M - k) by lane exchange
          cplx<T> y[C2];
#pragma unroll
          for (int i = 0; i < C2; i++) y[i] = buf[(C2 * ka + i) * PC + t];
          const int src = (j == 0 && t == 1) ? (l ^ 16) : (l ^ 17);
          const int kb0 = k1 + R * ka;
          cplx<T> wb = tw(kb0 >> 1);
          if (kb0 & 1) wb = cmul(wb, wn1);
          cplx<T> zo[C2];
#pragma unroll
          for (int i = 0; i < C2; i++) {
            const cplx<T> yp{shfl(y[C2 - 1 - i].x, src), shfl(y[C2 - 1 - i].y, src)};
            const int k = kb0 + R * C1 * i;
            const bool lo = k <= M - k;
            const cplx<T> wk = cmul(wb, twd[i]);
            const cplx<T> ws = lo ? wk : cplx<T>{-wk.x, wk.y};
            zo[i] = repack(lo ? y[i] : yp, lo ? yp : y[i], ws, lo);
          }
          if (j == 0 && t == 0) continue;  // row 0: below (its lanes only lent values)
          SgDft<C2, true, T>::run(zo);
#pragma unroll
          for (int n2 = 0; n2 < C2; n2++)
            buf[(C2 * ka + n2) * PC + t] =
                (ka == 0 || n2 == 0) ? zo[n2] : cmulc(zo[n2], twc[(n2 * ka) & (C - 1)]);
          continue;
        }
        cplx<T> z[C2];
#pragma unroll
        for (int i = 0; i < C2; i++) z[i] = buf[(C2 * ka + i) * PC + t];
        SgDft<C2, false, T>::run(z);
        const bool row0 = (j == 0 && t == 0);
        const int src = (j == 0 && t == 1) ? (l ^ 16) : (l ^ 17);
        const int kb0 = k1 + R * ka;  // k_i = kb0 + R C1 i
        T hk[C2];
#pragma unroll
        for (int i = 0; i < C2; i++) hk[i] = MODE == kSpecOut ? T(0) : h[kb0 + R * C1 * i];
        cplx<T> wb = tw(kb0 >> 1);
        if (kb0 & 1) wb = cmul(wb, wn1);  // W_N^{kb0}
        cplx<T> zo[C2];
#pragma unroll
        for (int i = 0; i < C2; i++) {
          const cplx<T> zp{shfl(z[C2 - 1 - i].x, src), shfl(z[C2 - 1 - i].y, src)};
          const T hp = shfl(hk[C2 - 1 - i], src);
          const int k = kb0 + R * C1 * i;
          const bool lo = k <= M - k;  // this unit holds the smaller frequency
          const cplx<T> wk = cmul(wb, twd[i]);          // W_N^k
          const cplx<T> ws = lo ? wk : cplx<T>{-wk.x, wk.y};  // W_N^{M-k} = -conj(W_N^k)
          cplx<T> x;
          zo[i] = split_filter(lo ? z[i] : zp, lo ? zp : z[i], lo ? hk[i] : hp, lo ? hp : hk[i],
                               ws, lo, x);
          if (!row0) c2 += hk[i] * (x.x * x.x + x.y * x.y);
          // X[k] at this unit's own frequency, stored in unit order (lanes write
          // consecutive slots); row 0's slots are its frequencies themselves
          if (MODE == kSpecOut && !row0) Xout[((i * C1 + ka) * S + j) * Rs + t] = x;
        }
        if constexpr (MODE == kSpecOut) {
          if (row0) {
#pragma unroll
            for (int i = 0; i < C2; i++) buf[(C2 * ka + i) * PC + t] = z[i];
          }
        } else if (!row0) {
          SgDft<C2, true, T>::run(zo);
#pragma unroll
          for (int n2 = 0; n2 < C2; n2++)
            buf[(C2 * ka + n2) * PC + t] =
                (ka == 0 || n2 == 0) ? zo[n2] : cmulc(zo[n2], twc[(n2 * ka) & (C - 1)]);
        } else {
#pragma unroll
          for (int i = 0; i < C2; i++) buf[(C2 * ka + i) * PC + t] = z[i];
        }
      }
      // row 0's lanes paired with row R/2 above and kept only their forward
      // values; row 0 is finished here through shared memory
      __syncthreads();
      if (j == 0) {
        // row 0 (k1 = 0, t = 0): partners k2 <-> C - k2 within the row
        T c0 = T(0);
        for (int pos = tid; pos < C; pos += NT) {
          const int k2 = pos / C2 + C1 * (pos % C2);
          if (k2 == 0) {  // bins 0 and M
            if constexpr (MODE == kSpecIn) {
              const T y0 = Yin[0].x, yM = Yin[M].x;
              buf[0] = cplx<T>{y0 + yM, y0 - yM};
              continue;
            }
            const cplx<T> zz = buf[0];
            const T x0 = zz.x + zz.y, xM = zz.x - zz.y;
            if constexpr (MODE == kSpecOut) {
              Xout[0] = cplx<T>{x0, T(0)};
              Xout[M] = cplx<T>{xM, T(0)};
              continue;
            }
            const T h0 = h[0], hM = h[M];
            c0 += h0 * x0 * x0 + hM * xM * xM;
            const T y0 = h0 * x0, yM = hM * xM;
            buf[0] = cplx<T>{y0 + yM, y0 - yM};
            continue;
          }
          const int k2p = C - k2;
          if (k2 > k2p) continue;
          const int posp = C2 * (k2p % C1) + k2p / C1;
          const int k = R * k2;
          const cplx<T> wk = tw(k >> 1);  // R even: k even
          if constexpr (MODE == kSpecIn) {
            const cplx<T> yk = Yin[k], ym = Yin[M - k];
            buf[pos * PC] = repack(yk, ym, wk, true);
            buf[posp * PC] = repack(yk, ym, wk, false);
            continue;
          }
          const cplx<T> zk = buf[pos * PC], zm = buf[posp * PC];
          cplx<T> xk, xm;
          if constexpr (MODE == kSpecOut) {
            split_filter(zk, zm, T(0), T(0), wk, true, xk);
            split_filter(zk, zm, T(0), T(0), wk, false, xm);
            Xout[k] = xk;
            Xout[M - k] = xm;
            continue;
          }
          const T hk0 = h[k], hm0 = h[M - k];
          const cplx<T> ok = split_filter(zk, zm, hk0, hm0, wk, true, xk);
          const cplx<T> om = split_filter(zk, zm, hk0, hm0, wk, false, xm);
          c0 += hk0 * (xk.x * xk.x + xk.y * xk.y) +
                (k2 == k2p ? T(0) : hm0 * (xm.x * xm.x + xm.y * xm.y));
          buf[pos * PC] = ok;
          buf[posp * PC] = om;
        }
        chi2 += (double)c0;
        __syncthreads();
        if (MODE != kSpecOut)
        for (int a1 = tid; a1 < C1; a1 += NT) {  // inverse row pass 1 of row 0
          cplx<T> b[C2];
#pragma unroll
          for (int i = 0; i < C2; i++) b[i] = buf[(C2 * a1 + i) * PC];
          SgDft<C2, true, T>::run(b);
#pragma unroll
          for (int n2 = 0; n2 < C2; n2++)
            buf[(C2 * a1 + n2) * PC] =
                (a1 == 0 || n2 == 0) ? b[n2] : cmulc(b[n2], twc[(n2 * a1) & (C - 1)]);
        }
        __syncthreads();
      }
      chi2 += (double)c2;
    }
    if constexpr (MODE == kSpecOut) {  // forward only: the spectrum is out, next tile
      __syncthreads();
      continue;
    }
    // ---- 7. inverse row pass 2: DFT_C1, conj four-step twiddle W_M^{n k1} ---
    run_pass<T, C1, true, Rs * C2, PAIR>(
        tid,
        [&](int u, auto& a) {
          const int t = u % Rs, n2 = u / Rs;
#pragma unroll
          for (int i = 0; i < C1; i++) a[i] = buf[(C2 * i + n2) * PC + t];
        },
        [&](int u, auto& a) {
          const int t = u % Rs, n2 = u / Rs;
          const int k1 = row_of<R>(j * Rs + t);
#pragma unroll
          for (int n1 = 0; n1 < C1; n1++) {
            const int n = C2 * n1 + n2;
            buf[n * PC + t] = cmulc(a[n1], tw((n * k1) & (M - 1)));
          }
        });
    cluster_arrive();
    cluster_wait();
    // ---- 8. transpose C -> A through registers -----------------------------
    {
      cplx<T> v[G::XE];
#pragma unroll
      for (int it = 0; it < G::XE; it++) {
        const int e = it * NT + tid;  // over (q, c, t) with t fastest
        if (E % NT != 0 && e >= E) break;
        const int t = e % Rs, r = e / Rs, c = r % Cs, q = r / Cs;
        v[it] = ld_cluster(cluster_map(buf + (j * Cs + c) * PC + t, q), (cplx<T>*)nullptr);
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
        buf[G::pa(posr, c)] = v[it];
      }
    }
    __syncthreads();
    // ---- 9. inverse column pass 1: DFT_R2, conj twiddle W_R^{n2 a1} --------
    run_pass<T, R2, true, Cs * R1, PAIR>(
        tid,
        [&](int u, auto& b) {
          const int c = u % Cs, a1 = u / Cs;
#pragma unroll
          for (int i = 0; i < R2; i++) b[i] = buf[G::pa(R2 * a1 + i, c)];
        },
        [&](int u, auto& b) {
          const int c = u % Cs, a1 = u / Cs;
#pragma unroll
          for (int n2 = 0; n2 < R2; n2++)
            buf[G::pa(R2 * a1 + n2, c)] =
                (a1 == 0 || n2 == 0) ? b[n2] : cmulc(b[n2], twr[(n2 * a1) & (R - 1)]);
        });
    __syncthreads();
    // ---- 10. inverse column pass 2: DFT_R1 ----------------------------------
    run_pass<T, R1, true, Cs * R2, PAIR>(
        tid,
        [&](int u, auto& a) {
          const int c = u % Cs, n2 = u / Cs;
#pragma unroll
          for (int i = 0; i < R1; i++) a[i] = buf[G::pa(R2 * i + n2, c)];
        },
        [&](int u, auto& a) {
          const int c = u % Cs, n2 = u / Cs;
#pragma unroll
          for (int n1 = 0; n1 < R1; n1++) buf[G::pa(R2 * n1 + n2, c)] = a[n1];
        });
    __syncthreads();
    // ---- 11. store -------------------------------------------------------------
    if (MODE != kSpecOut && p.ilv3) {
      // component (tile / nseg) % 3 of the [group sample / 8][3][8] layout P^T
      // reads, tile = (group * 3 + component) * nseg + segment: a sample pair
      // is 8 contiguous bytes (FP32), four lanes fill one 32-byte sector
      const long long nst = p.nseg;
      const long long grp = tile / (3 * nst), comp = (tile / nst) % 3, seg = tile % nst;
      T* dst = p.out + 3 * (grp * nst + seg) * (2LL * M) + 8 * comp;
#pragma unroll 16
      for (int it = 0; it < G::XE; it++) {
        const int e = it * NT + tid;
        if (E % NT != 0 && e >= E) break;
        const int c = e % Cs, n1 = e / Cs;
        const long long n = 2LL * (C * n1 + j * Cs + c);  // even: the pair stays in its block
        *reinterpret_cast<cplx<T>*>(dst + 24 * (n >> 3) + (n & 7)) = buf[G::pa(n1, c)];
      }
    } else if (kVec) {
#pragma unroll 8
      for (int it = 0; it < E / 2 / NT; it++) {
        const int e2 = it * NT + tid;
        const int c = 2 * (e2 % (Cs / 2)), n1 = e2 / (Cs / 2);
        const long long s0 = base + 2LL * (C * n1 + j * Cs + c);
        const cplx<T> a = buf[G::pa(n1, c)], b = buf[G::pa(n1, c + 1)];
        *reinterpret_cast<float4*>(p.out + s0) = make_float4((float)a.x, (float)a.y, (float)b.x, (float)b.y);
      }
    } else
#pragma unroll 16
    for (int it = 0; it < G::XE; it++) {
      const int e = it * NT + tid;
      if (E % NT != 0 && e >= E) break;
      const int c = e % Cs, n1 = e / Cs;
      const long long s0 = base + 2LL * (C * n1 + j * Cs + c);
      *reinterpret_cast<cplx<T>*>(p.out + s0) = buf[G::pa(n1, c)];
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
  return sizeof(cplx<T>) * ((size_t)G::BUF + G::TWN);
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

template <typename T, int LOGR, int LOGC, int S, int MODE>
static cudaError_t prepare() {
  auto fn = k_noise_filter<T, LOGR, LOGC, S, MODE>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem_bytes<T, LOGR, LOGC, S>());
  if (e == cudaSuccess && S > 8)
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  return e;
}

template <typename T, int LOGR, int LOGC, int S, int MODE>
static cudaError_t launch_one(const FilterArgs<T>& a, int nclusters, cudaStream_t st) {
  cudaError_t e = prepare<T, LOGR, LOGC, S, MODE>();
  if (e != cudaSuccess) return e;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = make_cfg<T, LOGR, LOGC, S>(attr, nclusters, st);
  return cudaLaunchKernelEx(&cfg, k_noise_filter<T, LOGR, LOGC, S, MODE>, a);
}

template <typename T, int LOGR, int LOGC, int S, int MODE>
static int max_clusters_one() {
  if (prepare<T, LOGR, LOGC, S, MODE>() != cudaSuccess) return 0;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = make_cfg<T, LOGR, LOGC, S>(attr, 1, nullptr);
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_noise_filter<T, LOGR, LOGC, S, MODE>, &cfg) !=
      cudaSuccess)
    return 0;
  return n;
}

// (LOGR, LOGC, S) per log2(M) and precision; S keeps the per-CTA share at
// 8192 (FP32) or 4096 (FP64) complex points.  For FP32 tiles of 2^14..2^17
// samples a second shape with 4096 points per CTA (twice the cluster) is
// compiled too; sg_autotune times both on the context's data.
#define SG_FILTER_CASES_F32(X)                                                               \
  X(float, 4, 3, 1) X(float, 4, 4, 1) X(float, 5, 4, 1) X(float, 5, 5, 1) X(float, 6, 5, 1)  \
  X(float, 6, 6, 1) X(float, 7, 6, 1) X(float, 7, 7, 2) X(float, 8, 7, 4) X(float, 8, 8, 8)  \
  X(float, 7, 6, 2) X(float, 7, 7, 4) X(float, 8, 7, 8) X(float, 8, 8, 16)
#define SG_FILTER_CASES_F64(X)                                                                 \
  X(double, 4, 3, 1) X(double, 4, 4, 1) X(double, 5, 4, 1) X(double, 5, 5, 1)                  \
  X(double, 6, 5, 1) X(double, 6, 6, 1) X(double, 7, 6, 2) X(double, 7, 7, 4)                 \
  X(double, 8, 7, 8) X(double, 8, 8, 16)

}  // namespace sg
