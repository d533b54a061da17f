// sg_fft3.cu -- the offset-group noise weighting (S0, S1, S2)^ = H[k] (a, b1, b2)^
// in FP32 as three in-place passes over the group timelines, each a plain
// grid of independent CTAs (no cluster, no distributed shared memory).
//
// The group timelines live in P^T's interleaved layout: per (group, segment)
// tile of ns = 2M samples and three components, sample i of component c at
// float offset 24 (i / 8) + 8 c + i % 8.  A sample pair (2m, 2m+1) of one
// component is the packed complex point z_c[m] = x_c[2m] + i x_c[2m+1] at
// float offset 24 (m / 4) + 8 c + 2 (m % 4), so the packed complex array and
// the real timelines share the same bytes and every pass can work in place.
//
// The length-M complex FFT is the four-step FFT M = R x C with m = C n1 + n2:
//   pass 1 (columns):  Y[k1][n2] = W_M^{n2 k1} sum_n1 z[C n1 + n2] W_R^{n1 k1},
//                      stored at m = C k1 + n2;
//   pass 2 (rows):     Z[k1 + R k2] = sum_n2 Y[k1][n2] W_C^{n2 k2}; the real
//                      spectrum split of the pair (k, M-k), the 3 x 3 mixing
//                      by H (or a scaling by h), the re-packing for the
//                      inverse, and the inverse row DFT
//                      U[k1][n2] = sum_k2 Z'[k1 + R k2] W_C^{-n2 k2};
//   pass 3 (columns):  z'[C n1 + n2] = sum_k1 W_R^{-n1 k1} W_M^{-n2 k1} U[k1][n2],
//                      whose real and imaginary parts are the output samples.
// A frequency k = k1 + R k2 (k1 > 0) has its real-FFT partner M - k =
// (R - k1) + R (C - 1 - k2), so pass 2 takes the rows k1 and R - k1 of all
// three components together (rows 0 and R/2 pair with themselves and share
// one CTA).  Between the passes the tiles go through L2 (75 MB for 48
// segments of 131,072 samples: with L2 warm the three passes read 54 MB from
// DRAM); each pass reads and writes every tile once.
//
// Every sub-DFT of length R or C is two in-register radix passes (R = R1 R2,
// sizes <= 16) with one exchange through shared memory, one unit (one small
// DFT) per thread; the first radix pass's units load straight from the tile
// and the last pass's units store straight to it, the lanes of a warp over
// columns (or row positions), so that every global access is a run of whole
// 32-byte sectors.
//
// The same passes serve single timelines (NC = 1): the right-hand side's
// per-detector half spectra (column pass + a forward row pass that stores
// the r2c values) and the per-detector operator's filter, both in batches of
// tiles through an L2-sized scratch.
// Conventions are FFTW's unnormalised r2c (sign -1) and c2r (sign +1), as in
// the reference's noise weighting (sanepic.cc:2390-2445, 2522-2582): the
// output is c2r(H r2c(x)) per group and segment, the same linear map as the
// cluster filter kernels (sg_filter.cuh) with the group mixing (sg_group.cu).
#include <cuda_runtime.h>

#include <algorithm>

#include "sg_cplx.cuh"
#include "sg_dft.cuh"
#include "sg_kernels.h"

namespace sg {
namespace f3 {

using cf = cplx<float>;

__device__ __forceinline__ cf ldg2(const cf* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return cf{v.x, v.y};
}
// W_M^j from the two-level table W_M^j = hi[j / 64] lo[j % 64]
__device__ __forceinline__ cf twm(const cf* lo, const cf* hi, int j) {
  return cmul(ldg2(hi + (j >> 6)), ldg2(lo + (j & 63)));
}

template <int LOGN>
struct Split {
  static constexpr int N = 1 << LOGN;
  static constexpr int N1 = 1 << ((LOGN + 1) / 2), N2 = N / N1;  // N = N1 N2, N1 >= N2
  static constexpr int LOGN2 = LOGN / 2;
  // shared layout of one length-N sequence: position p at p + p / N2, so that
  // both radix passes reach distinct bank pairs; an odd stride between
  // sequences
  static __device__ __forceinline__ int pad(int p) { return p + (p >> LOGN2); }
  static constexpr int QS = (N + N / N2) | 1;
};

// ---- passes 1 and 3: the column DFTs of CB columns -----------------------------
// NC = 3: the three components of a group tile in P^T's interleaved layout
// (sequence q = c CB + cc is column n2 = c0 + cc of component c; a row's CB
// columns of the three components are 6 CB contiguous floats); NC = 1: one
// timeline in natural order (sequence q is column c0 + q).  A column DFT of
// length R = R1 R2 (n1 = t + R2 j, k1 = ka + R1 kb) is two radix passes:
// units (q, t) take DFT_R1 over j straight from the tile, units (q, ka)
// DFT_R2 over t and write straight back; the lanes of a warp run over q, so
// every access to the tile is a run of whole 32-byte sectors.
template <int LOGR, int LOGC, int CB, int NC>
struct ColGeo {
  static constexpr int R = 1 << LOGR, C = 1 << LOGC, M = R * C;
  using S = Split<LOGR>;
  static constexpr int R1 = S::N1, R2 = S::N2, QS = S::QS;
  static constexpr int NSEQ = NC * CB;
  static constexpr int NT = NSEQ * R1;  // threads: the units of the R2 pass
  static constexpr int SMEM = NSEQ * QS + R + CB * R2;  // sequences, W_R, column steps
  static_assert(CB % 4 == 0 && CB <= C, "column blocks of whole 32-byte sectors");
  static_assert(NC == 1 || NC == 3, "one timeline or a group tile");
};

// complex point (row n, sequence q) of a tile, as an offset in complex units
template <int LOGC, int CB, int NC>
__device__ __forceinline__ long long col_elem(int c0, int q, int n) {
  if constexpr (NC == 1) {
    return (long long)(1 << LOGC) * n + c0 + q;
  } else {
    const int c = q / CB, cc = q % CB;
    return 3LL * (1 << LOGC) * n + 3 * c0 + 12 * (cc >> 2) + 4 * c + (cc & 3);
  }
}

template <int LOGR, int LOGC, int CB, int NC>
__device__ __forceinline__ void col_tables(cf* twr, cf* step, int c0, const cf* lo, const cf* hi,
                                           int tid) {
  using G = ColGeo<LOGR, LOGC, CB, NC>;
  for (int i = tid; i < G::R; i += G::NT) twr[i] = twm(lo, hi, i * G::C);  // W_R^i
  for (int i = tid; i < CB * G::R2; i += G::NT) {  // step[kb CB + cc] = W_M^{(c0 + cc) R1 kb}
    const int kb = i / CB, cc = i % CB;
    step[i] = twm(lo, hi, (c0 + cc) * G::R1 * kb);
  }
}

// pass 1: column DFTs and the four-step twiddle W_M^{n2 k1}; grid = tiles x C / CB.
// In place for NC = 3 (in == out); NC = 1 reads timelines and writes the
// transformed tiles elsewhere.
template <int LOGR, int LOGC, int CB, int NC, int MINB = 1>
__global__ void __launch_bounds__(ColGeo<LOGR, LOGC, CB, NC>::NT, MINB)
    k_f3_colfwd(const float* in, float* out, const cf* __restrict__ tw_lo,
                const cf* __restrict__ tw_hi) {
  using G = ColGeo<LOGR, LOGC, CB, NC>;
  using S = typename G::S;
  constexpr int R1 = G::R1, R2 = G::R2, QS = G::QS, NSEQ = G::NSEQ;
  extern __shared__ __align__(16) unsigned char f3_smem[];
  cf* s = reinterpret_cast<cf*>(f3_smem);
  cf* twr = s + NSEQ * QS;
  cf* step = twr + G::R;
  const int tid = threadIdx.x;
  const long long tile = blockIdx.x / (G::C / CB);
  const int c0 = (int)(blockIdx.x % (G::C / CB)) * CB;
  const cf* ti = reinterpret_cast<const cf*>(in) + tile * NC * (long long)G::M;
  cf* to = reinterpret_cast<cf*>(out) + tile * NC * (long long)G::M;
  // pass A: DFT_R1 over j of z[t + R2 j], twiddle W_R^{t ka}
  const bool unitA = tid < NSEQ * R2;
  const int qa = tid % NSEQ, ta = tid / NSEQ;
  cf a[R1];
  if (unitA) {
#pragma unroll
    for (int j = 0; j < R1; j++) {
      const cf* p = ti + col_elem<LOGC, CB, NC>(c0, qa, ta + R2 * j);
      if constexpr (NC == 1) {  // timelines read once: evict first, keep L2 for the batch
        const float2 v = __ldcs(reinterpret_cast<const float2*>(p));
        a[j] = cf{v.x, v.y};
      } else {
        a[j] = *p;
      }
    }
  }
  col_tables<LOGR, LOGC, CB, NC>(twr, step, c0, tw_lo, tw_hi, tid);
  __syncthreads();
  if (unitA) {
    SgDft<R1, false, float>::run(a);
#pragma unroll
    for (int ka = 0; ka < R1; ka++)
      s[qa * QS + S::pad(ta + R2 * ka)] = (ka == 0 || ta == 0) ? a[ka] : cmul(a[ka], twr[ta * ka]);
  }
  __syncthreads();
  // pass B: DFT_R2 over t, Y[ka + R1 kb] times W_M^{n2 (ka + R1 kb)}, to the tile
  {
    const int q = tid % NSEQ, ka = tid / NSEQ, cc = q % CB, n2 = c0 + cc;
    cf v[R2];
#pragma unroll
    for (int i = 0; i < R2; i++) v[i] = s[q * QS + S::pad(i + R2 * ka)];
    SgDft<R2, false, float>::run(v);
    const cf wa = twm(tw_lo, tw_hi, n2 * ka);
#pragma unroll
    for (int kb = 0; kb < R2; kb++) {
      const cf y = n2 == 0 ? v[kb] : cmul(v[kb], cmul(wa, step[kb * CB + cc]));
      to[col_elem<LOGC, CB, NC>(c0, q, ka + R1 * kb)] = y;
    }
  }
}

// pass 3: the conjugate four-step twiddle and the inverse column DFTs; in
// place on group tiles (NC = 3, in == out), or from the transformed tiles of
// single timelines back to the timelines (NC = 1)
template <int LOGR, int LOGC, int CB, int NC, int MINB = 1>
__global__ void __launch_bounds__(ColGeo<LOGR, LOGC, CB, NC>::NT, MINB)
    k_f3_colinv(const float* in, float* out, const cf* __restrict__ tw_lo,
                const cf* __restrict__ tw_hi) {
  using G = ColGeo<LOGR, LOGC, CB, NC>;
  using S = typename G::S;
  constexpr int R1 = G::R1, R2 = G::R2, QS = G::QS, NSEQ = G::NSEQ;
  extern __shared__ __align__(16) unsigned char f3_smem[];
  cf* s = reinterpret_cast<cf*>(f3_smem);
  cf* twr = s + NSEQ * QS;
  cf* step = twr + G::R;
  const int tid = threadIdx.x;
  const long long tile = blockIdx.x / (G::C / CB);
  const int c0 = (int)(blockIdx.x % (G::C / CB)) * CB;
  const cf* ti = reinterpret_cast<const cf*>(in) + tile * NC * (long long)G::M;
  cf* to = reinterpret_cast<cf*>(out) + tile * NC * (long long)G::M;
  // pass B': conj W_M^{n2 k1}, DFT_R2 (sign +) over kb of U[ka + R1 kb], conj W_R^{t ka}
  {
    const int q = tid % NSEQ, ka = tid / NSEQ, cc = q % CB, n2 = c0 + cc;
    cf v[R2];
#pragma unroll
    for (int kb = 0; kb < R2; kb++) v[kb] = ti[col_elem<LOGC, CB, NC>(c0, q, ka + R1 * kb)];
    col_tables<LOGR, LOGC, CB, NC>(twr, step, c0, tw_lo, tw_hi, tid);
    __syncthreads();
    if (n2 != 0) {
      const cf wa = twm(tw_lo, tw_hi, n2 * ka);
#pragma unroll
      for (int kb = 0; kb < R2; kb++) v[kb] = cmulc(v[kb], cmul(wa, step[kb * CB + cc]));
    }
    SgDft<R2, true, float>::run(v);
#pragma unroll
    for (int i = 0; i < R2; i++)
      s[q * QS + S::pad(i + R2 * ka)] = (ka == 0 || i == 0) ? v[i] : cmulc(v[i], twr[i * ka]);
  }
  __syncthreads();
  // pass A': DFT_R1 (sign +) over ka, z'[t + R2 j], to the tile
  if (tid < NSEQ * R2) {
    const int q = tid % NSEQ, ta = tid / NSEQ;
    cf a[R1];
#pragma unroll
    for (int ka = 0; ka < R1; ka++) a[ka] = s[q * QS + S::pad(ta + R2 * ka)];
    SgDft<R1, true, float>::run(a);
#pragma unroll
    for (int j = 0; j < R1; j++) to[col_elem<LOGC, CB, NC>(c0, q, ta + R2 * j)] = a[j];
  }
}

// ---- pass 2: rows ----------------------------------------------------------------
// A row CTA takes row pairs: pair p = 0 is rows {0, R/2}, pair p > 0 rows
// {p, R - p}, so that every frequency k = k1 + R k2 and its real-FFT partner
// M - k sit in the same CTA.  A row DFT of length C = C1 C2 (n2 = t + C2 j,
// k2 = ka + C1 kb): units (rr, t) read the tile, units (rr, ka) work in
// shared memory, the inverse's units (rr, t) write the tile.
__device__ __forceinline__ int row_k1(int R, int p, int side) {
  return p == 0 ? (side ? R / 2 : 0) : (side ? R - p : p);
}

// complex point n of row k1, component c of a group tile (complex units)
template <int LOGC>
__device__ __forceinline__ long long row3_elem(int k1, int c, int n) {
  return 3LL * (1 << LOGC) * k1 + 12 * (n >> 2) + 4 * c + (n & 3);
}

// the frequency pair of spectrum task tau (0 <= tau <= C) of row pair p:
// (side, column) of the smaller frequency k (A) and of M - k (B); special:
// bins 0 and M (row 0, column 0).  False if the task does not exist.
__device__ __forceinline__ bool pair_of(int C, int p, int tau, int& rowA, int& colA, int& rowB,
                                        int& colB, bool& special) {
  special = false;
  if (p != 0) {
    if (tau >= C) return false;
    if (tau < C / 2) { rowA = 0; colA = tau; rowB = 1; colB = C - 1 - tau; }
    else { rowA = 1; colA = C - 1 - tau; rowB = 0; colB = tau; }
  } else if (tau < C / 2) {  // row R/2: k2 <-> C-1-k2
    rowA = 1; colA = tau; rowB = 1; colB = C - 1 - tau;
  } else if (tau == C / 2) {  // bins 0 and M
    rowA = rowB = 0; colA = colB = 0; special = true;
  } else if (tau < C) {  // row 0: k2 <-> C - k2
    rowA = 0; colA = tau - C / 2; rowB = 0; colB = C - colA;
  } else {  // row 0, k2 = C/2: k = M/2, its own partner
    rowA = rowB = 0; colA = colB = C / 2;
  }
  return true;
}

// W_N^{k1} (N = 2M) of each of a CTA's 2 RP rows (row 2 pp + side of pair
// p0 + pp), from the W_M table and wn1 = W_N; the split twiddle of
// k = k1 + R col is then W_N^k = w1s[row] W_N^{R col} (wsp[col] = W_N^{R col};
// exact for k1 = 0, where w1s = 1), computed once per CTA instead of once per
// frequency pair
__device__ __forceinline__ void row_w1_table(cf* w1s, int nrows, int p0, int R, const cf* lo,
                                             const cf* hi, cf wn1, int tid, int nt) {
  for (int i = tid; i < nrows; i += nt) {
    const int k1 = row_k1(R, p0 + (i >> 1), i & 1);
    cf w1{1.f, 0.f};
    if (k1 != 0) {
      w1 = twm(lo, hi, k1 >> 1);
      if (k1 & 1) w1 = cmul(w1, wn1);
    }
    w1s[i] = w1;
  }
}
__device__ __forceinline__ cf split_tw_row(const cf* w1s, int row, int col, const cf* wsp) {
  return cmul(w1s[row], wsp[col]);
}

// r2c values X[k], X[M-k] from the packed spectrum values Z[k], Z[M-k]
__device__ __forceinline__ void split_pair(cf zk, cf zm, cf wk, cf& xk, cf& xm) {
  const cf Ev{0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y)};
  const cf Ov{0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x)};
  const cf wO = cmul(wk, Ov);
  xk = Ev + wO;
  xm = cconj(Ev - wO);
}
// the packed values at k and M-k for the inverse of the r2c values Y[k], Y[M-k]
__device__ __forceinline__ void repack_pair(cf yk, cf ym, cf wk, cf& zk, cf& zm) {
  const cf P = yk + cconj(ym), Q = yk - cconj(ym);
  const cf cwQ = cmulc(Q, wk);
  const cf iwQ{-cwQ.y, cwQ.x};
  zk = P + iwQ;
  zm = cconj(P - iwQ);
}

// the row tables: twA[ka C2 + t] = twB[t C1 + ka] = W_C^{t ka}, wsp[i] = W_N^{R i}
template <int LOGR, int LOGC>
__device__ __forceinline__ void row_tables(cf* twA, cf* twB, cf* wsp, const cf* lo, const cf* hi,
                                           int tid, int nt) {
  constexpr int R = 1 << LOGR, C = 1 << LOGC;
  constexpr int C1 = Split<LOGC>::N1, C2 = Split<LOGC>::N2;
  for (int i = tid; i < C; i += nt) {
    const int ka = i / C2, t = i % C2;
    twA[i] = twm(lo, hi, ((t * ka) & (C - 1)) * R);
    const int tb = i / C1, kb = i % C1;
    twB[i] = twm(lo, hi, ((tb * kb) & (C - 1)) * R);
    wsp[i] = twm(lo, hi, (R / 2) * i);
  }
}

// Forward row DFTs of NSEQ sequences into shared memory, natural order.
// rows_load: the pass-A units' inputs (point n of sequence rr from ld(rr, n));
// rows_forward_loaded: the rest, starting with a barrier that also orders the
// tables and the previous use of s.
template <int LOGC, int NSEQ, class Ld>
__device__ __forceinline__ void rows_load(int tid, Ld ld, cf (&a)[Split<LOGC>::N1]) {
  constexpr int C1 = Split<LOGC>::N1, C2 = Split<LOGC>::N2;
  if (tid < NSEQ * C2) {
    const int rra = tid / C2, ta = tid % C2;
#pragma unroll
    for (int j = 0; j < C1; j++) a[j] = ld(rra, ta + C2 * j);
  }
}
template <int LOGC, int NSEQ>
__device__ __forceinline__ void rows_forward_loaded(cf* s, const cf* twA, int tid,
                                                    cf (&a)[Split<LOGC>::N1]) {
  using S = Split<LOGC>;
  constexpr int C1 = S::N1, C2 = S::N2, QS = S::QS;
  const bool unitA = tid < NSEQ * C2;
  const int rra = tid / C2, ta = tid % C2;
  __syncthreads();
  if (unitA) {
    SgDft<C1, false, float>::run(a);
#pragma unroll
    for (int ka = 0; ka < C1; ka++)
      s[rra * QS + S::pad(ta + C2 * ka)] = (ka == 0 || ta == 0) ? a[ka] : cmul(a[ka], twA[ka * C2 + ta]);
  }
  __syncthreads();
  const int rrb = tid / C1, kab = tid % C1;
  cf v[C2];
#pragma unroll
  for (int i = 0; i < C2; i++) v[i] = s[rrb * QS + S::pad(i + C2 * kab)];
  SgDft<C2, false, float>::run(v);
  __syncthreads();
#pragma unroll
  for (int kb = 0; kb < C2; kb++) s[rrb * QS + S::pad(kab + C1 * kb)] = v[kb];
  __syncthreads();
}
template <int LOGC, int NSEQ, class Ld>
__device__ __forceinline__ void rows_forward(cf* s, const cf* twA, int tid, Ld ld) {
  cf a[Split<LOGC>::N1];
  rows_load<LOGC, NSEQ>(tid, ld, a);
  rows_forward_loaded<LOGC, NSEQ>(s, twA, tid, a);
}

// Inverse row DFTs of the NSEQ sequences in shared memory (natural order);
// st(rr, n, v) stores point n of sequence rr.
template <int LOGC, int NSEQ, class St>
__device__ __forceinline__ void rows_inverse(cf* s, const cf* twB, int tid, St st) {
  using S = Split<LOGC>;
  constexpr int C1 = S::N1, C2 = S::N2, QS = S::QS;
  const int rrb = tid / C1, kab = tid % C1;
  {
    cf v[C2];
#pragma unroll
    for (int kb = 0; kb < C2; kb++) v[kb] = s[rrb * QS + S::pad(kab + C1 * kb)];
    SgDft<C2, true, float>::run(v);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < C2; i++)
      s[rrb * QS + S::pad(i + C2 * kab)] = (kab == 0 || i == 0) ? v[i] : cmulc(v[i], twB[i * C1 + kab]);
  }
  __syncthreads();
  if (tid < NSEQ * C2) {
    const int rra = tid / C2, ta = tid % C2;
    cf a[C1];
#pragma unroll
    for (int ka = 0; ka < C1; ka++) a[ka] = s[rra * QS + S::pad(ta + C2 * ka)];
    SgDft<C1, true, float>::run(a);
#pragma unroll
    for (int j = 0; j < C1; j++) st(rra, ta + C2 * j, a[j]);
  }
}

// The weighting pass: RP row pairs of RSEG consecutive segments of one group
// per CTA, three components (sequence rr = (2 pp + side) 3 + c).  With HSTAGE
// the weights of its rows are staged in shared memory once and serve all RSEG
// segments; otherwise each frequency pair reads its weights from L2.
// MIX 1: the group's 3 x 3 H, hrow[g][pos][6] (H00 H01 H02 H11 H12 H22);
// MIX 0: one spectrum h per group, hrow[g][pos].  pos = C k1 + k2 for
// k = k1 + R k2 < M, pos = M for k = M.  Grid: groups x ceil(nseg / RSEG) x
// (R/2) / RP.
template <int LOGR, int LOGC, int RP, int MIX, bool HSTAGE = true>
struct RowGeo {
  static constexpr int R = 1 << LOGR, C = 1 << LOGC, M = R * C;
  using S = Split<LOGC>;
  static constexpr int C1 = S::N1, C2 = S::N2, QS = S::QS;
  static constexpr int NSEQ = 6 * RP;
  static constexpr int NT = NSEQ * C1;
  static constexpr int HW = MIX ? 6 : 1;  // weights per frequency
  // shared: sequences, W_C twice, split tables (complex) + with HSTAGE the
  // rows' weights (floats, padded to 8 B)
  static constexpr int SMEM =
      NSEQ * QS + 3 * C + 2 * RP + (HSTAGE ? (2 * RP * C * HW + HW + 1) / 2 : 0);
  static_assert((R / 2) % RP == 0, "row pairs per CTA divide R/2");
};

template <int LOGR, int LOGC, int RP, int MIX, int RSEG, int MINB = 1, bool HSTAGE = true>
__global__ void __launch_bounds__(RowGeo<LOGR, LOGC, RP, MIX, HSTAGE>::NT, MINB)
    k_f3_rows(float* __restrict__ data, const float* __restrict__ hrow, int nseg,
              const cf* __restrict__ tw_lo, const cf* __restrict__ tw_hi, cf wn1) {
  using G = RowGeo<LOGR, LOGC, RP, MIX, HSTAGE>;
  using S = typename G::S;
  constexpr int R = G::R, C = G::C, M = G::M, QS = S::QS, NT = G::NT, HW = G::HW;
  constexpr int NSEQ = G::NSEQ;
  extern __shared__ __align__(16) unsigned char f3_smem[];
  cf* s = reinterpret_cast<cf*>(f3_smem);
  cf* twA = s + NSEQ * QS;
  cf* twB = twA + C;
  cf* wsp = twB + C;
  cf* w1s = wsp + C;  // [2 RP]
  float* hs = reinterpret_cast<float*>(w1s + 2 * RP);  // [2 RP][C][HW], then bin M
  const int tid = threadIdx.x;
  constexpr int CPT = (R / 2) / RP;  // CTAs per segment
  const int nsb = (nseg + RSEG - 1) / RSEG;
  const int p0 = (int)(blockIdx.x % CPT) * RP;
  const long long rest = blockIdx.x / CPT;
  const int sb = (int)(rest % nsb);
  const long long grp = rest / nsb;
  const float* H = hrow + grp * (long long)(M + 1) * HW;
  row_tables<LOGR, LOGC>(twA, twB, wsp, tw_lo, tw_hi, tid, NT);
  row_w1_table(w1s, 2 * RP, p0, R, tw_lo, tw_hi, wn1, tid, NT);
  if constexpr (HSTAGE) {
    for (int i = tid; i < 2 * RP * C * HW; i += NT) {
      const int row = i / (C * HW), e = i % (C * HW);
      hs[i] = __ldg(H + (long long)C * HW * row_k1(R, p0 + (row >> 1), row & 1) + e);
    }
    if (tid < HW) hs[2 * RP * C * HW + tid] = __ldg(H + (long long)M * HW + tid);
  }
  const int s_end = min(nseg, (sb + 1) * RSEG);
  auto elem = [&](int rr, int n) {
    const int row = rr / 3;
    return row3_elem<LOGC>(row_k1(R, p0 + (row >> 1), row & 1), rr % 3, n);
  };
  // (loading the next segment's rows while this one is weighted was slower:
  // 56 -> 59-66 us at 48 x 131072 samples, registers for the prefetch)
  for (int seg = sb * RSEG; seg < s_end; seg++) {
    cf* t = reinterpret_cast<cf*>(data + (grp * nseg + seg) * 6LL * M);
    rows_forward<LOGC, NSEQ>(s, twA, tid, [&](int rr, int n) { return t[elem(rr, n)]; });
    // spectrum: pairs (k, M - k) of all three components
    for (int task = tid; task < RP * (C + 1); task += NT) {
      const int pp = task / (C + 1), tau = task % (C + 1);
      const int p = p0 + pp;
      int rowA, colA, rowB, colB;
      bool special;
      if (!pair_of(C, p, tau, rowA, colA, rowB, colB, special)) continue;
      cf* qa = s + ((2 * pp + rowA) * 3) * QS + S::pad(colA);
      cf* qb = s + ((2 * pp + rowB) * 3) * QS + S::pad(colB);
      // the weights: staged rows, or straight from L2 (read-only path)
      float hva[HW], hvb[HW];
      if constexpr (HSTAGE) {
        const float* hsb =
            special ? hs + 2 * RP * C * HW : hs + ((2 * pp + rowB) * C + colB) * HW;
#pragma unroll
        for (int i = 0; i < HW; i++) {
          hva[i] = hs[((2 * pp + rowA) * C + colA) * HW + i];
          hvb[i] = hsb[i];
        }
      } else {
        const long long pa = (long long)C * row_k1(R, p, rowA) + colA;
        const long long pb = special ? M : (long long)C * row_k1(R, p, rowB) + colB;
#pragma unroll
        for (int i = 0; i < HW; i++) {
          hva[i] = __ldg(H + pa * HW + i);
          hvb[i] = __ldg(H + pb * HW + i);
        }
      }
      const float* ha = hva;
      const float* hb = hvb;
      if (special) {
        const float* hm = hvb;  // bin M
        float x0[3], xm[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
          const cf z = qa[c * QS];
          x0[c] = z.x + z.y;
          xm[c] = z.x - z.y;
        }
        float y0[3], ym[3];
        if constexpr (MIX) {
          y0[0] = ha[0] * x0[0] + ha[1] * x0[1] + ha[2] * x0[2];
          y0[1] = ha[1] * x0[0] + ha[3] * x0[1] + ha[4] * x0[2];
          y0[2] = ha[2] * x0[0] + ha[4] * x0[1] + ha[5] * x0[2];
          ym[0] = hm[0] * xm[0] + hm[1] * xm[1] + hm[2] * xm[2];
          ym[1] = hm[1] * xm[0] + hm[3] * xm[1] + hm[4] * xm[2];
          ym[2] = hm[2] * xm[0] + hm[4] * xm[1] + hm[5] * xm[2];
        } else {
#pragma unroll
          for (int c = 0; c < 3; c++) {
            y0[c] = ha[0] * x0[c];
            ym[c] = hm[0] * xm[c];
          }
        }
#pragma unroll
        for (int c = 0; c < 3; c++) qa[c * QS] = cf{y0[c] + ym[c], y0[c] - ym[c]};
        continue;
      }
      const cf wk = split_tw_row(w1s, 2 * pp + rowA, colA, wsp);
      cf xk[3], xm[3];
#pragma unroll
      for (int c = 0; c < 3; c++) split_pair(qa[c * QS], qb[c * QS], wk, xk[c], xm[c]);
      cf yk[3], ym[3];
      if constexpr (MIX) {
#define SG_F3_MIX(Y, X, h)                                                       \
  Y[0] = cf{h[0] * X[0].x + h[1] * X[1].x + h[2] * X[2].x,                       \
            h[0] * X[0].y + h[1] * X[1].y + h[2] * X[2].y};                      \
  Y[1] = cf{h[1] * X[0].x + h[3] * X[1].x + h[4] * X[2].x,                       \
            h[1] * X[0].y + h[3] * X[1].y + h[4] * X[2].y};                      \
  Y[2] = cf{h[2] * X[0].x + h[4] * X[1].x + h[5] * X[2].x,                       \
            h[2] * X[0].y + h[4] * X[1].y + h[5] * X[2].y};
        SG_F3_MIX(yk, xk, ha)
        SG_F3_MIX(ym, xm, hb)
#undef SG_F3_MIX
      } else {
#pragma unroll
        for (int c = 0; c < 3; c++) {
          yk[c] = cscale(xk[c], ha[0]);
          ym[c] = cscale(xm[c], hb[0]);
        }
      }
#pragma unroll
      for (int c = 0; c < 3; c++) {
        cf zk, zm;
        repack_pair(yk[c], ym[c], wk, zk, zm);
        qa[c * QS] = zk;
        if (qb != qa) qb[c * QS] = zm;
      }
    }
    __syncthreads();
    rows_inverse<LOGC, NSEQ>(s, twB, tid, [&](int rr, int n, cf v) { t[elem(rr, n)] = v; });
  }
}

// The weighting pass of single timelines (the per-detector operator): RP
// row pairs of RSEG consecutive tiles of one detector per CTA (sequence rr =
// 2 pp + side), in place on the transformed tiles data [tiles][2M] (tile t of
// the batch is tile tile0 + t of the operator, detector (tile0 + t) / nseg);
// the spectrum of each frequency pair is scaled by the detector's filter row
// in position order (hpos [ndet][M+1]).  Grid: ceil(tiles / RSEG) x (R/2) / RP.
template <int LOGR, int LOGC, int RP>
struct Row1Geo {
  static constexpr int R = 1 << LOGR, C = 1 << LOGC, M = R * C;
  using S = Split<LOGC>;
  static constexpr int QS = S::QS, NSEQ = 2 * RP, NT = NSEQ * S::N1;
  // shared: sequences, W_C twice, split tables (complex) + the rows' weights
  static constexpr int SMEM = NSEQ * QS + 3 * C + 2 * RP + (2 * RP * C + 2) / 2;
  static_assert((R / 2) % RP == 0, "row pairs per CTA divide R/2");
};

template <int LOGR, int LOGC, int RP, int RSEG, int MINB = 1, bool HSTAGE = true>
__global__ void __launch_bounds__(Row1Geo<LOGR, LOGC, RP>::NT, MINB)
    k_f3_rows1(float* __restrict__ data, long long ntiles, long long tile0, int nseg,
               const float* __restrict__ hpos, const cf* __restrict__ tw_lo,
               const cf* __restrict__ tw_hi, cf wn1) {
  using G = Row1Geo<LOGR, LOGC, RP>;
  using S = typename G::S;
  constexpr int R = G::R, C = G::C, M = G::M, QS = G::QS, NT = G::NT, NSEQ = G::NSEQ;
  extern __shared__ __align__(16) unsigned char f3_smem[];
  cf* s = reinterpret_cast<cf*>(f3_smem);
  cf* twA = s + NSEQ * QS;
  cf* twB = twA + C;
  cf* wsp = twB + C;
  cf* w1s = wsp + C;  // [2 RP]
  float* hs = reinterpret_cast<float*>(w1s + 2 * RP);  // [2 RP][C], then bin M
  const int tid = threadIdx.x;
  constexpr int CPT = (R / 2) / RP;
  const int p0 = (int)(blockIdx.x % CPT) * RP;
  const long long tb = (blockIdx.x / CPT) * RSEG;  // first tile of the batch
  row_tables<LOGR, LOGC>(twA, twB, wsp, tw_lo, tw_hi, tid, NT);
  row_w1_table(w1s, 2 * RP, p0, R, tw_lo, tw_hi, wn1, tid, NT);
  long long det_staged = -1;
  const long long t_end = tb + RSEG < ntiles ? tb + RSEG : ntiles;
  for (long long tl = tb; tl < t_end; tl++) {
    const long long det = (tile0 + tl) / nseg;
    cf* t = reinterpret_cast<cf*>(data) + tl * (long long)M;
    auto elem = [&](int rr, int n) {
      return (long long)C * row_k1(R, p0 + (rr >> 1), rr & 1) + n;
    };
    const float* hdet = hpos + det * (long long)(M + 1);
    if (HSTAGE && det != det_staged) {  // the detector's filter values at this CTA's rows
      __syncthreads();  // the previous tile's last reads of hs
      const float* h = hpos + det * (long long)(M + 1);
      for (int i = tid; i < 2 * RP * C; i += NT)
        hs[i] = __ldg(h + (long long)C * row_k1(R, p0 + (i / C >> 1), (i / C) & 1) + i % C);
      if (tid == 0) hs[2 * RP * C] = __ldg(h + M);
      det_staged = det;
    }
    rows_forward<LOGC, NSEQ>(s, twA, tid, [&](int rr, int n) { return t[elem(rr, n)]; });
    for (int task = tid; task < RP * (C + 1); task += NT) {
      const int pp = task / (C + 1), tau = task % (C + 1);
      const int p = p0 + pp;
      int rowA, colA, rowB, colB;
      bool special;
      if (!pair_of(C, p, tau, rowA, colA, rowB, colB, special)) continue;
      cf* qa = s + (2 * pp + rowA) * QS + S::pad(colA);
      cf* qb = s + (2 * pp + rowB) * QS + S::pad(colB);
      float ha, hb;
      if constexpr (HSTAGE) {
        ha = hs[(2 * pp + rowA) * C + colA];
        hb = special ? hs[2 * RP * C] : hs[(2 * pp + rowB) * C + colB];
      } else {  // straight from L2
        ha = __ldg(hdet + (long long)C * row_k1(R, p, rowA) + colA);
        hb = __ldg(hdet + (special ? (long long)M : (long long)C * row_k1(R, p, rowB) + colB));
      }
      if (special) {
        const cf z = *qa;
        const float y0 = ha * (z.x + z.y), yM = hb * (z.x - z.y);
        *qa = cf{y0 + yM, y0 - yM};
        continue;
      }
      const cf wk = split_tw_row(w1s, 2 * pp + rowA, colA, wsp);
      cf xk, xm, zk, zm;
      split_pair(*qa, *qb, wk, xk, xm);
      repack_pair(cscale(xk, ha), cscale(xm, hb), wk, zk, zm);
      *qa = zk;
      if (qb != qa) *qb = zm;
    }
    __syncthreads();
    rows_inverse<LOGC, NSEQ>(s, twB, tid, [&](int rr, int n, cf v) { t[elem(rr, n)] = v; });
  }
}

// Forward row pass of single timelines with the half spectrum out: RP row
// pairs of one tile per CTA (sequence rr = 2 pp + side), the r2c values X[k]
// stored at their positions pos (as above) of spec[tile0 + tile][M+1].
// Grid: tiles x (R/2) / RP.
template <int LOGR, int LOGC, int RP>
struct RowSpecGeo {
  static constexpr int R = 1 << LOGR, C = 1 << LOGC, M = R * C;
  using S = Split<LOGC>;
  static constexpr int QS = S::QS, NSEQ = 2 * RP, NT = NSEQ * S::N1;
  static constexpr int SMEM = NSEQ * QS + 3 * C + 2 * RP;
  static_assert((R / 2) % RP == 0, "row pairs per CTA divide R/2");
};

template <int LOGR, int LOGC, int RP, int MINB = 1>
__global__ void __launch_bounds__(RowSpecGeo<LOGR, LOGC, RP>::NT, MINB)
    k_f3_rowspec(const float* __restrict__ in, cf* __restrict__ spec, long long tile0,
                 const cf* __restrict__ tw_lo, const cf* __restrict__ tw_hi, cf wn1) {
  using G = RowSpecGeo<LOGR, LOGC, RP>;
  using S = typename G::S;
  constexpr int R = G::R, C = G::C, M = G::M, QS = G::QS, NT = G::NT, NSEQ = G::NSEQ;
  extern __shared__ __align__(16) unsigned char f3_smem[];
  cf* s = reinterpret_cast<cf*>(f3_smem);
  cf* twA = s + NSEQ * QS;
  cf* twB = twA + C;
  cf* wsp = twB + C;
  const int tid = threadIdx.x;
  constexpr int CPT = (R / 2) / RP;
  const int p0 = (int)(blockIdx.x % CPT) * RP;
  const long long tile = blockIdx.x / CPT;
  const cf* t = reinterpret_cast<const cf*>(in) + tile * (long long)M;
  cf* X = spec + (tile0 + tile) * (long long)(M + 1);
  cf* w1s = wsp + C;
  row_tables<LOGR, LOGC>(twA, twB, wsp, tw_lo, tw_hi, tid, NT);
  row_w1_table(w1s, 2 * RP, p0, R, tw_lo, tw_hi, wn1, tid, NT);
  rows_forward<LOGC, NSEQ>(s, twA, tid, [&](int rr, int n) {
    const float2 v = __ldcs(reinterpret_cast<const float2*>(t) +
                            (long long)C * row_k1(R, p0 + (rr >> 1), rr & 1) + n);
    return cf{v.x, v.y};
  });
  for (int task = tid; task < RP * (C + 1); task += NT) {
    const int pp = task / (C + 1), tau = task % (C + 1);
    const int p = p0 + pp;
    int rowA, colA, rowB, colB;
    bool special;
    if (!pair_of(C, p, tau, rowA, colA, rowB, colB, special)) continue;
    const cf za = s[(2 * pp + rowA) * QS + S::pad(colA)];
    // the spectra go to DRAM and are read once: streaming stores
    float2* Xf = reinterpret_cast<float2*>(X);
    if (special) {
      __stcs(Xf, make_float2(za.x + za.y, 0.f));
      __stcs(Xf + M, make_float2(za.x - za.y, 0.f));
      continue;
    }
    const cf zb = s[(2 * pp + rowB) * QS + S::pad(colB)];
    const int k1A = row_k1(R, p, rowA), k1B = row_k1(R, p, rowB);
    cf xk, xm;
    split_pair(za, zb, split_tw_row(w1s, 2 * pp + rowA, colA, wsp), xk, xm);
    __stcs(Xf + (long long)C * k1A + colA, make_float2(xk.x, xk.y));
    if (k1A != k1B || colA != colB) __stcs(Xf + (long long)C * k1B + colB, make_float2(xm.x, xm.y));
  }
}

// Inverse row pass of group tiles from their weighted half spectra: gspec
// [G][3][nseg][M+1] (positions pos), RP row pairs of one group tile per CTA;
// the rows go into the tile in P^T's layout for k_f3_colinv.  Grid: G nseg x
// (R/2) / RP.
template <int LOGR, int LOGC, int RP>
struct RowInGeo {
  static constexpr int R = 1 << LOGR, C = 1 << LOGC, M = R * C;
  using S = Split<LOGC>;
  static constexpr int QS = S::QS, NSEQ = 6 * RP, NT = NSEQ * S::N1;
  static constexpr int SMEM = NSEQ * QS + 3 * C + 2 * RP;
  static_assert((R / 2) % RP == 0, "row pairs per CTA divide R/2");
};

template <int LOGR, int LOGC, int RP, int MINB = 1>
__global__ void __launch_bounds__(RowInGeo<LOGR, LOGC, RP>::NT, MINB)
    k_f3_rows_specin(const cf* __restrict__ gspec, float* __restrict__ data, int nseg,
                     const cf* __restrict__ tw_lo, const cf* __restrict__ tw_hi, cf wn1) {
  using G = RowInGeo<LOGR, LOGC, RP>;
  using S = typename G::S;
  constexpr int R = G::R, C = G::C, M = G::M, QS = G::QS, NT = G::NT, NSEQ = G::NSEQ;
  extern __shared__ __align__(16) unsigned char f3_smem[];
  cf* s = reinterpret_cast<cf*>(f3_smem);
  cf* twA = s + NSEQ * QS;
  cf* twB = twA + C;
  cf* wsp = twB + C;
  const int tid = threadIdx.x;
  constexpr int CPT = (R / 2) / RP;
  const int p0 = (int)(blockIdx.x % CPT) * RP;
  const long long tile = blockIdx.x / CPT;  // group * nseg + segment
  const long long grp = tile / nseg, seg = tile % nseg;
  cf* t = reinterpret_cast<cf*>(data + tile * 6LL * M);
  cf* w1s = wsp + C;
  row_tables<LOGR, LOGC>(twA, twB, wsp, tw_lo, tw_hi, tid, NT);
  row_w1_table(w1s, 2 * RP, p0, R, tw_lo, tw_hi, wn1, tid, NT);
  __syncthreads();
  for (int task = tid; task < RP * (C + 1); task += NT) {
    const int pp = task / (C + 1), tau = task % (C + 1);
    const int p = p0 + pp;
    int rowA, colA, rowB, colB;
    bool special;
    if (!pair_of(C, p, tau, rowA, colA, rowB, colB, special)) continue;
    const int k1A = row_k1(R, p, rowA), k1B = row_k1(R, p, rowB);
    cf* qa = s + ((2 * pp + rowA) * 3) * QS + S::pad(colA);
    cf* qb = s + ((2 * pp + rowB) * 3) * QS + S::pad(colB);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const cf* Y = gspec + ((grp * 3 + c) * nseg + seg) * (long long)(M + 1);
      if (special) {
        const float y0 = Y[0].x, yM = Y[M].x;
        qa[c * QS] = cf{y0 + yM, y0 - yM};
        continue;
      }
      const cf wk = split_tw_row(w1s, 2 * pp + rowA, colA, wsp);
      const cf yk = Y[(long long)C * k1A + colA], ym = Y[(long long)C * k1B + colB];
      cf zk, zm;
      repack_pair(yk, ym, wk, zk, zm);
      qa[c * QS] = zk;
      if (qb != qa) qb[c * QS] = zm;
    }
  }
  __syncthreads();
  rows_inverse<LOGC, NSEQ>(s, twB, tid, [&](int rr, int n, cf v) {
    const int row = rr / 3;
    t[row3_elem<LOGC>(row_k1(R, p0 + (row >> 1), row & 1), rr % 3, n)] = v;
  });
}

}  // namespace f3

// ---- host side -----------------------------------------------------------------
// Tile shapes per log2(M): R x C with C >= R.  Group tiles: CB = 8 columns
// per column CTA, RP = 2 row pairs and RSEG = 3 segments per row CTA; at
// M = 65536 the column kernels are capped for three CTAs per SM and the row
// kernel for four (fewer registers, more CTAs in flight: 149 -> 107 us per
// application of 48 tiles on a GB300).  Single timelines (the right-hand
// side's detectors): 16 columns per column CTA, 8 row pairs per row CTA,
// the column kernels capped for four CTAs per SM (64 registers, no spills;
// at 131072 samples 20.8 -> 20.5 us forward and 20.6 -> 19.3 us inverse per
// 96 tiles on a GB300, against three CTAs at 80 registers).
namespace {
constexpr int kCB = 8, kRP = 2, kCB1 = 16, kRP1 = 8, kMB1 = 4;

template <class K>
cudaError_t set_smem(K k, int bytes) {
  return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

// The weighting pass reads H straight from L2 (staging a CTA's rows of H in
// shared memory for three segments had been slower: 56 -> 47.7 us for the
// 3 x 3 mixing at 48 x 131072 samples, 47.3 -> 43.6 us for one spectrum, with
// more CTAs per SM in the freed shared memory).  RPR row pairs per CTA.
template <int LOGR, int LOGC, int MIX, int MBC, int RPR, int MBR>
cudaError_t f3_run(float* data, const float* hrow, long long ngroups, int nseg,
                   const cplx<float>* lo, const cplx<float>* hi, cplx<float> wn1, cudaStream_t st) {
  using CG = f3::ColGeo<LOGR, LOGC, kCB, 3>;
  using RG = f3::RowGeo<LOGR, LOGC, RPR, MIX, false>;
  auto kc = f3::k_f3_colfwd<LOGR, LOGC, kCB, 3, MBC>;
  auto kr = f3::k_f3_rows<LOGR, LOGC, RPR, MIX, 1, MBR, false>;
  auto ki = f3::k_f3_colinv<LOGR, LOGC, kCB, 3, MBC>;
  const int smc = CG::SMEM * (int)sizeof(cplx<float>), smr = RG::SMEM * (int)sizeof(cplx<float>);
  cudaError_t e = set_smem(kc, smc);
  if (e == cudaSuccess) e = set_smem(ki, smc);
  if (e == cudaSuccess) e = set_smem(kr, smr);
  if (e != cudaSuccess) return e;
  const long long ntiles = ngroups * nseg;
  const long long gc = ntiles * (CG::C / kCB);
  const long long gr = ntiles * (RG::R / 2 / RPR);
  if (gc > 0x7fffffffLL || gr > 0x7fffffffLL) return cudaErrorInvalidValue;
  kc<<<(unsigned)gc, CG::NT, smc, st>>>(data, data, lo, hi);
  kr<<<(unsigned)gr, RG::NT, smr, st>>>(data, hrow, nseg, lo, hi, wn1);
  ki<<<(unsigned)gc, CG::NT, smc, st>>>(data, data, lo, hi);
  return cudaGetLastError();
}

// row pass shape per MIX: (row pairs per CTA, register cap); the 3 x 3
// mixing at 2^15..2^16 points runs one row pair per CTA
template <int LOGR, int LOGC, int MBC, int MBR>
cudaError_t f3_run_mix(int mix, float* data, const float* hrow, long long ngroups, int nseg,
                       const cplx<float>* lo, const cplx<float>* hi, cplx<float> wn1,
                       cudaStream_t st) {
  constexpr bool big = LOGR + LOGC >= 15;
  if (mix)
    return f3_run<LOGR, LOGC, 1, MBC, big ? 1 : 2, big ? 2 * MBR : MBR>(data, hrow, ngroups, nseg,
                                                                       lo, hi, wn1, st);
  return f3_run<LOGR, LOGC, 0, MBC, 2, MBR + 1>(data, hrow, ngroups, nseg, lo, hi, wn1, st);
}

template <int LOGR, int LOGC>
cudaError_t f3_fwd1(const float* tod, float* scratch, cplx<float>* spec, long long ntiles,
                    long long batch, const cplx<float>* lo, const cplx<float>* hi, cplx<float> wn1,
                    cudaStream_t st) {
  using CG = f3::ColGeo<LOGR, LOGC, kCB1, 1>;
  using RG = f3::RowSpecGeo<LOGR, LOGC, kRP1>;
  auto kc = f3::k_f3_colfwd<LOGR, LOGC, kCB1, 1, kMB1>;
  auto kr = f3::k_f3_rowspec<LOGR, LOGC, kRP1, 4>;  // four CTAs per SM: 29.5 -> 28.4 us per 96 tiles
  const int smc = CG::SMEM * (int)sizeof(cplx<float>), smr = RG::SMEM * (int)sizeof(cplx<float>);
  cudaError_t e = set_smem(kc, smc);
  if (e == cudaSuccess) e = set_smem(kr, smr);
  if (e != cudaSuccess) return e;
  constexpr long long N = 2LL * CG::M;  // samples per tile
  for (long long t0 = 0; t0 < ntiles && e == cudaSuccess; t0 += batch) {
    const long long nb = ntiles - t0 < batch ? ntiles - t0 : batch;
    const long long gc = nb * (CG::C / kCB1), gr = nb * (RG::R / 2 / kRP1);
    if (gc > 0x7fffffffLL || gr > 0x7fffffffLL) return cudaErrorInvalidValue;
    kc<<<(unsigned)gc, CG::NT, smc, st>>>(tod + t0 * N, scratch, lo, hi);
    kr<<<(unsigned)gr, RG::NT, smr, st>>>(scratch, spec, t0, lo, hi, wn1);
    e = cudaGetLastError();
  }
  return e;
}

template <int LOGR, int LOGC, int MBC>
cudaError_t f3_inv3(const cplx<float>* gspec, float* data, long long ngroups, int nseg,
                    const cplx<float>* lo, const cplx<float>* hi, cplx<float> wn1, cudaStream_t st) {
  using CG = f3::ColGeo<LOGR, LOGC, kCB, 3>;
  using RG = f3::RowInGeo<LOGR, LOGC, kRP>;
  auto kr = f3::k_f3_rows_specin<LOGR, LOGC, kRP, 1>;
  auto ki = f3::k_f3_colinv<LOGR, LOGC, kCB, 3, MBC>;
  const int smc = CG::SMEM * (int)sizeof(cplx<float>), smr = RG::SMEM * (int)sizeof(cplx<float>);
  cudaError_t e = set_smem(ki, smc);
  if (e == cudaSuccess) e = set_smem(kr, smr);
  if (e != cudaSuccess) return e;
  const long long ntiles = ngroups * nseg;
  const long long gc = ntiles * (CG::C / kCB), gr = ntiles * (RG::R / 2 / kRP);
  if (gc > 0x7fffffffLL || gr > 0x7fffffffLL) return cudaErrorInvalidValue;
  kr<<<(unsigned)gr, RG::NT, smr, st>>>(gspec, data, nseg, lo, hi, wn1);
  ki<<<(unsigned)gc, CG::NT, smc, st>>>(data, data, lo, hi);
  return cudaGetLastError();
}

template <int LOGR, int LOGC>
cudaError_t f3_det(const float* x, float* y, float* scratch, const float* hpos, long long ntiles,
                   int nseg, long long batch, const cplx<float>* lo, const cplx<float>* hi,
                   cplx<float> wn1, cudaStream_t st) {
  // four tiles per row CTA (consecutive segments of one detector share the
  // filter row, staged once; one tile per CTA with the filter values read
  // from L2 measured the same, 2.57 against 2.64 ms at C2)
  constexpr int RS1 = 4;
  using CG = f3::ColGeo<LOGR, LOGC, kCB1, 1>;
  using RG = f3::Row1Geo<LOGR, LOGC, kRP1>;
  auto kc = f3::k_f3_colfwd<LOGR, LOGC, kCB1, 1, kMB1>;
  auto kr = f3::k_f3_rows1<LOGR, LOGC, kRP1, RS1, 3, true>;
  auto ki = f3::k_f3_colinv<LOGR, LOGC, kCB1, 1, kMB1>;
  const int smc = CG::SMEM * (int)sizeof(cplx<float>), smr = RG::SMEM * (int)sizeof(cplx<float>);
  cudaError_t e = set_smem(kc, smc);
  if (e == cudaSuccess) e = set_smem(ki, smc);
  if (e == cudaSuccess) e = set_smem(kr, smr);
  if (e != cudaSuccess) return e;
  constexpr long long N = 2LL * CG::M;
  for (long long t0 = 0; t0 < ntiles && e == cudaSuccess; t0 += batch) {
    const long long nb = ntiles - t0 < batch ? ntiles - t0 : batch;
    const long long gc = nb * (CG::C / kCB1), gr = (nb + RS1 - 1) / RS1 * (RG::R / 2 / kRP1);
    if (gc > 0x7fffffffLL || gr > 0x7fffffffLL) return cudaErrorInvalidValue;
    kc<<<(unsigned)gc, CG::NT, smc, st>>>(x + t0 * N, scratch, lo, hi);
    kr<<<(unsigned)gr, RG::NT, smr, st>>>(scratch, nb, t0, nseg, hpos, lo, hi, wn1);
    ki<<<(unsigned)gc, CG::NT, smc, st>>>(scratch, y + t0 * N, lo, hi);
    e = cudaGetLastError();
  }
  return e;
}

// (LOGR, LOGC) = (logm / 2, logm - logm / 2); register caps for three
// column CTAs and four row CTAs per SM, three where rows of 128 points would
// spill at four (uncapped, the row kernel took up to 158 registers at
// 2^13..2^15 points)
#define SG_F3_SHAPES(X) X(10, 5, 5, 3, 4) X(11, 5, 6, 3, 4) X(12, 6, 6, 3, 4) X(13, 6, 7, 3, 3) \
  X(14, 7, 7, 3, 3) X(15, 7, 8, 3, 4) X(16, 8, 8, 3, 4)

int f3_logr(int logm) { return logm / 2; }  // R = 2^(logm/2) <= C
}  // namespace

bool fft3_supported(int logm) { return logm >= 10 && logm <= 16; }

void fft3_pos_freq(int logm, std::vector<int>& kfreq) {
  const int M = 1 << logm, R = 1 << f3_logr(logm), C = M / R;
  kfreq.resize(M + 1);
  for (int pos = 0; pos < M; pos++) kfreq[pos] = pos / C + R * (pos % C);
  kfreq[M] = M;
}

cudaError_t fft3_group_weight(float* data, const float* hrow, int mix, long long ngroups, int nseg,
                              int logm, const cplx<float>* tw_lo, const cplx<float>* tw_hi,
                              cplx<float> wn1, cudaStream_t st) {
  if (!fft3_supported(logm) || ngroups < 1 || nseg < 1) return cudaErrorInvalidValue;
#define SG_F3_CASE(LM, LR, LC, MBC, MBR) \
  case LM:                              \
    return f3_run_mix<LR, LC, MBC, MBR>(mix, data, hrow, ngroups, nseg, tw_lo, tw_hi, wn1, st);
  switch (logm) { SG_F3_SHAPES(SG_F3_CASE) }
#undef SG_F3_CASE
  return cudaErrorInvalidValue;
}

// Tiles of 2M FP32 samples in 48 MB of scratch: a batch stays in L2 between
// its column and row passes.  (Batches rounded down to whole waves of the
// column kernels, 57 instead of 96 tiles of 131072 samples, were slower:
// C2 6.51 -> 6.62 ms, the per-detector filter 2.57 -> 2.77 ms.)
long long fft3_rhs_batch(int logm) { return std::max(1LL, (48LL << 20) / (8LL << logm)); }

cudaError_t fft3_forward_spectra(const float* tod, float* scratch, cplx<float>* spec,
                                 long long ntiles, long long batch, int logm,
                                 const cplx<float>* tw_lo, const cplx<float>* tw_hi,
                                 cplx<float> wn1, cudaStream_t st) {
  if (!fft3_supported(logm) || ntiles < 1 || batch < 1) return cudaErrorInvalidValue;
#define SG_F3_CASE(LM, LR, LC, MBC, MBR) \
  case LM:                              \
    return f3_fwd1<LR, LC>(tod, scratch, spec, ntiles, batch, tw_lo, tw_hi, wn1, st);
  switch (logm) { SG_F3_SHAPES(SG_F3_CASE) }
#undef SG_F3_CASE
  return cudaErrorInvalidValue;
}

cudaError_t fft3_detector_filter(const float* x, float* y, float* scratch, const float* hpos,
                                 long long ntiles, long long batch, int nseg, int logm,
                                 const cplx<float>* tw_lo, const cplx<float>* tw_hi,
                                 cplx<float> wn1, cudaStream_t st) {
  if (!fft3_supported(logm) || ntiles < 1 || nseg < 1 || batch < 1) return cudaErrorInvalidValue;
#define SG_F3_CASE(LM, LR, LC, MBC, MBR) \
  case LM:                              \
    return f3_det<LR, LC>(x, y, scratch, hpos, ntiles, nseg, batch, tw_lo, tw_hi, wn1, st);
  switch (logm) { SG_F3_SHAPES(SG_F3_CASE) }
#undef SG_F3_CASE
  return cudaErrorInvalidValue;
}

cudaError_t fft3_inverse_from_spectra(const cplx<float>* gspec, float* data, long long ngroups,
                                      int nseg, int logm, const cplx<float>* tw_lo,
                                      const cplx<float>* tw_hi, cplx<float> wn1, cudaStream_t st) {
  if (!fft3_supported(logm) || ngroups < 1 || nseg < 1) return cudaErrorInvalidValue;
#define SG_F3_CASE(LM, LR, LC, MBC, MBR) \
  case LM:                              \
    return f3_inv3<LR, LC, MBC>(gspec, data, ngroups, nseg, tw_lo, tw_hi, wn1, st);
  switch (logm) { SG_F3_SHAPES(SG_F3_CASE) }
#undef SG_F3_CASE
  return cudaErrorInvalidValue;
}

}  // namespace sg
