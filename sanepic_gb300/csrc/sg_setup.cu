// sg_setup.cu -- one-time setup kernels: observed-pixel compaction (indpix),
// the pixel-sorted sample index (CSR) used by the deterministic P^T, hit
// counts, cross-link sums and the two preconditioners.
//
// Reference counterparts: pixon/indpix sanepic.cc:828-915, hits 2613-2626,
// sumCross 2594-2597, compute_diagPtNPCorr 2680-2762.  The 3x3 block-Jacobi
// preconditioner has no reference counterpart.
#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include "sg_healpix.h"
#include "sg_kernels.h"

namespace sg {

static unsigned grid_for(long long n, int threads, long long cap = 152LL * 32) {
  long long b = (n + threads - 1) / threads;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

// detector samples per RING pixel: each group sample counts once per member
// detector (integer atomics: the result does not depend on their order)
__global__ void k_hist(const int* ring_pix, long long n, long long nsd, const int* gsize,
                       int* count) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int p = ring_pix[i];
    if (p >= 0) atomicAdd(count + p, gsize[i / nsd]);
  }
}

cudaError_t hist_launch(const int* ring_pix, long long n, long long nsd, const int* gsize,
                        int* count, cudaStream_t st) {
  k_hist<<<grid_for(n, 256), 256, 0, st>>>(ring_pix, n, nsd, gsize, count);
  return cudaGetLastError();
}

__global__ void k_compact(const int* ring_pix, const int* indpix, long long n, int* pix) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    pix[i] = indpix[ring_pix[i]];
}

cudaError_t compact_launch(const int* ring_pix, const int* indpix, long long n, int* pix,
                           cudaStream_t st) {
  k_compact<<<grid_for(n, 256), 256, 0, st>>>(ring_pix, indpix, n, pix);
  return cudaGetLastError();
}

__global__ void k_hits(const int* count, const int* indpix, long long npixfull, int* hits) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npixfull;
       i += (long long)gridDim.x * blockDim.x) {
    const int m = indpix[i];
    if (m >= 0) hits[m] = count[i];
  }
}

cudaError_t hits_launch(const int* count, const int* indpix, long long npixfull, int* hits,
                        cudaStream_t st) {
  k_hits<<<grid_for(npixfull, 256), 256, 0, st>>>(count, indpix, npixfull, hits);
  return cudaGetLastError();
}

// full[int2ring[m]] = compact[m]: a compact map into the full-sky RING map
// (the caller zeroes full first; unobserved pixels stay 0)
__global__ void k_expand(const double* __restrict__ compact, const long long* __restrict__ i2r,
                         long long npix, double* __restrict__ full) {
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < npix;
       m += (long long)gridDim.x * blockDim.x)
    full[i2r[m]] = compact[m];
}

cudaError_t expand_launch(const double* compact, const long long* i2r, long long npix,
                          double* full, cudaStream_t st) {
  k_expand<<<grid_for(npix, 256), 256, 0, st>>>(compact, i2r, npix, full);
  return cudaGetLastError();
}

// ---- pixel numbering -------------------------------------------------------
// The reference's indpix (rank of each observed pixel in ascending RING order,
// sanepic.cc:904-915) and the library's internal numbering (rank in NESTED
// order when nside is a power of two, else RING order), by two exclusive
// scans instead of a host sort.
__global__ void k_obs(const int* count, long long n, int* flag) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x)
    flag[p] = count[p] != 0;
}

__global__ void k_nest_mark(const int* count, long long n, long long nside, int nested,
                            int* mark, int* ring_of) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    if (count[p] == 0) continue;
    const long long q = nested ? hp_ring2nest_int(nside, p) : p;
    mark[q] = 1;
    ring_of[q] = (int)p;
  }
}

// internal index m of the q-th marked nested pixel; indpix in both orders
__global__ void k_number(const int* count, const int* mark, const int* mrank, const int* ring_of,
                         const int* rrank, long long n, long long* int2ring,
                         long long* int2ringc, int* indpix_int, int* indpix_ring) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    indpix_ring[q] = count[q] != 0 ? rrank[q] : -1;
    if (!mark[q]) continue;
    const int m = mrank[q], p = ring_of[q];
    int2ring[m] = p;
    int2ringc[m] = rrank[p];
    indpix_int[p] = m;
  }
}

__global__ void k_total(const int* flag, const int* rank, long long n, int* total) {
  *total = n > 0 ? rank[n - 1] + flag[n - 1] : 0;
}

size_t numbering_tmp_bytes(long long n) {
  size_t scan = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, scan, (const int*)nullptr, (int*)nullptr, (int)n);
  return 5 * sizeof(int) * (size_t)n + scan + 256;
}

cudaError_t numbering_launch(const int* count, long long n, long long nside, int nested,
                             long long* int2ring, long long* int2ringc, int* indpix_int,
                             int* indpix_ring, int* npix, void* tmp, size_t tmp_bytes,
                             cudaStream_t st) {
  int* flag = reinterpret_cast<int*>(tmp);
  int* rrank = flag + n;
  int* mark = rrank + n;
  int* mrank = mark + n;
  int* ring_of = mrank + n;
  void* scan_tmp = ring_of + n;
  size_t scan_bytes = tmp_bytes - 5 * sizeof(int) * (size_t)n;
  const unsigned g = grid_for(n, 256);
  cudaError_t e = cudaMemsetAsync(mark, 0, sizeof(int) * n, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(indpix_int, 0xff, sizeof(int) * n, st);
  if (e != cudaSuccess) return e;
  k_obs<<<g, 256, 0, st>>>(count, n, flag);
  k_nest_mark<<<g, 256, 0, st>>>(count, n, nside, nested, mark, ring_of);
  e = cub::DeviceScan::ExclusiveSum(scan_tmp, scan_bytes, flag, rrank, (int)n, st);
  if (e == cudaSuccess) e = cub::DeviceScan::ExclusiveSum(scan_tmp, scan_bytes, mark, mrank, (int)n, st);
  if (e != cudaSuccess) return e;
  k_number<<<g, 256, 0, st>>>(count, mark, mrank, ring_of, rrank, n, int2ring, int2ringc,
                              indpix_int, indpix_ring);
  k_total<<<1, 1, 0, st>>>(flag, rrank, n, npix);
  return cudaGetLastError();
}

// *flag = 1 if any entry is negative (NaN pointing leaves -1)
__global__ void k_any_negative(const int* v, long long n, int* flag) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    if (v[i] < 0) {
      *flag = 1;
      return;
    }
}

cudaError_t any_negative_launch(const int* v, long long n, int* flag, cudaStream_t st) {
  k_any_negative<<<grid_for(n, 256), 256, 0, st>>>(v, n, flag);
  return cudaGetLastError();
}

// *flag = 1 if any entry is NaN
__global__ void k_any_nan(const double* v, long long n, int* flag) {
  bool nan = false;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    nan |= !(v[i] > 0) && !(v[i] <= 0.0);
  if (__any_sync(0xffffffffu, nan) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

cudaError_t any_nan_launch(const double* v, long long n, int* flag, cudaStream_t st) {
  k_any_nan<<<grid_for(n, 256), 256, 0, st>>>(v, n, flag);
  return cudaGetLastError();
}

// ---- CSR: samples sorted by (pixel, sample index) ---------------------------
// Keys (pixel << 32 | sample) are unique, so the order is fully determined.
__global__ void k_make_keys(const int* pix, long long n, unsigned long long* keys) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    keys[i] = ((unsigned long long)(unsigned)pix[i] << 32) | (unsigned long long)i;
}

__global__ void k_keys_to_idx(const unsigned long long* keys, long long n, uint32_t* idx) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    idx[i] = (uint32_t)(keys[i] & 0xffffffffULL);
}

static int bits_for(long long v) {
  int b = 0;
  while ((1LL << b) <= v) b++;
  return b;
}

size_t csr_tmp_bytes(long long n, long long npix) {
  (void)npix;
  size_t sort_bytes = 0;
  cub::DoubleBuffer<unsigned long long> db(nullptr, nullptr);
  cub::DeviceRadixSort::SortKeys(nullptr, sort_bytes, db, n, 0, 64);
  return 2 * sizeof(unsigned long long) * (size_t)n + sort_bytes + 1024;
}

// row starts of the CSR: the first sorted key of every pixel (every observed
// pixel has at least one sample, so every entry is written)
__global__ void k_offsets(const unsigned long long* keys, long long n, long long npix,
                          long long* off) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n;
       j += (long long)gridDim.x * blockDim.x) {
    const long long p = (long long)(keys[j] >> 32);
    if (j == 0 || (long long)(keys[j - 1] >> 32) != p) off[p] = j;
    if (j == n - 1) off[npix] = n;
  }
}

cudaError_t csr_build(const int* pix, long long n, long long npix,
                      long long* csr_off, uint32_t* csr_idx, void* tmp, size_t tmp_bytes,
                      cudaStream_t st) {
  char* base = reinterpret_cast<char*>(tmp);
  unsigned long long* k0 = reinterpret_cast<unsigned long long*>(base);
  unsigned long long* k1 = k0 + n;
  char* cub_tmp = reinterpret_cast<char*>(k1 + n);
  size_t cub_bytes = tmp_bytes - 2 * sizeof(unsigned long long) * (size_t)n;
  k_make_keys<<<grid_for(n, 256), 256, 0, st>>>(pix, n, k0);
  cub::DoubleBuffer<unsigned long long> db(k0, k1);
  const int nbits = 32 + bits_for(npix);
  cudaError_t e = cub::DeviceRadixSort::SortKeys(cub_tmp, cub_bytes, db, n, 0, nbits, st);
  if (e != cudaSuccess) return e;
  k_keys_to_idx<<<grid_for(n, 256), 256, 0, st>>>(db.Current(), n, csr_idx);
  k_offsets<<<grid_for(n, 256), 256, 0, st>>>(db.Current(), n, npix, csr_off);
  return cudaGetLastError();
}

template <typename T>
__global__ void k_gather_cs(const T* cs, const uint32_t* idx, long long n, T* out) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n;
       j += (long long)gridDim.x * blockDim.x) {
    const long long i = idx[j];
    out[2 * j] = cs[2 * i];
    out[2 * j + 1] = cs[2 * i + 1];
  }
}

template <typename T>
cudaError_t gather_cs_launch(const T* cs, const uint32_t* csr_idx, long long n, T* csr_cs,
                             cudaStream_t st) {
  k_gather_cs<T><<<grid_for(n, 256), 256, 0, st>>>(cs, csr_idx, n, csr_cs);
  return cudaGetLastError();
}
template cudaError_t gather_cs_launch<float>(const float*, const uint32_t*, long long, float*,
                                             cudaStream_t);
template cudaError_t gather_cs_launch<double>(const double*, const uint32_t*, long long,
                                              double*, cudaStream_t);

// cos/sin of twice the group's base angle phi per group sample, rounded to T:
// phi = psi_o, or with a half-wave plate phi = -psi_o + 2 omega (ii + ns iseg)
// (sanepic.cc:757-766); the detector's own angle is applied as a rotation.
// For FP32 storage the FP64 angle is first reduced modulo 2pi (exact fmod)
// so that HWP angles of ~1e6 rad stay on the fast path.
// Without a half-wave plate the cross-link sums below need cos/sin of the
// same 2 psi_o in FP64: with cs64 set they are stored there too (one FP64
// sincos per sample serves both where the arguments agree bit for bit).
template <typename T>
__global__ void k_base_angles(const double* psio, long long n, long long ns, long long nsd,
                              int hwp, double omega, T* cs, double2* cs64) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double phi = psio[i];
    double s0 = 0.0, c0 = 0.0, araw = 0.0;
    if (cs64) {  // the cross-link argument, 2 (psi_o + 0)
      araw = 2.0 * (phi + 0.0);
      sincos(araw, &s0, &c0);
      cs64[i] = make_double2(c0, s0);
    }
    if (hwp) phi = -phi + 2.0 * omega * (double)(i % nsd);  // i % nsd = ii + ns * iseg
    double a = 2.0 * phi;
    if (sizeof(T) == 4) a = fmod(a, 6.2831853071795864769252867665590057683943387987502);
    double s, c;
    if (cs64 && __double_as_longlong(a) == __double_as_longlong(araw)) {
      s = s0;
      c = c0;
    } else {
      sincos(a, &s, &c);
    }
    cs[2 * i] = (T)c;
    cs[2 * i + 1] = (T)s;
  }
}

template <typename T>
cudaError_t base_angles_launch(const double* psio, long long n, long long ns, long long nsd,
                               int hwp, double omega, T* cs, double* cs64, cudaStream_t st) {
  (void)ns;
  k_base_angles<T><<<grid_for(n, 256), 256, 0, st>>>(psio, n, ns, nsd, hwp, omega, cs,
                                                     reinterpret_cast<double2*>(cs64));
  return cudaGetLastError();
}
template cudaError_t base_angles_launch<float>(const double*, long long, long long, long long,
                                               int, double, float*, double*, cudaStream_t);
template cudaError_t base_angles_launch<double>(const double*, long long, long long, long long,
                                                int, double, double*, double*, cudaStream_t);

// ---- per-pixel reductions over the CSR (one warp per pixel) -----------------
// COS2P/SIN2P (sanepic.cc:2594-2597): per pixel, the sum over detector
// samples of cos/sin(2 (psi_o + psi_det)).  Per group sample that is
// cos 2psi_o SC - sin 2psi_o SS (and sin 2psi_o SC + cos 2psi_o SS) with
// SC, SS the group's sums of cos/sin(2 psi_det).  FP64, warp per pixel.
// With tab set, cos/sin of 2 psi_o come from the table the base-angle pass
// filled (the same FP64 values) instead of one sincos per sample here.
__global__ void k_sumcross(const long long* off, const uint32_t* idx, const double* psio,
                           const double2* tab, long long nsd, const double* gsc,
                           const double* gss, long long npix, double* out) {
  const int lane = threadIdx.x & 31;
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long m = warp; m < npix; m += nwarps) {
    double c = 0.0, s = 0.0;
    for (long long j = off[m] + lane; j < off[m + 1]; j += 32) {
      const long long gs = idx[j];
      const int g = (int)(gs / nsd);
      double sn, cs;
      if (tab) {
        const double2 t = tab[gs];
        cs = t.x;
        sn = t.y;
      } else {
        sincos(2.0 * (psio[gs] + 0.0), &sn, &cs);
      }
      c += cs * gsc[g] - sn * gss[g];
      s += sn * gsc[g] + cs * gss[g];
    }
    for (int o = 16; o > 0; o >>= 1) {
      c += __shfl_xor_sync(0xffffffffu, c, o);
      s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    if (lane == 0) {
      out[m] = c;
      out[npix + m] = s;
      out[2 * npix + m] = 0.0;
    }
  }
}

cudaError_t sumcross_launch(const long long* csr_off, const uint32_t* csr_idx, const double* psio,
                            const double* tab, long long nsd, const double* gsc, const double* gss,
                            long long npix, double* sumcross, cudaStream_t st) {
  k_sumcross<<<grid_for(npix * 32, 256, 152LL * 64), 256, 0, st>>>(
      csr_off, csr_idx, psio, reinterpret_cast<const double2*>(tab), nsd, gsc, gss, npix,
      sumcross);
  return cudaGetLastError();
}

// 3x3 block-Jacobi: A_p = sum over detector samples of g0_det w w^T,
// w = (1, cos 2a, sin 2a), a = phi + delta_det.  Summed over a group's
// detectors in closed form from five group constants
//   gc = (sum g0, sum g0 cos 2d, sum g0 sin 2d, sum g0 cos 4d, sum g0 sin 4d)
// with cos^2 = (1 + cos 4a)/2, cos sin = sin 4a / 2.  Inverse in FP64.
template <typename T>
struct pair_of;
template <>
struct pair_of<float> {
  using type = float2;
};
template <>
struct pair_of<double> {
  using type = double2;
};

// Reciprocal condition number lambda_min / lambda_max of the symmetric 3 x 3
// matrix (a0 a1 a2; a1 a3 a4; a2 a4 a5), its eigenvalues from the
// trigonometric closed form for symmetric 3 x 3 matrices (O. K. Smith,
// "Eigenvalues of a symmetric 3 x 3 matrix", CACM 4(4), 1961).
__device__ double sym3_rcond(const double* a) {
  const double p1 = a[1] * a[1] + a[2] * a[2] + a[4] * a[4];
  const double q = (a[0] + a[3] + a[5]) / 3.0;
  const double d0 = a[0] - q, d1 = a[3] - q, d2 = a[5] - q;
  const double p2 = d0 * d0 + d1 * d1 + d2 * d2 + 2.0 * p1;
  if (!(q > 0.0)) return 0.0;
  if (p2 <= 0.0) return 1.0;  // a multiple of the identity
  const double p = sqrt(p2 / 6.0), ip = 1.0 / p;
  // B = (A - q I) / p, r = det(B) / 2
  const double b0 = d0 * ip, b1 = a[1] * ip, b2 = a[2] * ip, b3 = d1 * ip, b4 = a[4] * ip,
               b5 = d2 * ip;
  double r = 0.5 * (b0 * (b3 * b5 - b4 * b4) - b1 * (b1 * b5 - b4 * b2) + b2 * (b1 * b4 - b3 * b2));
  r = fmin(1.0, fmax(-1.0, r));
  const double phi = acos(r) / 3.0;
  const double lmax = q + 2.0 * p * cos(phi);
  const double lmin = q + 2.0 * p * cos(phi + 2.0943951023931954923);  // + 2 pi / 3
  return lmax > 0.0 ? fmax(lmin, 0.0) / lmax : 0.0;
}

// A team of L lanes per pixel (256 / L pixels per block), each lane taking
// its samples j, j + L, ... four at a time with the loads of all four in
// flight; FP64 sums, combined over the team with a fixed xor tree.
// A pixel's Q/U are masked when hits[m] < 2 (the reference's rule) or, with
// rcond_min > 0, when its block's reciprocal condition number is below
// rcond_min; polmask_out (optional) receives hits[m], or min(hits[m], 1)
// where the block is masked; minv (optional) the inverse blocks.
template <typename T, int L>
__global__ void __launch_bounds__(256)
    k_bj3(const long long* off, const uint32_t* idx, const T* ccs, long long npix, uint32_t nsd,
          int ngroups, const double* gc, const int* hits, double rcond_min, int* polmask_out,
          double* minv) {
  using P2 = typename pair_of<T>::type;
  constexpr int U = 4;
  const int lane = threadIdx.x % L;
  const long long m = (long long)blockIdx.x * (256 / L) + threadIdx.x / L;
  const P2* cs2 = reinterpret_cast<const P2*>(ccs);
  double a[6] = {0, 0, 0, 0, 0, 0};
  if (m < npix) {
    const long long jend = off[m + 1];
    for (long long j = off[m] + lane; j < jend; j += L * U) {
      int g[U];
      P2 w[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const long long k = j + L * u;
        const bool in = k < jend;
        g[u] = (in && ngroups > 1) ? (int)(idx[k] / nsd) : 0;
        w[u] = in ? cs2[k] : P2{};
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        if (j + L * u >= jend) break;
        const int gg = g[u];
        const double G0 = gc[gg], G2c = gc[ngroups + gg], G2s = gc[2 * ngroups + gg];
        const double G4c = gc[3 * ngroups + gg], G4s = gc[4 * ngroups + gg];
        const double c2 = (double)w[u].x, s2 = (double)w[u].y;
        const double c4 = c2 * c2 - s2 * s2, s4 = 2.0 * c2 * s2;
        const double C4 = c4 * G4c - s4 * G4s, S4 = s4 * G4c + c4 * G4s;
        a[0] += G0;
        a[1] += c2 * G2c - s2 * G2s;
        a[2] += s2 * G2c + c2 * G2s;
        a[3] += 0.5 * (G0 + C4);
        a[4] += 0.5 * S4;
        a[5] += 0.5 * (G0 - C4);
      }
    }
  }
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < 6; k++) a[k] += __shfl_xor_sync(0xffffffffu, a[k], o);
  if (lane == 0 && m < npix) {
    bool pol = hits[m] >= 2;
    if (pol && rcond_min > 0.0) pol = sym3_rcond(a) >= rcond_min;
    if (polmask_out) polmask_out[m] = pol ? hits[m] : min(hits[m], 1);
    if (!minv) return;
    double o6[6] = {0, 0, 0, 0, 0, 0};
    if (!pol) {
      o6[0] = a[0] != 0.0 ? 1.0 / a[0] : 0.0;
    } else {
      const double c00 = a[3] * a[5] - a[4] * a[4];
      const double c01 = a[2] * a[4] - a[1] * a[5];
      const double c02 = a[1] * a[4] - a[2] * a[3];
      const double c11 = a[0] * a[5] - a[2] * a[2];
      const double c12 = a[1] * a[2] - a[0] * a[4];
      const double c22 = a[0] * a[3] - a[1] * a[1];
      const double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
      const double scale = a[0] * a[0] * a[0];
      if (!(det > 1e-12 * scale)) {
        o6[0] = 1.0 / a[0];
        o6[3] = a[3] > 0.0 ? 1.0 / a[3] : 0.0;
        o6[5] = a[5] > 0.0 ? 1.0 / a[5] : 0.0;
      } else {
        const double id = 1.0 / det;
        o6[0] = c00 * id;
        o6[1] = c01 * id;
        o6[2] = c02 * id;
        o6[3] = c11 * id;
        o6[4] = c12 * id;
        o6[5] = c22 * id;
      }
    }
#pragma unroll
    for (int k = 0; k < 6; k++) minv[k * npix + m] = o6[k];
  }
}

template <typename T, int L>
static void bj3_team(const long long* csr_off, const uint32_t* csr_idx, const T* csr_cs,
                     long long npix, long long nsd, int ngroups, const double* gconst,
                     const int* hits_true, double rcond_min, int* polmask_out, double* minv,
                     cudaStream_t st) {
  const long long blocks = (npix + 256 / L - 1) / (256 / L);
  k_bj3<T, L><<<(unsigned)blocks, 256, 0, st>>>(csr_off, csr_idx, csr_cs, npix, (uint32_t)nsd,
                                                 ngroups, gconst, hits_true, rcond_min,
                                                 polmask_out, minv);
}

template <typename T>
cudaError_t bj3_launch(const long long* csr_off, const uint32_t* csr_idx, const T* csr_cs,
                       long long npix, long long nsd, int ngroups, const double* gconst,
                       const int* hits_true, double rcond_min, int* polmask_out, double* minv,
                       cudaStream_t st) {
  if (npix <= 0) return cudaSuccess;
#define SG_BJ3_TEAM(L)                                                                       \
  bj3_team<T, L>(csr_off, csr_idx, csr_cs, npix, nsd, ngroups, gconst, hits_true, rcond_min, \
                 polmask_out, minv, st)
  switch (pt_lanes((long long)ngroups * nsd, npix)) {  // every group sample is in the CSR
    case 1: SG_BJ3_TEAM(1); break;
    case 2: SG_BJ3_TEAM(2); break;
    case 4: SG_BJ3_TEAM(4); break;
    case 8: SG_BJ3_TEAM(8); break;
    case 16: SG_BJ3_TEAM(16); break;
    default: SG_BJ3_TEAM(32); break;
  }
#undef SG_BJ3_TEAM
  return cudaGetLastError();
}
template cudaError_t bj3_launch<float>(const long long*, const uint32_t*, const float*, long long,
                                       long long, int, const double*, const int*, double, int*,
                                       double*, cudaStream_t);
template cudaError_t bj3_launch<double>(const long long*, const uint32_t*, const double*,
                                        long long, long long, int, const double*, const int*,
                                        double, int*, double*, cudaStream_t);

// N_ of every detector summed over its group: the pixel stream is common to
// the group, so the reference's per-detector pair sums add up per group.
template <typename T>
__global__ void k_group_ntab(const T* ntab, long long ns, int ngroups, const int* grp_off,
                             const int* grp_det, T* out) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ns * ngroups;
       e += (long long)gridDim.x * blockDim.x) {
    const int g = (int)(e / ns);
    const long long t = e % ns;
    double acc = 0.0;
    for (int m = grp_off[g]; m < grp_off[g + 1]; m++) acc += (double)ntab[grp_det[m] * ns + t];
    out[e] = (T)acc;
  }
}

template <typename T>
cudaError_t group_ntab_launch(const T* ntab, long long ns, int ngroups, const int* grp_off,
                              const int* grp_det, T* out, cudaStream_t st) {
  k_group_ntab<T><<<grid_for(ns * ngroups, 256), 256, 0, st>>>(ntab, ns, ngroups, grp_off,
                                                              grp_det, out);
  return cudaGetLastError();
}
template cudaError_t group_ntab_launch<float>(const float*, long long, int, const int*,
                                              const int*, float*, cudaStream_t);
template cudaError_t group_ntab_launch<double>(const double*, long long, int, const int*,
                                               const int*, double*, cudaStream_t);

// Reference diagonal: for every tile and pixel, sum over sample pairs (i, j)
// of that pixel in the tile with |i - j| < ns/2 of N_[|i - j|], N_ = c2r|SpN|
// (sanepic.cc:2698-2752).  The reference adds it twice (Q1) and sets the Q/U
// blocks to I/2 (sanepic.cc:2561-2565).  One thread per pixel; the sample
// list is sorted by sample index, so a tile's samples are contiguous.
template <typename T>
__global__ void k_diag(const long long* off, const uint32_t* idx, long long npix, long long ns,
                       int nseg, const T* ntab, double* Mp) {
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < npix;
       m += (long long)gridDim.x * blockDim.x) {
    double acc = 0.0;
    long long j0 = off[m];
    const long long jend = off[m + 1];
    while (j0 < jend) {
      const long long tile = idx[j0] / ns;
      long long j1 = j0;
      while (j1 < jend && (long long)(idx[j1] / ns) == tile) j1++;
      const T* nt = ntab + (tile / nseg) * ns;
      for (long long a = j0; a < j1; a++) {
        const long long ia = idx[a] % ns;
        for (long long b = j0; b < j1; b++) {
          const long long ib = idx[b] % ns;
          const long long dd = ia > ib ? ia - ib : ib - ia;
          if (dd < ns / 2) acc += (double)nt[dd];
        }
      }
      j0 = j1;
    }
    Mp[m] = 2.0 * acc;
    Mp[npix + m] = acc;
    Mp[2 * npix + m] = acc;
  }
}

template <typename T>
cudaError_t diag_launch(const long long* csr_off, const uint32_t* csr_idx, long long npix,
                        long long ns, int nseg, const T* ntab, double* Mp, cudaStream_t st) {
  k_diag<T><<<grid_for(npix, 128), 128, 0, st>>>(csr_off, csr_idx, npix, ns, nseg, ntab, Mp);
  return cudaGetLastError();
}
template cudaError_t diag_launch<float>(const long long*, const uint32_t*, long long, long long,
                                        int, const float*, double*, cudaStream_t);
template cudaError_t diag_launch<double>(const long long*, const uint32_t*, long long,
                                         long long, int, const double*, double*, cudaStream_t);

// ---- timeline ingest (sg_set_tod) ---------------------------------------------
// out = (T) in; any NaN sets *nan_flag (the patch below then runs)
template <typename T>
__global__ void k_ingest(const double* __restrict__ in, long long n, T* __restrict__ out,
                         int* nan_flag) {
  bool nan = false;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = in[i];
    nan |= !(v > 0) && !(v <= 0.0);
    out[i] = (T)v;
  }
  if (__any_sync(0xffffffffu, nan) && (threadIdx.x & 31) == 0) atomicOr(nan_flag, 1);
}

// four samples per thread, 16-byte loads (in and out 16-byte aligned, n % 4 == 0):
// fewer, larger requests, which matters when `in` is host memory read over
// the CPU-GPU link
template <typename T>
__global__ void k_ingest4(const double2* __restrict__ in, long long n4, T* __restrict__ out,
                          int* nan_flag) {
  bool nan = false;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4;
       i += (long long)gridDim.x * blockDim.x) {
    const double2 a = in[2 * i], b = in[2 * i + 1];
    nan |= !(a.x > 0) && !(a.x <= 0.0);
    nan |= !(a.y > 0) && !(a.y <= 0.0);
    nan |= !(b.x > 0) && !(b.x <= 0.0);
    nan |= !(b.y > 0) && !(b.y <= 0.0);
    out[4 * i] = (T)a.x;
    out[4 * i + 1] = (T)a.y;
    out[4 * i + 2] = (T)b.x;
    out[4 * i + 3] = (T)b.y;
  }
  if (__any_sync(0xffffffffu, nan) && (threadIdx.x & 31) == 0) atomicOr(nan_flag, 1);
}

template <typename T>
cudaError_t ingest_launch(const double* in, long long n, T* out, int* nan_flag, cudaStream_t st) {
  if (n % 4 == 0 && (reinterpret_cast<uintptr_t>(in) & 15) == 0) {
    const long long b = (n / 4 + 255) / 256;
    k_ingest4<T><<<(int)(b < 8192 ? b : 8192), 256, 0, st>>>(
        reinterpret_cast<const double2*>(in), n / 4, out, nan_flag);
    return cudaGetLastError();
  }
  const long long b = (n + 255) / 256;
  k_ingest<T><<<(int)(b < 4096 ? b : 4096), 256, 0, st>>>(in, n, out, nan_flag);
  return cudaGetLastError();
}
template cudaError_t ingest_launch<float>(const double*, long long, float*, int*, cudaStream_t);
template cudaError_t ingest_launch<double>(const double*, long long, double*, int*, cudaStream_t);

// One detector's filter row from its iSpf values (sanepic.cc:524-538):
// h[k] = iSpf[(long)(k / nssp * ns)] / ns / ns for k = 0..M, h[0] replaced by
// iSpf[1] 1e-6 / ns / ns; part[block] = this block's share of
// g0 = h[0] + 2 sum_{0<k<M} h[k] + h[M] (the diagonal of the circulant N^-1).
template <typename T>
__global__ void __launch_bounds__(256)
    k_noise_row(const double* __restrict__ ispf, long long nssp, long long ns, T* __restrict__ row,
                double* part) {
  const long long M = ns / 2;
  const double dns = (double)ns;
  double g = 0.0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k <= M;
       k += (long long)gridDim.x * blockDim.x) {
    const long long idx = (long long)((double)k / (double)nssp * dns);
    const double h = k == 0 ? ispf[1] * 1e-6 / dns / dns : ispf[idx] / dns / dns;
    row[k] = (T)h;
    g += (k == 0 || k == M) ? h : 2.0 * h;
  }
  __shared__ double sh[8];
  for (int o = 16; o > 0; o >>= 1) g += __shfl_xor_sync(0xffffffffu, g, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = g;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; w++) t += sh[w];
    part[blockIdx.x] = t;
  }
}

__global__ void k_sum_parts(const double* part, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < n; i++) t += part[i];
    *out = t;
  }
}

template <typename T>
cudaError_t noise_row_launch(const double* ispf, long long nssp, long long ns, T* row, double* g0,
                             double* part, cudaStream_t st) {
  k_noise_row<T><<<kNoiseRowBlocks, 256, 0, st>>>(ispf, nssp, ns, row, part);
  k_sum_parts<<<1, 32, 0, st>>>(part, kNoiseRowBlocks, g0);
  return cudaGetLastError();
}
template cudaError_t noise_row_launch<float>(const double*, long long, long long, float*, double*,
                                             double*, cudaStream_t);
template cudaError_t noise_row_launch<double>(const double*, long long, long long, double*,
                                              double*, double*, cudaStream_t);

// a NaN sample takes the previous sample's value, within each segment, in
// sample order (sanepic.cc:784-790): one thread walks one segment
template <typename T>
__global__ void k_nan_patch(T* v, long long ns, long long nseg) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= nseg) return;
  T* s = v + g * ns;
  for (long long i = 1; i < ns; i++)
    if (isnan(s[i])) s[i] = s[i - 1];
}

template <typename T>
cudaError_t nan_patch_launch(T* v, long long ns, long long nseg, cudaStream_t st) {
  k_nan_patch<T><<<(int)((nseg + 63) / 64), 64, 0, st>>>(v, ns, nseg);
  return cudaGetLastError();
}
template cudaError_t nan_patch_launch<float>(float*, long long, long long, cudaStream_t);
template cudaError_t nan_patch_launch<double>(double*, long long, long long, cudaStream_t);

}  // namespace sg
