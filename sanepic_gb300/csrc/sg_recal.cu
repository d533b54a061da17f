// sg_recal.cu -- detector gains and their fit: the recalibration loop of the
// reference (-r, -R; sanepic.cc:1041-1130, 2123-2316, MPI_compute_chi2
// 3206-3260) on the GPU operator.
//
// Model: d = g P m + n with one gain g per (detector, segment) tile.  The
// map is made with the gains of the previous fit, A = P^T G N^-1 G P and
// b = P^T G N^-1 d (the reference divides the data by g and multiplies the
// noise weights by g^2, sanepic.cc:1044-1053, 2545; the same system), and
// the gains are then refitted with the map held fixed, tile by tile:
//     g = s^T N^-1 d / s^T N^-1 s,   s = P m,
// the weighted least-squares gain of sanepic.cc:2166-2226 (relCalib =
// sPNd / cPNPc); with -R one gain per detector from the sums over its
// segments (zeta_all / gamma_all, sanepic.cc:2254-2271).  The mean gain is
// then held at the mean of the gains the map was made with: the map and the
// gains are only determined up to a common factor, which the reference's
// absrecal sets (sanepic.cc:2157-2159, 2281-2291).
//
// What differs from the reference on purpose (its -r does not run: each fit
// quadruples the gains and the CG of the next loop diverges, and without -R
// absrecal turns NaN):
//  * sPNd carries a factor 2 and cPNPc a factor 1/2 (sanepic.cc:2196-2201,
//    2217-2220), so each of its fits returns four times the gain; here both
//    sums carry the same factor (below);
//  * absrecal divides by gamma_all, which only -R fills (997-998, 2254-2271):
//    here the mean of the new gains is scaled to the mean of the old ones in
//    closed form instead of its fixed-point reruns;
//  * the data are divided by relCalib[idet + iseg + iseg_min * ndet]
//    (sanepic.cc:1049-1052), an index unlike the tile's own
//    idet + (iseg + iseg_min) * ndet used everywhere else: here every tile
//    uses its own gain;
//  * the orbital dipole (-o, fodipole) is taken as zero.
// The sums are the reference's half-spectrum sums with one factor on both,
//     b = 2 sum_{k <= ns/2} Re(D_k conj S_k) SpN_k,  c = 2 sum |S_k|^2 SpN_k,
// formed in the time domain: (N^-1 s)^T d is the same sum with bins 0 and
// ns/2 counted once, so b = (N^-1 d)^T s + SpN_0 S_0 D_0 + SpN_M S_M D_M
// with S_0 = sum s_i and S_M = sum (-1)^i s_i (likewise c); no spectrum is
// stored.  chi^2 before and after the fit is the reference's (2 sum over the
// half spectrum of |F(d - g s)|^2 SpN, sanepic.cc:3228-3246), from the noise
// filter's own chi^2 sums.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "sanepic_gpu.h"
#include "sg_ctx.h"
#include "sg_kernels.h"

namespace sg {
namespace {

constexpr int kRT = 256;

template <typename T>
__global__ void __launch_bounds__(kRT) k_tile_scale(T* __restrict__ y, const T* __restrict__ tsc,
                                                   long long ns, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] *= tsc[i / ns];
}

// one block per tile; FP64 products, a fixed per-thread order and a fixed tree
template <typename T>
__global__ void __launch_bounds__(kRT) k_tile_dots(const T* __restrict__ a,
                                                  const T* __restrict__ b, long long ns,
                                                  double* __restrict__ out) {
  const long long t = blockIdx.x;
  const T* pa = a + t * ns;
  const T* pb = b + t * ns;
  double s = 0.0;
  for (long long i = threadIdx.x; i < ns; i += kRT) s += (double)pa[i] * (double)pb[i];
  __shared__ double sh[kRT / 32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int w = 0; w < kRT / 32; w++) tot += sh[w];
    out[t] = tot;
  }
}

// out[2 t] = sum of the tile's samples, out[2 t + 1] = sum (-1)^i x_i (the
// r2c bins 0 and ns/2), FP64 in a fixed order
template <typename T>
__global__ void __launch_bounds__(kRT) k_tile_edges(const T* __restrict__ x, long long ns,
                                                   double* __restrict__ out) {
  const long long t = blockIdx.x;
  const T* px = x + t * ns;
  double s0 = 0.0, s1 = 0.0;
  // kRT is even: a thread's samples all have the parity of threadIdx.x
  for (long long i = threadIdx.x; i < ns; i += kRT) s0 += (double)px[i];
  s1 = (threadIdx.x & 1) ? -s0 : s0;
  __shared__ double sh[2][kRT / 32];
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = s0;
    sh[1][threadIdx.x >> 5] = s1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < kRT / 32; w++) {
      a += sh[0][w];
      b += sh[1][w];
    }
    out[2 * t] = a;
    out[2 * t + 1] = b;
  }
}

template <typename T>
cudaError_t tile_edges_launch(const T* x, long long ntiles, long long ns, double* out,
                              cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  k_tile_edges<T><<<(unsigned)ntiles, kRT, 0, st>>>(x, ns, out);
  return cudaGetLastError();
}

}  // namespace

template <typename T>
cudaError_t tile_scale_launch(T* y, const T* tsc, long long ntiles, long long ns, cudaStream_t st) {
  const long long n = ntiles * ns;
  long long blocks = (n + kRT - 1) / kRT;
  if (blocks > 152LL * 16) blocks = 152LL * 16;
  k_tile_scale<T><<<(unsigned)blocks, kRT, 0, st>>>(y, tsc, ns, n);
  return cudaGetLastError();
}

template <typename T>
cudaError_t tile_dots_launch(const T* a, const T* b, long long ntiles, long long ns, double* out,
                             cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  k_tile_dots<T><<<(unsigned)ntiles, kRT, 0, st>>>(a, b, ns, out);
  return cudaGetLastError();
}

template cudaError_t tile_scale_launch<float>(float*, const float*, long long, long long,
                                              cudaStream_t);
template cudaError_t tile_scale_launch<double>(double*, const double*, long long, long long,
                                               cudaStream_t);
template cudaError_t tile_dots_launch<float>(const float*, const float*, long long, long long,
                                             double*, cudaStream_t);
template cudaError_t tile_dots_launch<double>(const double*, const double*, long long, long long,
                                              double*, cudaStream_t);

}  // namespace sg

using namespace sg;

namespace {

// g per tile [det][seg] in the operator's type
cudaError_t upload_tiles(sg_ctx* c, const std::vector<double>& g, DevBuf& dst, bool squared) {
  const long long nt = c->ntiles;
  cudaError_t e = dst.alloc((size_t)nt * c->esize);
  if (e != cudaSuccess) return e;
  if (c->f32) {
    std::vector<float> h(nt);
    for (long long t = 0; t < nt; t++) h[t] = (float)(squared ? g[t] * g[t] : g[t]);
    e = cudaMemcpyAsync(dst.p, h.data(), sizeof(float) * nt, cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);  // h is a host temporary
  } else {
    std::vector<double> h(nt);
    for (long long t = 0; t < nt; t++) h[t] = squared ? g[t] * g[t] : g[t];
    e = cudaMemcpyAsync(dst.p, h.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  }
  return e;
}

// chi^2 of d - G P m for the map in dmap (G from the device array g, or 1)
cudaError_t chi2_of(sg_ctx* c, const DevBuf* g, double* out) {
  cudaError_t e = c->launch_project(g, c->y.p);
  double* dchi2 = &c->sc.as<CgScalars>()->chi2;
  if (e == cudaSuccess)
    e = c->launch_filter(kLoadTodMinus, c->tod.p, c->yb.p, c->ntiles, (int)c->nseg, 0, c->y.p,
                         dchi2);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, dchi2, sizeof(double), cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  return e;
}

}  // namespace

extern "C" int sg_gains_from_sums(long ndet, long nseg, int per_detector, const double* dots_ds,
                                  const double* dots_ss, const double* edges_s,
                                  const double* edges_d, const double* spn_edge,
                                  const double* g_old, double* g_new) {
  if (ndet < 1 || nseg < 1 || !dots_ds || !dots_ss || !edges_s || !edges_d || !spn_edge || !g_old ||
      !g_new)
    return SG_ERR_ARG;
  const long long nt = (long long)ndet * nseg;
  // the half-spectrum sums (bins 0 and ns/2 counted twice, as the reference)
  std::vector<double> bd(nt), cs(nt);
  for (long long t = 0; t < nt; t++) {
    const long long d = t / nseg;
    const double w0 = spn_edge[2 * d], wm = spn_edge[2 * d + 1];
    const double s0 = edges_s[2 * t], sm = edges_s[2 * t + 1];
    const double d0 = edges_d[2 * t], dm = edges_d[2 * t + 1];
    bd[t] = dots_ds[t] + w0 * s0 * d0 + wm * sm * dm;
    cs[t] = dots_ss[t] + w0 * s0 * s0 + wm * sm * sm;
  }
  if (per_detector) {  // -R: one gain per detector (sanepic.cc:2254-2271)
    for (long long d = 0; d < ndet; d++) {
      double zeta = 0.0, gamma = 0.0;
      for (long long s = 0; s < nseg; s++) {
        zeta += bd[d * nseg + s];
        gamma += cs[d * nseg + s];
      }
      for (long long s = 0; s < nseg; s++)
        g_new[d * nseg + s] = gamma > 0.0 ? zeta / gamma : g_old[d * nseg + s];
    }
  } else {
    for (long long t = 0; t < nt; t++) g_new[t] = cs[t] > 0.0 ? bd[t] / cs[t] : g_old[t];
  }
  // the mean gain held at that of the gains the map was made with
  double m0 = 0.0, m1 = 0.0;
  for (long long t = 0; t < nt; t++) {
    m0 += g_old[t];
    m1 += g_new[t];
  }
  if (!(m1 > 0.0 && std::isfinite(m1))) return SG_ERR_NOT_CONVERGED;
  const double f = m0 / m1;
  for (long long t = 0; t < nt; t++) g_new[t] *= f;
  return SG_OK;
}

extern "C" int sg_set_gains(sg_ctx* c, const double* gains) {
  if (!c) return SG_ERR_ARG;
  const long long nd = c->ndet, nsg = c->nseg, nt = nd * nsg;
  std::vector<double> g(nt, 1.0);
  if (gains) {
    for (long long s = 0; s < nsg; s++)
      for (long long d = 0; d < nd; d++) {
        const double v = gains[d + s * nd];  // relCalib's layout, sanepic.cc:993, 2224
        if (!(std::isfinite(v) && v > 0.0))
          return c->fail(SG_ERR_ARG, "gain of detector %lld, segment %lld is %g (must be > 0)",
                         d, s, v);
        g[d * nsg + s] = v;
      }
  }
  cudaSetDevice(c->desc.device);
  bool ones = true;
  for (double v : g) ones = ones && v == 1.0;
  cudaError_t e = cudaSuccess;
  if (!ones) {
    e = upload_tiles(c, g, c->gain_t, false);
    if (e == cudaSuccess) e = upload_tiles(c, g, c->gain2_t, true);
    if (e != cudaSuccess) return c->cuda_fail(e, "gains");
  }
  c->gains_h = g;
  c->gains_on = !ones;
  // b and the learned part were made with the old operator; the map stays
  // (a start map for the next solve), the preconditioners too (the
  // reference keeps the diagonal of its first loop, sanepic.cc:1352)
  c->have_rhs = false;
  c->coarse_k = 0;
  c->set_learned_kind(0);
  c->learned_enabled = false;
  c->drop_graphs();  // captured iterations embed the operator's launch sequence
  return SG_OK;
}

extern "C" int sg_fit_gains(sg_ctx* c, int per_detector, double* gains_out, double* chi2_before,
                            double* chi2_after) {
  if (!c) return SG_ERR_ARG;
  if (!gains_out) return c->fail(SG_ERR_ARG, "null gains array");
  if (!c->have_pointing) return c->fail(SG_ERR_STATE, "pointing not set");
  for (long long dd = 0; dd < c->ndet; dd++) {
    if (!c->have_noise[dd]) return c->fail(SG_ERR_STATE, "noise of detector %lld not set", dd);
    if (!c->have_tod[dd]) return c->fail(SG_ERR_STATE, "TOD of detector %lld not set", dd);
  }
  if (!c->have_solution) return c->fail(SG_ERR_STATE, "no map: call sg_solve first");
  int rc = prepare_operator(c);
  if (rc) return rc;
  cudaSetDevice(c->desc.device);
  const long long nd = c->ndet, nsg = c->nseg, nt = c->ntiles;
  if (c->gains_h.size() != (size_t)nt) c->gains_h.assign(nt, 1.0);
  cudaError_t e = c->yb.alloc((size_t)nt * c->ns * c->esize);
  if (e == cudaSuccess) e = c->tdots.alloc(sizeof(double) * 6 * nt);
  // s = P m; (N^-1 d)^T s (N^-1 is symmetric), (N^-1 s)^T s, and the bins 0
  // and ns/2 of s and d
  double* dots = c->tdots.as<double>();
  if (e == cudaSuccess) e = c->to_map(c->x.as<double>());
  if (e == cudaSuccess) e = c->detector_weight_step(c->tod.p, c->yb.p);
  if (e == cudaSuccess) e = c->launch_project(nullptr, c->y.p);
  if (c->f32) {
    if (e == cudaSuccess)
      e = tile_dots_launch<float>(c->yb.as<float>(), c->y.as<float>(), nt, c->ns, dots, c->st);
    if (e == cudaSuccess) e = tile_edges_launch<float>(c->y.as<float>(), nt, c->ns, dots + 2 * nt, c->st);
    if (e == cudaSuccess)
      e = tile_edges_launch<float>(c->tod.as<float>(), nt, c->ns, dots + 4 * nt, c->st);
    if (e == cudaSuccess) e = c->detector_weight_step(c->y.p, c->yb.p);
    if (e == cudaSuccess)
      e = tile_dots_launch<float>(c->yb.as<float>(), c->y.as<float>(), nt, c->ns, dots + nt, c->st);
  } else {
    if (e == cudaSuccess)
      e = tile_dots_launch<double>(c->yb.as<double>(), c->y.as<double>(), nt, c->ns, dots, c->st);
    if (e == cudaSuccess)
      e = tile_edges_launch<double>(c->y.as<double>(), nt, c->ns, dots + 2 * nt, c->st);
    if (e == cudaSuccess)
      e = tile_edges_launch<double>(c->tod.as<double>(), nt, c->ns, dots + 4 * nt, c->st);
    if (e == cudaSuccess) e = c->detector_weight_step(c->y.p, c->yb.p);
    if (e == cudaSuccess)
      e = tile_dots_launch<double>(c->yb.as<double>(), c->y.as<double>(), nt, c->ns, dots + nt,
                                   c->st);
  }
  c->launches += 4;
  std::vector<double> h(6 * nt);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h.data(), dots, sizeof(double) * 6 * nt, cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) return c->cuda_fail(e, "gain fit");
  std::vector<double> g(nt);
  if (sg_gains_from_sums(nd, nsg, per_detector, h.data(), h.data() + nt, h.data() + 2 * nt,
                         h.data() + 4 * nt, c->spn_edge.data(), c->gains_h.data(), g.data()) != SG_OK)
    return c->fail(SG_ERR_NOT_CONVERGED,
                   "gain fit: no positive mean gain (the map does not fit the data)");
  // chi^2 with the gains the map was made with, and with the new ones
  double x2b = 0.0, x2a = 0.0;
  DevBuf gnew;
  e = chi2_of(c, c->gains_on ? &c->gain_t : nullptr, &x2b);
  if (e == cudaSuccess) e = upload_tiles(c, g, gnew, false);
  if (e == cudaSuccess) e = chi2_of(c, &gnew, &x2a);
  if (e != cudaSuccess) return c->cuda_fail(e, "gain fit chi2");
  for (long long s = 0; s < nsg; s++)
    for (long long d = 0; d < nd; d++) gains_out[d + s * nd] = g[d * nsg + s];
  if (chi2_before) *chi2_before = x2b;
  if (chi2_after) *chi2_after = x2a;
  return SG_OK;
}
