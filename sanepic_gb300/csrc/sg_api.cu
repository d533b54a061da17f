// sg_api.cu -- host side of libsanepic_gpu: the context, the setup pipeline
// and the PCG driver behind the C ABI in include/sanepic_gpu.h.
//
// All device memory is owned here (cudaMalloc at setup, nothing allocated
// inside the iteration loop).  One CG iteration is a fixed sequence of
// launches on one stream -- P, the noise filter, the per-group detector sums,
// P^T, three vector kernels -- captured once into a CUDA graph and replayed;
// the host reads back the CG scalars once per iteration to test convergence.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/sanepic_gpu.h"
#include "sg_ctx.h"
#include "sg_healpix.h"
#include "sg_kernels.h"


// ---------------------------------------------------------------------------
static bool is_pow2(long long v) { return v > 0 && (v & (v - 1)) == 0; }

extern "C" int sg_create(sg_ctx** out, const sg_desc* desc) {
  if (!out || !desc) return SG_ERR_ARG;
  *out = nullptr;
  sg_ctx* c = new sg_ctx();
  c->desc = *desc;
  auto bad = [&](int code, const char* msg) {
    // a failed create still returns the context so sg_last_error works
    c->err = msg;
    *out = c;
    return code;
  };
  if (desc->pol != 1) return bad(SG_ERR_UNSUPPORTED, "pol must be 1 (pol=0 is broken in the reference)");
  if (!is_pow2(desc->ns) || desc->ns < 256 || desc->ns > 131072)
    return bad(SG_ERR_UNSUPPORTED, "ns must be a power of two in [256, 131072]");
  if (desc->nseg < 1 || desc->ndet < 1) return bad(SG_ERR_ARG, "nseg and ndet must be >= 1");
  if (desc->nside < 1 || desc->nside > 8192) return bad(SG_ERR_ARG, "nside out of range");
  const long long nsamp = (long long)desc->ns * desc->nseg * desc->ndet;
  if (nsamp >= (1LL << 32)) return bad(SG_ERR_UNSUPPORTED, "more than 2^32 samples");
  cudaError_t e = cudaSetDevice(desc->device);
  if (e != cudaSuccess) return bad(SG_ERR_CUDA, cudaGetErrorString(e));
  e = cudaStreamCreateWithFlags(&c->own_st, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bad(SG_ERR_CUDA, cudaGetErrorString(e));
  c->st = c->own_st;
  c->f32 = desc->precision == SG_F32;
  c->esize = c->f32 ? 4 : 8;
  c->ns = desc->ns;
  c->nseg = desc->nseg;
  c->ndet = desc->ndet;
  c->ntiles = c->nseg * c->ndet;
  c->nsamp = nsamp;
  c->npixfull = 12LL * desc->nside * desc->nside;
  const long long M = c->ns / 2;
  int logm = 0;
  while ((1LL << logm) < M) logm++;
  c->logm = logm;
  const long long emax = c->f32 ? 8192 : 4096;  // complex elements per CTA buffer
  c->S = (int)std::max<long long>(1, M / emax);
  c->nclusters = c->f32 ? filter_max_clusters<float>(logm, c->S)
                        : filter_max_clusters<double>(logm, c->S);
  if (c->nclusters <= 0) return bad(SG_ERR_CUDA, "noise-filter kernel cannot be scheduled");
  c->have_noise.assign(c->ndet, 0);
  c->have_tod.assign(c->ndet, 0);
  // twiddle tables W_M^j = W_M^{64 jh} W_M^{jl}, computed in FP64
  {
    std::vector<double> lo(2 * 64), hi(2 * (M / 64));
    for (int jl = 0; jl < 64; jl++) {
      double a = kD2PI * (double)jl / (double)M;
      lo[2 * jl] = cos(a);
      lo[2 * jl + 1] = -sin(a);
    }
    for (long long jh = 0; jh < M / 64; jh++) {
      double a = kD2PI * (double)(64 * jh) / (double)M;
      hi[2 * jh] = cos(a);
      hi[2 * jh + 1] = -sin(a);
    }
    const double a1 = kD2PI / (double)(2 * M);
    c->wn1d = cplx<double>{cos(a1), -sin(a1)};
    c->wn1f = cplx<float>{(float)cos(a1), (float)-sin(a1)};
    if ((e = c->tw_lo.alloc(lo.size() * c->esize)) != cudaSuccess ||
        (e = c->tw_hi.alloc(hi.size() * c->esize)) != cudaSuccess)
      return bad(SG_ERR_CUDA, cudaGetErrorString(e));
    if (c->f32) {
      std::vector<float> lf(lo.begin(), lo.end()), hf(hi.begin(), hi.end());
      cudaMemcpy(c->tw_lo.p, lf.data(), lf.size() * 4, cudaMemcpyHostToDevice);
      cudaMemcpy(c->tw_hi.p, hf.data(), hf.size() * 4, cudaMemcpyHostToDevice);
    } else {
      cudaMemcpy(c->tw_lo.p, lo.data(), lo.size() * 8, cudaMemcpyHostToDevice);
      cudaMemcpy(c->tw_hi.p, hi.data(), hi.size() * 8, cudaMemcpyHostToDevice);
    }
  }
  if ((e = c->filt.alloc((size_t)c->ndet * (M + 1) * c->esize)) != cudaSuccess ||
      (e = c->g0.alloc(sizeof(double) * c->ndet)) != cudaSuccess ||
      (e = c->y.alloc((size_t)nsamp * c->esize)) != cudaSuccess ||
      (e = c->tod.alloc((size_t)nsamp * c->esize)) != cudaSuccess ||
      (e = c->chi2p.alloc(sizeof(double) * c->S * c->nclusters)) != cudaSuccess)
    return bad(SG_ERR_CUDA, cudaGetErrorString(e));
  if ((e = cudaMallocHost(&c->sc_host, sizeof(CgScalars))) != cudaSuccess)
    return bad(SG_ERR_CUDA, cudaGetErrorString(e));
  *out = c;
  return SG_OK;
}

extern "C" void sg_destroy(sg_ctx* c) { delete c; }

extern "C" int sg_set_stream(sg_ctx* c, void* stream) {
  if (!c) return SG_ERR_ARG;
  cudaStream_t s = stream ? reinterpret_cast<cudaStream_t>(stream) : c->own_st;
  if (s != c->st) {
    cudaStreamSynchronize(c->st);
    c->drop_graphs();  // graphs were captured on the old stream
    c->st = s;
  }
  return SG_OK;
}

extern "C" const char* sg_last_error(const sg_ctx* c) {
  return c ? c->err.c_str() : "null context";
}

extern "C" long sg_npix(const sg_ctx* c) { return c ? (long)c->npix : -1; }

extern "C" long sg_kernel_launches(const sg_ctx* c) { return c ? (long)c->launches : -1; }

extern "C" int sg_weighting(const sg_ctx* c) {
  if (!c) return SG_ERR_ARG;
  return (c->grouped() ? 1 : 0) | (c->use_f3 ? 2 : 0);
}

extern "C" int sg_group_mode(const sg_ctx* c, long* ngroups) {
  if (!c) return 0;
  if (ngroups) *ngroups = c->ngroups;
  return c->grouped() ? (c->use_f3 ? 2 : 1) : 0;
}

// ---------------------------------------------------------------------------
extern "C" int sg_set_pointing(sg_ctx* c, const double* ra, const double* dec,
                               const double* psi, long nsamp_total, const long* isampmin,
                               const sg_det* dets) {
  if (!c) return SG_ERR_ARG;
  if (!ra || !dec || !psi || !dets) return c->fail(SG_ERR_ARG, "null pointing array");
  cudaSetDevice(c->desc.device);
  const long long ns = c->ns, nseg = c->nseg, ndet = c->ndet, nsd = ns * nseg;
  const bool hwp = c->desc.hwp != 0;
  c->isampmin.resize(nseg);
  for (long long g = 0; g < nseg; g++) {
    c->isampmin[g] = isampmin ? isampmin[g] : g * ns;
    if (c->isampmin[g] < 0 || c->isampmin[g] + ns > nsamp_total)
      return c->fail(SG_ERR_ARG, "segment %lld [%lld, %lld] outside the %ld-sample timeline",
                     g, c->isampmin[g], c->isampmin[g] + ns - 1, nsamp_total);
  }
  cudaError_t e;
#define SG_TRY(x)                                     \
  do {                                                \
    e = (x);                                          \
    if (e != cudaSuccess) return c->cuda_fail(e, #x); \
  } while (0)
  // device scratch of the set-up, kept in the context so that a caller who
  // sets the pointing again (one scan after another) does not pay for
  // allocating and freeing it each time
  sg_ctx::PointingScratch& P = c->pscr;
  DevBuf &dra = P.ra, &ddec = P.dec, &dpsi = P.psi, &doffx = P.offx, &doffy = P.offy,
         &ring = P.ring, &psio = P.psio, &flag = P.flag, &count = P.count, &scratch = P.scratch,
         &gsz = P.gsz, &gsc = P.gsc, &gss = P.gss;
  SG_TRY(dra.alloc(sizeof(double) * nsd));
  SG_TRY(ddec.alloc(sizeof(double) * nsd));
  SG_TRY(dpsi.alloc(sizeof(double) * nsd));
  SG_TRY(flag.alloc(2 * sizeof(int)));
  // the segments' boresight goes to the device as it is (one copy per array if
  // the segments are contiguous); psi's NaN samples take the previous sample's
  // value within the segment there (sanepic.cc:722-727)
  {
    bool contiguous = true;
    for (long long g = 1; g < nseg; g++) contiguous &= c->isampmin[g] == c->isampmin[0] + g * ns;
    const double* src[3] = {ra, dec, psi};
    DevBuf* dst[3] = {&dra, &ddec, &dpsi};
    for (int a = 0; a < 3; a++) {
      if (contiguous) {
        SG_TRY(cudaMemcpyAsync(dst[a]->p, src[a] + c->isampmin[0], sizeof(double) * nsd,
                               cudaMemcpyHostToDevice, c->st));
      } else {
        for (long long g = 0; g < nseg; g++)
          SG_TRY(cudaMemcpyAsync(dst[a]->as<double>() + g * ns, src[a] + c->isampmin[g],
                                 sizeof(double) * ns, cudaMemcpyHostToDevice, c->st));
      }
    }
    // the sequential rule runs only where psi has a NaN at all
    int hnan = 0;
    SG_TRY(cudaMemsetAsync(flag.p, 0, sizeof(int), c->st));
    SG_TRY(any_nan_launch(dpsi.as<double>(), nsd, flag.as<int>(), c->st));
    SG_TRY(cudaMemcpyAsync(&hnan, flag.p, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    SG_TRY(cudaStreamSynchronize(c->st));
    if (hnan) SG_TRY(nan_patch_launch<double>(dpsi.as<double>(), ns, nseg, c->st));
  }
  // offset groups: detectors with identical (offx, offy) share the pixelisation
  // (pass 1); if any pointing sample is NaN, every detector gets its own
  // stream (pass 2) so the reference's previous-pixel rule, which carries
  // across detectors, is applied exactly.
  std::vector<int> hring;
  for (int pass = 0; pass < 2; pass++) {
    std::vector<int> goff, gdet;
    std::vector<char> used(ndet, 0);
    for (long long dd = 0; dd < ndet; dd++) {
      if (used[dd]) continue;
      goff.push_back((int)gdet.size());
      for (long long e2 = dd; e2 < ndet; e2++)
        if (!used[e2] && (pass == 1 ? e2 == dd
                                    : (dets[e2].offx == dets[dd].offx &&
                                       dets[e2].offy == dets[dd].offy))) {
          used[e2] = 1;
          gdet.push_back((int)e2);
        }
    }
    goff.push_back((int)gdet.size());
    const int G = (int)goff.size() - 1;
    std::vector<double> offx(G), offy(G);
    for (int g = 0; g < G; g++) {
      offx[g] = dets[gdet[goff[g]]].offx;
      offy[g] = dets[gdet[goff[g]]].offy;
    }
    const long long ng = (long long)G * nsd;
    SG_TRY(doffx.alloc(sizeof(double) * G));
    SG_TRY(doffy.alloc(sizeof(double) * G));
    SG_TRY(ring.alloc(sizeof(int) * ng));
    SG_TRY(psio.alloc(sizeof(double) * ng));
    SG_TRY(cudaMemcpyAsync(doffx.p, offx.data(), sizeof(double) * G, cudaMemcpyHostToDevice, c->st));
    SG_TRY(cudaMemcpyAsync(doffy.p, offy.data(), sizeof(double) * G, cudaMemcpyHostToDevice, c->st));
    SG_TRY(cudaMemsetAsync(flag.p, 0, 2 * sizeof(int), c->st));
    PointingArgs pa{};
    pa.ns = ns;
    pa.nseg = (int)nseg;
    pa.ngroups = G;
    pa.ra = dra.as<double>();
    pa.dec = ddec.as<double>();
    pa.psi = dpsi.as<double>();
    pa.offx = doffx.as<double>();
    pa.offy = doffy.as<double>();
    pa.nside = c->desc.nside;
    pa.ring_pix = ring.as<int>();
    pa.psio = psio.as<double>();
    pa.error_flag = flag.as<int>();
    SG_TRY(pointing_launch(pa, c->st));
    SG_TRY(any_negative_launch(ring.as<int>(), ng, flag.as<int>() + 1, c->st));
    int hflag[2] = {0, 0};
    SG_TRY(cudaMemcpyAsync(hflag, flag.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->st));
    SG_TRY(cudaStreamSynchronize(c->st));
    if (hflag[0])
      return c->fail(SG_ERR_POINTING, "theta out of range in ang2pix (the reference exits here)");
    const bool any_invalid = hflag[1] != 0;  // NaN pointing somewhere
    c->ngroups = G;
    c->ngsamp = ng;
    c->grp_off_h = goff;
    c->grp_det_h = gdet;
    if (!any_invalid) break;
    if (pass == 1 || G == ndet) {
      // NaN pointing: reuse the previous pixel in the reference's loop order
      // (det, seg, sample; sanepic.cc:851-873), streams are per detector here
      hring.resize(ng);
      SG_TRY(cudaMemcpy(hring.data(), ring.p, sizeof(int) * ng, cudaMemcpyDeviceToHost));
      int prev = 0;
      for (long long i = 0; i < ng; i++) {
        if (hring[i] < 0) hring[i] = prev;
        prev = hring[i];
      }
      SG_TRY(cudaMemcpy(ring.p, hring.data(), sizeof(int) * ng, cudaMemcpyHostToDevice));
      break;
    }
  }
  const int G = c->ngroups;
  const long long ng = c->ngsamp;
  std::vector<int> gsize(G);
  for (int g = 0; g < G; g++) gsize[g] = c->grp_off_h[g + 1] - c->grp_off_h[g];
  SG_TRY(gsz.alloc(sizeof(int) * G));
  SG_TRY(cudaMemcpy(gsz.p, gsize.data(), sizeof(int) * G, cudaMemcpyHostToDevice));
  SG_TRY(c->grp_off.alloc(sizeof(int) * (G + 1)));
  SG_TRY(c->grp_det.alloc(sizeof(int) * ndet));
  SG_TRY(cudaMemcpy(c->grp_off.p, c->grp_off_h.data(), sizeof(int) * (G + 1), cudaMemcpyHostToDevice));
  SG_TRY(cudaMemcpy(c->grp_det.p, c->grp_det_h.data(), sizeof(int) * ndet, cudaMemcpyHostToDevice));
  // detector rotations: the detector's angle relative to its group's base
  // angle phi is +psi_det, or -psi_det under a half-wave plate
  // (psip = -(psi_o + psi_det) + 2 omega t, sanepic.cc:765)
  c->psidet_h.resize(ndet);
  {
    std::vector<double> r(2 * ndet);
    for (long long dd = 0; dd < ndet; dd++) {
      c->psidet_h[dd] = dets[dd].psi;
      const double a = 2.0 * (hwp ? -dets[dd].psi : dets[dd].psi);
      r[2 * dd] = cos(a);
      r[2 * dd + 1] = sin(a);
    }
    SG_TRY(c->dcs.alloc((size_t)2 * ndet * c->esize));
    if (c->f32) {
      std::vector<float> f(r.begin(), r.end());
      SG_TRY(cudaMemcpy(c->dcs.p, f.data(), 4 * f.size(), cudaMemcpyHostToDevice));
    } else {
      SG_TRY(cudaMemcpy(c->dcs.p, r.data(), 8 * r.size(), cudaMemcpyHostToDevice));
    }
  }
  // detector samples per RING pixel
  SG_TRY(count.alloc(sizeof(int) * c->npixfull));
  SG_TRY(cudaMemsetAsync(count.p, 0, sizeof(int) * c->npixfull, c->st));
  SG_TRY(hist_launch(ring.as<int>(), ng, nsd, gsz.as<int>(), count.as<int>(), c->st));
  // indpix in the reference's RING order (sanepic.cc:904-915), and the
  // library's internal numbering: observed pixels in NESTED order
  const std::vector<long long> old_int2ring = c->int2ring;
  long long npix = 0;
  {
    const long long nf = c->npixfull, nside = c->desc.nside;
    const size_t ntb = numbering_tmp_bytes(nf);
    DevBuf &ntmp = P.ntmp, &d_i2r = P.i2r, &d_i2rc = P.i2rc, &d_ipr = P.ipr, &d_np = P.np;
    SG_TRY(ntmp.alloc(ntb));
    SG_TRY(d_i2r.alloc(sizeof(long long) * nf));
    SG_TRY(d_i2rc.alloc(sizeof(long long) * nf));
    SG_TRY(d_ipr.alloc(sizeof(int) * nf));
    SG_TRY(d_np.alloc(sizeof(int)));
    SG_TRY(c->indpix.alloc(sizeof(int) * nf));
    SG_TRY(numbering_launch(count.as<int>(), nf, nside, (nside & (nside - 1)) == 0 ? 1 : 0,
                            d_i2r.as<long long>(), d_i2rc.as<long long>(), c->indpix.as<int>(),
                            d_ipr.as<int>(), d_np.as<int>(), ntmp.p, ntb, c->st));
    int hnp = 0;
    SG_TRY(cudaMemcpyAsync(&hnp, d_np.p, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    SG_TRY(cudaStreamSynchronize(c->st));
    npix = hnp;
    c->npix = npix;
    c->int2ring.resize(npix);
    c->int2ringc.resize(npix);
    c->indpix_host.resize(nf);
    SG_TRY(cudaMemcpyAsync(c->int2ring.data(), d_i2r.p, sizeof(long long) * npix,
                           cudaMemcpyDeviceToHost, c->st));
    SG_TRY(cudaMemcpyAsync(c->int2ringc.data(), d_i2rc.p, sizeof(long long) * npix,
                           cudaMemcpyDeviceToHost, c->st));
    SG_TRY(cudaMemcpyAsync(c->indpix_host.data(), d_ipr.p, sizeof(int) * nf,
                           cudaMemcpyDeviceToHost, c->st));
    SG_TRY(cudaStreamSynchronize(c->st));
  }
  SG_TRY(c->pix.alloc(sizeof(int) * ng));
  SG_TRY(compact_launch(ring.as<int>(), c->indpix.as<int>(), ng, c->pix.as<int>(), c->st));
  SG_TRY(c->hits.alloc(sizeof(int) * npix));
  SG_TRY(hits_launch(count.as<int>(), c->indpix.as<int>(), c->npixfull, c->hits.as<int>(), c->st));
  // pixel-sorted group-sample index (CSR) for P^T
  const size_t ctb = csr_tmp_bytes(ng, npix);
  SG_TRY(scratch.alloc(ctb));
  SG_TRY(c->csr_off.alloc(sizeof(long long) * (npix + 1)));
  SG_TRY(c->csr_idx.alloc(sizeof(uint32_t) * ng));
  SG_TRY(csr_build(c->pix.as<int>(), ng, npix, c->csr_off.as<long long>(),
                   c->csr_idx.as<uint32_t>(), scratch.p, ctb, c->st));
  // base angles (cos 2phi, sin 2phi) in time order and in CSR order
  SG_TRY(c->cs.alloc((size_t)2 * ng * c->esize));
  SG_TRY(c->csr_cs.alloc((size_t)2 * ng * c->esize));
  DevBuf& cs64 = P.cs64;  // FP64 (cos, sin) 2 psi_o for the cross-link sums (no half-wave plate)
  if (!hwp) SG_TRY(cs64.alloc(sizeof(double) * 2 * ng));
  if (c->f32) {
    SG_TRY(base_angles_launch<float>(psio.as<double>(), ng, ns, nsd, hwp ? 1 : 0, c->desc.omega,
                                     c->cs.as<float>(), cs64.as<double>(), c->st));
    SG_TRY(gather_cs_launch<float>(c->cs.as<float>(), c->csr_idx.as<uint32_t>(), ng,
                                   c->csr_cs.as<float>(), c->st));
  } else {
    SG_TRY(base_angles_launch<double>(psio.as<double>(), ng, ns, nsd, hwp ? 1 : 0, c->desc.omega,
                                      c->cs.as<double>(), cs64.as<double>(), c->st));
    SG_TRY(gather_cs_launch<double>(c->cs.as<double>(), c->csr_idx.as<uint32_t>(), ng,
                                    c->csr_cs.as<double>(), c->st));
  }
  // cross-link sums with psipFP = psi_o + psi_det (sanepic.cc:760-762, 2594-2597)
  {
    std::vector<double> sc_(G, 0.0), ss_(G, 0.0);
    for (int g = 0; g < G; g++)
      for (int k = c->grp_off_h[g]; k < c->grp_off_h[g + 1]; k++) {
        sc_[g] += cos(2.0 * c->psidet_h[c->grp_det_h[k]]);
        ss_[g] += sin(2.0 * c->psidet_h[c->grp_det_h[k]]);
      }
    SG_TRY(gsc.alloc(sizeof(double) * G));
    SG_TRY(gss.alloc(sizeof(double) * G));
    SG_TRY(cudaMemcpy(gsc.p, sc_.data(), sizeof(double) * G, cudaMemcpyHostToDevice));
    SG_TRY(cudaMemcpy(gss.p, ss_.data(), sizeof(double) * G, cudaMemcpyHostToDevice));
  }
  SG_TRY(c->sumcross.alloc(sizeof(double) * 3 * npix));
  SG_TRY(sumcross_launch(c->csr_off.as<long long>(), c->csr_idx.as<uint32_t>(), psio.as<double>(),
                         cs64.as<double>(), nsd, gsc.as<double>(), gss.as<double>(), npix,
                         c->sumcross.as<double>(), c->st));
  SG_TRY(c->ys.alloc((size_t)3 * ng * c->esize));  // [ng / 8][3][8]
  // the offset-group operator when every group is large enough (three
  // timelines per group instead of one per detector); SANEPIC_GPU_GROUP_FILTER=0
  // keeps the per-detector operator
  {
    int gmin = (int)ndet;
    for (int g = 0; g < G; g++) gmin = std::min(gmin, c->grp_off_h[g + 1] - c->grp_off_h[g]);
    const char* env = getenv("SANEPIC_GPU_GROUP_FILTER");
    c->group_mode = gmin >= sg_ctx::kGroupMin && !(env && env[0] == '0');
    c->have_hmix = false;
    if (c->group_mode) {
      const long long M1 = ns / 2 + 1;
      SG_TRY(c->gtl.alloc((size_t)3 * ng * c->esize));
      SG_TRY(c->gspec.alloc((size_t)3 * G * nseg * M1 * 2 * c->esize));
      SG_TRY(c->hmix.alloc((size_t)G * M1 * 6 * c->esize));
      SG_TRY(c->dspec.alloc((size_t)ndet * nseg * M1 * 2 * c->esize));
      SG_TRY(c->rhs_part.alloc(sizeof(double) * kGroupRhsBlocks));
    } else {
      c->gtl.release();
      c->gspec.release();
      c->hmix.release();
      c->dspec.release();
      c->rhs_part.release();
    }
  }
  // CG vectors
  const size_t vb = sizeof(double) * 3 * npix;
  SG_TRY(c->x.alloc(vb));
  SG_TRY(c->r.alloc(vb));
  SG_TRY(c->d.alloc(vb));
  SG_TRY(c->q.alloc(vb));
  SG_TRY(c->z.alloc(vb));
  SG_TRY(c->rprev.alloc(vb));
  SG_TRY(c->b.alloc(vb));
  SG_TRY(c->minv.alloc(sizeof(double) * 6 * npix));
  SG_TRY(c->mdiag.alloc(vb));
  SG_TRY(c->mp_raw.alloc(vb));
  SG_TRY(c->part.alloc(sizeof(double) * 4 * kCgBlocks));
  SG_TRY(c->sc.alloc(sizeof(CgScalars)));
  SG_TRY(c->dmap.alloc((size_t)4 * npix * c->esize));
  SG_TRY(cudaMemsetAsync(c->x.p, 0, vb, c->st));
  SG_TRY(cudaStreamSynchronize(c->st));
  c->drop_graphs();
  if (c->int2ring != old_int2ring) {
    // another pixel set: the network's patch geometry is rebuilt on demand and
    // the coarse space (vectors over the old pixels) is dropped.  With the same
    // pixel set a coarse space built on other pointing or noise stays a valid
    // (symmetric positive definite) preconditioner, only a weaker one.
    c->npatch = c->npatch_pad = 0;
    c->coarse_k = 0;
    if (c->learned_kind == 2) {
      c->set_learned_kind(0);
      c->learned_enabled = false;
    }
  }
  c->have_pointing = true;
  c->have_rhs = c->have_solution = c->have_bj3 = c->have_diag = false;
  return build_polmask(c);
}

extern "C" int sg_set_pol_rcond(sg_ctx* c, double rcond_min) {
  if (!c) return SG_ERR_ARG;
  if (!(rcond_min >= 0.0 && rcond_min < 1.0))
    return c->fail(SG_ERR_ARG, "rcond_min %g outside [0, 1)", rcond_min);
  cudaSetDevice(c->desc.device);
  c->pol_rcond = rcond_min;
  // b, the block-Jacobi blocks and any learned part were made with the old mask
  c->have_rhs = c->have_solution = c->have_bj3 = false;
  c->coarse_k = 0;
  c->set_learned_kind(0);
  c->learned_enabled = false;
  c->drop_graphs();
  return c->have_pointing ? build_polmask(c) : SG_OK;
}

// the filter rows of detectors d0 .. d0 + n - 1 from their iSpf values (n
// rows of nssp values, ispf_host: the caller's array), one copy and one wait
static int set_noise_rows(sg_ctx* c, long d0, long n, const double* ispf, long nssp) {
  const long long ns = c->ns, M = ns / 2;
  // the largest index read (sanepic.cc:535; monotonic in k)
  const long long idx_max = (long long)((double)M / nssp * ns);
  if (idx_max < 0 || idx_max >= nssp)
    return c->fail(SG_ERR_ARG, "noise spectrum of %ld values is too short for ns=%lld", nssp, ns);
  cudaSetDevice(c->desc.device);
  // the iSpf values go to the device as they are; the row, its 1/ns^2 scale,
  // the bin-0 override (sanepic.cc:536-537) and g0 are computed there
  const size_t bytes = sizeof(double) * (size_t)n * nssp;
  cudaError_t e = cudaSuccess;
  if (c->noise_stage.bytes < bytes) e = c->noise_stage.alloc(bytes);
  if (e == cudaSuccess && !c->noise_part.p) e = c->noise_part.alloc(sizeof(double) * kNoiseRowBlocks);
  if (e == cudaSuccess && !c->ev_copy) e = cudaEventCreateWithFlags(&c->ev_copy, cudaEventDisableTiming);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->noise_stage.p, ispf, bytes, cudaMemcpyHostToDevice, c->st);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev_copy, c->st);
  for (long k = 0; k < n && e == cudaSuccess; k++) {
    const long det = d0 + k;
    const double* row = c->noise_stage.as<double>() + (size_t)k * nssp;
    e = c->f32 ? noise_row_launch<float>(row, nssp, ns, c->filt.as<float>() + det * (M + 1),
                                         c->g0.as<double>() + det, c->noise_part.as<double>(), c->st)
               : noise_row_launch<double>(row, nssp, ns, c->filt.as<double>() + det * (M + 1),
                                          c->g0.as<double>() + det, c->noise_part.as<double>(),
                                          c->st);
    c->launches += 2;
  }
  if (e == cudaSuccess) e = cudaEventSynchronize(c->ev_copy);  // the caller's array is read
  if (e != cudaSuccess) return c->cuda_fail(e, "set_noise");
  // the weights of bins 0 and ns/2 in FP64 (sanepic.cc:533-537), which the
  // gain fit's half-spectrum sums count twice (sg_recal.cu)
  if (c->spn_edge.size() != (size_t)(2 * c->ndet)) c->spn_edge.assign(2 * c->ndet, 0.0);
  for (long k = 0; k < n; k++) {
    const double* r = ispf + (size_t)k * nssp;
    c->spn_edge[2 * (d0 + k)] = r[1] * 1e-6 / (double)ns / (double)ns;
    c->spn_edge[2 * (d0 + k) + 1] = r[idx_max] / (double)ns / (double)ns;
    c->have_noise[d0 + k] = 1;
  }
  c->have_bj3 = c->have_diag = c->have_rhs = c->have_hmix = false;
  return SG_OK;
}

extern "C" int sg_set_noise(sg_ctx* c, long det, const double* ispf, long nssp) {
  if (!c) return SG_ERR_ARG;
  if (det < 0 || det >= c->ndet || !ispf || nssp < 2)
    return c->fail(SG_ERR_ARG, "bad detector index or noise spectrum");
  return set_noise_rows(c, det, 1, ispf, nssp);
}

extern "C" int sg_set_noise_all(sg_ctx* c, const double* ispf, long nssp) {
  if (!c) return SG_ERR_ARG;
  if (!ispf || nssp < 2) return c->fail(SG_ERR_ARG, "bad noise spectra");
  return set_noise_rows(c, 0, c->ndet, ispf, nssp);
}

// TOD of detectors d0 .. d0 + n - 1 (rows of nsamp_total samples in the
// caller's array): each detector's segments are copied to the device as they
// are by the copy engine, into one of two staging buffers on the context's
// copy stream, and converted and NaN-patched there (sanepic.cc:776-803) on
// its stream while the next detector's copy runs; one wait for all.  (On a
// GB300 machine 64 rows of 50 MB from pinned memory take 16.7 ms this way,
// ~193 GB/s, against 16.9 ms for an ingest kernel reading the pinned rows
// itself; bare copies reach ~208 GB/s over that link, with one stream or
// several.)
static int set_tod_rows(sg_ctx* c, long d0, long n, const double* tod, long nsamp_total) {
  if (!c->have_pointing) return c->fail(SG_ERR_STATE, "set the pointing before the TOD");
  cudaSetDevice(c->desc.device);
  const long long ns = c->ns, nseg = c->nseg, nsd = ns * nseg;
  for (long long g = 0; g < nseg; g++)
    if (c->isampmin[g] + ns > nsamp_total)
      return c->fail(SG_ERR_ARG, "TOD shorter than the segment list");
  cudaError_t e = cudaSuccess;
  if (c->nanflag.bytes < sizeof(int) * (size_t)c->ndet) e = c->nanflag.alloc(sizeof(int) * c->ndet);
  if (e == cudaSuccess && c->stage.bytes < 2 * sizeof(double) * nsd)
    e = c->stage.alloc(2 * sizeof(double) * nsd);
  if (e == cudaSuccess && !c->copy_st) e = cudaStreamCreateWithFlags(&c->copy_st, cudaStreamNonBlocking);
  for (int q = 0; q < 2 && e == cudaSuccess; q++) {
    if (!c->ev_staged[q]) e = cudaEventCreateWithFlags(&c->ev_staged[q], cudaEventDisableTiming);
    if (e == cudaSuccess && !c->ev_ingested[q])
      e = cudaEventCreateWithFlags(&c->ev_ingested[q], cudaEventDisableTiming);
  }
  bool contiguous = true;
  for (long long g = 1; g < nseg; g++) contiguous &= c->isampmin[g] == c->isampmin[0] + g * ns;
  if (e == cudaSuccess) e = cudaMemsetAsync(c->nanflag.p, 0, sizeof(int) * n, c->st);
  // the copy stream starts after the context's earlier work
  if (e == cudaSuccess) e = cudaEventRecord(c->ev_ingested[0], c->st);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(c->copy_st, c->ev_ingested[0], 0);
  for (long k = 0; k < n && e == cudaSuccess; k++) {
    const double* row = tod + (size_t)k * nsamp_total;
    const long det = d0 + k;
    const int q = (int)(k & 1);
    double* buf = c->stage.as<double>() + (size_t)q * nsd;
    // buffer q is free once the conversion of detector k - 2 has read it
    if (k >= 2) e = cudaStreamWaitEvent(c->copy_st, c->ev_ingested[q], 0);
    if (e == cudaSuccess && contiguous) {
      e = cudaMemcpyAsync(buf, row + c->isampmin[0], sizeof(double) * nsd, cudaMemcpyHostToDevice,
                          c->copy_st);
    } else {
      for (long long g = 0; g < nseg && e == cudaSuccess; g++)
        e = cudaMemcpyAsync(buf + g * ns, row + c->isampmin[g], sizeof(double) * ns,
                            cudaMemcpyHostToDevice, c->copy_st);
    }
    if (e == cudaSuccess) e = cudaEventRecord(c->ev_staged[q], c->copy_st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->st, c->ev_staged[q], 0);
    if (e == cudaSuccess)
      e = c->f32 ? ingest_launch<float>(buf, nsd, c->tod.as<float>() + det * nsd,
                                        c->nanflag.as<int>() + k, c->st)
                 : ingest_launch<double>(buf, nsd, c->tod.as<double>() + det * nsd,
                                         c->nanflag.as<int>() + k, c->st);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev_ingested[q], c->st);
    c->launches++;
  }
  std::vector<int> nan(n, 0);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(nan.data(), c->nanflag.p, sizeof(int) * n, cudaMemcpyDeviceToHost, c->st);
  // every copy was waited on by a conversion on c->st: the caller's rows are read
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  for (long k = 0; k < n && e == cudaSuccess; k++)
    if (nan[k]) {
      e = c->f32 ? nan_patch_launch<float>(c->tod.as<float>() + (d0 + k) * nsd, ns, nseg, c->st)
                 : nan_patch_launch<double>(c->tod.as<double>() + (d0 + k) * nsd, ns, nseg, c->st);
      c->launches++;
    }
  if (e != cudaSuccess) return c->cuda_fail(e, "set_tod");
  for (long k = 0; k < n; k++) c->have_tod[d0 + k] = 1;
  c->have_rhs = false;
  return SG_OK;
}

extern "C" int sg_set_tod(sg_ctx* c, long det, const double* tod, long nsamp_total) {
  if (!c) return SG_ERR_ARG;
  if (det < 0 || det >= c->ndet || !tod) return c->fail(SG_ERR_ARG, "bad detector or TOD");
  return set_tod_rows(c, det, 1, tod, nsamp_total);
}

extern "C" int sg_set_tod_all(sg_ctx* c, const double* tod, long nsamp_total) {
  if (!c) return SG_ERR_ARG;
  if (!tod) return c->fail(SG_ERR_ARG, "null TOD");
  return set_tod_rows(c, 0, c->ndet, tod, nsamp_total);
}

static int check_ready(sg_ctx* c, bool need_tod) {
  if (!c->have_pointing) return c->fail(SG_ERR_STATE, "pointing not set");
  for (long long dd = 0; dd < c->ndet; dd++) {
    if (!c->have_noise[dd]) return c->fail(SG_ERR_STATE, "noise of detector %lld not set", dd);
    if (need_tod && !c->have_tod[dd]) return c->fail(SG_ERR_STATE, "TOD of detector %lld not set", dd);
  }
  return prepare_operator(c);
}

int prepare_operator(sg_ctx* c) {
  cudaSetDevice(c->desc.device);
  const cudaError_t e = c->ensure_hmix();
  return e == cudaSuccess ? SG_OK : c->cuda_fail(e, "group operator set-up");
}

extern "C" int sg_rhs(sg_ctx* c, double* chi2) {
  if (!c) return SG_ERR_ARG;
  int rc = check_ready(c, true);
  if (rc) return rc;
  cudaSetDevice(c->desc.device);
  // chi2_0 only when asked for: without it, offset groups whose detectors
  // share one noise spectrum skip the per-detector FFTs (rhs_of)
  double* dchi2 = chi2 ? &c->sc.as<CgScalars>()->chi2 : nullptr;
  cudaError_t e = c->rhs_of(c->tod.p, c->b.as<double>(), dchi2);
  double h = 0.0;
  if (e == cudaSuccess && chi2)
    e = cudaMemcpyAsync(&h, dchi2, sizeof(double), cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) return c->cuda_fail(e, "rhs");
  if (chi2) *chi2 = h;  // chi2_0 (sanepic.cc:1089-1110)
  c->have_rhs = true;
  return SG_OK;
}

extern "C" int sg_apply(sg_ctx* c, const double* xin, double* yout, int masked) {
  if (!c) return SG_ERR_ARG;
  int rc = check_ready(c, false);
  if (rc) return rc;
  if (!xin || !yout) return c->fail(SG_ERR_ARG, "null vector");
  cudaSetDevice(c->desc.device);
  const size_t vb = sizeof(double) * 3 * c->npix;
  std::vector<double> tmp(3 * c->npix);
  c->to_internal(xin, tmp.data());
  cudaError_t e = cudaMemcpyAsync(c->z.p, tmp.data(), vb, cudaMemcpyHostToDevice, c->st);
  if (e == cudaSuccess) e = c->apply_dev(c->z.as<double>(), c->q.as<double>(), masked != 0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tmp.data(), c->q.p, vb, cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) return c->cuda_fail(e, "apply");
  c->to_ring(tmp.data(), yout);
  return SG_OK;
}

extern "C" int sg_noise_filter(sg_ctx* c, const double* in, double* out) {
  if (!c) return SG_ERR_ARG;
  if (!in || !out) return c->fail(SG_ERR_ARG, "null array");
  for (long long dd = 0; dd < c->ndet; dd++)
    if (!c->have_noise[dd]) return c->fail(SG_ERR_STATE, "noise of detector %lld not set", dd);
  cudaSetDevice(c->desc.device);
  const long long n = c->nsamp;
  DevBuf din;
  cudaError_t e = din.alloc((size_t)n * c->esize);
  if (e != cudaSuccess) return c->cuda_fail(e, "noise_filter alloc");
  if (c->f32) {
    std::vector<float> f(in, in + n);
    e = cudaMemcpy(din.p, f.data(), 4 * n, cudaMemcpyHostToDevice);
  } else {
    e = cudaMemcpy(din.p, in, 8 * n, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = c->launch_filter(kLoadTod, din.p, c->y.p, c->ntiles, (int)c->nseg, 0);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  if (e == cudaSuccess) {
    if (c->f32) {
      std::vector<float> f(n);
      e = cudaMemcpy(f.data(), c->y.p, 4 * n, cudaMemcpyDeviceToHost);
      for (long long i = 0; i < n; i++) out[i] = f[i];
    } else {
      e = cudaMemcpy(out, c->y.p, 8 * n, cudaMemcpyDeviceToHost);
    }
  }
  if (e != cudaSuccess) return c->cuda_fail(e, "noise_filter");
  return SG_OK;
}

// ---------------------------------------------------------------------------
// The pol mask of the CG steps: the true hits where the pixel's Q/U are
// solved for, min(hits, 1) where they are masked -- fewer than 2 hits (the
// reference's rule, sanepic.cc:1316-1330) or, with pol_rcond > 0, a 3 x 3
// block sum_i w_i w_i^T (w = (1, cos 2psi, sin 2psi), every detector sample
// weighted 1) whose reciprocal condition number is below pol_rcond.
int build_polmask(sg_ctx* c) {
  const long long npix = c->npix;
  cudaError_t e = c->polmask.alloc(sizeof(int) * npix);
  if (e == cudaSuccess && c->pol_rcond <= 0.0)
    e = cudaMemcpyAsync(c->polmask.p, c->hits.p, sizeof(int) * npix, cudaMemcpyDeviceToDevice,
                        c->st);
  if (e == cudaSuccess && c->pol_rcond > 0.0) {
    const int G = c->ngroups;
    std::vector<double> gc(5 * G, 0.0);
    for (int g = 0; g < G; g++)
      for (int k = c->grp_off_h[g]; k < c->grp_off_h[g + 1]; k++) {
        const int dd = c->grp_det_h[k];
        const double d2 = 2.0 * (c->desc.hwp ? -c->psidet_h[dd] : c->psidet_h[dd]);
        gc[g] += 1.0;
        gc[G + g] += cos(d2);
        gc[2 * G + g] += sin(d2);
        gc[3 * G + g] += cos(2.0 * d2);
        gc[4 * G + g] += sin(2.0 * d2);
      }
    DevBuf ones;
    e = ones.alloc(sizeof(double) * 5 * G);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(ones.p, gc.data(), sizeof(double) * 5 * G, cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess) {
      if (c->f32)
        e = bj3_launch<float>(c->csr_off.as<long long>(), c->csr_idx.as<uint32_t>(),
                              c->csr_cs.as<float>(), npix, c->ns * c->nseg, G, ones.as<double>(),
                              c->hits.as<int>(), c->pol_rcond, c->polmask.as<int>(), nullptr,
                              c->st);
      else
        e = bj3_launch<double>(c->csr_off.as<long long>(), c->csr_idx.as<uint32_t>(),
                               c->csr_cs.as<double>(), npix, c->ns * c->nseg, G,
                               ones.as<double>(), c->hits.as<int>(), c->pol_rcond,
                               c->polmask.as<int>(), nullptr, c->st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);  // before `ones` is freed
  }
  if (e != cudaSuccess) return c->cuda_fail(e, "pol mask");
  return SG_OK;
}

int build_bj3(sg_ctx* c) {
  if (c->have_bj3) return SG_OK;
  // group constants (sum g0, sum g0 cos 2d', sum g0 sin 2d', sum g0 cos 4d',
  // sum g0 sin 4d') over each group's detectors, d' = the detector rotation
  const int G = c->ngroups;
  std::vector<double> gc(5 * G, 0.0);
  c->g0_h.resize(c->ndet);
  cudaError_t e0 = cudaMemcpyAsync(c->g0_h.data(), c->g0.p, sizeof(double) * c->ndet,
                                   cudaMemcpyDeviceToHost, c->st);
  if (e0 == cudaSuccess) e0 = cudaStreamSynchronize(c->st);
  if (e0 != cudaSuccess) return c->cuda_fail(e0, "bj3 build");
  for (int g = 0; g < G; g++)
    for (int k = c->grp_off_h[g]; k < c->grp_off_h[g + 1]; k++) {
      const int dd = c->grp_det_h[k];
      const double d2 = 2.0 * (c->desc.hwp ? -c->psidet_h[dd] : c->psidet_h[dd]);
      const double g0 = c->g0_h[dd];
      gc[g] += g0;
      gc[G + g] += g0 * cos(d2);
      gc[2 * G + g] += g0 * sin(d2);
      gc[3 * G + g] += g0 * cos(2.0 * d2);
      gc[4 * G + g] += g0 * sin(2.0 * d2);
    }
  cudaError_t e = c->gconst.alloc(sizeof(double) * 5 * G);
  if (e == cudaSuccess) e = cudaMemcpy(c->gconst.p, gc.data(), sizeof(double) * 5 * G,
                                       cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    if (c->f32)
      e = bj3_launch<float>(c->csr_off.as<long long>(), c->csr_idx.as<uint32_t>(),
                            c->csr_cs.as<float>(), c->npix, c->ns * c->nseg, G,
                            c->gconst.as<double>(), c->polmask.as<int>(), 0.0, nullptr,
                            c->minv.as<double>(), c->st);
    else
      e = bj3_launch<double>(c->csr_off.as<long long>(), c->csr_idx.as<uint32_t>(),
                             c->csr_cs.as<double>(), c->npix, c->ns * c->nseg, G,
                             c->gconst.as<double>(), c->polmask.as<int>(), 0.0, nullptr,
                             c->minv.as<double>(), c->st);
  }
  if (e == cudaSuccess && c->f32) {
    e = c->minv32.alloc(sizeof(float) * 6 * c->npix);
    if (e == cudaSuccess) e = to_f32_launch(c->minv.as<double>(), c->minv32.as<float>(),
                                            6 * c->npix, c->st);
    c->launches++;
  }
  if (e != cudaSuccess) return c->cuda_fail(e, "bj3 build");
  c->have_bj3 = true;
  return SG_OK;
}

// The reference's diagonal (also needed for the NVAR outputs).
int build_diag(sg_ctx* c) {
  if (c->have_diag) return SG_OK;
  cudaError_t e;
  const long long ns = c->ns, npix = c->npix;
  // N_ = c2r(|SpN|) per detector: the filter with |h| applied to a unit impulse
  if ((e = c->ntab.alloc((size_t)c->ndet * ns * c->esize)) != cudaSuccess)
    return c->cuda_fail(e, "diag alloc");
  e = c->launch_filter(kLoadDelta, nullptr, c->ntab.p, c->ndet, 1, 1);
  // the group's pixel stream is shared, so the detectors' tables add up
  DevBuf gtab;
  if (e == cudaSuccess) e = gtab.alloc((size_t)c->ngroups * ns * c->esize);
  if (e == cudaSuccess) {
    if (c->f32) {
      e = group_ntab_launch<float>(c->ntab.as<float>(), ns, c->ngroups, c->grp_off.as<int>(),
                                   c->grp_det.as<int>(), gtab.as<float>(), c->st);
      if (e == cudaSuccess)
        e = diag_launch<float>(c->csr_off.as<long long>(), c->csr_idx.as<uint32_t>(), npix, ns,
                               (int)c->nseg, gtab.as<float>(), c->mp_raw.as<double>(), c->st);
    } else {
      e = group_ntab_launch<double>(c->ntab.as<double>(), ns, c->ngroups, c->grp_off.as<int>(),
                                    c->grp_det.as<int>(), gtab.as<double>(), c->st);
      if (e == cudaSuccess)
        e = diag_launch<double>(c->csr_off.as<long long>(), c->csr_idx.as<uint32_t>(), npix, ns,
                                (int)c->nseg, gtab.as<double>(), c->mp_raw.as<double>(), c->st);
    }
  }
  if (e == cudaSuccess) e = mask_qu(c->mp_raw.as<double>(), c->hits.as<int>(), npix, c->st);
  std::vector<double> mp(3 * npix);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(mp.data(), c->mp_raw.p, sizeof(double) * 3 * npix, cudaMemcpyDeviceToHost,
                        c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) return c->cuda_fail(e, "diag build");
  for (long long m = 0; m < npix; m++)
    if (mp[m] == 0.0) return c->fail(SG_ERR_PRECOND, "Mp[%lld] has elements = 0", m);
  for (auto& v : mp) v = v != 0.0 ? 1.0 / v : 0.0;
  e = cudaMemcpy(c->mdiag.p, mp.data(), sizeof(double) * 3 * npix, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return c->cuda_fail(e, "diag upload");
  c->ntab.release();
  c->have_diag = true;
  return SG_OK;
}

extern "C" int sg_solve(sg_ctx* c, const sg_solve_opts* o, sg_report* rep) {
  if (!c || !o) return SG_ERR_ARG;
  int rc = check_ready(c, false);
  if (rc) return rc;
  if (!c->have_rhs) return c->fail(SG_ERR_STATE, "call sg_rhs before sg_solve");
  if (o->precond != SG_PRECOND_BJ3 && o->precond != SG_PRECOND_DIAG &&
      o->precond != SG_PRECOND_LEARNED)
    return c->fail(SG_ERR_UNSUPPORTED, "preconditioner %d not available", o->precond);
  if (o->precond == SG_PRECOND_LEARNED && !c->have_mlp && c->coarse_k == 0)
    return c->fail(SG_ERR_STATE, "train (sg_learn_train) or load (sg_learn_set_params) the network first");
  cudaSetDevice(c->desc.device);
  const double t0 = now_s();
  rc = (o->precond == SG_PRECOND_DIAG) ? build_diag(c) : build_bj3(c);
  if (rc == SG_OK && o->precond == SG_PRECOND_LEARNED && c->learned_kind == 1)
    rc = ensure_patches(c);
  if (rc) return rc;
  // chi^2 of the refresh iterations is computed only where it is seen
  c->refresh_chi2 = o->verbose != 0 || o->on_iteration != nullptr;
  // 0: reference diagonal, 1: block-Jacobi, 2: block-Jacobi + a learned part
  // (the network or the coarse space; flexible PCG)
  int pc = (o->precond == SG_PRECOND_BJ3) ? 1 : (o->precond == SG_PRECOND_DIAG ? 0 : 2);
  int fallback_iter = -1;
  if (pc == 2 && !c->learned_enabled) {  // plain PCG judged the network: it did not gain
    pc = 1;
    fallback_iter = 0;
  }
  const long long npix = c->npix;
  const size_t vb = sizeof(double) * 3 * npix;
  cudaError_t e;
  // x0 (masked, sanepic.cc:1209-1227, 1316-1330), r = A x0
  std::vector<double> x0i;
  if (o->x0) {
    x0i.resize(3 * npix);
    c->to_internal(o->x0, x0i.data());
    e = cudaMemcpyAsync(c->x.p, x0i.data(), vb, cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess) e = mask_qu(c->x.as<double>(), c->polmask.as<int>(), npix, c->st);
    if (e == cudaSuccess) e = c->apply_dev(c->x.as<double>(), c->r.as<double>(), true);
  } else {
    e = cudaMemsetAsync(c->x.p, 0, vb, c->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->r.p, 0, vb, c->st);
  }
  CgVecs v = c->vecs(pc == 2 ? 1 : pc);
  if (!c->ev0) cudaEventCreate(&c->ev0);
  if (!c->ev1) cudaEventCreate(&c->ev1);
  const long long launches0 = c->launches;
  if (e == cudaSuccess) e = cudaEventRecord(c->ev0, c->st);
  if (e == cudaSuccess) e = c->f32 ? cg_init<float>(v, c->st) : cg_init<double>(v, c->st);
  c->launches += 2;
  if (pc == 2) {  // z0 = M_bj3 r0 + correction, d0 = z0
    CgVecs v2 = c->vecs(2);
    if (e == cudaSuccess) e = c->learned_z(0);
    if (e == cudaSuccess)
      e = c->f32 ? cg_reinit_d<float>(v2, c->dmap.as<float>(), c->st)
                 : cg_reinit_d<double>(v2, c->dmap.as<double>(), c->st);
    c->launches += 1;
  } else if (e == cudaSuccess) {
    e = c->to_map(c->d.as<double>());
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->sc_host, c->sc.p, sizeof(CgScalars), cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) return c->cuda_fail(e, "solve init");
  const double t1 = now_s();
  const double var00 = c->sc_host->var00, delta0 = c->sc_host->delta0;
  double crit = c->sc_host->var / var00;
  const double crit0 = crit;
  const int refresh_every = o->refresh_every > 0 ? o->refresh_every : 10;
  // the reference's diagonal mode, and any solve that prints or reports chi2,
  // keeps the reference's true residual at iteration 0
  const int skip0 = (pc != 0 && !c->refresh_chi2) ? 1 : 0;
  const int maxiter = o->maxiter > 0 ? o->maxiter : 2000;
  c->crit_hist.clear();
  c->have_solution = true;  // the callback may read the current map
  int iter = 0;
  bool loop_done = false;
  // With nothing to report per iteration (no printed line, no callback) the
  // whole loop runs on the device: one graph launch, the convergence test in
  // a kernel (SANEPIC_GPU_DEVICE_LOOP=0 keeps the host-driven loop).
  const char* dl_env = getenv("SANEPIC_GPU_DEVICE_LOOP");
  if (o->use_graph && !o->verbose && !o->on_iteration && !(dl_env && dl_env[0] == '0')) {
    sg_ctx::LoopGraph* lg = nullptr;
    LoopState ls{0, maxiter, refresh_every, 0, o->stop_crit, 0, 0, skip0};
    e = c->ensure_loop_buffers(maxiter);
    if (e == cudaSuccess) e = c->solve_loop_graph(pc, &lg);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(c->loop_state.p, &ls, sizeof(ls), cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess) e = cudaGraphLaunch(lg->exec, c->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&ls, c->loop_state.p, sizeof(ls), cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(c->sc_host, c->sc.p, sizeof(CgScalars), cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) return c->cuda_fail(e, "device solve loop");
    iter = ls.iter;
    c->crit_hist.resize(iter);
    if (iter > 0)
      e = cudaMemcpy(c->crit_hist.data(), c->loop_hist.p, sizeof(double) * iter, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return c->cuda_fail(e, "device solve loop");
    const long long nref = refresh_count(iter, refresh_every, skip0);
    c->launches += nref * lg->launches_refresh + (iter - nref) * lg->launches_plain + 2LL * iter;
    crit = c->sc_host->var / var00;
    // a breakdown of the learned part falls back below; any other stop is final
    loop_done = !(ls.done == 3 && pc == 2 && crit > o->stop_crit);
    if (ls.done == 3 && pc == 2 && crit > o->stop_crit) {
      fallback_iter = iter;
      pc = 1;
      CgVecs v1 = c->vecs(1);
      e = c->apply_dev(c->x.as<double>(), c->r.as<double>(), true);
      if (e == cudaSuccess) e = c->f32 ? cg_init<float>(v1, c->st) : cg_init<double>(v1, c->st);
      if (e == cudaSuccess) e = c->to_map(c->d.as<double>());
      c->launches += 7;
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->sc_host, c->sc.p, sizeof(CgScalars), cudaMemcpyDeviceToHost, c->st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
      if (e != cudaSuccess) return c->cuda_fail(e, "fallback restart");
    }
  }
  while (!loop_done && ((iter < maxiter && crit > o->stop_crit) || iter == 0)) {
    const bool refresh = refresh_at(iter, refresh_every, skip0);
    e = c->run_iteration(pc, refresh, o->use_graph != 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(c->sc_host, c->sc.p, sizeof(CgScalars), cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) return c->cuda_fail(e, "solve iteration");
    crit = c->sc_host->var / var00;
    c->crit_hist.push_back(crit);
    const double crit2 = c->sc_host->delta / delta0, chi2 = c->sc_host->chi2;
    if (o->verbose)
      printf("iter = %d, crit = %10.15g, crit2 = %10.15g, chi2 = %10.15g\n", iter, crit, crit2,
             chi2);
    const int stop = o->on_iteration ? o->on_iteration(o->user, iter, crit, crit2, chi2) : 0;
    iter++;
    if (stop) break;
    if (c->sc_host->flag && pc == 2 && crit > o->stop_crit) {
      // the network's correction broke flexible PCG: restart from the current
      // map with plain block-Jacobi PCG (r = b - A x, z = M r, d = z)
      fallback_iter = iter;
      pc = 1;
      CgVecs v1 = c->vecs(1);
      e = c->apply_dev(c->x.as<double>(), c->r.as<double>(), true);
      if (e == cudaSuccess) e = c->f32 ? cg_init<float>(v1, c->st) : cg_init<double>(v1, c->st);
      if (e == cudaSuccess) e = c->to_map(c->d.as<double>());
      c->launches += 7;
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->sc_host, c->sc.p, sizeof(CgScalars), cudaMemcpyDeviceToHost, c->st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
      if (e != cudaSuccess) return c->cuda_fail(e, "fallback restart");
      continue;
    }
    // d^T A d <= 0 or r^T z <= 0: the recurrence has hit rounding level (or a
    // non-SPD preconditioner); stop with the current map
    if (c->sc_host->flag) break;
  }
  e = cudaEventRecord(c->ev1, c->st);
  if (e == cudaSuccess) e = cudaEventSynchronize(c->ev1);
  float dev_ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&dev_ms, c->ev0, c->ev1);
  if (e != cudaSuccess) return c->cuda_fail(e, "solve timing");
  const double t2 = now_s();
  c->have_solution = true;
  if (rep) {
    rep->iterations = iter;
    rep->converged = crit <= o->stop_crit;
    rep->crit = crit;
    rep->var00 = var00;
    rep->solve_seconds = t2 - t1;
    rep->iter_per_sec = iter / (t2 - t1 > 0 ? t2 - t1 : 1e-30);
    rep->setup_seconds = t1 - t0;
    rep->device_seconds = dev_ms * 1e-3;
    rep->kernel_launches = (long)(c->launches - launches0);
    rep->breakdown = c->sc_host->flag;
    rep->fallback_iter = fallback_iter;
    rep->crit0 = crit0;
  }
  return SG_OK;
}

// ---------------------------------------------------------------------------
static void expand(const sg_ctx* c, const double* compact, double* full) {
  for (long long p = 0; p < c->npixfull; p++) full[p] = 0.0;
  for (long long m = 0; m < c->npix; m++) full[c->int2ring[m]] = compact[m];
}

extern "C" int sg_get_map(sg_ctx* c, int kind, double* out) {
  if (!c || !out) return SG_ERR_ARG;
  if (!c->have_pointing) return c->fail(SG_ERR_STATE, "pointing not set");
  cudaSetDevice(c->desc.device);
  const long long npix = c->npix;
  std::vector<double> v;
  if (kind < SG_MAP_I || kind > SG_MAP_U) v.resize(3 * npix);
  cudaError_t e = cudaSuccess;
  const double* blk = nullptr;
  switch (kind) {
    case SG_MAP_I:
    case SG_MAP_Q:
    case SG_MAP_U: {
      // only the requested component, expanded to the full-sky RING map on
      // the device (the int -> RING table kept from sg_set_pointing) and
      // copied out once
      if (!c->have_solution) return c->fail(SG_ERR_STATE, "no solution yet");
      const size_t fb = sizeof(double) * c->npixfull;
      e = c->map_full.alloc(fb);
      if (e == cudaSuccess) e = cudaMemsetAsync(c->map_full.p, 0, fb, c->st);
      if (e == cudaSuccess)
        e = expand_launch(c->x.as<double>() + (kind - SG_MAP_I) * npix,
                          c->pscr.i2r.as<long long>(), npix, c->map_full.as<double>(), c->st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(out, c->map_full.p, fb, cudaMemcpyDeviceToHost, c->st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
      if (e != cudaSuccess) return c->cuda_fail(e, "get_map");
      return SG_OK;
    }
    case SG_MAP_NVAR:
    case SG_MAP_Q_NVAR:
    case SG_MAP_U_NVAR: {
      int rc = build_diag(c);
      if (rc) return rc;
      e = cudaMemcpy(v.data(), c->mdiag.p, sizeof(double) * 3 * npix, cudaMemcpyDeviceToHost);
      blk = v.data() + (kind - SG_MAP_NVAR) * npix;
      break;
    }
    case SG_MAP_HITS:
    case SG_MAP_POL_HITS: {
      std::vector<int> h(npix);
      e = cudaMemcpy(h.data(), c->hits.p, sizeof(int) * npix, cudaMemcpyDeviceToHost);
      for (long long m = 0; m < npix; m++) v[m] = 2.0 * h[m];  // doubled (Q1)
      blk = v.data();
      break;
    }
    case SG_MAP_COS2P:
    case SG_MAP_SIN2P: {
      std::vector<int> h(npix);
      e = cudaMemcpy(v.data(), c->sumcross.p, sizeof(double) * 3 * npix, cudaMemcpyDeviceToHost);
      if (e == cudaSuccess) e = cudaMemcpy(h.data(), c->hits.p, sizeof(int) * npix, cudaMemcpyDeviceToHost);
      if (kind == SG_MAP_SIN2P)
        for (long long m = 0; m < npix; m++)
          if (h[m] < 2) v[npix + m] = 0.0;  // Q2 (sanepic.cc:1325-1328)
      blk = v.data() + (kind - SG_MAP_COS2P) * npix;
      break;
    }
    default:
      return c->fail(SG_ERR_ARG, "unknown map kind %d", kind);
  }
  if (e != cudaSuccess) return c->cuda_fail(e, "get_map");
  expand(c, blk, out);
  return SG_OK;
}

extern "C" int sg_get_solution(sg_ctx* c, double* out) {
  if (!c || !out) return SG_ERR_ARG;
  if (!c->have_solution) return c->fail(SG_ERR_STATE, "no solution yet");
  std::vector<double> tmp(3 * c->npix);
  cudaError_t e =
      cudaMemcpy(tmp.data(), c->x.p, sizeof(double) * 3 * c->npix, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return c->cuda_fail(e, "get_solution");
  c->to_ring(tmp.data(), out);
  return SG_OK;
}

extern "C" int sg_get_pixels(sg_ctx* c, long* ring_out) {
  if (!c || !ring_out) return SG_ERR_ARG;
  if (!c->have_pointing) return c->fail(SG_ERR_STATE, "pointing not set");
  std::vector<int> comp(c->ngsamp);
  cudaError_t e =
      cudaMemcpy(comp.data(), c->pix.p, sizeof(int) * c->ngsamp, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return c->cuda_fail(e, "get_pixels");
  const long long nsd = c->ns * c->nseg;
  for (int g = 0; g < c->ngroups; g++)
    for (int k = c->grp_off_h[g]; k < c->grp_off_h[g + 1]; k++) {
      const long long dd = c->grp_det_h[k];
      for (long long w = 0; w < nsd; w++) ring_out[dd * nsd + w] = (long)c->int2ring[comp[g * nsd + w]];
    }
  return SG_OK;
}

extern "C" int sg_get_indpix(sg_ctx* c, long* out) {
  if (!c || !out) return SG_ERR_ARG;
  if (!c->have_pointing) return c->fail(SG_ERR_STATE, "pointing not set");
  for (long long p = 0; p < c->npixfull; p++) out[p] = c->indpix_host[p];
  return SG_OK;
}

extern "C" int sg_profile_operator(sg_ctx* c, int reps, double* ms) {
  if (!c || !ms || reps < 1) return SG_ERR_ARG;
  int rc = check_ready(c, false);
  if (rc) return rc;
  cudaSetDevice(c->desc.device);
  cudaEvent_t ev[5];
  for (auto& x : ev) cudaEventCreate(&x);
  cudaError_t e = c->to_map(c->d.as<double>());
  float tot[4] = {0.f, 0.f, 0.f, 0.f};
  for (int i = 0; i < reps && e == cudaSuccess; i++) {
    e = cudaEventRecord(ev[0], c->st);
    if (c->grouped()) {
      // projection = (a, b1, b2) (mixed by W for uniform groups); N^-1 into
      // P^T's layout (the three-pass weighting, or the cluster FFT kernels);
      // no detector sums
      if (e == cudaSuccess) e = c->group_project_step();
      if (e == cudaSuccess) e = cudaEventRecord(ev[1], c->st);
      if (e == cudaSuccess) e = c->group_weight_step();
      if (e == cudaSuccess) e = cudaEventRecord(ev[2], c->st);
    } else {
      if (e == cudaSuccess) e = c->launch_project(c->gains_on ? &c->gain2_t : nullptr);
      if (e == cudaSuccess) e = cudaEventRecord(ev[1], c->st);
      if (e == cudaSuccess) e = c->detector_weight_step(c->y.p, c->y.p);
      if (e == cudaSuccess) e = cudaEventRecord(ev[2], c->st);
      if (e == cudaSuccess) e = c->launch_detsum();
    }
    if (e == cudaSuccess) e = cudaEventRecord(ev[3], c->st);
    if (e == cudaSuccess) e = c->launch_pt(c->q.as<double>(), true);
    if (e == cudaSuccess) e = cudaEventRecord(ev[4], c->st);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[4]);
    for (int k = 0; k < 4 && e == cudaSuccess; k++) {
      float t = 0.f;
      e = cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
      tot[k] += t;
    }
  }
  for (auto& x : ev) cudaEventDestroy(x);
  if (e != cudaSuccess) return c->cuda_fail(e, "profile_operator");
  for (int k = 0; k < 4; k++) ms[k] = tot[k] / reps;
  return SG_OK;
}

extern "C" int sg_get_crit_history(sg_ctx* c, double* out, int max) {
  if (!c || !out) return SG_ERR_ARG;
  const int n = std::min<int>(max, (int)c->crit_hist.size());
  for (int i = 0; i < n; i++) out[i] = c->crit_hist[i];
  return n;
}
