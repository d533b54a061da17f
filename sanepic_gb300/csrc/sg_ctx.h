// sg_ctx.h -- the library context behind the C ABI (internal): problem
// sizes, the pixelisation, device buffers, the operator pieces A = P^T N^-1 P
// and the PCG iteration as a launch sequence (captured in CUDA graphs).
#pragma once
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "../../include/sanepic_gpu.h"
#include "sg_kernels.h"
#include "sg_mlp.h"

using namespace sg;

struct sg_ctx;
void forget_batch_graphs(const sg_ctx* c);  // sg_batch.cu: drop cached batch graphs using c

namespace sg {

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  // contents are undefined after alloc; a buffer of the same size is kept
  // (no cudaFree / cudaMalloc when a setter runs again on same-sized data)
  cudaError_t alloc(size_t n) {
    if (p && bytes == n) return cudaSuccess;
    release();
    bytes = n;
    if (n == 0) return cudaSuccess;
    return cudaMalloc(&p, n);
  }
  template <typename U>
  U* as() const {
    return reinterpret_cast<U*>(p);
  }
};

inline double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

constexpr double kD2PI = 6.2831853071795864769252867665590057683943387987502;

}  // namespace sg

struct sg_ctx {
  sg_desc desc{};
  std::string err;
  cudaStream_t st = nullptr;
  cudaStream_t own_st = nullptr;  // the stream the context created
  int f32 = 0;       // precision
  int esize = 8;     // bytes per real
  long long ns = 0, nseg = 0, ndet = 0, ntiles = 0, nsamp = 0, npixfull = 0;
  int logm = 0, S = 1, nclusters = 1;
  long long npix = 0;
  std::vector<int> indpix_host;        // RING pixel -> RING-order compact index (reference)
  std::vector<long long> int2ring;     // internal index -> RING pixel
  std::vector<long long> int2ringc;    // internal index -> RING-order compact index
  std::vector<long long> isampmin;

  // Detectors with identical focal-plane offsets share one pixel stream (an
  // offset group).  pix, cs, csr_* live per group sample (ngsamp of them);
  // y and tod per detector sample (nsamp).
  int ngroups = 0;
  long long ngsamp = 0;
  std::vector<int> grp_off_h, grp_det_h;
  std::vector<double> g0_h, psidet_h;
  DevBuf pix, cs, y, tod, csr_off, csr_idx, csr_cs, hits, indpix, sumcross;
  // the pol mask every CG step uses: true hits, or min(hits, 1) where the Q/U
  // block is masked -- the reference's rule (fewer than 2 hits) and, with
  // pol_rcond > 0, blocks whose reciprocal condition number is below it
  DevBuf polmask;
  double pol_rcond = 0.0;
  DevBuf grp_off, grp_det, dcs, ys, gconst;
  DevBuf filt, tw_lo, tw_hi, g0, ntab;
  DevBuf x, r, d, q, z, rprev, b, minv, mdiag, mp_raw, part, sc, dmap;
  DevBuf minv32;  // FP32 operators: the bj3 blocks in FP32 as well
  DevBuf chi2p;  // per-CTA chi^2 partials of the noise filter
  // offset-group operator (sg_group.cu): used when every group has at least
  // kGroupMin detectors; gtl [G][3][nsd], gspec [G][3][nseg][M+1] complex,
  // hmix [G][M+1][6]
  static constexpr int kGroupMin = 4;
  bool group_mode = false, have_hmix = false;
  // per (detector, segment) gains of the recalibration loop (sg_set_gains,
  // sanepic.cc:1044-1053 and 2508-2510): A = P^T G N^-1 G P and
  // b = P^T G N^-1 d with G = diag(g) tile by tile.  Gains of one tile break
  // the sums of an offset group, so the operator runs per detector while
  // they are set.
  bool gains_on = false;
  DevBuf gain_t, gain2_t;       // g and g^2 per tile [det][seg], in the operator's type
  std::vector<double> gains_h;  // g per tile [det][seg]
  DevBuf yb, tdots;             // the gain fit's second timeline buffer and per-tile sums
  std::vector<double> spn_edge;  // per detector: the weights of bins 0 and ns/2 (FP64)
  bool grouped() const { return group_mode && !gains_on; }
  DevBuf gtl, gspec, hmix, dspec, rhs_part;  // + data spectra [ndet][nseg][M+1], chi^2 partials
  DevBuf kslot, filt_slot;  // frequency of each spectrum slot; filter rows in slot order
  int kslot_S = -1;         // the tile shape kslot was made for
  int hmix_S = 0;           // the tile shape (cluster size) the slot order was built for
  DevBuf stage, nanflag;  // FP64 staging of two detectors' timelines, NaN flags
  // the timelines' copies run on their own stream, two staging buffers deep
  // (sg_set_tod_all: the copy of detector k + 1 overlaps the conversion of k)
  cudaStream_t copy_st = nullptr;
  cudaEvent_t ev_staged[2] = {nullptr, nullptr}, ev_ingested[2] = {nullptr, nullptr};
  DevBuf map_full;        // a full-sky RING map being read out
  // sg_set_pointing's device scratch (boresight, pixels, numbering and sort
  // temporaries), kept between calls
  struct PointingScratch {
    DevBuf ra, dec, psi, offx, offy, ring, psio, flag, count, scratch, gsz, gsc, gss;
    DevBuf ntmp, i2r, i2rc, ipr, np, cs64;
  } pscr;
  DevBuf noise_stage, noise_part;  // one detector's iSpf values; g0 partial sums
  cudaEvent_t ev_copy = nullptr;   // host->device copy of a caller's array done

  // learned preconditioner: the network, the nested patch geometry
  // (patch_idx [npatch_pad][256] internal pixel or -1), per-patch scales, and
  // the synthetic timeline used while generating training pairs
  std::unique_ptr<Mlp> mlp;
  DevBuf patch_idx, patch_sig, tod_syn, filt_noise;
  int npatch = 0, npatch_pad = 0;
  bool have_mlp = false, use_syn = false;
  bool learned_enabled = false;  // validation: a learned component beat plain PCG
  // learned coarse space: U, AU = A U [3 npix][coarse_pad(kc)] BF16, E^-1 [kc][kc] FP64
  DevBuf cs_u, cs_au, cs_einv, cs_coef, cs_part;
  int coarse_k = 0;
  int learned_kind = 0;  // SG_PRECOND_LEARNED applies 1: the network, 2: the coarse space
  // captured learned iterations embed the kind: change it only through here
  void set_learned_kind(int k) {
    if (k != learned_kind) drop_graphs();
    learned_kind = k;
  }
  const void* tod_active() const { return use_syn ? tod_syn.p : tod.p; }
  cplx<float> wn1f{1.f, 0.f};
  cplx<double> wn1d{1.0, 0.0};
  CgScalars* sc_host = nullptr;  // pinned

  bool have_pointing = false, have_rhs = false, have_solution = false;
  bool have_bj3 = false, have_diag = false;
  std::vector<char> have_noise, have_tod;
  std::vector<double> crit_hist;
  std::map<std::pair<int, int>, cudaGraphExec_t> graphs;
  std::map<std::pair<int, int>, long long> graph_launches;
  long long launches = 0;  // kernels launched by this context
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;

  int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    err = buf;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    return fail(SG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  }
  ~sg_ctx() {
    forget_batch_graphs(this);
    for (auto& kv : loop_graphs) cudaGraphExecDestroy(kv.second.exec);
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    if (ev0) cudaEventDestroy(ev0);
    if (ev_copy) cudaEventDestroy(ev_copy);
    for (int b = 0; b < 2; b++) {
      if (ev_staged[b]) cudaEventDestroy(ev_staged[b]);
      if (ev_ingested[b]) cudaEventDestroy(ev_ingested[b]);
    }
    if (copy_st) cudaStreamDestroy(copy_st);
    if (ev1) cudaEventDestroy(ev1);
    if (sc_host) cudaFreeHost(sc_host);
    if (own_st) cudaStreamDestroy(own_st);
  }

  // compact vectors [I|Q|U]: RING-order compact (API) <-> internal order
  void to_internal(const double* ringc, double* out) const {
    for (int cc = 0; cc < 3; cc++)
      for (long long m = 0; m < npix; m++) out[cc * npix + m] = ringc[cc * npix + int2ringc[m]];
  }
  void to_ring(const double* internal, double* out) const {
    for (int cc = 0; cc < 3; cc++)
      for (long long m = 0; m < npix; m++) out[cc * npix + int2ringc[m]] = internal[cc * npix + m];
  }

  // ---- operator pieces ---------------------------------------------------
  template <typename T>
  FilterArgs<T> filter_args(int mode, const T* in, T* out, long long ntiles_, int nseg_,
                            int filt_abs, const T* sub, double* chi2_part,
                            const T* table = nullptr) {
    FilterArgs<T> a{};
    a.ntiles = ntiles_;
    a.nseg = nseg_;
    a.mode = mode;
    a.filt_abs = filt_abs;
    a.tod = in;
    a.sub = sub;
    a.chi2_part = chi2_part;
    a.filt = table ? table : filt.as<T>();
    a.out = out;
    a.tw_lo = tw_lo.as<cplx<T>>();
    a.tw_hi = tw_hi.as<cplx<T>>();
    return a;
  }

  // chi2_out (device double) receives 2 sum h |X|^2 over all tiles when set
  cudaError_t launch_filter(int mode, const void* in, void* out, long long ntiles_, int nseg_,
                            int filt_abs, const void* sub = nullptr, double* chi2_out = nullptr,
                            const void* table = nullptr, int ilv3 = 0) {
    const int ncl = (int)std::min<long long>(nclusters, ntiles_);
    double* part = chi2_out ? chi2p.as<double>() : nullptr;
    cudaError_t e;
    launches++;
    if (f32) {
      auto a = filter_args<float>(mode, (const float*)in, (float*)out, ntiles_, nseg_, filt_abs,
                                  (const float*)sub, part, (const float*)table);
      a.wn1 = wn1f;
      a.ilv3 = ilv3;
      e = filter_launch<float>(a, logm, S, ncl, st);
    } else {
      auto a = filter_args<double>(mode, (const double*)in, (double*)out, ntiles_, nseg_,
                                   filt_abs, (const double*)sub, part, (const double*)table);
      a.wn1 = wn1d;
      a.ilv3 = ilv3;
      e = filter_launch<double>(a, logm, S, ncl, st);
    }
    if (e == cudaSuccess && chi2_out) {
      launches++;
      e = chi2_sum(part, S * ncl, chi2_out, st);
    }
    return e;
  }

  // per group sample detector sums of y, then the CSR reduction into a map
  cudaError_t launch_detsum() {
    launches++;
    if (f32)
      return detsum_launch<float>(y.as<float>(), ngsamp, ns * nseg, grp_off.as<int>(),
                                  grp_det.as<int>(), dcs.as<float>(), ys.as<float>(), st);
    return detsum_launch<double>(y.as<double>(), ngsamp, ns * nseg, grp_off.as<int>(),
                                 grp_det.as<int>(), dcs.as<double>(), ys.as<double>(), st);
  }

  // lanes per pixel of the FP32 P^T (0: from the mean samples per pixel;
  // sg_autotune may choose another)
  int pt_L = 0;
  int pt_team() const { return pt_L > 0 ? pt_L : pt_lanes(ngsamp, npix); }
  cudaError_t launch_pt(double* out, bool masked) {
    const int* h = masked ? polmask.as<int>() : nullptr;
    launches++;
    if (f32)
      return pt_launch<float>(csr_off.as<long long>(), csr_idx.as<uint32_t>(), csr_cs.as<float>(),
                              ys.as<float>(), npix, h, out, pt_team(), st);
    return pt_launch<double>(csr_off.as<long long>(), csr_idx.as<uint32_t>(), csr_cs.as<double>(),
                             ys.as<double>(), npix, h, out, 32, st);
  }

  // out = P^T y (y in time order, one row per detector)
  cudaError_t pt_of_y(double* out, bool masked) {
    cudaError_t e = launch_detsum();
    if (e == cudaSuccess) e = launch_pt(out, masked);
    return e;
  }

  cudaError_t to_map(const double* v) {
    launches++;
    if (f32) return to_map4<float>(v, npix, dmap.as<float>(), st);
    return to_map4<double>(v, npix, dmap.as<double>(), st);
  }

  // y = P map (time order, every detector), each tile times tsc[tile] when
  // tsc is set (the gains: g^2 in A, g in the residual d - G P x)
  cudaError_t launch_project(const DevBuf* tsc = nullptr, void* out = nullptr) {
    launches++;
    void* o = out ? out : y.p;
    if (f32)
      return project_launch<float>(pix.as<int>(), cs.as<float>(), dmap.as<float>(), ngsamp,
                                   ns * nseg, grp_off.as<int>(), grp_det.as<int>(),
                                   dcs.as<float>(), (float*)o, tsc ? tsc->as<float>() : nullptr,
                                   ns, st);
    return project_launch<double>(pix.as<int>(), cs.as<double>(), dmap.as<double>(), ngsamp,
                                  ns * nseg, grp_off.as<int>(), grp_det.as<int>(),
                                  dcs.as<double>(), (double*)o, tsc ? tsc->as<double>() : nullptr,
                                  ns, st);
  }
  // y *= g per tile (G after N^-1: b = P^T G N^-1 d, r = P^T G N^-1 (d - G P x))
  cudaError_t scale_by_gain(void* t) {
    launches++;
    return f32 ? tile_scale_launch<float>((float*)t, gain_t.as<float>(), ntiles, ns, st)
               : tile_scale_launch<double>((double*)t, gain_t.as<double>(), ntiles, ns, st);
  }

  cudaError_t apply_map(double* out, bool masked) {
    if (grouped()) return apply_map_group(out, masked);
    cudaError_t e = launch_project(gains_on ? &gain2_t : nullptr);
    if (e == cudaSuccess) e = detector_weight_step(y.p, y.p);
    if (e == cudaSuccess) e = pt_of_y(out, masked);
    return e;
  }

  // N^-1 of the per-detector operator, out = N^-1 in (timelines [ntiles][ns],
  // in == out allowed): the three-pass FP32 filter in batches through L2, or
  // the fused cluster filter
  cudaError_t detector_weight_step(const void* in, void* out) {
    if (!use_f3) return launch_filter(kLoadTod, in, out, ntiles, (int)nseg, 0);
    launches += 3 * ((ntiles + f3_batch - 1) / f3_batch);
    return fft3_detector_filter((const float*)in, (float*)out, f3scratch.as<float>(),
                                filt_pos.as<float>(), ntiles, f3_batch, (int)nseg, logm,
                                tw_lo.as<cplx<float>>(), tw_hi.as<cplx<float>>(), wn1f, st);
  }

  // forward FFT of tiles to spec_out, or inverse FFT of spec_in to tiles
  cudaError_t launch_filter_spec(const void* in, void* out, void* spec_out, const void* spec_in,
                                 long long ntiles_, int ilv3 = 0) {
    const int ncl = (int)std::min<long long>(nclusters, ntiles_);
    launches++;
    if (f32) {
      auto a = filter_args<float>(kLoadTod, (const float*)in, (float*)out, ntiles_, (int)nseg, 0,
                                  nullptr, nullptr);
      a.wn1 = wn1f;
      a.spec_out = (cplx<float>*)spec_out;
      a.spec_in = (const cplx<float>*)spec_in;
      a.ilv3 = ilv3;
      return filter_spec_launch<float>(a, logm, S, ncl, st);
    }
    auto a = filter_args<double>(kLoadTod, (const double*)in, (double*)out, ntiles_, (int)nseg, 0,
                                 nullptr, nullptr);
    a.wn1 = wn1d;
    a.spec_out = (cplx<double>*)spec_out;
    a.spec_in = (const cplx<double>*)spec_in;
    a.ilv3 = ilv3;
    return filter_spec_launch<double>(a, logm, S, ncl, st);
  }

  // the per-group mixing matrices from the filter rows (before any group apply)
  // (the slot order depends on the tile shape: rebuilt when the autotuner
  // changes the cluster size)
  // the per-detector operator's three-pass filter: the filter rows in
  // position order and the batches' scratch (made here, not while a graph
  // is being captured)
  cudaError_t ensure_f3_detector() {
    if (have_hmix) return cudaSuccess;
    const long long M1 = ns / 2 + 1;
    const char* f3env = getenv("SANEPIC_GPU_FFT3");
    use_f3 = f32 && fft3_supported(logm) && !(f3env && f3env[0] == '0');
    cudaError_t e = cudaSuccess;
    if (use_f3) {
      std::vector<int> kf;
      fft3_pos_freq(logm, kf);
      e = krow.alloc(sizeof(int) * M1);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(krow.p, kf.data(), sizeof(int) * M1, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // kf is a host temporary
      if (e == cudaSuccess) e = filt_pos.alloc((size_t)ndet * M1 * esize);
      if (e == cudaSuccess)
        e = permute_rows_launch<float>(filt.as<float>(), krow.as<int>(), ndet, M1,
                                       filt_pos.as<float>(), st);
      f3_batch = std::min<long long>(ntiles, fft3_rhs_batch(logm));
      if (e == cudaSuccess) e = f3scratch.alloc((size_t)f3_batch * ns * sizeof(float));
      launches += 1;
    }
    if (e == cudaSuccess) have_hmix = true;
    return e;
  }

  cudaError_t ensure_hmix() {
    if (!group_mode) return ensure_f3_detector();
    if (have_hmix && hmix_S == S) return cudaSuccess;
    const long long M1 = ns / 2 + 1;
    cudaError_t e = filt_slot.alloc((size_t)ndet * M1 * esize);
    if (e == cudaSuccess && kslot_S != S) {  // the slot order depends on the tile shape only
      std::vector<int> kf;
      spec_slot_freq(logm, S, kf);
      e = kslot.alloc(sizeof(int) * M1);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(kslot.p, kf.data(), sizeof(int) * M1, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // kf is a host temporary
      if (e == cudaSuccess) kslot_S = S;
    }
    if (e != cudaSuccess) return e;
    if (f32) {
      e = group_hmix_launch<float>(filt.as<float>(), dcs.as<float>(), grp_off.as<int>(),
                                   grp_det.as<int>(), kslot.as<int>(), ngroups, M1,
                                   hmix.as<float>(), st);
      if (e == cudaSuccess)
        e = permute_rows_launch<float>(filt.as<float>(), kslot.as<int>(), ndet, M1,
                                       filt_slot.as<float>(), st);
    } else {
      e = group_hmix_launch<double>(filt.as<double>(), dcs.as<double>(), grp_off.as<int>(),
                                    grp_det.as<int>(), kslot.as<int>(), ngroups, M1,
                                    hmix.as<double>(), st);
      if (e == cudaSuccess)
        e = permute_rows_launch<double>(filt.as<double>(), kslot.as<int>(), ndet, M1,
                                        filt_slot.as<double>(), st);
    }
    launches += 2;
    // do all detectors of each group share one noise spectrum?  Then the
    // right-hand side needs no per-detector FFT (rhs_of)
    DevBuf same;
    if (e == cudaSuccess) e = same.alloc(sizeof(int) * ndet);
    if (e == cudaSuccess) e = cudaMemsetAsync(same.p, 0, sizeof(int) * ndet, st);
    if (e == cudaSuccess)
      e = f32 ? rows_match_group_launch<float>(filt.as<float>(), M1, grp_off.as<int>(),
                                               grp_det.as<int>(), ngroups, grp_off_h[ngroups],
                                               same.as<int>(), st)
              : rows_match_group_launch<double>(filt.as<double>(), M1, grp_off.as<int>(),
                                                grp_det.as<int>(), ngroups, grp_off_h[ngroups],
                                                same.as<int>(), st);
    std::vector<int> same_h(ndet, 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(same_h.data(), same.p, sizeof(int) * ndet, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    groups_uniform = e == cudaSuccess;
    for (long long d = 0; d < ndet && groups_uniform; d++) groups_uniform = same_h[d] == 1;
    launches += 1;
    // uniform groups: W per group and the group's filter row for each of its
    // three timelines (tile row g * 3 + component), natural frequency order
    if (e == cudaSuccess && groups_uniform) {
      e = wmix.alloc((size_t)6 * ngroups * esize);
      if (e == cudaSuccess) e = gfilt.alloc((size_t)3 * ngroups * M1 * esize);
      if (e == cudaSuccess)
        e = f32 ? group_wmix_launch<float>(dcs.as<float>(), grp_off.as<int>(), grp_det.as<int>(),
                                           ngroups, wmix.as<float>(), st)
                : group_wmix_launch<double>(dcs.as<double>(), grp_off.as<int>(), grp_det.as<int>(),
                                            ngroups, wmix.as<double>(), st);
      for (long long g = 0; g < ngroups && e == cudaSuccess; g++) {
        const long long d0 = grp_det_h[grp_off_h[g]];
        for (int comp = 0; comp < 3 && e == cudaSuccess; comp++)
          e = cudaMemcpyAsync((char*)gfilt.p + (size_t)(3 * g + comp) * M1 * esize,
                              (const char*)filt.p + (size_t)d0 * M1 * esize, (size_t)M1 * esize,
                              cudaMemcpyDeviceToDevice, st);
      }
      launches += 1;
    }
    // the three-pass weighting: FP32, supported lengths, not switched off
    const char* f3env = getenv("SANEPIC_GPU_FFT3");
    use_f3 = e == cudaSuccess && f32 && fft3_supported(logm) && !(f3env && f3env[0] == '0');
    if (use_f3) {
      std::vector<int> kf;
      fft3_pos_freq(logm, kf);
      e = krow.alloc(sizeof(int) * M1);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(krow.p, kf.data(), sizeof(int) * M1, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // kf is a host temporary
      if (e == cudaSuccess) e = hrow.alloc((size_t)ngroups * M1 * (groups_uniform ? 1 : 6) * esize);
      if (e == cudaSuccess) e = filt_pos.alloc((size_t)ndet * M1 * esize);
      if (e == cudaSuccess)
        e = permute_rows_launch<float>(filt.as<float>(), krow.as<int>(), ndet, M1,
                                       filt_pos.as<float>(), st);
      f3_batch = std::min<long long>(ntiles, fft3_rhs_batch(logm));
      if (e == cudaSuccess) e = f3scratch.alloc((size_t)f3_batch * ns * sizeof(float));
      if (e == cudaSuccess && groups_uniform) {
        for (long long g = 0; g < ngroups && e == cudaSuccess; g++)
          e = permute_rows_launch<float>(filt.as<float>() + grp_det_h[grp_off_h[g]] * M1,
                                         krow.as<int>(), 1, M1, hrow.as<float>() + g * M1, st);
        launches += ngroups;
      } else if (e == cudaSuccess) {
        e = group_hmix_launch<float>(filt.as<float>(), dcs.as<float>(), grp_off.as<int>(),
                                     grp_det.as<int>(), krow.as<int>(), ngroups, M1,
                                     hrow.as<float>(), st);
        launches += 1;
      }
    }
    if (e == cudaSuccess) {
      have_hmix = true;
      hmix_S = S;
    }
    return e;
  }
  bool groups_uniform = false;  // every offset group's detectors share one noise spectrum
  DevBuf wmix, gfilt;           // uniform groups: W [G][6]; filter rows [3 G][M+1]
  // the three-pass weighting (sg_fft3.cu, FP32): the group timelines live in
  // P^T's layout (ys) and the weights in its row order, hrow [G][M+1][6] (H)
  // or [G][M+1] (one spectrum per group)
  bool use_f3 = false;
  DevBuf krow, hrow;
  DevBuf filt_pos, f3scratch;  // filter rows in position order; the forward batches' scratch
  long long f3_batch = 1;      // tiles per batch of the single-timeline passes

  // b = P^T N^-1 d for the timelines d (device, one row per detector) and
  // chi^2 of d into *chi2_dev.  Offset groups: the detectors' forward FFTs,
  // their weighted sums per group and frequency, three inverse FFTs per group.
  // With chi2_dev null and one noise spectrum per group, the detectors'
  // timelines are summed per group first: 3 FFT pairs per group and segment
  // instead of one forward FFT per detector and segment (same map; only the
  // rounding differs).
  cudaError_t rhs_of(const void* d, double* bout, double* chi2_dev) {
    if (!grouped()) {
      // with gains, G N^-1 d: chi^2_0 stays that of the raw data, as the
      // reference's calibrated data times its g^2 weights give
      // (sanepic.cc:1044-1053, 1089-1110)
      cudaError_t e = chi2_dev ? launch_filter(kLoadTod, d, y.p, ntiles, (int)nseg, 0, nullptr, chi2_dev)
                               : detector_weight_step(d, y.p);
      if (e == cudaSuccess && gains_on) e = scale_by_gain(y.p);
      if (e == cudaSuccess) e = pt_of_y(bout, true);
      return e;
    }
    const long long nsd = ns * nseg, M1 = ns / 2 + 1, gt = 3LL * ngroups * nseg;
    if (!chi2_dev && groups_uniform && use_f3) {
      // the detectors' timelines summed per group into P^T's layout, weighted
      // there by the group's one spectrum in place (the passes and P^T count
      // their own launches)
      launches += 1;
      cudaError_t e = group_tod_rhs_launch<float>((const float*)d, nsd, grp_off.as<int>(),
                                                  grp_det.as<int>(), dcs.as<float>(), ngroups,
                                                  ys.as<float>(), 1, st);
      if (e == cudaSuccess) e = fft3_weight();
      if (e == cudaSuccess) e = launch_pt(bout, true);
      return e;
    }
    if (!chi2_dev && groups_uniform) {
      cudaError_t e;
      launches += 2;  // sums, scaling
      if (f32) {
        e = group_tod_rhs_launch<float>((const float*)d, nsd, grp_off.as<int>(), grp_det.as<int>(),
                                        dcs.as<float>(), ngroups, gtl.as<float>(), 0, st);
        if (e == cudaSuccess) e = launch_filter_spec(gtl.p, nullptr, gspec.p, nullptr, gt);
        if (e == cudaSuccess)
          e = group_scale_launch<float>(gspec.as<cplx<float>>(), filt_slot.as<float>(),
                                        grp_off.as<int>(), grp_det.as<int>(), ngroups, nseg, M1, st);
      } else {
        e = group_tod_rhs_launch<double>((const double*)d, nsd, grp_off.as<int>(),
                                         grp_det.as<int>(), dcs.as<double>(), ngroups,
                                         gtl.as<double>(), 0, st);
        if (e == cudaSuccess) e = launch_filter_spec(gtl.p, nullptr, gspec.p, nullptr, gt);
        if (e == cudaSuccess)
          e = group_scale_launch<double>(gspec.as<cplx<double>>(), filt_slot.as<double>(),
                                         grp_off.as<int>(), grp_det.as<int>(), ngroups, nseg, M1,
                                         st);
      }
      if (e == cudaSuccess) e = launch_filter_spec(nullptr, ys.p, nullptr, gspec.p, gt, 1);
      if (e == cudaSuccess) e = launch_pt(bout, true);
      return e;
    }
    if (use_f3) {
      // every detector's half spectrum (three-pass forward in batches that
      // stay in L2), the group sums (and chi^2) in position order, the
      // inverse into P^T's layout
      const long long nbatches = (ntiles + f3_batch - 1) / f3_batch;
      // the batches' column and row passes, the group sums (and the chi^2
      // sum), the inverse row and column passes; P^T counts itself
      launches += 2 * nbatches + 1 + (chi2_dev ? 1 : 0) + 2;
      cudaError_t e = fft3_forward_spectra((const float*)d, f3scratch.as<float>(),
                                           dspec.as<cplx<float>>(), ntiles, f3_batch, logm,
                                           tw_lo.as<cplx<float>>(), tw_hi.as<cplx<float>>(), wn1f,
                                           st);
      if (e == cudaSuccess)
        e = group_rhs_launch<float>(dspec.as<cplx<float>>(), filt_pos.as<float>(), dcs.as<float>(),
                                    grp_off.as<int>(), grp_det.as<int>(), ngroups, nseg, M1,
                                    gspec.as<cplx<float>>(), rhs_part.as<double>(),
                                    kGroupRhsBlocks, st);
      if (e == cudaSuccess && chi2_dev)
        e = chi2_sum(rhs_part.as<double>(), kGroupRhsBlocks, chi2_dev, st);
      if (e == cudaSuccess)
        e = fft3_inverse_from_spectra(gspec.as<cplx<float>>(), ys.as<float>(), ngroups, (int)nseg,
                                      logm, tw_lo.as<cplx<float>>(), tw_hi.as<cplx<float>>(), wn1f,
                                      st);
      if (e == cudaSuccess) e = launch_pt(bout, true);
      return e;
    }
    cudaError_t e = launch_filter_spec(d, nullptr, dspec.p, nullptr, ntiles);
    launches += 2;  // sums, chi^2
    if (f32) {
      if (e == cudaSuccess)
        e = group_rhs_launch<float>(dspec.as<cplx<float>>(), filt_slot.as<float>(), dcs.as<float>(),
                                    grp_off.as<int>(), grp_det.as<int>(), ngroups, nseg, M1,
                                    gspec.as<cplx<float>>(), rhs_part.as<double>(),
                                    kGroupRhsBlocks, st);
    } else {
      if (e == cudaSuccess)
        e = group_rhs_launch<double>(dspec.as<cplx<double>>(), filt_slot.as<double>(),
                                     dcs.as<double>(),
                                     grp_off.as<int>(), grp_det.as<int>(), ngroups, nseg, M1,
                                     gspec.as<cplx<double>>(), rhs_part.as<double>(),
                                     kGroupRhsBlocks, st);
    }
    if (e == cudaSuccess && chi2_dev)
      e = chi2_sum(rhs_part.as<double>(), kGroupRhsBlocks, chi2_dev, st);
    if (e == cudaSuccess) e = launch_filter_spec(nullptr, ys.p, nullptr, gspec.p, gt, 1);
    if (e == cudaSuccess) e = launch_pt(bout, true);
    return e;
  }

  // the three passes of the FP32 group weighting, in place on ys
  cudaError_t fft3_weight() {
    launches += 3;
    return fft3_group_weight(ys.as<float>(), hrow.as<float>(), groups_uniform ? 0 : 1, ngroups,
                             (int)nseg, logm, tw_lo.as<cplx<float>>(), tw_hi.as<cplx<float>>(),
                             wn1f, st);
  }

  // A for offset groups in three steps: the projection to the group
  // timelines (a, b1, b2) (mixed by W for uniform groups), N^-1 on them into
  // P^T's layout ys, then P^T.  N^-1: the three-pass weighting in place
  // (FP32), else the cluster FFT kernels: the fused filter per timeline
  // (uniform groups), or forward FFTs, the 3 x 3 mixing per frequency and
  // the inverse FFTs.
  cudaError_t group_project_step() {
    const long long nsd = ns * nseg;
    launches += 1;
    void* out = use_f3 ? ys.p : gtl.p;
    const int ilv = use_f3 ? 1 : 0;
    if (groups_uniform)
      return f32 ? group_project_w_launch<float>(pix.as<int>(), cs.as<float>(), dmap.as<float>(),
                                                 wmix.as<float>(), ngsamp, nsd, (float*)out, ilv, st)
                 : group_project_w_launch<double>(pix.as<int>(), cs.as<double>(),
                                                  dmap.as<double>(), wmix.as<double>(), ngsamp,
                                                  nsd, (double*)out, ilv, st);
    return f32 ? group_project_launch<float>(pix.as<int>(), cs.as<float>(), dmap.as<float>(), ngsamp,
                                             nsd, (float*)out, ilv, st)
               : group_project_launch<double>(pix.as<int>(), cs.as<double>(), dmap.as<double>(),
                                              ngsamp, nsd, (double*)out, ilv, st);
  }
  cudaError_t group_weight_step() {
    if (use_f3) return fft3_weight();
    const long long M1 = ns / 2 + 1, gt = 3LL * ngroups * nseg;
    if (groups_uniform)
      return launch_filter(kLoadTod, gtl.p, ys.p, gt, (int)nseg, 0, nullptr, nullptr, gfilt.p, 1);
    launches += 1;  // mixing
    cudaError_t e = launch_filter_spec(gtl.p, nullptr, gspec.p, nullptr, gt);
    if (e == cudaSuccess)
      e = f32 ? group_mix_launch<float>(gspec.as<cplx<float>>(), hmix.as<float>(), ngroups, nseg,
                                        M1, st)
              : group_mix_launch<double>(gspec.as<cplx<double>>(), hmix.as<double>(), ngroups,
                                         nseg, M1, st);
    if (e == cudaSuccess) e = launch_filter_spec(nullptr, ys.p, nullptr, gspec.p, gt, 1);
    return e;
  }
  cudaError_t apply_map_group(double* out, bool masked) {
    cudaError_t e = group_project_step();
    if (e == cudaSuccess) e = group_weight_step();
    if (e == cudaSuccess) e = launch_pt(out, masked);
    return e;
  }

  // out = A v (masked or not); v is a device compact vector
  cudaError_t apply_dev(const double* v, double* out, bool masked) {
    cudaError_t e = to_map(v);
    if (e == cudaSuccess) e = apply_map(out, masked);
    return e;
  }

  CgVecs vecs(int precond) {
    CgVecs v{};
    v.npix = npix;
    v.x = x.as<double>();
    v.r = r.as<double>();
    v.d = d.as<double>();
    v.q = q.as<double>();
    v.z = z.as<double>();
    v.rprev = rprev.as<double>();
    v.b = b.as<double>();
    v.minv = minv.as<double>();
    v.minv32 = f32 ? minv32.as<float>() : nullptr;
    v.mdiag = mdiag.as<double>();
    v.hits_true = polmask.as<int>();
    v.precond = precond;
    v.part = part.as<double>();
    v.sc = sc.as<CgScalars>();
    return v;
  }

  // one PCG iteration (sanepic.cc:1417-1610) as a launch sequence
  cudaError_t enqueue_iteration(int precond, bool refresh) {
    if (precond == 2) return enqueue_learned_iteration(refresh);
    CgVecs v = vecs(precond);
    cudaError_t e = apply_map(q.as<double>(), true);
    if (e == cudaSuccess) e = cg_step_a(v, st);
    if (e == cudaSuccess) e = cg_step_b(v, refresh ? 1 : 0, 0, st);
    launches += 3;  // step a, b, c
    if (refresh && e == cudaSuccess) e = enqueue_true_residual(v, 0);
    if (e == cudaSuccess)
      e = f32 ? cg_step_c<float>(v, dmap.as<float>(), 0, st)
              : cg_step_c<double>(v, dmap.as<double>(), 0, st);
    return e;
  }

  // the refresh of sanepic.cc:1483-1572: r = b - A x recomputed, not updated.
  // Exact form: r = P^T N^-1 (d - P x), one pass per detector, which also
  // gives chi^2 of the residual timeline.  With the offset-group operator and
  // no chi^2 wanted (no printed line, no callback) r = b - A x through the
  // group operator instead, a few percent of the cost.
  bool refresh_chi2 = true;
  int refresh_kind() const { return (grouped() && !refresh_chi2) ? 2 : 1; }
  cudaError_t enqueue_true_residual(const CgVecs& v, int flexible) {
    cudaError_t e = to_map(x.as<double>());
    launches++;  // cg_refresh_r
    if (refresh_kind() == 2) {
      if (e == cudaSuccess) e = apply_map_group(q.as<double>(), true);
      if (e == cudaSuccess) e = cg_refresh_r(v, flexible, 0, st);
      return e;
    }
    // with gains: chi^2 of d - G P x (sanepic.cc:1500-1535), then G N^-1
    if (e == cudaSuccess) e = launch_project(gains_on ? &gain_t : nullptr);
    if (e == cudaSuccess)
      e = launch_filter(kLoadTodMinus, tod_active(), y.p, ntiles, (int)nseg, 0, y.p,
                        &sc.as<CgScalars>()->chi2);
    if (e == cudaSuccess && gains_on) e = scale_by_gain(y.p);
    if (e == cudaSuccess) e = pt_of_y(q.as<double>(), true);
    if (e == cudaSuccess) e = cg_refresh_r(v, flexible, 1, st);
    return e;
  }

  // flexible PCG with z = M_bj3 r + network correction (Polak-Ribiere beta)
  cudaError_t enqueue_learned_iteration(bool refresh) {
    CgVecs v = vecs(2);
    cudaError_t e = apply_map(q.as<double>(), true);
    if (e == cudaSuccess) e = cg_step_a(v, st);
    if (e == cudaSuccess) e = cg_step_b(v, refresh ? 1 : 0, 1, st);
    launches += 2;
    if (refresh && e == cudaSuccess) e = enqueue_true_residual(v, 1);
    if (e == cudaSuccess) e = learned_z(1);
    if (e == cudaSuccess)
      e = f32 ? cg_step_c<float>(v, dmap.as<float>(), 1, st)
              : cg_step_c<double>(v, dmap.as<double>(), 1, st);
    launches += 1;
    return e;
  }
  // z from r by the network (sg_learn.cu) or the coarse space, then the CG's
  // partial dots r.z, r.r (and z.r_prev when flexible)
  cudaError_t learned_z(int flexible);
  CoarseSpace coarse() const {
    CoarseSpace c{};
    c.kc = coarse_k;
    c.u = cs_u.as<uint16_t>();
    c.au = cs_au.as<uint16_t>();
    c.einv = cs_einv.as<double>();
    c.coef = cs_coef.as<double>();
    c.part = cs_part.as<double>();
    return c;
  }

  // captured iterations hold raw device pointers: drop them whenever a buffer
  // they use is reallocated
  unsigned long long graph_gen = 0;  // bumped whenever captured work is invalidated
  void drop_graphs() {
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
    graph_launches.clear();
    for (auto& kv : loop_graphs) cudaGraphExecDestroy(kv.second.exec);
    loop_graphs.clear();
    graph_gen++;
  }

  // ---- the whole PCG loop as one graph: a conditional WHILE node whose body
  // is one iteration (the refresh or the plain variant under two IF nodes)
  // and a decision kernel; loop_state holds the limits and the count, so one
  // captured loop serves every solve of the same preconditioner
  DevBuf loop_state, loop_hist;
  struct LoopGraph {
    cudaGraphExec_t exec = nullptr;
    long long launches_refresh = 0, launches_plain = 0;  // per iteration of each variant
  };
  std::map<std::pair<int, int>, LoopGraph> loop_graphs;

  // appends [WHILE loop] to g after deps; counts the launches of each variant
  cudaError_t add_solve_loop(cudaGraph_t g, const cudaGraphNode_t* deps, size_t ndeps, int precond,
                             cudaGraphNode_t* node_out, long long* n_refresh, long long* n_plain) {
    cudaGraphConditionalHandle hw, hr, hn;
    cudaError_t e = cudaGraphConditionalHandleCreate(&hw, g, 1, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&hr, g, 0, 0);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&hn, g, 0, 0);
    if (e != cudaSuccess) return e;
    cudaGraphNodeParams wp = {};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = hw;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    e = cudaGraphAddNode(node_out, g, deps, nullptr, ndeps, &wp);
    if (e != cudaSuccess) return e;
    cudaGraph_t body = wp.conditional.phGraph_out[0];
    const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
    LoopState* ls = loop_state.as<LoopState>();
    // begin: pick this iteration's variant
    cudaGraph_t cap;
    e = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, mode);
    if (e != cudaSuccess) return e;
    e = loop_begin_launch(ls, hr, hn, st);
    cudaError_t e2 = cudaStreamEndCapture(st, &cap);
    if (e != cudaSuccess) return e;
    if (e2 != cudaSuccess) return e2;
    cudaGraphNode_t begin;
    size_t nn = 1;
    e = cudaGraphGetNodes(body, &begin, &nn);
    if (e != cudaSuccess) return e;
    if (nn != 1) return cudaErrorInvalidValue;
    // the two variants, each under an IF node
    cudaGraphNode_t ifs[2];
    for (int v = 0; v < 2 && e == cudaSuccess; v++) {
      cudaGraphNodeParams ip = {};
      ip.type = cudaGraphNodeTypeConditional;
      ip.conditional.handle = v == 0 ? hr : hn;
      ip.conditional.type = cudaGraphCondTypeIf;
      ip.conditional.size = 1;
      e = cudaGraphAddNode(&ifs[v], body, &begin, nullptr, 1, &ip);
      if (e != cudaSuccess) break;
      e = cudaStreamBeginCaptureToGraph(st, ip.conditional.phGraph_out[0], nullptr, nullptr, 0, mode);
      if (e != cudaSuccess) break;
      const long long before = launches;
      e = enqueue_iteration(precond, v == 0);
      (v == 0 ? *n_refresh : *n_plain) = launches - before;
      launches = before;
      e2 = cudaStreamEndCapture(st, &cap);
      if (e == cudaSuccess) e = e2;
    }
    if (e != cudaSuccess) return e;
    // end: record crit, count, decide
    e = cudaStreamBeginCaptureToGraph(st, body, ifs, nullptr, 2, mode);
    if (e != cudaSuccess) return e;
    e = loop_end_launch(ls, sc.as<CgScalars>(), loop_hist.as<double>(), hw, st);
    e2 = cudaStreamEndCapture(st, &cap);
    return e != cudaSuccess ? e : e2;
  }

  // the single-solve loop graph for (precond, refresh kind), captured on first use
  cudaError_t solve_loop_graph(int precond, LoopGraph** out) {
    auto key = std::make_pair(precond, refresh_kind());
    auto it = loop_graphs.find(key);
    if (it == loop_graphs.end()) {
      cudaGraph_t g;
      cudaError_t e = cudaGraphCreate(&g, 0);
      if (e != cudaSuccess) return e;
      LoopGraph lg;
      cudaGraphNode_t node;
      e = add_solve_loop(g, nullptr, 0, precond, &node, &lg.launches_refresh, &lg.launches_plain);
      if (e == cudaSuccess) e = cudaGraphInstantiate(&lg.exec, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return e;
      it = loop_graphs.emplace(key, lg).first;
    }
    *out = &it->second;
    return cudaSuccess;
  }

  // loop_state / loop_hist for a solve of at most maxiter iterations
  cudaError_t ensure_loop_buffers(int maxiter) {
    cudaError_t e = cudaSuccess;
    if (!loop_state.p) e = loop_state.alloc(sizeof(LoopState));
    if (e == cudaSuccess && loop_hist.bytes < sizeof(double) * (size_t)maxiter) {
      drop_graphs();  // captured loops point at the old history buffer
      e = loop_hist.alloc(sizeof(double) * (size_t)maxiter);
    }
    return e;
  }

  // the captured iteration for (precond, refresh), captured on first use
  cudaError_t iteration_graph(int precond, bool refresh, cudaGraphExec_t* out) {
    auto key = std::make_pair(precond, refresh ? refresh_kind() : 0);
    auto it = graphs.find(key);
    if (it == graphs.end()) {
      cudaGraph_t g;
      cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
      if (e != cudaSuccess) return e;
      const long long before = launches;
      e = enqueue_iteration(precond, refresh);
      graph_launches[key] = launches - before;
      launches = before;
      cudaError_t e2 = cudaStreamEndCapture(st, &g);
      if (e != cudaSuccess) return e;
      if (e2 != cudaSuccess) return e2;
      cudaGraphExec_t ge;
      e = cudaGraphInstantiate(&ge, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return e;
      it = graphs.emplace(key, ge).first;
    }
    *out = it->second;
    return cudaSuccess;
  }

  cudaError_t run_iteration(int precond, bool refresh, bool use_graph) {
    if (!use_graph) return enqueue_iteration(precond, refresh);
    cudaGraphExec_t ge;
    cudaError_t e = iteration_graph(precond, refresh, &ge);
    if (e != cudaSuccess) return e;
    launches += graph_launches[std::make_pair(precond, refresh ? refresh_kind() : 0)];
    return cudaGraphLaunch(ge, st);
  }
};

int build_bj3(sg_ctx* c);  // 3x3 block-Jacobi blocks for the current pointing and noise
int build_polmask(sg_ctx* c);  // the CG's pol mask for the current pointing and pol_rcond
int ensure_patches(sg_ctx* c);  // nested patch geometry of the learned preconditioner
int build_diag(sg_ctx* c);      // the reference's diagonal preconditioner
int prepare_operator(sg_ctx* c);  // set-up the operator needs before its first application
