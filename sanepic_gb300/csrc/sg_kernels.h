// sg_kernels.h -- device kernel entry points of the map-making library
// (internal; the public C ABI is include/sanepic_gpu.h).
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include <vector>

#include "sg_cplx.cuh"

namespace sg {

// ---- noise filter (sg_filter.cu) --------------------------------------------
enum { kLoadTod = 0, kLoadDelta = 2, kLoadTodMinus = 3 };

template <typename T>
struct FilterArgs {
  long long ntiles;  // (det, seg) tiles, each ns = 2M samples, tile-major
  int nseg;          // det = tile / nseg selects the filter row
  int mode;          // kLoadTod / kLoadDelta / kLoadTodMinus
  int filt_abs;      // multiply by |h| instead of h
  const T* tod;      // kLoadTod, kLoadTodMinus: [ntiles][ns]
  const T* sub;      // kLoadTodMinus: the input is tod - sub
  double* chi2_part; // if set: per-CTA sums of h[k] |X[k]|^2, k = 0..ns/2 [gridDim]
  const T* filt;     // [ndet][M+1]
  T* out;            // [ntiles][ns]
  cplx<T>* spec_out;       // if set: forward FFT only, X[k] (k = 0..M) [ntiles][M+1]
  const cplx<T>* spec_in;  // if set: inverse FFT only of Y[k] [ntiles][M+1]
  int ilv3;                // with spec_in or the fused filter: out is [groups][nseg * ns / 8][3][8], tile = (group * 3 + component) * nseg + segment
  const cplx<T>* tw_lo;
  const cplx<T>* tw_hi;
  cplx<T> wn1;
};

template <typename T>
cudaError_t filter_launch(const FilterArgs<T>& a, int logm, int S, int nclusters,
                          cudaStream_t st);
template <typename T>
int filter_max_clusters(int logm, int S);
// frequency of each of the M+1 slots of a split-filter spectrum (tile shape logm, S)
void spec_slot_freq(int logm, int S, std::vector<int>& kfreq);
// forward FFT to a.spec_out, or inverse FFT from a.spec_in (exactly one set)
template <typename T>
cudaError_t filter_spec_launch(const FilterArgs<T>& a, int logm, int S, int nclusters,
                               cudaStream_t st);
size_t filter_smem_bytes(int logm, int S, int esize);
int filter_cluster_size(int logm, int esize);

// ---- pointing expansion + pixelisation (sg_pointing.cu, FP64, no FMA) --------
// Per offset group g (detectors with identical (offx, offy)) and group sample
// w = iseg * ns + ii: RING pixel and psi_o (the angle before the detector's
// own angle is added, sanepic.cc:742-759).
struct PointingArgs {
  long long ns;          // samples per segment
  int nseg, ngroups;
  const double* ra;      // [nseg][ns] boresight, psi already NaN-patched
  const double* dec;
  const double* psi;
  const double* offx;    // [ngroups] radians
  const double* offy;
  long long nside;
  int* ring_pix;         // [ngroups][nseg][ns]; -1 invalid (NaN), -2 out of range
  double* psio;          // [ngroups][nseg][ns]
  int* error_flag;       // set to 1 when theta is outside [0, pi]
};
cudaError_t pointing_launch(const PointingArgs& a, cudaStream_t st);

// ---- setup helpers (sg_setup.cu) ------------------------------------------------
// Group samples are indexed gs = g * nsd + iseg * ns + ii (nsd = nseg * ns).
// detector samples per RING pixel (each group sample counts gsize[g] times)
cudaError_t hist_launch(const int* ring_pix, long long n, long long nsd, const int* gsize,
                        int* count, cudaStream_t st);
cudaError_t compact_launch(const int* ring_pix, const int* indpix, long long n, int* pix,
                           cudaStream_t st);
// hits_true[m] = count[ring(m)] via indpix
// full[i2r[m]] = compact[m] for the npix observed pixels (full zeroed before)
cudaError_t expand_launch(const double* compact, const long long* i2r, long long npix,
                          double* full, cudaStream_t st);
cudaError_t hits_launch(const int* count, const int* indpix, long long npixfull,
                        int* hits_true, cudaStream_t st);
// pixel numbering from the per-RING-pixel sample counts [n = 12 nside^2]:
// indpix_ring (reference order, -1 if unobserved), indpix_int (internal
// index), int2ring / int2ringc [capacity n] (ring pixel and RING-order compact
// index of each internal index), *npix (device int) the observed pixels
size_t numbering_tmp_bytes(long long n);
cudaError_t numbering_launch(const int* count, long long n, long long nside, int nested,
                             long long* int2ring, long long* int2ringc, int* indpix_int,
                             int* indpix_ring, int* npix, void* tmp, size_t tmp_bytes,
                             cudaStream_t st);
cudaError_t any_negative_launch(const int* v, long long n, int* flag, cudaStream_t st);
cudaError_t any_nan_launch(const double* v, long long n, int* flag, cudaStream_t st);
// CSR by pixel over group samples: csr_off [npix+1], csr_idx [n]
size_t csr_tmp_bytes(long long n, long long npix);
cudaError_t csr_build(const int* pix, long long n, long long npix,
                      long long* csr_off, uint32_t* csr_idx, void* tmp, size_t tmp_bytes,
                      cudaStream_t st);
template <typename T>
cudaError_t gather_cs_launch(const T* cs, const uint32_t* csr_idx, long long n, T* csr_cs,
                             cudaStream_t st);
// (cos 2phi, sin 2phi) of the group base angle per group sample; cs64
// (optional, no half-wave plate): FP64 (cos, sin) of 2 psi_o for sumcross
template <typename T>
cudaError_t base_angles_launch(const double* psio, long long n, long long ns, long long nsd,
                               int hwp, double omega, T* cs, double* cs64, cudaStream_t st);
// COS2P/SIN2P sums over the CSR; gsc/gss [ngroups] = group sums of cos/sin 2psi_det;
// tab (optional): the cs64 table of base_angles_launch instead of sincos of psio
cudaError_t sumcross_launch(const long long* csr_off, const uint32_t* csr_idx, const double* psio,
                            const double* tab, long long nsd, const double* gsc, const double* gss,
                            long long npix, double* sumcross, cudaStream_t st);
// 3x3 block-Jacobi build+invert; gconst [5][ngroups]; minv [6][npix] (00 01 02 11 12 22)
// or null.  Q/U of a pixel are masked when hits_true < 2 or (rcond_min > 0)
// its block's reciprocal condition number is below rcond_min; polmask_out
// (optional) receives hits_true, or min(hits_true, 1) where masked.
template <typename T>
cudaError_t bj3_launch(const long long* csr_off, const uint32_t* csr_idx, const T* csr_cs,
                       long long npix, long long nsd, int ngroups, const double* gconst,
                       const int* hits_true, double rcond_min, int* polmask_out, double* minv,
                       cudaStream_t st);
// per-group sum of the detectors' N_ tables: out [ngroups][ns]
template <typename T>
cudaError_t group_ntab_launch(const T* ntab, long long ns, int ngroups, const int* grp_off,
                              const int* grp_det, T* out, cudaStream_t st);
// reference diagonal (compute_diagPtNPCorr x2, sanepic.cc:2680-2762): Mp [3][npix];
// ntab is per group [ngroups][ns] (group tile = idx / ns, group = tile / nseg)
template <typename T>
cudaError_t diag_launch(const long long* csr_off, const uint32_t* csr_idx, long long npix,
                        long long ns, int nseg, const T* ntab, double* Mp, cudaStream_t st);

// one detector's filter row from its iSpf file values, and g0 (the time-domain
// diagonal of its N^-1) into *g0 (part: kNoiseRowBlocks doubles of scratch)
constexpr int kNoiseRowBlocks = 64;
template <typename T>
cudaError_t noise_row_launch(const double* ispf, long long nssp, long long ns, T* row, double* g0,
                             double* part, cudaStream_t st);
// timeline ingest: out = (T) in over n samples, *nan_flag |= any NaN; then, if
// flagged, NaNs take the previous sample's value within each segment
template <typename T>
cudaError_t ingest_launch(const double* in, long long n, T* out, int* nan_flag, cudaStream_t st);
template <typename T>
cudaError_t nan_patch_launch(T* v, long long ns, long long nseg, cudaStream_t st);

// ---- P, detector sums, P^T (sg_pt.cu) ------------------------------------------
// Groups: grp_off [ngroups+1] / grp_det list the detectors of each offset group;
// dcs [ndet] = (cos 2d', sin 2d') rotates the group base angle to the detector's.
// P: t[det][w] = I + cos(2phi+2d') Q + sin(2phi+2d') U at the group's pixel
// (n = group samples, multiple of 4); map is [npix][4].
template <typename T>
cudaError_t project_launch(const int* gpix, const T* gcs, const T* map, long long n,
                           long long nsd, const int* grp_off, const int* grp_det, const T* dcs,
                           T* t, const T* tsc, long long ns, cudaStream_t st);
// per (detector, segment) tile of ns samples (tile = det * nseg + seg):
// y[tile][:] *= tsc[tile]
template <typename T>
cudaError_t tile_scale_launch(T* y, const T* tsc, long long ntiles, long long ns, cudaStream_t st);
// out[tile] = sum over the tile's samples of a * b (FP64, fixed order)
template <typename T>
cudaError_t tile_dots_launch(const T* a, const T* b, long long ntiles, long long ns, double* out,
                             cudaStream_t st);
// detector sums per group sample: ys[gs] = (sum y, sum cos2d' y, sum sin2d' y, 0)
template <typename T>
cudaError_t detsum_launch(const T* y, long long n, long long nsd, const int* grp_off,
                          const int* grp_det, const T* dcs, T* ys, cudaStream_t st);
// q[c*npix + m]: sums over the group samples of pixel m of (S0, cos2phi A - sin2phi B,
// sin2phi A + cos2phi B); Q/U zeroed where the pol mask applies (hits_true < 2).
// lanes per pixel (FP32: 1..32, from pt_lanes; FP64 ignores it)
template <typename T>
cudaError_t pt_launch(const long long* csr_off, const uint32_t* csr_idx, const T* csr_cs,
                      const T* ys, long long npix, const int* hits_true, double* q, int lanes,
                      cudaStream_t st);
int pt_lanes(long long nsamples, long long npix);

// ---- the offset-group operator (sg_group.cu) -------------------------------------
// gtl = (a, b1, b2) = (I, Q c + U s, U c - Q s) per group sample, in the
// layout [G][3][nsd], or with ilv in P^T's interleaved [G][nsd / 8][3][8]
template <typename T>
cudaError_t group_project_launch(const int* gpix, const T* gcs, const T* map, long long ng,
                                 long long nsd, T* gtl, int ilv, cudaStream_t st);
// half spectra [G][3][nseg][M+1] <- H (a, b1, b2) per frequency, hmix [G][M+1][6]
template <typename T>
cudaError_t group_mix_launch(cplx<T>* spec, const T* hmix, long long G, long long nseg,
                             long long M1, cudaStream_t st);
// right-hand side spectra of each group from the detectors' data spectra
// dspec [ndet][nseg][M+1] (slot order, filt rows in slot order too):
// gspec (S0, S1, S2)^ = sum_d h_d X_d (1, c, s);
// chi2_part [nblocks] = partial sums of h_d |X_d|^2
constexpr int kGroupRhsBlocks = 152 * 8;
template <typename T>
cudaError_t group_rhs_launch(const cplx<T>* dspec, const T* filt, const T* dcs, const int* grp_off,
                             const int* grp_det, long long G, long long nseg, long long M1,
                             cplx<T>* gspec, double* chi2_part, int nblocks, cudaStream_t st);
// uniform groups in the operator: gtl = W (a, b1, b2) with wmix [G][6] =
// sum_d (1, c, s, cc, cs, ss); N^-1 then filters each timeline on its own
template <typename T>
cudaError_t group_project_w_launch(const int* gpix, const T* gcs, const T* map, const T* wmix,
                                   long long ng, long long nsd, T* gtl, int ilv, cudaStream_t st);
template <typename T>
cudaError_t group_wmix_launch(const T* dcs, const int* grp_off, const int* grp_det, long long G,
                              T* wmix, cudaStream_t st);
// groups whose detectors share one noise spectrum: gtl (layout as for the
// projection) = the detectors' timelines summed with weights (1, c_d, s_d);
// then the group's half spectra [G][3][nseg][M+1] scaled by its (first
// detector's) filter row
template <typename T>
cudaError_t group_tod_rhs_launch(const T* tod, long long nsd, const int* grp_off,
                                 const int* grp_det, const T* dcs, long long G, T* gtl, int ilv,
                                 cudaStream_t st);
template <typename T>
cudaError_t group_scale_launch(cplx<T>* spec, const T* filt, const int* grp_off, const int* grp_det,
                               long long G, long long nseg, long long M1, cudaStream_t st);
// same[d] = 1 if detector d's filter row equals its group's first detector's
// (one block per listed detector, ndet_listed = grp_off[G])
template <typename T>
cudaError_t rows_match_group_launch(const T* filt, long long M1, const int* grp_off,
                                    const int* grp_det, long long G, long long ndet_listed,
                                    int* same, cudaStream_t st);
// hmix [G][slot][6] = sum_d h_d[kslot[slot]] (1, c, s, cc, cs, ss) over each group's detectors
template <typename T>
cudaError_t group_hmix_launch(const T* filt, const T* dcs, const int* grp_off, const int* grp_det,
                              const int* kslot, long long G, long long M1, T* hmix,
                              cudaStream_t st);
// out [rows][slot] = in [rows][kslot[slot]] (filter rows into spectrum slot order)
template <typename T>
cudaError_t permute_rows_launch(const T* in, const int* kslot, long long rows, long long M1, T* out,
                                cudaStream_t st);

// ---- the offset-group noise weighting in three passes (sg_fft3.cu, FP32) ----------
// In place on the group timelines in P^T's interleaved layout, tile (group g,
// segment s) at float offset (g nseg + s) 3 ns:  y = c2r(H r2c(x)) per tile,
// with the weights in row order (hrow: [G][M+1][6] symmetric 3 x 3 H with
// mix, else [G][M+1] one spectrum per group; position pos = C k1 + k2 holds
// frequency k = k1 + R k2, position M the Nyquist bin; fft3_pos_freq lists
// them).  tw_lo / tw_hi: W_M^j = hi[j / 64] lo[j % 64], wn1 = W_{2M}.
bool fft3_supported(int logm);
void fft3_pos_freq(int logm, std::vector<int>& kfreq);
cudaError_t fft3_group_weight(float* data, const float* hrow, int mix, long long ngroups, int nseg,
                              int logm, const cplx<float>* tw_lo, const cplx<float>* tw_hi,
                              cplx<float> wn1, cudaStream_t st);
// The right-hand side's halves: the half spectra X[k] (positions pos) of
// single timelines tod [ntiles][2M] into spec [ntiles][M+1], in batches of
// `batch` tiles through scratch [batch][2M]; and the inverse of weighted
// group spectra gspec [G][3][nseg][M+1] (positions pos) into the group tiles
// in P^T's layout.  fft3_rhs_batch: tiles small enough that a batch stays in
// L2 between its column and row passes.
long long fft3_rhs_batch(int logm);
// y [ntiles][2M] <- c2r(h_d r2c(x)) per tile (detector d = tile / nseg,
// hpos [ndet][M+1] the filter rows in position order; x == y allowed), in
// batches of `batch` tiles through scratch [batch][2M]
cudaError_t fft3_detector_filter(const float* x, float* y, float* scratch, const float* hpos,
                                 long long ntiles, long long batch, int nseg, int logm,
                                 const cplx<float>* tw_lo, const cplx<float>* tw_hi,
                                 cplx<float> wn1, cudaStream_t st);
cudaError_t fft3_forward_spectra(const float* tod, float* scratch, cplx<float>* spec,
                                 long long ntiles, long long batch, int logm,
                                 const cplx<float>* tw_lo, const cplx<float>* tw_hi,
                                 cplx<float> wn1, cudaStream_t st);
cudaError_t fft3_inverse_from_spectra(const cplx<float>* gspec, float* data, long long ngroups,
                                      int nseg, int logm, const cplx<float>* tw_lo,
                                      const cplx<float>* tw_hi, cplx<float> wn1, cudaStream_t st);

// ---- CG vector algebra (sg_cg.cu) ------------------------------------------------
struct CgScalars {
  double delta;      // current r^T z
  double delta_old;  // previous r^T z
  double delta0;
  double var;        // r^T r
  double var00;      // b^T b
  double alpha, beta, rtq;
  double chi2;       // 2 sum h |F(d - P x)|^2 at the last refresh
  int flag;          // bit 0: d^T A d <= 0, bit 1: r^T z <= 0
  int pad;
};
constexpr int kCgBlocks = 304;  // 2 x 152 SMs, grid-stride
constexpr int kCgThreads = 256;

struct CgVecs {
  long long npix;
  double* x;
  double* r;
  double* d;
  double* q;
  double* z;            // preconditioned residual
  double* rprev;        // flexible PCG: previous residual (or nullptr)
  const double* b;
  const double* minv;   // bj3 [6][npix] (00 01 02 11 12 22)
  // the same blocks in FP32 (FP32 operators only, else null): the coarse
  // space's pre-smoothing applies M_bj3 on the FP32 pipe (flexible PCG)
  const float* minv32;
  const double* mdiag;  // reference diagonal, inverted [3][npix]
  const int* hits_true;
  int precond;          // 0 diag, 1 bj3, 2 z supplied externally
  double* part;         // [4][kCgBlocks] partial sums
  CgScalars* sc;
};
// r = b - r (r holds the masked A x0); z = M r; d = z; scalars
template <typename T>
cudaError_t cg_init(const CgVecs& v, cudaStream_t st);
cudaError_t cg_step_a(const CgVecs& v, cudaStream_t st);  // partial q.d
cudaError_t cg_step_b(const CgVecs& v, int refresh, int flexible, cudaStream_t st);
// refresh: r = b - q, or r = q when q already holds the residual (direct)
cudaError_t cg_refresh_r(const CgVecs& v, int flexible, int direct, cudaStream_t st);
// out[i] = (float)in[i]
cudaError_t to_f32_launch(const double* in, float* out, long long n, cudaStream_t st);
// out = 2 * sum of n per-CTA chi^2 partials (fixed order)
cudaError_t chi2_sum(const double* part, int n, double* out, cudaStream_t st);
cudaError_t cg_dots(const CgVecs& v, int flexible, cudaStream_t st);
template <typename T>
cudaError_t cg_step_c(const CgVecs& v, T* dmap, int flexible, cudaStream_t st);
// d = z, delta = delta0 = r.z after cg_dots (start of a flexible PCG)
template <typename T>
cudaError_t cg_reinit_d(const CgVecs& v, T* dmap, cudaStream_t st);
template <typename T>
cudaError_t to_map4(const double* x, long long npix, T* map, cudaStream_t st);
cudaError_t mask_qu(double* v, const int* hits_true, long long npix, cudaStream_t st);
cudaError_t apply_precond(const CgVecs& v, const double* x, double* y, cudaStream_t st);

// ---- the PCG loop on the device (a conditional WHILE node of a CUDA graph) ----
struct LoopState {
  int iter;           // iterations done
  int maxiter;
  int refresh_every;  // the true residual every refresh_every-th iteration (0, r, 2r, ...)
  int done;           // 1: converged, 2: iteration limit, 3: breakdown flag
  double stop;        // |r|^2 / |b|^2 at which to stop
  unsigned long long t_first, t_last;  // device clock (ns) at the first and last iteration's end
  int skip0;          // 1: no true residual at iteration 0 (see refresh_at)
};

// Whether iteration `iter` recomputes the true residual b - A x: every
// refresh_every-th, as the reference (sanepic.cc:1483-1572).  With skip0 the
// first one (iteration 0) is left out: after one step from x0 = 0 the
// recurrence's residual equals b - A x to rounding, so that pass only costs
// an operator application.  The reference-compatible mode keeps it (its
// printed chi2 line comes from it).
__host__ __device__ inline bool refresh_at(int iter, int refresh_every, int skip0) {
  if (skip0 && iter == 0) return false;
  return refresh_every <= 1 || (iter % refresh_every) == 0;
}
// refresh iterations among the first `iters`
inline long long refresh_count(int iters, int refresh_every, int skip0) {
  if (iters <= 0) return 0;
  long long n = refresh_every <= 1 ? iters : (iters + refresh_every - 1) / refresh_every;
  return (skip0 && refresh_every > 1) ? n - 1 : n;
}
// sets the IF handles of this iteration's variant (refresh or not)
cudaError_t loop_begin_launch(const LoopState* s, cudaGraphConditionalHandle refresh,
                              cudaGraphConditionalHandle normal, cudaStream_t st);
// records crit = var / var00 in hist[iter], counts the iteration, and sets the
// WHILE handle to continue unless converged, at the limit or broken down
cudaError_t loop_end_launch(LoopState* s, const CgScalars* sc, double* hist,
                            cudaGraphConditionalHandle loop, cudaStream_t st);

// two-level preconditioner: coarse space U [3 npix][kp] (BF16, element-major,
// kp = coarse_pad(kc) columns, the last kp - kc zero), AU = A U, E^-1 [kc][kc]
constexpr int kCoarseMax = 32;
int coarse_pad(int kc);
struct CoarseSpace {
  int kc;             // columns (1..kCoarseMax)
  const uint16_t* u;   // BF16 bit patterns
  const uint16_t* au;
  const double* einv;
  double* coef;       // [kCoarseMax] scratch
  double* part;       // [2][kCoarseMax][kCgBlocks] scratch
};
// v.z = z(v.r) of the balancing two-level preconditioner around v's M, and
// the CG partial dots r.z, r.r (z.r_prev if flexible) as cg_dots leaves them
cudaError_t coarse_apply(const CgVecs& v, const CoarseSpace& cs, int flexible, cudaStream_t st);
// part [nsplit][m][m]: split-K partial Gram matrices X Y^T of FP64 rows [m][ld] over n
cudaError_t gram_launch(const double* X, const double* Y, long long ld, int m, long long n,
                        int nsplit, double* part, cudaStream_t st);
// out [n][coarse_pad(kc)] (BF16, element-major) = (C^T V)^T, V [m][ld] FP64, C [m][kc] FP64
cudaError_t combine_launch(const double* V, long long ld, int m, const double* C, int kc,
                           long long n, uint16_t* out, cudaStream_t st);

// ---- tensor-core BF16 GEMM (sg_gemm.cu) -----------------------------------------
// C[M x N] (FP32, row-major, ldc = N) = A[M x K] . B[N x K]^T (+ C if beta);
// A, B row-major BF16 with K contiguous; M % 128 == 0, N % 128 == 0, K % 64 == 0.
// *err (device int) receives a nonzero code if a pipeline wait timed out.
bool gemm_shape_ok(int M, int N, int K);
cudaError_t gemm_prepare();  // one-time kernel attributes on the current device
cudaError_t gemm_bf16(const void* A, const void* B, float* C, int M, int N, int K, int beta,
                      int* err, cudaStream_t st);

}  // namespace sg
