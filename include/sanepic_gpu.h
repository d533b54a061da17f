/*
 * sanepic_gpu.h -- C ABI of libsanepic_gpu, the GB300 (sm_103a) map-making
 * library that replaces the reference's PCG hot path (patanch/SANEPIC,
 * src/sanepic.cc).  Plain pointers and sizes only; callers own every host
 * buffer (it is copied in or out), the library owns all device memory.
 *
 * The reference has no library interface: its hot path sits between its
 * binary readers and map writers inside main().  Each entry point below names
 * the part of sanepic.cc it replaces.  The drop-in `sanepic` executable
 * (same getopt string, files and outputs) is built on these calls.
 *
 * Errors: every int-returning call returns SG_OK (0) or a negative SG_ERR_*
 * code and never exits the process (the reference calls exit()).  The last
 * error message of a context is available from sg_last_error().
 * Threading: one context per host thread.  Contexts share only this
 * process-wide state, each piece guarded by a mutex: the cache of batch
 * graphs of sg_solve_batch (keyed by the contexts it solves, dropped when one
 * is destroyed), the per-device shared-memory opt-in of the tensor-core GEMM,
 * and the no-allocation entry point's device table and its address per GPU.
 * Layouts: per-sample arrays are [det][seg][sample] (sanepic.cc:749, 874);
 * compact maps are [I | Q | U], npix each, observed pixels in ascending RING
 * order (sanepic.cc:904-921); full maps are 12*nside^2 RING doubles with 0 at
 * unobserved pixels (sanepic.cc:2364-2388).
 */
#ifndef SANEPIC_GPU_H
#define SANEPIC_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define SG_OK 0
#define SG_ERR_ARG (-1)         /* invalid argument or size */
#define SG_ERR_CUDA (-2)        /* a CUDA call failed (message has details) */
#define SG_ERR_STATE (-3)       /* call out of order (e.g. solve before rhs) */
#define SG_ERR_POINTING (-4)    /* theta outside [0, pi]: the reference exits */
#define SG_ERR_UNSUPPORTED (-5) /* e.g. ns not a power of two in [256, 131072] */
#define SG_ERR_PRECOND (-6)     /* zero preconditioner entry (sanepic.cc:1344) */
#define SG_ERR_NOT_CONVERGED (-7)

#define SG_F64 0 /* every per-sample quantity in FP64 */
#define SG_F32 1 /* TOD, cos/sin, FFT in FP32; P^T sums and CG in FP64 */

#define SG_PRECOND_BJ3 0  /* 3x3 block-Jacobi (not in the reference) */
#define SG_PRECOND_DIAG 1 /* the reference's diagonal, sanepic.cc:1351-1355 */
#define SG_PRECOND_LEARNED 2 /* BJ3 + trained MLP correction, flexible PCG */

/* map kinds for sg_get_map (output names: sanepic.cc:1618-1690, 1786-1801) */
#define SG_MAP_I 0
#define SG_MAP_Q 1
#define SG_MAP_U 2
#define SG_MAP_NVAR 3
#define SG_MAP_Q_NVAR 4
#define SG_MAP_U_NVAR 5
#define SG_MAP_HITS 6
#define SG_MAP_POL_HITS 7
#define SG_MAP_COS2P 8
#define SG_MAP_SIN2P 9

typedef struct sg_ctx sg_ctx;

typedef struct sg_desc {
  long ns;          /* -l samples per segment (power of two, 256..131072) */
  long nseg;        /* -n number of segments */
  long ndet;        /* -d number of detectors */
  long nside;       /* -N HEALPix nside */
  int pol;          /* -p, must be 1 (pol=0 is broken in the reference) */
  int hwp;          /* -h */
  double omega;     /* -w HWP step, rad/sample (sanepic.cc:765) */
  int precision;    /* SG_F64 or SG_F32 */
  int device;       /* CUDA device ordinal */
} sg_desc;

typedef struct sg_det {
  double offx; /* lel * pi/180 (sanepic.cc:460) */
  double offy; /* xel * pi/180 (sanepic.cc:461) */
  double psi;  /* detector angle, rad (sanepic.cc:462) */
} sg_det;

typedef struct sg_solve_opts {
  int precond;       /* SG_PRECOND_* */
  double stop_crit;  /* stop when |r|^2/|b|^2 <= stop_crit (reference 1e-15) */
  int maxiter;       /* reference: 2000 (sanepic.cc:1415) */
  int refresh_every; /* true residual b - A x every k iterations (reference 10) */
  int verbose;       /* print the reference's "iter = ..., crit = ..." lines */
  const double *x0;  /* -I start map, compact [3*npix], or NULL for zeros */
  int use_graph;     /* replay each iteration from a captured CUDA graph */
  /* Called after every iteration with the values the reference prints
   * (sanepic.cc:1607-1609; chi2 is refreshed every refresh_every iterations,
   * sanepic.cc:1483-1546), or NULL.  A nonzero return ends the solve.  Inside
   * the call, sg_get_solution and sg_get_map(I, Q, U) read the current map
   * (the reference's per-iteration map writes, sanepic.cc:1709-1745). */
  int (*on_iteration)(void *user, int iter, double crit, double crit2, double chi2);
  void *user;
} sg_solve_opts;

typedef struct sg_report {
  int iterations;
  int converged;
  double crit;          /* final |r|^2/|b|^2 */
  double var00;         /* |b|^2 */
  double solve_seconds; /* wall time of the iterations */
  double iter_per_sec;
  double setup_seconds; /* preconditioner build inside sg_solve */
  double device_seconds;  /* CUDA-event time of the solve on the GPU (sg_solve_batch:
                             device clock from the batch's first iteration to this
                             problem's last) */
  long kernel_launches;   /* kernels this library launched during the solve */
  int breakdown;          /* nonzero: stopped early because d^T A d <= 0 (bit 0) or
                             r^T M r <= 0 (bit 1) -- the residual reached rounding level */
  int fallback_iter;      /* SG_PRECOND_LEARNED: iteration at which the solve fell back
                             to plain block-Jacobi PCG, or -1 */
  double crit0;           /* sg_solve: |r0|^2/|b|^2 of the start map, the reference's
                             var0/var00 (sanepic.cc:1362-1384); sg_solve_batch: 0 */
} sg_report;

/* Creates a context on desc->device.  Replaces the parameter handling of
 * main (sanepic.cc:315-446) and the MPI layout (sanepic.cc:591-632). */
int sg_create(sg_ctx **ctx, const sg_desc *desc);

/* Run this context's work on an existing CUDA stream (a cudaStream_t passed
 * as void*; NULL restores the context's own stream).  The caller keeps
 * ownership.  No reference counterpart (the reference has no GPU). */
int sg_set_stream(sg_ctx *ctx, void *cuda_stream);

/* Boresight pointing (full timelines of nsamp_total samples, read at
 * isampmin[iseg], sanepic.cc:680-692; NULL isampmin = i*ns) and per-detector
 * offsets/angles.  Runs the pointing expansion, HEALPix ang2pix, indpix
 * compaction, hit counts and cross-link sums on the GPU.  Replaces
 * sanepic.cc:452-464, 722-773, 828-951, 2594-2597, 2613-2626. */
int sg_set_pointing(sg_ctx *ctx, const double *ra, const double *dec, const double *psi,
                    long nsamp_total, const long *isampmin, const sg_det *dets);

/* Extends the pol degeneracy mask of every solve: besides the reference's
 * pixels with fewer than 2 hits (sanepic.cc:1316-1330, 1455-1459), Q and U
 * are masked (zeroed, not solved for) in pixels whose 3 x 3 block
 * sum_i w_i w_i^T, w = (1, cos 2psi_i, sin 2psi_i) over the pixel's detector
 * samples, has a reciprocal condition number below rcond_min.  With one
 * detector angle most such blocks are nearly singular and the system has
 * (near) null vectors, on which PCG stalls (the reference stops at its
 * iteration limit); 1e-6 is a working threshold.  0 (the default) keeps the
 * reference's rule.  Output maps (HITS, NVAR, SIN2P) keep the reference's
 * rule either way.  Invalidates b, the preconditioners and any learned part:
 * call before sg_rhs and sg_learn_train.  No reference counterpart. */
int sg_set_pol_rcond(sg_ctx *ctx, double rcond_min);

/* Inverse-noise spectrum of one detector (nssp values, the -u file).
 * Replaces sanepic.cc:507-539 (including the bin-0 override, 536-537). */
int sg_set_noise(sg_ctx *ctx, long det, const double *ispf, long nssp);

/* The same for every detector at once: ispf holds ndet rows of nssp values
 * (detector d's -u file in row d).  One copy and one wait instead of one
 * per detector; the rows are the ones sg_set_noise makes. */
int sg_set_noise_all(sg_ctx *ctx, const double *ispf, long nssp);

/* TOD of one detector (full timeline; NaNs patched as sanepic.cc:784-790).
 * Replaces sanepic.cc:776-803. */
int sg_set_tod(sg_ctx *ctx, long det, const double *tod, long nsamp_total);

/* The same for every detector at once: tod holds ndet rows of nsamp_total
 * samples (detector d's timeline in row d).  One wait for all detectors
 * instead of one per detector. */
int sg_set_tod_all(sg_ctx *ctx, const double *tod, long nsamp_total);

/* b = P^T N^-1 d (sanepic.cc:1069-1125).  chi2 (may be NULL) receives the
 * reference's chi2_0 = 2 sum |F d|^2 SpN (sanepic.cc:1089-1110).  Without
 * it, offset groups whose detectors all have the same noise spectrum sum
 * their timelines before the FFTs (three FFT pairs per group and segment
 * instead of one FFT per detector; the same b up to rounding). */
int sg_rhs(sg_ctx *ctx, double *chi2);

/* Detector gains of the recalibration loop (-r / -R, sanepic.cc:1041-1130,
 * 2123-2316): one gain per (detector, segment) tile, gains[idet + iseg *
 * ndet] (the layout of the reference's relCalib and of its relCalib.dat<n>
 * files), every gain finite and > 0; NULL restores 1.  The operator then
 * solves P^T G N^-1 G P m = P^T G N^-1 d with G = diag(g) tile by tile (the
 * reference's calibrated data d/g with its noise weights times g^2,
 * sanepic.cc:1044-1053, 2545).  While gains other than 1 are set the
 * operator runs per detector (gains break the sums of an offset group).
 * Invalidates b (call sg_rhs again) and any learned part; the current map
 * stays readable and the preconditioners are kept, as the reference keeps
 * those of its first loop (sanepic.cc:1352). */
int sg_set_gains(sg_ctx *ctx, const double *gains);

/* Gain fit with the current map m held fixed (after sg_solve), the
 * reference's relCalib = sPNd / cPNPc (sanepic.cc:2166-2226) as the
 * weighted least-squares gain of d = g P m + n per tile:
 *   g = (P m)^T N^-1 d / (P m)^T N^-1 (P m),
 * per_detector != 0 (-R): one gain per detector from the sums over its
 * segments (sanepic.cc:2254-2271).  The new gains are scaled so that their
 * mean equals the mean of the gains m was made with (the common factor the
 * map absorbs; the reference's absrecal, sanepic.cc:2281-2291).  gains_out
 * [nseg * ndet] as sg_set_gains takes them (not applied: pass them to
 * sg_set_gains); chi2_before / chi2_after (may be NULL): the reference's
 * chi^2 of d - g P m with the old and the new gains (sanepic.cc:3206-3260).
 * Differences from the reference (whose -r diverges): its fits carry a
 * factor 4 (sPNd x 2, cPNPc x 1/2), its absrecal reads arrays only -R fills,
 * and the orbital dipole (-o) is taken as zero here. */
int sg_fit_gains(sg_ctx *ctx, int per_detector, double *gains_out, double *chi2_before,
                 double *chi2_after);

/* The host arithmetic of sg_fit_gains on given per-tile sums (no GPU; for
 * checking): tile t = idet * nseg + iseg, dots_ds[t] = (N^-1 d)^T s,
 * dots_ss[t] = (N^-1 s)^T s with s = P m, edges_s[2t..2t+1] = (sum s_i,
 * sum (-1)^i s_i), edges_d likewise for d, spn_edge[2 idet..] the detector's
 * weights of bins 0 and ns/2; g_old / g_new per tile [idet][iseg].  Returns
 * SG_ERR_NOT_CONVERGED when the new gains have no positive mean. */
int sg_gains_from_sums(long ndet, long nseg, int per_detector, const double *dots_ds,
                       const double *dots_ss, const double *edges_s, const double *edges_d,
                       const double *spn_edge, const double *g_old, double *g_new);

/* Number of observed pixels (npix, sanepic.cc:915). */
long sg_npix(const sg_ctx *ctx);
/* 1 if the operator runs per offset group (detectors with identical
 * focal-plane offsets, at least 4 in every group, share one pixel stream:
 * three timelines per group instead of one per detector), 2 if it does and
 * weights the group timelines with the three-pass FP32 FFT (in place in the
 * layout P^T reads; known once the operator was prepared by a first apply,
 * right-hand side or solve), else 0; *ngroups (if non-null) receives the
 * number of groups.  No reference counterpart. */
int sg_group_mode(const sg_ctx *ctx, long *ngroups);

/* How the operator applies N^-1, as bits: 1 = per offset group (three
 * timelines per group, see sg_group_mode), 2 = with the three-pass FP32 FFT
 * through L2 (else the cluster FFT kernels).  Known once the operator was
 * prepared by a first apply, right-hand side or solve.  No reference
 * counterpart. */
int sg_weighting(const sg_ctx *ctx);

/* Kernels this context has launched so far (a CUDA graph's kernel nodes
 * counted one by one), for callers that account for device work; -1 for a
 * null context.  No reference counterpart. */
long sg_kernel_launches(const sg_ctx *ctx);

/* y = P^T N^-1 P x for a compact host vector [3*npix] (one operator pass,
 * sanepic.cc:1428-1448); masked != 0 applies the pol degeneracy mask
 * (sanepic.cc:1455-1459). */
int sg_apply(sg_ctx *ctx, const double *x, double *y, int masked);

/* N^-1 applied tile by tile to a [ndet][nseg][ns] host array (the
 * r2c -> x SpN -> c2r of sanepic.cc:2429-2436, 2549-2582). */
int sg_noise_filter(sg_ctx *ctx, const double *in, double *out);

/* N^-1 (r2c -> x h -> c2r, as sg_noise_filter) on ntiles tiles of ns FP32
 * samples that the caller already holds in DEVICE memory, allocating no GPU
 * memory: for callers that cannot call cudaMalloc -- applications whose GPU
 * memory belongs to their own pool, code running while a CUDA graph is being
 * captured, real-time loops that cannot take cudaMalloc's synchronisation.
 * No counterpart in the reference (it has no GPU code).
 * in/out: [ntiles][ns]; filt: [ntiles / tiles_per_filter][ns/2 + 1] inverse-
 * noise rows (tile t uses row t / tiles_per_filter); stream: a cudaStream_t or
 * NULL.  The work is enqueued on the stream of the current device.
 * Limit: ns a power of two in [256, 131072]; larger ns returns
 * SG_ERR_UNSUPPORTED.  The FFT twiddle table lives in one 8.5 KiB
 * library-static device array per GPU, shared by every call: calls that
 * overlap on the GPU race on it.  The first call on a device looks the array
 * up (cudaGetSymbolAddress) and the first call for each ns prepares that
 * kernel, so make one call per device and ns before any stream capture. */
int sg_noise_filter_noalloc(const float *in, float *out, const float *filt, long ns,
                            long ntiles, long tiles_per_filter, void *stream);

/* ---- learned preconditioner (no reference counterpart) ----------------------
 * Two learned parts, both trained on residuals that the plain block-Jacobi
 * solver produces on synthetic skies for this context's pointing and noise:
 * (1) a 4-layer MLP (768 -> 256 -> 256 -> 256 -> 768, BF16 weights on the
 * tensor cores, FP32 accumulate) that maps 3 x 256-pixel nested-HEALPix
 * patches of the block-Jacobi-preconditioned residual to a correction
 * (needs nside a power of two >= 16); (2) a coarse space U of kc vectors, the
 * Ritz vectors of M_bj3 A with the smallest Ritz values on the span of the
 * solver's preconditioned residuals, applied as the two-level balancing
 * preconditioner z = (I - U E^-1 (AU)^T) M_bj3 (I - AU E^-1 U^T) r
 * + U E^-1 U^T r, E = U^T A U (symmetric positive definite).
 * SG_PRECOND_LEARNED runs flexible PCG with the part that validation chose
 * and falls back to plain block-Jacobi PCG if r^T z turns non-positive. */
typedef struct sg_learn_opts {
  int npairs;        /* residual/solution pairs from the plain solver (0: 512) */
  long seed;         /* first synthetic sky/noise seed (0: 5000) */
  int steps;         /* Adam steps (0: 1500; < 0: no network) */
  int batch;         /* patches per step, multiple of 128 (0: 4096) */
  float lr;          /* Adam learning rate (0: 1e-3) */
  double pair_crit;  /* plain-solver |r|^2/|b|^2 that defines each solution (0: 1e-13) */
  double val_crit;   /* stop of the validation solves (0: 1e-12) */
  int force;         /* 2: use the coarse space, other nonzero: the network, even
                        if validation shows no gain */
  int coarse_k;      /* coarse-space vectors, at most 32 (0: 24, and the validation also
                        tries the first 16 and 8 and keeps the fastest; < 0: no coarse
                        space) */
  int coarse_vectors; /* stored residuals the coarse space is built from (0: 256) */
} sg_learn_opts;

typedef struct sg_learn_report {
  int pairs, skies; /* pairs kept, synthetic skies solved */
  long rows;        /* training patches (pairs x observed patches) */
  int steps;
  float loss_first, loss_last;  /* batch MSE (normalised units) at the first / last step */
  double gen_seconds, train_seconds;
  double gemm_tflop;            /* tensor-core work of the training, TFLOP */
  /* validation on two held-out synthetic skies and noise realisations:
   * iterations and CUDA-event time of a solve, the mean of the two */
  int val_plain_iters, val_learned_iters;
  double val_plain_ms, val_learned_ms;
  int enabled;  /* 1: SG_PRECOND_LEARNED uses a learned part; 0: it runs plain
                   block-Jacobi PCG because neither part beat it */
  int coarse_k, coarse_vectors;  /* coarse-space vectors kept, residuals used */
  double coarse_seconds;         /* building the coarse space */
  int val_coarse_iters;
  double val_coarse_ms;
  int kind;  /* what SG_PRECOND_LEARNED applies: 0 nothing (plain PCG),
                1 the network, 2 the coarse space */
} sg_learn_report;

/* Generates training data on this context's pointing and noise model
 * (synthetic skies and noise on the GPU; the residuals of plain block-Jacobi
 * solves run to pair_crit), builds the coarse space from the first
 * coarse_vectors residuals (one operator application each, then a
 * Rayleigh-Ritz step) and trains the network with the library's own
 * forward/backward kernels: each step maximises the A-cosine
 * (r^T z)^2 / ((z^T A z)(r^T M_bj3 r)) of the corrected direction z for one
 * stored residual, differentiated through one application of A.  Plain PCG
 * then judges both on two held-out problems (report->kind, report->enabled).
 * The coarse space belongs to this operator: a context with other pointing
 * or noise must be trained again.  `batch` is unused (one residual's patches
 * per step).  Overwrites b and the solution: call sg_rhs again before
 * sg_solve. */
int sg_learn_train(sg_ctx *ctx, const sg_learn_opts *opts, sg_learn_report *report);
long sg_learn_nparams(void);
/* FP32 parameters, per layer W [out x in] row-major then b [out]. */
int sg_learn_get_params(sg_ctx *ctx, float *params);
int sg_learn_set_params(sg_ctx *ctx, const float *params);
/* The Rayleigh-Ritz step of the coarse space on host arrays (no GPU): from
 * H = V^T A V and G = V^T M^-1 V [m][m] (row-major), writes C [m][k] (U = V C)
 * for the k <= kc Ritz vectors of M A with the smallest positive Ritz values
 * theta [k], and E^-1 [k][k] for E = C^T H C.  Returns k (0: none usable). */
int sg_coarse_from_gram(int m, int kc, const double *H, const double *G, double *C,
                        double *einv, double *theta);

/* Tests and measurements on host arrays.  sg_mlp_gemm_host: C[M x N] =
 * A[M x K] . B[N x K]^T, BF16 bit patterns in, FP32 out (M, N multiples of
 * 128, K of 64); with reps > 0, *ms = mean CUDA-event time of one GEMM.
 * sg_mlp_grad_host: one forward + backward of the network (B rows, a
 * multiple of 128): Y [B x 768], loss = mean (Y - T)^2, grads like params. */
int sg_mlp_gemm_host(const unsigned short *A, const unsigned short *B, float *C, int M, int N,
                     int K, int reps, double *ms);
int sg_mlp_grad_host(const float *params, const float *X, const float *T, int B, float *Y,
                     float *loss, float *grads);

/* Preconditioned CG (sanepic.cc:1177-1761).  With use_graph and nothing to
 * report per iteration (verbose 0, no on_iteration) the whole loop is one
 * CUDA-graph launch: a conditional WHILE node over the captured iteration,
 * its convergence test and iteration limit evaluated on the device
 * (SANEPIC_GPU_DEVICE_LOOP=0 keeps the host-driven loop). */
int sg_solve(sg_ctx *ctx, const sg_solve_opts *opts, sg_report *report);

/* Solves n independent problems (contexts, each after sg_rhs) at once.  With
 * use_graph: one CUDA graph holds every problem's solve start and WHILE loop
 * as independent branches, so the batch is a single launch (the graph is kept
 * for the same contexts); otherwise every context iterates on its own stream
 * and the host advances each as its last iteration finishes.  Same options
 * for all (x0 must be NULL); reports[i] as sg_solve's.  No reference
 * counterpart (one problem per run). */
int sg_solve_batch(sg_ctx **ctxs, int n, const sg_solve_opts *opts, sg_report *reports);

/* Times this context's noise filter with each compiled tile shape for its
 * segment length (FP32 tiles of 2^14..2^17 samples: 8192 or 4096 complex
 * points per CTA of the thread-block cluster) on its own timeline, or with
 * the offset-group operator one whole operator application, and keeps the
 * faster; *cluster_size and *ms (may be NULL) receive the choice and its
 * time per launch.  Then times the P^T reduction's team of lanes per pixel
 * (FP32: half, the same and twice the team chosen from the mean samples per
 * pixel) and keeps the fastest.  Needs the pointing and every detector's
 * noise (SG_ERR_STATE otherwise).  No reference counterpart. */
int sg_autotune(sg_ctx *ctx, int *cluster_size, double *ms);

/* The tile shapes in use: cluster size of the noise filter and lanes per
 * pixel of the P^T reduction (32 = a warp, the FP64 kernel).  No reference
 * counterpart. */
int sg_tile_shapes(const sg_ctx *ctx, int *cluster_size, int *pt_lanes);

/* A full 12*nside^2 RING map (write_reduced_map, sanepic.cc:2364-2388). */
int sg_get_map(sg_ctx *ctx, int kind, double *out_full);

/* The compact solution [3*npix], i.e. the map__A_* output (sanepic.cc:1786-1788). */
int sg_get_solution(sg_ctx *ctx, double *out_compact);

/* RING pixel of every sample [ndet][nseg][ns] (the reference's datatopix). */
int sg_get_pixels(sg_ctx *ctx, long *ring_pix);

/* indpix [12*nside^2] (sanepic.cc:904-915). */
int sg_get_indpix(sg_ctx *ctx, long *indpix);

/* crit = |r|^2/|b|^2 after each iteration of the last solve (up to max). */
int sg_get_crit_history(sg_ctx *ctx, double *out, int max);

/* Diagnostics: average CUDA-event time (ms) of the four operator kernels over
 * `reps` applications of A to the current search direction: ms[0] = P,
 * ms[1] = noise filter N^-1, ms[2] = per-sample detector sums, ms[3] = P^T.
 * Overwrites only scratch buffers.
 * No reference counterpart (the reference has no profiling). */
int sg_profile_operator(sg_ctx *ctx, int reps, double *ms);

const char *sg_last_error(const sg_ctx *ctx);
void sg_destroy(sg_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
