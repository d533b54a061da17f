/*
 * oracle.h -- FP64 single-process CPU restatement of the reference's
 * map-making hot path (patanch/SANEPIC src/sanepic.cc), used ONLY as the
 * checker: by tests/, by __graft_entry__.smoke() and by bench.py's
 * cpu_baseline leg.  The shipped GPU library never links or calls it.
 *
 * Parity of this restatement is pinned against the unmodified reference
 * compiled with project-written FFTW/MPI shims (oracle/Makefile, target
 * `ref`); the fixtures under tests/golden/ come from that build.
 *
 * Layouts follow the reference: per-sample arrays are [det][seg][sample]
 * (index ii + ns*iseg + ns*nseg*idet, sanepic.cc:749, 874); compact maps are
 * [I block | Q block | U block] of npix each (sanepic.cc:919-921); spectra are
 * [det][ns] (the diagonal of SpN_all, sanepic.cc:534).
 * Polarisation is always on (pol=1, the only mode the reference runs
 * correctly), polardet = 1 and polarang = 0 (sanepic.cc:545-550).
 */
#ifndef SANEPIC_ORACLE_H
#define SANEPIC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* sanepic.cc:3412-3476 */
void orc_pointingshift(double x, double y, long nn, const double *thetap,
                       const double *phip, const double *psip, double *theta,
                       double *phi, double *psi);

/* sanepic.cc:2764-2843.  Returns the RING pixel, or -1 when the reference
 * would exit (nside or theta out of range). */
long orc_ang2pix_ring(long nside, double theta, double phi);

/* Per-detector pointing expansion + pixelisation (sanepic.cc:722-773,
 * 848-875).  ra/dec/psi are full boresight timelines read at
 * isampmin[iseg] (sanepic.cc:680-692); psi is NaN-patched in a private copy
 * (sanepic.cc:722-727).  Outputs per [det][seg][sample]: RING pixel, psip
 * (HWP-modulated when hwp) and psipFP (sanepic.cc:757-766).  `prev_pix`
 * carries the reference's "reuse the previous pixel" rule across calls
 * (sanepic.cc:859-872).  Returns 0, or -1 on an ang2pix range error. */
int orc_expand_detector(long ns, long nseg, const long *isampmin,
                        const double *ra, const double *dec, const double *psi,
                        double offx, double offy, double psidet, int hwp,
                        double omega, long nside, long *pix, double *psip,
                        double *psipfp, long *prev_pix);

/* indpix compaction (sanepic.cc:904-915); returns npix (observed pixels). */
long orc_indpix(long nside, long nsamp, const long *pix, long *indpix);

/* Inverse-noise weights for one detector (sanepic.cc:533-537):
 * spn[k] = ispf[(long)((double)k / nssp * ns)] / ns / ns, spn[0] replaced by
 * ispf[1] * 1e-6 / ns / ns.  spn has ns entries. */
void orc_noise_weights(long ns, long nssp, const double *ispf, double *spn);

/* P for one (det, seg) tile, deproject (sanepic.cc:2845-2873). */
void orc_deproject(const double *S, const long *indpix, const long *pix,
                   const double *psip, long ns, long npix, double *Ps);

/* N^-1 for one tile: r2c, multiply by spn[k] (k <= ns/2), c2r
 * (sanepic.cc:2429-2436 then 2549-2582). */
void orc_noise_filter(long ns, const double *in, const double *spn,
                      double *out);

/* P^T accumulation for one tile (sanepic.cc:2584-2611, sumCross == NULL). */
void orc_backproject(double *PNd, const long *indpix, const long *pix,
                     const double *psip, long ns, long npix, const double *Nd);

/* y = A x = sum_tiles P^T N^-1 P x (sanepic.cc:1428-1439); y overwritten. */
void orc_apply(long ns, long nseg, long ndet, long npix, const long *indpix,
               const long *pix, const double *psip, const double *spn,
               const double *x, double *y);

/* b = sum_tiles P^T N^-1 d (sanepic.cc:1076-1117) and chi2_0
 * (sanepic.cc:1089-1110); tod is [det][seg][sample], NaN-patched. */
double orc_rhs(long ns, long nseg, long ndet, long npix, const long *indpix,
               const long *pix, const double *psip, const double *spn,
               const double *tod, double *b);

/* Gain fit of the recalibration loop with the map x held fixed
 * (sanepic.cc:2166-2226, one factor 2 on both sums where the reference has
 * 2 on sPNd and 1/2 on cPNPc): per tile t = idet * nseg + iseg, s = P x,
 * dots[t] = 2 sum_{k <= ns/2} Re(D_k conj S_k) spn[k] and
 * dots[ndet * nseg + t] = 2 sum_{k <= ns/2} |S_k|^2 spn[k]. */
void orc_gain_dots(long ns, long nseg, long ndet, long npix, const long *indpix,
                   const long *pix, const double *psip, const double *spn,
                   const double *tod, const double *x, double *dots);

/* chi^2 of d - g P x (MPI_compute_chi2, sanepic.cc:3206-3260, no dipole);
 * gains per tile [idet][iseg], NULL for 1. */
double orc_gain_chi2(long ns, long nseg, long ndet, long npix, const long *indpix,
                     const long *pix, const double *psip, const double *spn,
                     const double *tod, const double *x, const double *gains);

/* Hit counts as the reference accumulates them: do_PtNd runs twice with
 * hits != NULL (sanepic.cc:1258-1266), so every count is doubled.
 * hits has 2*npix entries (I then pol), sanepic.cc:2613-2626. */
void orc_hits(long nsamp, long npix, const long *indpix, const long *pix,
              long *hits);

/* Cross-link sums (sanepic.cc:2594-2597) with psipFP; sumcross has 3*npix
 * entries (only the first 2*npix are written, as in the reference). */
void orc_sumcross(long nsamp, long npix, const long *indpix, const long *pix,
                  const double *psipfp, double *sumcross);

/* The reference's preconditioner diagonal, compute_diagPtNPCorr
 * (sanepic.cc:2680-2762), applied for every tile twice (doubling, Q1) and
 * with the Q/U blocks set to I/2 (sanepic.cc:2561-2565).  Mp has 3*npix
 * entries and is overwritten. */
void orc_diag_precond(long ns, long nseg, long ndet, long npix,
                      const long *indpix, const long *pix, const double *spn,
                      double *Mp);

/* compute_diagPtNPCorr for one tile (sanepic.cc:2680-2762): adds to
 * dPtNP[m] (the I block) sum_{i,j at pixel m, |i-j| < ns/2} N_[|i-j|] with
 * N_ = c2r(|Nk|). */
void orc_diag_tile(const double *Nk, const long *pix, long ns, const long *indpix,
                   double *dPtNP);

/* The whole path on nthreads threads in the reference's parallel layout
 * (cgpar.c): the CPU baseline's timed run. */
int cp_run(long ns, long nseg, long ndet, long nside, const double *ra, const double *dec,
           const double *psi, const long *isampmin, const double *psidet, int hwp,
           double omega, const double *ispf, long nssp, const double *tod, int nthreads,
           double stop_crit, int maxiter, double *x, double *crit_hist, double *times,
           long *npix_out, int *iters_out);

/* 3x3 block-Jacobi preconditioner (not in the reference): per pixel
 * sum_i g0_det * w w^T with w = (1, cos 2psi, sin 2psi), g0 = the diagonal of
 * N^-1 for that detector (c2r(spn)[0]); inverted in FP64.  Pixels whose pol
 * block is masked (hits[npix+m] < 4) keep only 1/A_II.  minv has 9*npix
 * entries (row-major 3x3 per pixel). */
void orc_block_jacobi(long ns, long nseg, long ndet, long npix,
                      const long *indpix, const long *pix, const double *psip,
                      const double *spn, const long *hits, double *minv);

/* PCG exactly as the reference runs it (sanepic.cc:1250-1761): x0 given
 * (zeros or -I), degeneracy mask from hits (sanepic.cc:1316-1330, 1455-1459),
 * true residual every 10th iteration (sanepic.cc:1483-1572).  precond 0 =
 * the reference's diagonal (Mp from orc_diag_precond, inverted here), 1 =
 * 3x3 block-Jacobi (minv).  Stops when crit = var_n/var00 <= stop_crit or
 * after maxiter (the reference uses 1e-15 and 2000).  x (3*npix) receives
 * the map; crit_hist (maxiter+1 entries, may be NULL) receives crit per
 * iteration; returns the iteration count.  verbose prints the reference's
 * "iter = ..." lines. */
int orc_pcg(long ns, long nseg, long ndet, long npix, const long *indpix,
            const long *pix, const double *psip, const double *spn,
            const double *b, const long *hits, const double *Mp_raw,
            const double *minv, int precond, const double *x0,
            double stop_crit, int maxiter, int verbose, double *x,
            double *crit_hist);

/* Expand a compact npix vector to a full RING map, 0 where unobserved
 * (write_reduced_map, sanepic.cc:2364-2388). */
void orc_expand_map(long nside, const long *indpix, const double *mapr,
                    double *full);

#ifdef __cplusplus
}
#endif
#endif
