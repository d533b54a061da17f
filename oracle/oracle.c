/*
 * oracle.c -- FP64 CPU restatement of the reference's map-making hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h): the checker for the GPU library,
 * never part of it.  Each function restates the reference routine cited in
 * its comment with the same operation order, compiled with
 * -ffp-contract=off so that results are identical on x86-64 and aarch64.
 */
#include "oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fft64.h"

#define ORC_D2PI 6.2831853071795864769252867665590057683943387987502

/* ---------------------------------------------------------------------- */
/* sanepic.cc:3412-3476                                                    */
void orc_pointingshift(double x, double y, long nn, const double *thetap,
                       const double *phip, const double *psip, double *theta,
                       double *phi, double *psi) {
  double theta_ = asin(sqrt(x * x + y * y));
  double phi_ = atan2(y, x);
  for (long ii = 0; ii < nn; ii++) {
    theta[ii] = acos(sin(thetap[ii]) * sin(theta_) * cos(phi_ + psip[ii]) +
                     cos(thetap[ii]) * cos(theta_));
    phi[ii] = atan2(-sin(theta_) * sin(phi_ + psip[ii]),
                    (-cos(thetap[ii]) * sin(theta_) * cos(phi_ + psip[ii]) +
                     sin(thetap[ii]) * cos(theta_))) +
              phip[ii];
  }
  double drp[3], dr[3], eph[3], R[3][3];
  drp[2] = -sin(theta_) * cos(phi_);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) R[i][j] = 0.0;
  R[1][1] = -1.0;
  eph[2] = 0.0;
  for (long ii = 0; ii < nn; ii++) {
    drp[0] = cos(psip[ii]) * cos(theta_);
    drp[1] = sin(psip[ii]) * cos(theta_);
    R[0][0] = -cos(thetap[ii]);
    R[0][2] = sin(thetap[ii]);
    R[2][0] = sin(thetap[ii]);
    R[2][2] = cos(thetap[ii]);
    for (int k = 0; k < 3; k++) dr[k] = 0.0;
    for (int j = 0; j < 3; j++)
      for (int k = 0; k < 3; k++) dr[k] += R[k][j] * drp[j];
    eph[0] = -sin(phi[ii] - phip[ii]);
    eph[1] = cos(phi[ii] - phip[ii]);
    double aaa = 0.0, rrr = 0.0;
    for (int k = 0; k < 3; k++) {
      rrr += dr[k] * dr[k];
      aaa += dr[k] * eph[k];
    }
    aaa = aaa / sqrt(rrr);
    if (aaa > 1.0) aaa = 1.0;
    if (aaa < -1.0) aaa = -1.0;
    double psitmp = acos(aaa);
    if (dr[2] < 0) psitmp = -psitmp;
    psitmp = (fmod(psitmp + ORC_D2PI / 4.0 + 2.0 * ORC_D2PI, ORC_D2PI)) -
             ORC_D2PI / 2.0;
    psi[ii] = psitmp;
  }
}

/* ---------------------------------------------------------------------- */
/* sanepic.cc:2764-2843                                                    */
long orc_ang2pix_ring(long nside, double theta, double phi) {
  int nl2, nl4, ncap, npix, jp, jm, ipix1;
  double z, za, tt, tp, tmp;
  int ir, ip, kshift;
  double piover2 = 0.5 * M_PI;
  double PI = M_PI;
  double twopi = 2.0 * M_PI;
  double z0 = 2.0 / 3.0;
  if (nside < 1 || nside > 8192) return -1;
  if (theta < 0. || theta > PI) return -1;
  z = cos(theta);
  za = fabs(z);
  if (phi >= twopi) phi = phi - twopi;
  if (phi < 0.) phi = phi + twopi;
  tt = phi / piover2;
  nl2 = 2 * nside;
  nl4 = 4 * nside;
  ncap = nl2 * (nside - 1);
  npix = 12 * nside * nside;
  if (za <= z0) {
    jp = (int)floor(nside * (0.5 + tt - z * 0.75));
    jm = (int)floor(nside * (0.5 + tt + z * 0.75));
    ir = nside + 1 + jp - jm;
    kshift = 0;
    if ((ir & 1) == 0) kshift = 1;
    ip = (int)floor((jp + jm - nside + kshift + 1) / 2) + 1;
    if (ip > nl4) ip = ip - nl4;
    ipix1 = ncap + nl4 * (ir - 1) + ip;
  } else {
    tp = tt - floor(tt);
    tmp = sqrt(3. * (1. - za));
    jp = (int)floor(nside * tp * tmp);
    jm = (int)floor(nside * (1. - tp) * tmp);
    ir = jp + jm + 1;
    ip = (int)floor(tt * ir) + 1;
    if (ip > 4 * ir) ip = ip - 4 * ir;
    ipix1 = 2 * ir * (ir - 1) + ip;
    if (z <= 0.) ipix1 = npix - 2 * ir * (ir + 1) + ip;
  }
  return ipix1 - 1;
}

/* ---------------------------------------------------------------------- */
/* sanepic.cc:722-773 (pointing) and 848-875 (pixels)                      */
int orc_expand_detector(long ns, long nseg, const long *isampmin,
                        const double *ra, const double *dec, const double *psi,
                        double offx, double offy, double psidet, int hwp,
                        double omega, long nside, long *pix, double *psip,
                        double *psipfp, long *prev_pix) {
  double *psis = (double *)malloc(sizeof(double) * ns);
  long npixfull = 12 * nside * nside;
  for (long iseg = 0; iseg < nseg; iseg++) {
    const double *ras = ra + isampmin[iseg];
    const double *decs = dec + isampmin[iseg];
    memcpy(psis, psi + isampmin[iseg], sizeof(double) * ns);
    for (long ii = 0; ii < ns; ii++)
      if (!(psis[ii] > 0) && !(psis[ii] <= 0.0))
        if (ii > 0) psis[ii] = psis[ii - 1];
    for (long ii = 0; ii < ns; ii++) {
      double thetap_i = ORC_D2PI / 4.0 - decs[ii];
      double phip_i = ras[ii];
      double psip_i = psis[ii];
      double theta_o, phi_o, psi_o;
      orc_pointingshift(offx, offy, 1, &thetap_i, &phip_i, &psip_i, &theta_o,
                        &phi_o, &psi_o);
      double ra_rad = phi_o;
      double dec_rad = ORC_D2PI / 4.0 - theta_o;
      long pos = ii + ns * iseg;
      psip[pos] = psi_o + psidet;
      psipfp[pos] = psip[pos];
      if (hwp) psip[pos] = -(psi_o + psidet) + 2.0 * omega * (ii + ns * iseg);
      double theta = ORC_D2PI / 4.0 - dec_rad;
      double phi = fmod(ra_rad + ORC_D2PI, ORC_D2PI);
      long ipr;
      if (theta != theta || phi != phi) {
        ipr = -2; /* NaN pointing: invalid, keep the previous pixel below */
      } else {
        ipr = orc_ang2pix_ring(nside, theta, phi);
        if (ipr == -1) {
          free(psis);
          return -1;
        }
      }
      if (ipr < 0 || ipr > npixfull - 1) ipr = *prev_pix;
      *prev_pix = ipr;
      pix[pos] = ipr;
    }
  }
  free(psis);
  return 0;
}

/* sanepic.cc:904-915 */
long orc_indpix(long nside, long nsamp, const long *pix, long *indpix) {
  long npixfull = 12 * nside * nside;
  long *pixon = (long *)calloc(npixfull, sizeof(long));
  for (long i = 0; i < nsamp; i++) pixon[pix[i]] += 1;
  long ll = 0;
  for (long ii = 0; ii < npixfull; ii++) {
    indpix[ii] = -1;
    if (pixon[ii] != 0) indpix[ii] = ll++;
  }
  free(pixon);
  return ll;
}

/* sanepic.cc:533-537 */
void orc_noise_weights(long ns, long nssp, const double *ispf, double *spn) {
  for (long ii = 0; ii < ns; ii++)
    spn[ii] = ispf[(long)((double)ii / nssp * ns)] / (double)ns / (double)ns;
  spn[0] = ispf[1] * 1e-6 / (double)ns / (double)ns;
}

/* sanepic.cc:2845-2873 with polar, polard = 1, polara = 0, GalBP = 0 */
void orc_deproject(const double *S, const long *indpix, const long *pix,
                   const double *psip, long ns, long npix, double *Ps) {
  const double polard = 1.0, polara = 0.0;
  for (long ii = 0; ii < ns; ii++) {
    long mpos = indpix[pix[ii]];
    if (mpos < 0) mpos = -mpos - 2;
    Ps[ii] = 0.0;
    Ps[ii] = S[mpos] + polard * (S[npix + mpos] * cos(2.0 * (psip[ii] + polara)) +
                                 S[2 * npix + mpos] * sin(2.0 * (psip[ii] + polara)));
  }
}

/* sanepic.cc:2429-2436, 2549-2552, 2579-2581 */
void orc_noise_filter(long ns, const double *in, const double *spn,
                      double *out) {
  long nk = ns / 2 + 1;
  double *f = (double *)malloc(sizeof(double) * 2 * nk);
  fft64_r2c(ns, in, f);
  for (long k = 0; k < nk; k++) {
    f[2 * k] = 0.0 + f[2 * k] * spn[k];
    f[2 * k + 1] = 0.0 + f[2 * k + 1] * spn[k];
  }
  fft64_c2r(ns, f, out);
  free(f);
}

/* sanepic.cc:2584-2611 (sumCross == NULL), polardet = 1, polarang = 0 */
void orc_backproject(double *PNd, const long *indpix, const long *pix,
                     const double *psip, long ns, long npix, const double *Nd) {
  for (long ii = 0; ii < ns; ii++) {
    long mpos = indpix[pix[ii]];
    if (mpos >= 0) {
      PNd[mpos] += Nd[ii];
      PNd[npix + mpos] += 1.0 * cos(2.0 * (psip[ii] + 0.0)) * Nd[ii];
      PNd[2 * npix + mpos] += 1.0 * sin(2.0 * (psip[ii] + 0.0)) * Nd[ii];
    }
  }
}

/* sanepic.cc:1428-1439 (one operator application over every tile) */
void orc_apply(long ns, long nseg, long ndet, long npix, const long *indpix,
               const long *pix, const double *psip, const double *spn,
               const double *x, double *y) {
  double *Ps = (double *)malloc(sizeof(double) * ns);
  double *Nd = (double *)malloc(sizeof(double) * ns);
  memset(y, 0, sizeof(double) * 3 * npix);
  for (long iseg = 0; iseg < nseg; iseg++)
    for (long idet = 0; idet < ndet; idet++) {
      long off = ns * iseg + ns * nseg * idet;
      orc_deproject(x, indpix, pix + off, psip + off, ns, npix, Ps);
      orc_noise_filter(ns, Ps, spn + ns * idet, Nd);
      orc_backproject(y, indpix, pix + off, psip + off, ns, npix, Nd);
    }
  free(Ps);
  free(Nd);
}

/* sanepic.cc:1076-1117 */
double orc_rhs(long ns, long nseg, long ndet, long npix, const long *indpix,
               const long *pix, const double *psip, const double *spn,
               const double *tod, double *b) {
  long nk = ns / 2 + 1;
  double *f = (double *)malloc(sizeof(double) * 2 * nk);
  double *Nd = (double *)malloc(sizeof(double) * ns);
  double chi20 = 0.0;
  memset(b, 0, sizeof(double) * 3 * npix);
  for (long iseg = 0; iseg < nseg; iseg++)
    for (long idet = 0; idet < ndet; idet++) {
      long off = ns * iseg + ns * nseg * idet;
      const double *sp = spn + ns * idet;
      fft64_r2c(ns, tod + off, f);
      for (long k = 0; k < nk; k++) {
        double fr = f[2 * k] * sqrt(sp[k]) * 1.0;
        double fi = f[2 * k + 1] * sqrt(sp[k]) * 1.0;
        chi20 += (fr * fr + fi * fi) / 1.0 * 2.0;
      }
      for (long k = 0; k < nk; k++) {
        f[2 * k] = 0.0 + f[2 * k] * sp[k];
        f[2 * k + 1] = 0.0 + f[2 * k + 1] * sp[k];
      }
      fft64_c2r(ns, f, Nd);
      orc_backproject(b, indpix, pix + off, psip + off, ns, npix, Nd);
    }
  free(f);
  free(Nd);
  return chi20;
}

/* The gain fit's sums with the map x held fixed, as the reference forms
 * sPNd and cPNPc (sanepic.cc:2166-2226) but with one factor on both: for
 * tile t = idet * nseg + iseg, s = P x on the tile (deproject,
 * sanepic.cc:2173-2176), S = r2c(s), D = r2c(d) and
 *   dots[t]          = 2 sum_{k <= ns/2} Re(D_k conj S_k) spn[k]
 *   dots[ntiles + t] = 2 sum_{k <= ns/2} |S_k|^2 spn[k]
 * (the reference's sPNd carries 2, its cPNPc 1/2: its ratio is 4x this). */
void orc_gain_dots(long ns, long nseg, long ndet, long npix, const long *indpix,
                   const long *pix, const double *psip, const double *spn,
                   const double *tod, const double *x, double *dots) {
  long nt = ndet * nseg, nk = ns / 2 + 1;
  double *s = (double *)malloc(sizeof(double) * ns);
  double *fs = (double *)malloc(sizeof(double) * 2 * nk);
  double *fd = (double *)malloc(sizeof(double) * 2 * nk);
  for (long idet = 0; idet < ndet; idet++)
    for (long iseg = 0; iseg < nseg; iseg++) {
      long off = ns * iseg + ns * nseg * idet, t = idet * nseg + iseg;
      const double *sp = spn + ns * idet;
      orc_deproject(x, indpix, pix + off, psip + off, ns, npix, s);
      fft64_r2c(ns, s, fs);
      fft64_r2c(ns, tod + off, fd);
      double bd = 0.0, cs = 0.0;
      for (long k = 0; k < nk; k++) {
        bd += (fd[2 * k] * fs[2 * k] + fd[2 * k + 1] * fs[2 * k + 1]) * sp[k] * 2.0;
        cs += (fs[2 * k] * fs[2 * k] + fs[2 * k + 1] * fs[2 * k + 1]) * sp[k] * 2.0;
      }
      dots[t] = bd;
      dots[nt + t] = cs;
    }
  free(s);
  free(fs);
  free(fd);
}

/* chi^2 of d - g P x over every tile as MPI_compute_chi2 forms it
 * (sanepic.cc:3206-3260, the orbital dipole zero): 2 sum_{k <= ns/2}
 * |F(d - g s)_k|^2 spn[k]; gains per tile [idet][iseg], NULL for 1. */
double orc_gain_chi2(long ns, long nseg, long ndet, long npix, const long *indpix,
                     const long *pix, const double *psip, const double *spn,
                     const double *tod, const double *x, const double *gains) {
  long nk = ns / 2 + 1;
  double *s = (double *)malloc(sizeof(double) * ns);
  double *f = (double *)malloc(sizeof(double) * 2 * nk);
  double chi2 = 0.0;
  for (long iseg = 0; iseg < nseg; iseg++)
    for (long idet = 0; idet < ndet; idet++) {
      long off = ns * iseg + ns * nseg * idet;
      double g = gains ? gains[idet * nseg + iseg] : 1.0;
      orc_deproject(x, indpix, pix + off, psip + off, ns, npix, s);
      for (long i = 0; i < ns; i++) s[i] = tod[off + i] - g * s[i];
      fft64_r2c(ns, s, f);
      const double *sp = spn + ns * idet;
      for (long k = 0; k < nk; k++) {
        double fr = f[2 * k] * sqrt(sp[k]), fi = f[2 * k + 1] * sqrt(sp[k]);
        chi2 += (fr * fr + fi * fi) * 2.0;
      }
    }
  free(s);
  free(f);
  return chi2;
}

/* sanepic.cc:2613-2626, run twice (sanepic.cc:1258-1266) */
void orc_hits(long nsamp, long npix, const long *indpix, const long *pix,
              long *hits) {
  memset(hits, 0, sizeof(long) * 2 * npix);
  for (int pass = 0; pass < 2; pass++)
    for (long i = 0; i < nsamp; i++) {
      long mpos = indpix[pix[i]];
      if (mpos >= 0) {
        hits[mpos] += 1;
        hits[npix + mpos] += 1;
      }
    }
}

/* sanepic.cc:2594-2597 */
void orc_sumcross(long nsamp, long npix, const long *indpix, const long *pix,
                  const double *psipfp, double *sumcross) {
  memset(sumcross, 0, sizeof(double) * 3 * npix);
  for (long i = 0; i < nsamp; i++) {
    long mpos = indpix[pix[i]];
    if (mpos >= 0) {
      sumcross[mpos] += cos(2.0 * (psipfp[i] + 0.0));
      sumcross[npix + mpos] += sin(2.0 * (psipfp[i] + 0.0));
    }
  }
}

/* ---------------------------------------------------------------------- */
/* compute_diagPtNPCorr, sanepic.cc:2680-2762                              */
typedef struct {
  long key;
  long idx;
} orc_kv;

static int orc_kv_cmp(const void *a, const void *b) {
  const orc_kv *x = (const orc_kv *)a, *y = (const orc_kv *)b;
  if (x->key != y->key) return (x->key > y->key) - (x->key < y->key);
  return (x->idx > y->idx) - (x->idx < y->idx);
}

void orc_diag_tile(const double *Nk, const long *pix, long ns, const long *indpix,
                   double *dPtNP) {
  long nk = ns / 2 + 1;
  double *Nk_ = (double *)malloc(sizeof(double) * 2 * nk);
  double *N_ = (double *)malloc(sizeof(double) * ns);
  orc_kv *kv = (orc_kv *)malloc(sizeof(orc_kv) * ns);
  for (long k = 0; k < nk; k++) {
    Nk_[2 * k] = fabs(Nk[k]);
    Nk_[2 * k + 1] = 0.0;
  }
  fft64_c2r(ns, Nk_, N_);
  for (long ii = 0; ii < ns; ii++) {
    kv[ii].key = indpix[pix[ii]];
    kv[ii].idx = ii;
  }
  qsort(kv, ns, sizeof(orc_kv), orc_kv_cmp);
  long c0 = 0;
  while (c0 < ns && kv[c0].key < 0) c0++;
  while (c0 < ns) {
    long c1 = c0;
    while (c1 < ns && kv[c1].key == kv[c0].key) c1++;
    double *acc = dPtNP + kv[c0].key;
    for (long i = c0; i < c1; i++) {
      long ii2 = kv[i].idx;
      for (long k = c0; k < c1; k++) {
        long kk2 = kv[k].idx;
        if (labs(kk2 - ii2) < ns / 2) *acc += N_[labs(ii2 - kk2)];
      }
    }
    c0 = c1;
  }
  free(Nk_);
  free(N_);
  free(kv);
}

void orc_diag_precond(long ns, long nseg, long ndet, long npix,
                      const long *indpix, const long *pix, const double *spn,
                      double *Mp) {
  memset(Mp, 0, sizeof(double) * 3 * npix);
  for (long iseg = 0; iseg < nseg; iseg++)
    for (int pass = 0; pass < 2; pass++)
      for (long idet = 0; idet < ndet; idet++) {
        long off = ns * iseg + ns * nseg * idet;
        orc_diag_tile(spn + ns * idet, pix + off, ns, indpix, Mp);
        for (long ii = 0; ii < npix; ii++) {
          Mp[ii + npix] = Mp[ii] / 2.0;
          Mp[ii + 2 * npix] = Mp[ii] / 2.0;
        }
      }
}

/* ---------------------------------------------------------------------- */
/* 3x3 block-Jacobi (new, not in the reference)                            */
static double orc_g0(long ns, const double *spn) {
  /* c2r(spn)[0]: the (constant) diagonal of the circulant N^-1 */
  double acc = spn[0];
  for (long k = 1; k < ns / 2; k++) acc += 2.0 * spn[k];
  if (ns % 2 == 0) acc += spn[ns / 2];
  else acc += 2.0 * spn[ns / 2];
  return acc;
}

void orc_block_jacobi(long ns, long nseg, long ndet, long npix,
                      const long *indpix, const long *pix, const double *psip,
                      const double *spn, const long *hits, double *minv) {
  double *A = (double *)calloc(6 * npix, sizeof(double)); /* II IQ IU QQ QU UU */
  for (long idet = 0; idet < ndet; idet++) {
    double g0 = orc_g0(ns, spn + ns * idet);
    for (long iseg = 0; iseg < nseg; iseg++)
      for (long ii = 0; ii < ns; ii++) {
        long pos = ii + ns * iseg + ns * nseg * idet;
        long m = indpix[pix[pos]];
        if (m < 0) continue;
        double c = cos(2.0 * psip[pos]), s = sin(2.0 * psip[pos]);
        double *a = A + 6 * m;
        a[0] += g0;
        a[1] += g0 * c;
        a[2] += g0 * s;
        a[3] += g0 * c * c;
        a[4] += g0 * c * s;
        a[5] += g0 * s * s;
      }
  }
  for (long m = 0; m < npix; m++) {
    const double *a = A + 6 * m;
    double *o = minv + 9 * m;
    for (int i = 0; i < 9; i++) o[i] = 0.0;
    if (hits[npix + m] < 4) {
      o[0] = a[0] != 0.0 ? 1.0 / a[0] : 0.0;
      continue;
    }
    double c00 = a[3] * a[5] - a[4] * a[4];
    double c01 = a[2] * a[4] - a[1] * a[5];
    double c02 = a[1] * a[4] - a[2] * a[3];
    double c11 = a[0] * a[5] - a[2] * a[2];
    double c12 = a[1] * a[2] - a[0] * a[4];
    double c22 = a[0] * a[3] - a[1] * a[1];
    double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
    double scale = a[0] * a[0] * a[0];
    if (!(det > 1e-12 * scale)) {
      /* numerically singular block: plain diagonal inverse */
      o[0] = 1.0 / a[0];
      o[4] = a[3] > 0.0 ? 1.0 / a[3] : 0.0;
      o[8] = a[5] > 0.0 ? 1.0 / a[5] : 0.0;
      continue;
    }
    double id = 1.0 / det;
    o[0] = c00 * id; o[1] = c01 * id; o[2] = c02 * id;
    o[3] = c01 * id; o[4] = c11 * id; o[5] = c12 * id;
    o[6] = c02 * id; o[7] = c12 * id; o[8] = c22 * id;
  }
  free(A);
}

/* ---------------------------------------------------------------------- */
/* PCG, sanepic.cc:1250-1761                                               */
static int orc_masked(long ii, long npix, const long *hits) {
  return ii >= npix && ii < 3 * npix && hits[(ii % npix) + npix] < 4;
}

static void orc_apply_precond(int precond, long npix, const double *M,
                              const double *minv, const double *r, double *z) {
  if (precond == 0) {
    for (long ii = 0; ii < 3 * npix; ii++) z[ii] = M[ii] * r[ii];
  } else {
    for (long m = 0; m < npix; m++) {
      const double *o = minv + 9 * m;
      double r0 = r[m], r1 = r[npix + m], r2 = r[2 * npix + m];
      z[m] = o[0] * r0 + o[1] * r1 + o[2] * r2;
      z[npix + m] = o[3] * r0 + o[4] * r1 + o[5] * r2;
      z[2 * npix + m] = o[6] * r0 + o[7] * r1 + o[8] * r2;
    }
  }
}

int orc_pcg(long ns, long nseg, long ndet, long npix, const long *indpix,
            const long *pix, const double *psip, const double *spn,
            const double *b_in, const long *hits, const double *Mp_raw,
            const double *minv, int precond, const double *x0,
            double stop_crit, int maxiter, int verbose, double *x,
            double *crit_hist) {
  long n = 3 * npix;
  double *b = (double *)malloc(sizeof(double) * n);
  double *M = (double *)malloc(sizeof(double) * n);
  double *r = (double *)malloc(sizeof(double) * n);
  double *d = (double *)malloc(sizeof(double) * n);
  double *q = (double *)malloc(sizeof(double) * n);
  double *z = (double *)malloc(sizeof(double) * n);
  memcpy(b, b_in, sizeof(double) * n);
  for (long ii = 0; ii < n; ii++) {
    x[ii] = x0 ? x0[ii] : 0.0;
    M[ii] = Mp_raw ? Mp_raw[ii] : 0.0;
  }
  orc_apply(ns, nseg, ndet, npix, indpix, pix, psip, spn, x, r); /* A x0 */
  for (long ii = 0; ii < n; ii++)
    if (orc_masked(ii, npix, hits)) {
      r[ii] = 0.0;
      x[ii] = 0.0;
      b[ii] = 0.0;
      M[ii] = 0.0;
    }
  for (long ii = 0; ii < n; ii++) {
    if (precond == 0 && M[ii] != 0.0) M[ii] = 1.0 / M[ii];
    r[ii] = b[ii] - r[ii];
  }
  orc_apply_precond(precond, npix, M, minv, r, d);
  double delta_n = 0.0, var_n = 0.0, var00 = 0.0;
  for (long ii = 0; ii < n; ii++) delta_n += r[ii] * d[ii];
  for (long ii = 0; ii < n; ii++) var_n += r[ii] * r[ii];
  for (long ii = 0; ii < n; ii++) var00 += b[ii] * b[ii];
  double delta0 = delta_n;
  int iter = 0;
  while ((iter < maxiter && var_n / var00 > stop_crit) || iter == 0) {
    orc_apply(ns, nseg, ndet, npix, indpix, pix, psip, spn, d, q);
    for (long ii = 0; ii < n; ii++)
      if (orc_masked(ii, npix, hits)) q[ii] = 0.0;
    double rtq = 0.0;
    for (long ii = 0; ii < n; ii++) rtq += q[ii] * d[ii];
    double alpha = delta_n / rtq;
    for (long ii = 0; ii < n; ii++) x[ii] += alpha * d[ii];
    if ((iter % 10) == 0) {
      orc_apply(ns, nseg, ndet, npix, indpix, pix, psip, spn, x, r);
      for (long ii = 0; ii < n; ii++)
        if (orc_masked(ii, npix, hits)) r[ii] = 0.0;
      for (long ii = 0; ii < n; ii++) r[ii] = b[ii] - r[ii];
    } else {
      for (long ii = 0; ii < n; ii++) r[ii] -= alpha * q[ii];
    }
    double delta_o = delta_n;
    delta_n = 0.0;
    var_n = 0.0;
    if (precond == 0) {
      for (long ii = 0; ii < n; ii++) delta_n += r[ii] * M[ii] * r[ii];
    } else {
      orc_apply_precond(precond, npix, M, minv, r, z);
      for (long ii = 0; ii < n; ii++) delta_n += r[ii] * z[ii];
    }
    for (long ii = 0; ii < n; ii++) var_n += r[ii] * r[ii];
    double beta = delta_n / delta_o;
    if (precond == 0) {
      for (long ii = 0; ii < n; ii++) d[ii] = M[ii] * r[ii] + beta * d[ii];
    } else {
      for (long ii = 0; ii < n; ii++) d[ii] = z[ii] + beta * d[ii];
    }
    if (crit_hist) crit_hist[iter] = var_n / var00;
    if (verbose)
      printf("iter = %d, crit = %10.15g, crit2 = %10.15g\n", iter,
             var_n / var00, delta_n / delta0);
    iter++;
  }
  free(b);
  free(M);
  free(r);
  free(d);
  free(q);
  free(z);
  return iter;
}

/* write_reduced_map, sanepic.cc:2364-2388 */
void orc_expand_map(long nside, const long *indpix, const double *mapr,
                    double *full) {
  for (long ii = 0; ii < 12 * nside * nside; ii++) {
    full[ii] = 0.0;
    if (indpix[ii] != -1) {
      if (indpix[ii] < 0) full[ii] = mapr[-indpix[ii] - 2];
      else full[ii] = mapr[indpix[ii]];
    }
  }
}
