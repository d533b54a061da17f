/*
 * cgpar.c -- the reference's whole map-making path (patanch/SANEPIC
 * src/sanepic.cc) on every host core, for the CPU baseline that bench.py
 * times.  Measurement infrastructure like the rest of oracle/: the GPU
 * library never links or calls it.
 *
 * It runs the restated functions of oracle.c in the reference's parallel
 * layout (sanepic.cc:591-632): worker threads own contiguous blocks of
 * (detector, segment) tiles, as the reference's MPI ranks own segments, and
 * accumulate P^T into private maps that are summed in fixed worker order
 * (the MPI_Reduce of sanepic.cc:1124, 1448); the CG vector algebra runs on
 * one thread, as on the reference's rank 0 (sanepic.cc:1336-1411,
 * 1455-1610).  Phases, as the reference orders them:
 *   setup     pointing expansion and ang2pix per tile (sanepic.cc:722-875),
 *             indpix (904-915), noise weights (507-539)
 *   rhs       b = P^T N^-1 d and chi2_0, ending where the reference prints
 *             "PtNd Computed..." (1069-1132)
 *   precond   the first operator pass A x0 together with hits and the
 *             diagonal preconditioner, both accumulated twice per tile as
 *             the reference's two do_PtNd calls do (1250-1266, 2680-2762),
 *             and the pol mask (1316-1330)
 *   solve     PCG iterations (1415-1610), the true residual b - A x every
 *             10th, until crit = |r|^2/|b|^2 <= stop_crit or maxiter.
 * Every tile's FFTs use fft64.c (the same transforms as the FFTW shim the
 * reference was built with here).
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "fft64.h"
#include "oracle.h"

#define CP_MAXW 256

typedef struct cp_ctx cp_ctx;
typedef struct {
  cp_ctx *c;
  int w;
} cp_arg;

struct cp_ctx {
  long ns, nseg, ndet, nside, nssp, npixfull, npix;
  const double *ra, *dec, *psi, *psidet, *ispf, *tod;
  const long *isampmin;
  int hwp;
  double omega;
  int nw;
  long t0[CP_MAXW], t1[CP_MAXW];   /* tile range of each worker */
  long *pix[CP_MAXW];              /* [tiles][ns] RING pixel */
  double *psip[CP_MAXW];           /* [tiles][ns] */
  unsigned char *seen[CP_MAXW];    /* [npixfull] */
  double *priv[CP_MAXW];           /* [3 npix] private P^T sums */
  long *hits[CP_MAXW];             /* [npix] */
  double *mp[CP_MAXW];             /* [npix] */
  double chi2[CP_MAXW];
  int err[CP_MAXW];
  long *indpix;
  double *spn;                     /* [ndet][ns] */
  int task;
  const double *vin;               /* the map an apply reads */
  double *vout;                    /* where the reduction writes */
  pthread_barrier_t start, done, mid;
  cp_arg args[CP_MAXW];            /* the workers' arguments (live as long as c) */
};

enum { T_EXIT, T_POINTING, T_SEEN, T_RHS, T_PRECOND, T_APPLY };

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* sum the workers' private arrays over this worker's share of [0, n) */
/* which: 0 the maps (into vout), 1 the hits (into vout), 2 Mp (into
 * vout + npix) */
static void reduce_share(cp_ctx *c, int w, int which, long n) {
  long a = n * w / c->nw, b = n * (w + 1) / c->nw;
  double *out = which == 2 ? c->vout + c->npix : c->vout;
  for (long i = a; i < b; i++) {
    double s = 0.0;
    for (int v = 0; v < c->nw; v++)
      s += which == 0 ? c->priv[v][i] : (which == 1 ? (double)c->hits[v][i] : c->mp[v][i]);
    out[i] = s;
  }
}

static void tile_rhs(cp_ctx *c, int w, long t, double *f, double *nd) {
  long idet = t / c->nseg, iseg = t % c->nseg, off = (t - c->t0[w]) * c->ns;
  long nk = c->ns / 2 + 1;
  const double *sp = c->spn + c->ns * idet;
  const double *d = c->tod + idet * c->nseg * c->ns + iseg * c->ns;
  fft64_r2c(c->ns, d, f);
  for (long k = 0; k < nk; k++) {
    double fr = f[2 * k] * sqrt(sp[k]), fi = f[2 * k + 1] * sqrt(sp[k]);
    c->chi2[w] += (fr * fr + fi * fi) * 2.0;
  }
  for (long k = 0; k < nk; k++) {
    f[2 * k] *= sp[k];
    f[2 * k + 1] *= sp[k];
  }
  fft64_c2r(c->ns, f, nd);
  orc_backproject(c->priv[w], c->indpix, c->pix[w] + off, c->psip[w] + off, c->ns, c->npix, nd);
}

static void tile_apply(cp_ctx *c, int w, long t, double *ps, double *nd) {
  long idet = t / c->nseg, off = (t - c->t0[w]) * c->ns;
  orc_deproject(c->vin, c->indpix, c->pix[w] + off, c->psip[w] + off, c->ns, c->npix, ps);
  orc_noise_filter(c->ns, ps, c->spn + c->ns * idet, nd);
  orc_backproject(c->priv[w], c->indpix, c->pix[w] + off, c->psip[w] + off, c->ns, c->npix, nd);
}

static void *worker(void *p) {
  cp_arg *a = (cp_arg *)p;
  cp_ctx *c = a->c;
  int w = a->w;
  long ns = c->ns;
  double *buf1 = (double *)malloc(sizeof(double) * (ns + 2));
  double *buf2 = (double *)malloc(sizeof(double) * (ns + 2));
  for (;;) {
    pthread_barrier_wait(&c->start);
    int task = c->task;
    if (task == T_EXIT) break;
    if (task == T_POINTING) {
      long prev = 0;
      for (long t = c->t0[w]; t < c->t1[w] && !c->err[w]; t++) {
        long idet = t / c->nseg, iseg = t % c->nseg, off = (t - c->t0[w]) * ns;
        /* one segment per call; buf2 receives psipFP (the angle before the
         * HWP term) */
        if (orc_expand_detector(ns, 1, c->isampmin + iseg, c->ra, c->dec, c->psi, 0.0, 0.0,
                                c->psidet[idet], c->hwp, c->omega, c->nside, c->pix[w] + off,
                                c->psip[w] + off, buf2, &prev) != 0)
          c->err[w] = 1;
        /* the HWP angle uses the absolute sample index ii + ns * iseg
         * (sanepic.cc:765), which a one-segment call cannot see */
        if (c->hwp)
          for (long ii = 0; ii < ns; ii++)
            c->psip[w][off + ii] = -buf2[ii] + 2.0 * c->omega * (double)(ii + ns * iseg);
      }
    } else if (task == T_SEEN) {
      memset(c->seen[w], 0, (size_t)c->npixfull);
      long n = (c->t1[w] - c->t0[w]) * ns;
      for (long i = 0; i < n; i++) c->seen[w][c->pix[w][i]] = 1;
    } else if (task == T_RHS || task == T_APPLY) {
      memset(c->priv[w], 0, sizeof(double) * 3 * c->npix);
      c->chi2[w] = 0.0;
      for (long t = c->t0[w]; t < c->t1[w]; t++) {
        if (task == T_RHS) tile_rhs(c, w, t, buf1, buf2);
        else tile_apply(c, w, t, buf1, buf2);
      }
      pthread_barrier_wait(&c->mid);
      reduce_share(c, w, 0, 3 * c->npix);
    } else if (task == T_PRECOND) {
      memset(c->hits[w], 0, sizeof(long) * c->npix);
      memset(c->mp[w], 0, sizeof(double) * c->npix);
      for (long t = c->t0[w]; t < c->t1[w]; t++) {
        long idet = t / c->nseg, off = (t - c->t0[w]) * ns;
        for (int pass = 0; pass < 2; pass++) {
          for (long ii = 0; ii < ns; ii++) {
            long m = c->indpix[c->pix[w][off + ii]];
            if (m >= 0) c->hits[w][m] += 1;
          }
          orc_diag_tile(c->spn + ns * idet, c->pix[w] + off, ns, c->indpix, c->mp[w]);
        }
      }
      pthread_barrier_wait(&c->mid);
      reduce_share(c, w, 1, c->npix);   /* hits into vout[0, npix) */
      reduce_share(c, w, 2, c->npix);   /* Mp into vout[npix, 2 npix) */
    }
    pthread_barrier_wait(&c->done);
  }
  free(buf1);
  free(buf2);
  return NULL;
}

static void run(cp_ctx *c, int task) {
  c->task = task;
  pthread_barrier_wait(&c->start);
  if (task != T_EXIT) pthread_barrier_wait(&c->done); /* workers leave at T_EXIT */
}

/*
 * The whole path on nthreads worker threads.  ra/dec/psi: boresight
 * timelines (segment iseg read at isampmin[iseg], no NaNs); psidet: detector
 * angles in rad; ispf: [ndet][nssp]; tod: [ndet][nseg*ns].  Outputs: x
 * (3 * 12 nside^2 doubles; the first 3*npix hold the compact solution in the
 * reference's order), crit_hist (maxiter doubles), times[0..4] = setup, rhs,
 * precond, solve seconds and the seconds from the end of setup until crit
 * first reached stop_crit, *npix_out, *iters_out.  Returns 0, -1 on an
 * ang2pix range error, -2 on bad arguments, -3 if a worker thread could not
 * be started.
 */
int cp_run(long ns, long nseg, long ndet, long nside, const double *ra, const double *dec,
           const double *psi, const long *isampmin, const double *psidet, int hwp,
           double omega, const double *ispf, long nssp, const double *tod, int nthreads,
           double stop_crit, int maxiter, double *x, double *crit_hist, double *times,
           long *npix_out, int *iters_out) {
  if (nthreads < 1 || nthreads > CP_MAXW || ns < 4 || nseg < 1 || ndet < 1) return -2;
  cp_ctx *c = (cp_ctx *)calloc(1, sizeof(cp_ctx));
  c->ns = ns;
  c->nseg = nseg;
  c->ndet = ndet;
  c->nside = nside;
  c->nssp = nssp;
  c->npixfull = 12 * nside * nside;
  c->ra = ra;
  c->dec = dec;
  c->psi = psi;
  c->isampmin = isampmin;
  c->psidet = psidet;
  c->hwp = hwp;
  c->omega = omega;
  c->ispf = ispf;
  c->tod = tod;
  long ntiles = ndet * nseg;
  int nw = nthreads < ntiles ? nthreads : (int)ntiles;
  c->nw = nw;
  for (int w = 0; w < nw; w++) {
    c->t0[w] = ntiles * w / nw;
    c->t1[w] = ntiles * (w + 1) / nw;
    long n = (c->t1[w] - c->t0[w]) * ns;
    c->pix[w] = (long *)malloc(sizeof(long) * n);
    c->psip[w] = (double *)malloc(sizeof(double) * n);
    c->seen[w] = (unsigned char *)malloc((size_t)c->npixfull);
  }
  /* every worker uses the plan of length ns: create it before they start */
  {
    double *a = (double *)calloc(ns + 2, sizeof(double));
    double *b = (double *)calloc(ns + 2, sizeof(double));
    fft64_r2c(ns, a, b);
    free(a);
    free(b);
  }
  pthread_barrier_init(&c->start, NULL, nw + 1);
  pthread_barrier_init(&c->done, NULL, nw + 1);
  pthread_barrier_init(&c->mid, NULL, nw);
  pthread_t th[CP_MAXW];
  for (int w = 0; w < nw; w++) {
    c->args[w].c = c;
    c->args[w].w = w;
    if (pthread_create(&th[w], NULL, worker, &c->args[w]) != 0) {
      /* the workers already started wait on a barrier that can no longer
       * fill: leave them (and c, which they read) and report the failure */
      return -3;
    }
  }
  const double t_begin = now_s();
  int rc = 0;
  /* ---- setup ---------------------------------------------------------- */
  run(c, T_POINTING);
  for (int w = 0; w < nw; w++)
    if (c->err[w]) rc = -1;
  long npix = 0, n3 = 0;
  double *b = NULL, *M = NULL, *r = NULL, *d = NULL, *q = NULL;
  long *hits = NULL;
  int iter = 0;
  double t_setup = 0, t_rhs = 0, t_pre = 0, t_solve = 0, t_to_stop = -1.0;
  if (rc == 0) {
    run(c, T_SEEN);
    c->indpix = (long *)malloc(sizeof(long) * c->npixfull);
    for (long p = 0; p < c->npixfull; p++) {
      int on = 0;
      for (int w = 0; w < nw && !on; w++) on = c->seen[w][p];
      c->indpix[p] = on ? npix++ : -1;
    }
    c->npix = npix;
    n3 = 3 * npix;
    c->spn = (double *)malloc(sizeof(double) * ndet * ns);
    for (long idet = 0; idet < ndet; idet++)
      orc_noise_weights(ns, nssp, ispf + idet * nssp, c->spn + idet * ns);
    for (int w = 0; w < nw; w++) {
      c->priv[w] = (double *)malloc(sizeof(double) * n3);
      c->hits[w] = (long *)malloc(sizeof(long) * npix);
      c->mp[w] = (double *)malloc(sizeof(double) * npix);
    }
    b = (double *)malloc(sizeof(double) * n3);
    M = (double *)calloc(n3, sizeof(double));
    r = (double *)malloc(sizeof(double) * n3);
    d = (double *)malloc(sizeof(double) * n3);
    q = (double *)malloc(sizeof(double) * n3);
    hits = (long *)malloc(sizeof(long) * npix);
    const double t_a = now_s();
    t_setup = t_a - t_begin;
    /* ---- rhs: b = P^T N^-1 d ------------------------------------------ */
    c->vout = b;
    run(c, T_RHS);
    const double t_b = now_s();
    t_rhs = t_b - t_a;
    /* ---- hits, diagonal preconditioner (doubled), A x0 ----------------- */
    double *hd = (double *)malloc(sizeof(double) * 2 * npix);
    c->vout = hd;
    run(c, T_PRECOND);
    for (long m = 0; m < npix; m++) {
      hits[m] = (long)hd[m];
      M[m] = hd[npix + m];
      M[npix + m] = M[m] / 2.0; /* sanepic.cc:2561-2565 */
      M[2 * npix + m] = M[m] / 2.0;
    }
    free(hd);
    for (long ii = 0; ii < n3; ii++) x[ii] = 0.0;
    c->vin = x;
    c->vout = r;
    run(c, T_APPLY); /* A x0 (x0 = 0 here, as the reference runs it) */
    for (long m = 0; m < npix; m++)
      if (hits[m] < 4) { /* pol hits, doubled (sanepic.cc:1316-1330) */
        r[npix + m] = r[2 * npix + m] = 0.0;
        b[npix + m] = b[2 * npix + m] = 0.0;
        M[npix + m] = M[2 * npix + m] = 0.0;
      }
    for (long ii = 0; ii < n3; ii++) {
      if (M[ii] != 0.0) M[ii] = 1.0 / M[ii];
      r[ii] = b[ii] - r[ii];
      d[ii] = M[ii] * r[ii];
    }
    double delta_n = 0.0, var_n = 0.0, var00 = 0.0;
    for (long ii = 0; ii < n3; ii++) delta_n += r[ii] * d[ii];
    for (long ii = 0; ii < n3; ii++) var_n += r[ii] * r[ii];
    for (long ii = 0; ii < n3; ii++) var00 += b[ii] * b[ii];
    const double t_c = now_s();
    t_pre = t_c - t_b;
    /* ---- PCG (sanepic.cc:1415-1610) ------------------------------------ */
    while ((iter < maxiter && var_n / var00 > stop_crit) || iter == 0) {
      c->vin = d;
      c->vout = q;
      run(c, T_APPLY);
      for (long m = 0; m < npix; m++)
        if (hits[m] < 4) q[npix + m] = q[2 * npix + m] = 0.0;
      double rtq = 0.0;
      for (long ii = 0; ii < n3; ii++) rtq += q[ii] * d[ii];
      double alpha = delta_n / rtq;
      for (long ii = 0; ii < n3; ii++) x[ii] += alpha * d[ii];
      if ((iter % 10) == 0) {
        c->vin = x;
        c->vout = r;
        run(c, T_APPLY);
        for (long m = 0; m < npix; m++)
          if (hits[m] < 4) r[npix + m] = r[2 * npix + m] = 0.0;
        for (long ii = 0; ii < n3; ii++) r[ii] = b[ii] - r[ii];
      } else {
        for (long ii = 0; ii < n3; ii++) r[ii] -= alpha * q[ii];
      }
      double delta_o = delta_n;
      delta_n = 0.0;
      var_n = 0.0;
      for (long ii = 0; ii < n3; ii++) delta_n += r[ii] * M[ii] * r[ii];
      for (long ii = 0; ii < n3; ii++) var_n += r[ii] * r[ii];
      double beta = delta_n / delta_o;
      for (long ii = 0; ii < n3; ii++) d[ii] = M[ii] * r[ii] + beta * d[ii];
      if (crit_hist) crit_hist[iter] = var_n / var00;
      if (t_to_stop < 0.0 && var_n / var00 <= stop_crit) t_to_stop = now_s() - t_a;
      iter++;
    }
    t_solve = now_s() - t_c;
  }
  run(c, T_EXIT);
  for (int w = 0; w < nw; w++) pthread_join(th[w], NULL);
  times[0] = t_setup;
  times[1] = t_rhs;
  times[2] = t_pre;
  times[3] = t_solve;
  times[4] = t_to_stop;
  *npix_out = npix;
  *iters_out = iter;
  pthread_barrier_destroy(&c->start);
  pthread_barrier_destroy(&c->done);
  pthread_barrier_destroy(&c->mid);
  for (int w = 0; w < nw; w++) {
    free(c->pix[w]);
    free(c->psip[w]);
    free(c->seen[w]);
    free(c->priv[w]);
    free(c->hits[w]);
    free(c->mp[w]);
  }
  free(c->indpix);
  free(c->spn);
  free(b);
  free(M);
  free(r);
  free(d);
  free(q);
  free(hits);
  free(c);
  return rc;
}
