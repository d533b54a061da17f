/*
 * fft64.c -- FP64 FFT for the CPU oracle and the FFTW shim (test
 * infrastructure; see fft64.h for the transform conventions).
 *
 * Power-of-two n: the real signal is packed into n/2 complex points
 * z[m] = x[2m] + i x[2m+1], transformed with an iterative radix-2
 * decimation-in-time FFT, and split into the real spectrum with the standard
 * even/odd identity X[k] = E[k] + W_n^k O[k].  Other n: direct DFT.
 * Twiddles are computed once per length with libm cos/sin and cached.
 * Not thread-safe (the cache is a process-global table); the oracle and the
 * shimmed reference are single-threaded processes.
 */
#include "fft64.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define FFT64_TWO_PI 6.28318530717958647692528676655900576839433879875021

typedef struct {
  long n;        /* real length n (power of two) */
  double *wm;    /* exp(-2 pi i k / (n/2)), k < n/4   (complex FFT twiddles) */
  double *wn;    /* exp(-2 pi i k / n),     k <= n/2  (split twiddles)       */
  long *rev;     /* bit reversal permutation of length n/2 */
} fft64_plan;

#define FFT64_CACHE 16
static fft64_plan g_cache[FFT64_CACHE];
static int g_ncache = 0;

static int is_pow2(long n) { return n > 0 && (n & (n - 1)) == 0; }

static fft64_plan *get_plan(long n) {
  for (int i = 0; i < g_ncache; i++)
    if (g_cache[i].n == n) return &g_cache[i];
  int slot = g_ncache < FFT64_CACHE ? g_ncache++ : (int)(n % FFT64_CACHE);
  fft64_plan *p = &g_cache[slot];
  if (p->n) {
    free(p->wm);
    free(p->wn);
    free(p->rev);
  }
  long m = n / 2;
  p->n = n;
  p->wm = (double *)malloc(sizeof(double) * 2 * (m / 2 + 1));
  p->wn = (double *)malloc(sizeof(double) * 2 * (m + 1));
  p->rev = (long *)malloc(sizeof(long) * (m > 0 ? m : 1));
  for (long k = 0; k <= m / 2; k++) {
    double a = FFT64_TWO_PI * (double)k / (double)m;
    p->wm[2 * k] = cos(a);
    p->wm[2 * k + 1] = -sin(a);
  }
  for (long k = 0; k <= m; k++) {
    double a = FFT64_TWO_PI * (double)k / (double)n;
    p->wn[2 * k] = cos(a);
    p->wn[2 * k + 1] = -sin(a);
  }
  int bits = 0;
  while ((1L << bits) < m) bits++;
  for (long i = 0; i < m; i++) {
    long r = 0;
    for (int b = 0; b < bits; b++)
      if (i & (1L << b)) r |= 1L << (bits - 1 - b);
    p->rev[i] = r;
  }
  return p;
}

/* In-place complex FFT of length m (power of two); sign -1 forward, +1
 * backward (unnormalised). */
static void cfft(fft64_plan *p, double *z, long m, int sign) {
  for (long i = 0; i < m; i++) {
    long r = p->rev[i];
    if (r > i) {
      double t0 = z[2 * i], t1 = z[2 * i + 1];
      z[2 * i] = z[2 * r];
      z[2 * i + 1] = z[2 * r + 1];
      z[2 * r] = t0;
      z[2 * r + 1] = t1;
    }
  }
  for (long len = 2; len <= m; len <<= 1) {
    long half = len / 2, step = m / len;
    for (long base = 0; base < m; base += len) {
      for (long j = 0; j < half; j++) {
        double wr = p->wm[2 * j * step];
        double wi = p->wm[2 * j * step + 1] * (sign < 0 ? 1.0 : -1.0);
        double *a = z + 2 * (base + j), *b = z + 2 * (base + j + half);
        double tr = b[0] * wr - b[1] * wi;
        double ti = b[0] * wi + b[1] * wr;
        b[0] = a[0] - tr;
        b[1] = a[1] - ti;
        a[0] = a[0] + tr;
        a[1] = a[1] + ti;
      }
    }
  }
}

static void dft_r2c(long n, const double *in, double *out) {
  for (long k = 0; k <= n / 2; k++) {
    double re = 0.0, im = 0.0;
    for (long j = 0; j < n; j++) {
      double a = FFT64_TWO_PI * (double)((j * k) % n) / (double)n;
      re += in[j] * cos(a);
      im -= in[j] * sin(a);
    }
    out[2 * k] = re;
    out[2 * k + 1] = im;
  }
}

static void dft_c2r(long n, const double *in, double *out) {
  for (long j = 0; j < n; j++) {
    double acc = 0.0;
    for (long k = 0; k < n; k++) {
      double re, im;
      if (k <= n / 2) {
        re = in[2 * k];
        im = in[2 * k + 1];
      } else {
        re = in[2 * (n - k)];
        im = -in[2 * (n - k) + 1];
      }
      if (k == 0 || (n % 2 == 0 && k == n / 2)) im = 0.0;
      double a = FFT64_TWO_PI * (double)((j * k) % n) / (double)n;
      acc += re * cos(a) - im * sin(a);
    }
    out[j] = acc;
  }
}

void fft64_r2c(long n, const double *in, double *out) {
  if (!is_pow2(n) || n < 4) {
    dft_r2c(n, in, out);
    return;
  }
  long m = n / 2;
  fft64_plan *p = get_plan(n);
  double *z = (double *)malloc(sizeof(double) * 2 * m);
  memcpy(z, in, sizeof(double) * n); /* z[j] = x[2j] + i x[2j+1] */
  cfft(p, z, m, -1);
  /* k = 0 and k = m */
  out[0] = z[0] + z[1];
  out[1] = 0.0;
  out[2 * m] = z[0] - z[1];
  out[2 * m + 1] = 0.0;
  for (long k = 1; k < m; k++) {
    double ar = z[2 * k], ai = z[2 * k + 1];
    double br = z[2 * (m - k)], bi = -z[2 * (m - k) + 1]; /* conj(Z[m-k]) */
    double er = 0.5 * (ar + br), ei = 0.5 * (ai + bi);
    /* O = -i/2 (Z[k] - conj(Z[m-k])) */
    double dr = ar - br, di = ai - bi;
    double orr = 0.5 * di, oi = -0.5 * dr;
    double wr = p->wn[2 * k], wi = p->wn[2 * k + 1];
    out[2 * k] = er + (orr * wr - oi * wi);
    out[2 * k + 1] = ei + (orr * wi + oi * wr);
  }
  free(z);
}

void fft64_c2r(long n, const double *in, double *out) {
  if (!is_pow2(n) || n < 4) {
    dft_c2r(n, in, out);
    return;
  }
  long m = n / 2;
  fft64_plan *p = get_plan(n);
  double *z = (double *)malloc(sizeof(double) * 2 * m);
  for (long k = 0; k < m; k++) {
    /* Y[k] and Y[k+m] = conj(Y[m-k]); imaginary parts of Y[0], Y[m] ignored */
    double ar = in[2 * k], ai = (k == 0) ? 0.0 : in[2 * k + 1];
    double br = in[2 * (m - k)], bi = (k == 0) ? 0.0 : -in[2 * (m - k) + 1];
    double sr = ar + br, si = ai + bi;
    double dr = ar - br, di = ai - bi;
    /* W_n^{-k} = conj(wn[k]) */
    double wr = p->wn[2 * k], wi = -p->wn[2 * k + 1];
    double tr = dr * wr - di * wi, ti = dr * wi + di * wr;
    /* Z''[k] = S + i T */
    z[2 * k] = sr - ti;
    z[2 * k + 1] = si + tr;
  }
  cfft(p, z, m, +1);
  memcpy(out, z, sizeof(double) * n);
  free(z);
}
