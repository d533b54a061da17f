/*
 * fftw_shim.c -- FFTW 3 subset on top of oracle/fft64.c (see fftw3.h).
 * Plans only record the length and the buffers; creating one is cheap, which
 * matters because the reference creates a plan per call (sanepic.cc:2429).
 * TEST INFRASTRUCTURE ONLY.
 */
#include "fftw3.h"

#include <stdlib.h>

#include "../fft64.h"

struct shim_fftw_plan_s {
  int kind; /* 0 = r2c, 1 = c2r */
  long n;
  void *in;
  void *out;
};

static fftw_plan make(int kind, int n, void *in, void *out) {
  fftw_plan p = (fftw_plan)malloc(sizeof(*p));
  p->kind = kind;
  p->n = n;
  p->in = in;
  p->out = out;
  return p;
}

fftw_plan fftw_plan_dft_r2c_1d(int n, double *in, fftw_complex *out,
                               unsigned flags) {
  (void)flags;
  return make(0, n, in, out);
}

fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex *in, double *out,
                               unsigned flags) {
  (void)flags;
  return make(1, n, in, out);
}

void fftw_execute(const fftw_plan p) {
  if (p->kind == 0)
    fft64_r2c(p->n, (const double *)p->in, (double *)p->out);
  else
    fft64_c2r(p->n, (const double *)p->in, (double *)p->out);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }
