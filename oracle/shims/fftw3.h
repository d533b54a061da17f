/*
 * fftw3.h -- project-written stand-in for the subset of the FFTW 3 API that
 * the reference calls (sanepic.cc:709-711, 795-797, 2429-2431, 2579-2581,
 * 2705-2706, 2932-2945).  It exists only so that the unmodified reference
 * source compiles in this image, which has no FFTW; the transforms come from
 * oracle/fft64.c and follow FFTW's documented unnormalised conventions.
 * TEST INFRASTRUCTURE ONLY.
 */
#ifndef SANEPIC_SHIM_FFTW3_H
#define SANEPIC_SHIM_FFTW3_H

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct shim_fftw_plan_s *fftw_plan;

#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_dft_r2c_1d(int n, double *in, fftw_complex *out,
                               unsigned flags);
fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex *in, double *out,
                               unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#ifdef __cplusplus
}
#endif
#endif
