/*
 * fft64.h -- FP64 real<->complex FFT used by the CPU oracle and by the FFTW
 * shim that lets the unmodified reference compile here.
 *
 * TEST INFRASTRUCTURE ONLY: nothing in the shipped GPU library links this.
 *
 * Transform definitions follow FFTW 3's documented (unnormalised) conventions,
 * which is what the reference relies on (sanepic.cc:795-797, 2429-2431,
 * 2579-2581, 2705-2706):
 *   r2c:  X[k] = sum_{j<n} x[j] exp(-2 pi i j k / n),       k = 0 .. n/2
 *   c2r:  y[j] = sum_{k<n} Y[k] exp(+2 pi i j k / n),       j = 0 .. n-1
 *         with Y[n-k] = conj(Y[k]); the imaginary parts of Y[0] and (n even)
 *         Y[n/2] are ignored.
 * FFTW itself is not in this image; the algorithm here is a textbook
 * radix-2 decimation-in-time FFT on the half-length packed signal (powers of
 * two) and a direct O(n^2) DFT for any other length.
 */
#ifndef SANEPIC_ORACLE_FFT64_H
#define SANEPIC_ORACLE_FFT64_H

#ifdef __cplusplus
extern "C" {
#endif

/* in: n reals; out: n/2+1 complex values stored as (re, im) pairs. */
void fft64_r2c(long n, const double *in, double *out);
/* in: n/2+1 complex (re, im) pairs; out: n reals.  `in` is not modified. */
void fft64_c2r(long n, const double *in, double *out);

#ifdef __cplusplus
}
#endif
#endif
