/*
 * qs_fft.h -- CPU discrete Fourier transforms for the multislice oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the arithmetic behind
 *   (1) the FFTW entry-point shim that lets the reference's own CPU path
 *       (stem3/stemlib.cpp, which calls fftwf_* at stemlib.cpp:1492,2108,
 *       2308,2331,2423,2438 and libs/data_containers.cpp:50-51) link on a
 *       machine without libfftw3f, and
 *   (2) the C restatement of that path in qs_oracle.c.
 * Nothing in the shipped library (qstem_gb300/) links it.
 *
 * Conventions follow FFTW's documented interface: unnormalised transforms,
 * sign -1 = forward (exp(-2 pi i jk/n)), +1 = backward, row-major
 * multi-dimensional layout with the last index fastest.  Arithmetic is done in
 * double precision internally; single-precision entry points convert on the
 * way in and out.
 *
 * Algorithm: self-sorting (Stockham) mixed-radix passes with radices 4, 2, 3,
 * 5 and generic small odd primes (<= 61); lengths with a larger prime factor
 * use Bluestein's chirp-z re-expression as a power-of-two cyclic convolution.
 */
#ifndef QS_FFT_H
#define QS_FFT_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct qs_fft1d qs_fft1d;

/* Plans are immutable after creation and may be shared between threads. */
qs_fft1d *qs_fft1d_create(int n);
void qs_fft1d_destroy(qs_fft1d *p);
int qs_fft1d_len(const qs_fft1d *p);
/* Number of doubles of scratch space qs_fft1d_exec needs. */
size_t qs_fft1d_work_doubles(const qs_fft1d *p);
/* In-place transform of n interleaved complex doubles.  `work` must hold
 * qs_fft1d_work_doubles(p) doubles (NULL: allocated per call). */
void qs_fft1d_exec(const qs_fft1d *p, double *x, int sign, double *work);

/* Cached plan lookup (thread-safe); plans live until process exit. */
const qs_fft1d *qs_fft1d_get(int n);

/* Multi-dimensional, in place, on interleaved complex data.
 * dims[0] is the slowest index.  `howmany` transforms spaced `dist`
 * complex elements apart. */
void qs_fftnd_c64(int rank, const int *dims, int howmany, ptrdiff_t dist,
                  float *data, int sign);
void qs_fftnd_c128(int rank, const int *dims, int howmany, ptrdiff_t dist,
                   double *data, int sign);

/* Convenience 2-D single-precision transform of an n0 x n1 array. */
void qs_fft2d_c64(int n0, int n1, float *data, int sign);

#ifdef __cplusplus
}
#endif
#endif
