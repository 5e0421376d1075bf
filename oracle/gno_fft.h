/*
 * Oracle FFT (test infrastructure only).
 *
 * A plain-C mixed-radix Stockham FFT in double and float precision, written
 * from the published Stockham autosort formulation.  It stands in for FFTW3
 * (single precision), which the reference CPU path calls through
 * src/libguanaco/fft.cpp:38-71 (fftwf_plan_dft_1d/2d, FFTW_ESTIMATE) and
 * which is not installed here.  Both transforms are unnormalised, forward uses
 * exp(-2*pi*i*k*n/N) and inverse exp(+2*pi*i*k*n/N), as FFTW does.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * this code; the product path never links it.
 */
#ifndef GNO_FFT_H
#define GNO_FFT_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* In-place complex transform of n points; data is interleaved (re, im). */
void gno_fft_c2c_d(double *data, size_t n, int inverse);
void gno_fft_c2c_f(float *data, size_t n, int inverse);

/* In-place 2D complex transform of a row-major (ysize, xsize) array. */
void gno_fft2_c2c_d(double *data, size_t xsize, size_t ysize, int inverse);
void gno_fft2_c2c_f(float *data, size_t xsize, size_t ysize, int inverse);

#ifdef __cplusplus
}
#endif

#endif
