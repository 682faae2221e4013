/*
 * cpu_fft.h -- double-precision mixed-radix complex FFT for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This file belongs to the oracle: it is used by
 * the CPU restatement of the reference algorithm (fftperm_oracle.c) and by the
 * FFTW-API shim that lets the reference's own FFTWBackend
 * (src/fft/FFTWBackend.cpp:185-299 plans, :301-362 forward, :364-420 inverse)
 * be compiled here without FFTW.  No product code links it.
 *
 * The reference's FFT contract (src/fft/FFTWBackend.cpp:221-237) is FFTW's:
 *   out[k] = sum_j in[j] * exp(sign * 2*pi*i * j.k / n),  sign = -1 forward,
 *   +1 backward, unnormalised, row-major (n0 slowest).
 * The transform here is an iterative Stockham auto-sort FFT with radix 4, 2
 * and generic odd-prime stages, twiddles from one table exp(-2*pi*i*j/n).
 */
#ifndef FFTPERM_ORACLE_CPU_FFT_H
#define FFTPERM_ORACLE_CPU_FFT_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cfft_plan cfft_plan;

/* 1-D plan for length n >= 1. */
cfft_plan* cfft_plan_create(int n);
void cfft_plan_destroy(cfft_plan* p);
int cfft_plan_length(const cfft_plan* p);

/* In-place 1-D transform of n interleaved complex values (re, im).
 * scratch must hold 2*n doubles.  sign = -1 or +1. */
void cfft_exec_1d(const cfft_plan* p, double* data, double* scratch, int sign);

/* 3-D row-major transform of n0 x n1 x n2 complex values (n2 fastest),
 * in place, unnormalised.  threads <= 0 means the OpenMP default. */
void cfft_exec_3d(int n0, int n1, int n2, double* data, int sign, int threads);

#ifdef __cplusplus
}
#endif

#endif
