/*
 * fftw3.h -- minimal FFTW-3-API shim, TEST INFRASTRUCTURE ONLY.
 *
 * FFTW3 is a third-party dependency of the reference that is not vendored
 * and is not installed in this image (the reference's CMakeLists.txt:192-196
 * looks it up with find_library, no pinned version).  To compile the
 * reference's own FFTWBackend (src/fft/FFTWBackend.cpp) unmodified for the
 * oracle, this header declares the handful of double-precision entry points
 * that file calls, with FFTW's documented meaning:
 *   fftw_plan_dft_3d(n0, n1, n2, in, out, sign, flags): out-of-place
 *   unnormalised complex DFT of a row-major n0 x n1 x n2 array, n2 fastest,
 *   out[k] = sum_j in[j] exp(sign 2 pi i j.k / n), FFTW_FORWARD = -1.
 * The transform itself is the oracle's own CPU FFT (oracle/cpu_fft.c).
 * Only the names and the contract follow FFTW; no FFTW code is used.
 */
#ifndef FFTPERM_FFTW_SHIM_H
#define FFTPERM_FFTW_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct fftw_shim_plan_s* fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex* in, fftw_complex* out,
                           int sign, unsigned flags);
fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
void fftw_execute(const fftw_plan plan);
void fftw_destroy_plan(fftw_plan plan);
void* fftw_malloc(unsigned long n);
void fftw_free(void* p);

#ifdef __cplusplus
}
#endif

#endif
