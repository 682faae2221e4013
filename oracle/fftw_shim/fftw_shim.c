/*
 * fftw_shim.c -- implementation of the FFTW-API shim (fftw3.h), TEST
 * INFRASTRUCTURE ONLY: it lets the reference's FFTWBackend run on the
 * oracle's CPU FFT (cpu_fft.c).  Plans remember the dimensions, the buffers
 * and the sign; fftw_execute copies in -> out and transforms out in place.
 */
#include "fftw3.h"

#include <stdlib.h>
#include <string.h>

#include "../cpu_fft.h"

struct fftw_shim_plan_s {
    int n0, n1, n2;
    double* in;
    double* out;
    int sign;
};

static int g_threads = 1;

int fftw_init_threads(void) { return 1; }

void fftw_plan_with_nthreads(int nthreads) { g_threads = nthreads > 0 ? nthreads : 1; }

fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex* in, fftw_complex* out,
                           int sign, unsigned flags) {
    (void)flags;
    if (n0 < 1 || n1 < 1 || n2 < 1) return NULL;
    fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
    p->n0 = n0; p->n1 = n1; p->n2 = n2;
    p->in = (double*)in; p->out = (double*)out;
    p->sign = sign;
    return p;
}

fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned flags) {
    return fftw_plan_dft_3d(1, 1, n, in, out, sign, flags);
}

void fftw_execute(const fftw_plan p) {
    const size_t n = (size_t)p->n0 * p->n1 * p->n2;
    if (p->out != p->in) memcpy(p->out, p->in, sizeof(double) * 2 * n);
    cfft_exec_3d(p->n0, p->n1, p->n2, p->out, p->sign, g_threads);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }

void* fftw_malloc(unsigned long n) { return malloc(n); }

void fftw_free(void* p) { free(p); }
