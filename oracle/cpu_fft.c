/*
 * cpu_fft.c -- double-precision mixed-radix complex FFT for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY (see cpu_fft.h).  The transform is the textbook
 * Stockham auto-sort formulation: stage s with radix R reads element
 * j + r*(n/R), applies the twiddle exp(sign*2*pi*i*(j mod Ns)*r/(Ns*R)),
 * does a length-R DFT and writes element (j/Ns)*Ns*R + (j mod Ns) + r*Ns,
 * ping-ponging between the data and a scratch buffer.  Radix-4 and radix-2
 * butterflies are written out; other prime factors use a direct DFT driven by
 * the same twiddle table, so every length n >= 1 is supported.
 */
#include "cpu_fft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define CFFT_MAX_STAGES 64

struct cfft_plan {
    int n;
    int nstage;
    int radix[CFFT_MAX_STAGES];
    int max_radix;
    double* tw; /* 2*n doubles: cos(2 pi j/n), -sin(2 pi j/n) */
};

static int factorize(int n, int* radix) {
    int k = 0;
    while (n % 4 == 0) { radix[k++] = 4; n /= 4; }
    while (n % 2 == 0) { radix[k++] = 2; n /= 2; }
    for (int p = 3; p * p <= n; p += 2) {
        while (n % p == 0) { radix[k++] = p; n /= p; }
    }
    if (n > 1) radix[k++] = n;
    return k;
}

cfft_plan* cfft_plan_create(int n) {
    if (n < 1) return NULL;
    cfft_plan* p = (cfft_plan*)calloc(1, sizeof(cfft_plan));
    if (!p) return NULL;
    p->n = n;
    p->nstage = (n == 1) ? 0 : factorize(n, p->radix);
    p->max_radix = 1;
    for (int s = 0; s < p->nstage; ++s)
        if (p->radix[s] > p->max_radix) p->max_radix = p->radix[s];
    p->tw = (double*)malloc(sizeof(double) * 2 * (size_t)n);
    const double two_pi = 6.283185307179586476925286766559;
    for (int j = 0; j < n; ++j) {
        const double a = two_pi * (double)j / (double)n;
        p->tw[2 * j + 0] = cos(a);
        p->tw[2 * j + 1] = -sin(a);
    }
    return p;
}

void cfft_plan_destroy(cfft_plan* p) {
    if (!p) return;
    free(p->tw);
    free(p);
}

int cfft_plan_length(const cfft_plan* p) { return p ? p->n : 0; }

/* w = exp(sign * 2 pi i t / n) from the forward table. */
static inline void twiddle(const cfft_plan* p, long t, int sign, double* wr, double* wi) {
    const int idx = (int)(t % p->n);
    *wr = p->tw[2 * idx];
    *wi = (sign < 0) ? p->tw[2 * idx + 1] : -p->tw[2 * idx + 1];
}

void cfft_exec_1d(const cfft_plan* p, double* data, double* scratch, int sign) {
    const int n = p->n;
    if (n <= 1) return;
    double* src = data;
    double* dst = scratch;
    double vr[64], vi[64];
    double* gvr = NULL;
    double* gvi = NULL;
    if (p->max_radix > 64) {
        gvr = (double*)malloc(sizeof(double) * 2 * (size_t)p->max_radix);
        gvi = gvr + p->max_radix;
    }
    int ns = 1;
    for (int s = 0; s < p->nstage; ++s) {
        const int R = p->radix[s];
        const int m = n / R;
        const long step = n / (ns * R);
        double* ar = (R > 64) ? gvr : vr;
        double* ai = (R > 64) ? gvi : vi;
        for (int j = 0; j < m; ++j) {
            const int k = j % ns;
            for (int r = 0; r < R; ++r) {
                const double xr = src[2 * (j + r * m)];
                const double xi = src[2 * (j + r * m) + 1];
                if (r == 0 || k == 0) {
                    ar[r] = xr;
                    ai[r] = xi;
                } else {
                    double wr, wi;
                    twiddle(p, (long)k * r * step, sign, &wr, &wi);
                    ar[r] = xr * wr - xi * wi;
                    ai[r] = xr * wi + xi * wr;
                }
            }
            const int base = (j / ns) * ns * R + k;
            if (R == 2) {
                const double y0r = ar[0] + ar[1], y0i = ai[0] + ai[1];
                const double y1r = ar[0] - ar[1], y1i = ai[0] - ai[1];
                dst[2 * base] = y0r; dst[2 * base + 1] = y0i;
                dst[2 * (base + ns)] = y1r; dst[2 * (base + ns) + 1] = y1i;
            } else if (R == 4) {
                const double s02r = ar[0] + ar[2], s02i = ai[0] + ai[2];
                const double d02r = ar[0] - ar[2], d02i = ai[0] - ai[2];
                const double s13r = ar[1] + ar[3], s13i = ai[1] + ai[3];
                const double d13r = ar[1] - ar[3], d13i = ai[1] - ai[3];
                /* sign*i*(d13) */
                const double jr = (sign < 0) ? d13i : -d13i;
                const double ji = (sign < 0) ? -d13r : d13r;
                dst[2 * base] = s02r + s13r;
                dst[2 * base + 1] = s02i + s13i;
                dst[2 * (base + ns)] = d02r + jr;
                dst[2 * (base + ns) + 1] = d02i + ji;
                dst[2 * (base + 2 * ns)] = s02r - s13r;
                dst[2 * (base + 2 * ns) + 1] = s02i - s13i;
                dst[2 * (base + 3 * ns)] = d02r - jr;
                dst[2 * (base + 3 * ns) + 1] = d02i - ji;
            } else {
                const long tstep = n / R; /* W_R^x = W_n^(x*n/R) */
                for (int q = 0; q < R; ++q) {
                    double yr = ar[0], yi = ai[0];
                    for (int r = 1; r < R; ++r) {
                        double wr, wi;
                        twiddle(p, ((long)q * r % R) * tstep, sign, &wr, &wi);
                        yr += ar[r] * wr - ai[r] * wi;
                        yi += ar[r] * wi + ai[r] * wr;
                    }
                    dst[2 * (base + q * ns)] = yr;
                    dst[2 * (base + q * ns) + 1] = yi;
                }
            }
        }
        double* t = src;
        src = dst;
        dst = t;
        ns *= R;
    }
    if (src != data) memcpy(data, src, sizeof(double) * 2 * (size_t)n);
    free(gvr);
}

#define CFFT_COL_BATCH 8

/* Transform every line along one axis of a row-major n0 x n1 x n2 array.
 * outer = product of dims before the axis, len = axis length,
 * inner = product of dims after the axis (element stride of the line). */
static void transform_axis(double* data, long outer, int len, long inner, int sign, int threads) {
    if (len <= 1) return;
    cfft_plan* p = cfft_plan_create(len);
    if (inner == 1) {
#pragma omp parallel num_threads(threads)
        {
            double* scratch = (double*)malloc(sizeof(double) * 2 * (size_t)len);
#pragma omp for schedule(static)
            for (long o = 0; o < outer; ++o) {
                cfft_exec_1d(p, data + 2 * o * len, scratch, sign);
            }
            free(scratch);
        }
    } else {
        const long nchunk = (inner + CFFT_COL_BATCH - 1) / CFFT_COL_BATCH;
#pragma omp parallel num_threads(threads)
        {
            double* buf = (double*)malloc(sizeof(double) * 2 * (size_t)len * CFFT_COL_BATCH);
            double* scratch = (double*)malloc(sizeof(double) * 2 * (size_t)len);
#pragma omp for schedule(static)
            for (long w = 0; w < outer * nchunk; ++w) {
                const long o = w / nchunk;
                const long c0 = (w % nchunk) * CFFT_COL_BATCH;
                const long nb = (inner - c0 < CFFT_COL_BATCH) ? inner - c0 : CFFT_COL_BATCH;
                double* base = data + 2 * (o * len * inner + c0);
                for (int j = 0; j < len; ++j) {
                    const double* row = base + 2 * (long)j * inner;
                    for (long b = 0; b < nb; ++b) {
                        buf[2 * (b * len + j)] = row[2 * b];
                        buf[2 * (b * len + j) + 1] = row[2 * b + 1];
                    }
                }
                for (long b = 0; b < nb; ++b) cfft_exec_1d(p, buf + 2 * b * len, scratch, sign);
                for (int j = 0; j < len; ++j) {
                    double* row = base + 2 * (long)j * inner;
                    for (long b = 0; b < nb; ++b) {
                        row[2 * b] = buf[2 * (b * len + j)];
                        row[2 * b + 1] = buf[2 * (b * len + j) + 1];
                    }
                }
            }
            free(buf);
            free(scratch);
        }
    }
    cfft_plan_destroy(p);
}

void cfft_exec_3d(int n0, int n1, int n2, double* data, int sign, int threads) {
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#else
    threads = 1;
#endif
    transform_axis(data, (long)n0 * n1, n2, 1, sign, threads);
    transform_axis(data, n0, n1, n2, sign, threads);
    transform_axis(data, 1, n0, (long)n1 * n2, sign, threads);
}
