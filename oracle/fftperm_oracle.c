/*
 * fftperm_oracle.c -- plain-C FP64 restatement of the reference's
 * permeability hot path.  TEST INFRASTRUCTURE ONLY (see fftperm_oracle.h).
 *
 * Every function follows the reference line by line in meaning and, where it
 * is cheap, in operation order, so that results agree with the reference
 * built in FP64 to round-off.  Citations are to files inside the reference
 * project.  The FFT is the oracle's own CPU FFT (cpu_fft.c), standing in for
 * FFTW, which the reference links but does not ship.
 */
#include "fftperm_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "cpu_fft.h"

#ifdef _OPENMP
#include <omp.h>
#endif

static const double kPi = 3.14159265358979323846;

/* ---- support (src/geometry/InterfaceVoxels.cpp:7-43,
 *               src/bignonnet/ForceSupport.cpp:9-25) ---------------------- */

static long wrap(long v, long n) {
    long m = v % n;
    if (m < 0) m += n;
    return m;
}

long long orc_support(int nx, int ny, int nz, const unsigned char* fluid_mask, int mode,
                      long long* out) {
    const long n = (long)nx * ny * nz;
    long long count = 0;
    for (long flat = 0; flat < n; ++flat) {
        if (fluid_mask[flat] != 0) continue; /* fluid voxels are never support */
        int take = 0;
        if (mode == 1) {
            take = 1; /* FullSolid: every solid voxel (ForceSupport.cpp:13-19) */
        } else {
            const long i = flat % nx;
            const long j = (flat / nx) % ny;
            const long k = flat / ((long)nx * ny);
            for (int dk = -1; dk <= 1 && !take; ++dk)
                for (int dj = -1; dj <= 1 && !take; ++dj)
                    for (int di = -1; di <= 1; ++di) {
                        if (di == 0 && dj == 0 && dk == 0) continue;
                        const long nidx = (wrap(k + dk, nz) * ny + wrap(j + dj, ny)) * nx +
                                          wrap(i + di, nx);
                        if (fluid_mask[nidx] != 0) {
                            take = 1;
                            break;
                        }
                    }
        }
        /* The flat scan is ascending, which is the reference's sorted,
         * de-duplicated order (InterfaceVoxels.cpp:40-41). */
        if (take) {
            if (out) out[count] = flat;
            ++count;
        }
    }
    return count;
}

/* ---- background force (src/bignonnet/BackgroundForce.cpp:14-60) ---------- */

void orc_background_force(int nx, int ny, int nz, const unsigned char* fluid_mask,
                          const long long* support, long long nb, const double grad[3],
                          double* f0) {
    const long n = (long)nx * ny * nz;
    memset(f0, 0, sizeof(double) * 3 * (size_t)n);
    long nf = 0;
    for (long i = 0; i < n; ++i) nf += fluid_mask[i] != 0;
    if (nb == 0) return;
    const double c_fluid = -1.0;
    const double c_support = -(double)nf / (double)nb;
    for (long i = 0; i < n; ++i) {
        if (fluid_mask[i] != 0) {
            f0[i] += c_fluid * grad[0];
            f0[n + i] += c_fluid * grad[1];
            f0[2 * n + i] += c_fluid * grad[2];
        }
    }
    for (long long s = 0; s < nb; ++s) {
        const long v = (long)support[s];
        f0[v] += c_support * grad[0];
        f0[n + v] += c_support * grad[1];
        f0[2 * n + v] += c_support * grad[2];
    }
}

/* ---- Green tensor (src/bignonnet/GreenOperator.cpp:95-178) --------------- */

static double sinc(double x) {
    /* GreenOperator.cpp:13-19 */
    if (fabs(x) < 1e-12) return 1.0;
    return sin(x) / x;
}

void orc_green_tensor(int nx, int ny, int nz, double h, double mu, int p_radius, double* g6,
                      int threads) {
    const long n = (long)nx * ny * nz;
    const double lx = h * nx, ly = h * ny, lz = h * nz; /* Grid3D.hpp:19-21 */
    const int P = p_radius < 0 ? 0 : p_radius;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#else
    (void)threads;
#endif
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads)
    for (long idx = 0; idx < n; ++idx) {
        const long ki = idx % nx;
        const long kj = (idx / nx) % ny;
        const long kk = idx / ((long)nx * ny);
        double gxx = 0, gxy = 0, gxz = 0, gyy = 0, gyz = 0, gzz = 0;
        if (!(ki == 0 && kj == 0 && kk == 0)) { /* G(0) = 0, :110-118 */
            for (int px = -P; px <= P; ++px)
                for (int py = -P; py <= P; ++py)
                    for (int pz = -P; pz <= P; ++pz) {
                        /* Unshifted wave numbers: m = k + p*n with k in [0, n) (:130-132) */
                        const long mx = ki + (long)px * nx;
                        const long my = kj + (long)py * ny;
                        const long mz = kk + (long)pz * nz;
                        const double sx = sinc(kPi * (double)mx / (double)nx);
                        const double sy = sinc(kPi * (double)my / (double)ny);
                        const double sz = sinc(kPi * (double)mz / (double)nz);
                        const double weight = (sx * sx) * (sy * sy) * (sz * sz);
                        if (weight == 0.0) continue;
                        const double qx = (2.0 * kPi * (double)mx) / lx;
                        const double qy = (2.0 * kPi * (double)my) / ly;
                        const double qz = (2.0 * kPi * (double)mz) / lz;
                        const double q2 = qx * qx + qy * qy + qz * qz;
                        if (q2 <= DBL_EPSILON) continue;
                        const double inv_mu_q2 = 1.0 / (mu * q2);
                        const double inv_q2 = 1.0 / q2;
                        const double fac = weight * inv_mu_q2;
                        gxx += fac * (1.0 - qx * qx * inv_q2);
                        gxy += fac * (-qx * qy * inv_q2);
                        gxz += fac * (-qx * qz * inv_q2);
                        gyy += fac * (1.0 - qy * qy * inv_q2);
                        gyz += fac * (-qy * qz * inv_q2);
                        gzz += fac * (1.0 - qz * qz * inv_q2);
                    }
        }
        g6[idx] = gxx;
        g6[n + idx] = gxy;
        g6[2 * n + idx] = gxz;
        g6[3 * n + idx] = gyy;
        g6[4 * n + idx] = gyz;
        g6[5 * n + idx] = gzz;
    }
}

/* ---- context ------------------------------------------------------------- */

struct orc_ctx {
    int nx, ny, nz;
    long n;
    double h, mu;
    int threads;
    unsigned char* mask;
    long long* support;
    long long nb;
    double* green;  /* 6 x N */
    double* spec;   /* 3 x N complex (force spectrum) */
    double* spec_u; /* 3 x N complex (velocity spectrum) */
    double* full_f; /* 3 x N real */
    double* full_u; /* 3 x N real */
    double* cin;    /* 3 x N_B */
    double* cout;   /* 3 x N_B */
};

orc_ctx* orc_create(int nx, int ny, int nz, double h, double mu, int p_radius,
                    const unsigned char* fluid_mask, int mode, int threads) {
    if (nx < 1 || ny < 1 || nz < 1 || !(mu > 0.0)) return NULL;
    orc_ctx* c = (orc_ctx*)calloc(1, sizeof(orc_ctx));
    c->nx = nx;
    c->ny = ny;
    c->nz = nz;
    c->n = (long)nx * ny * nz;
    c->h = h;
    c->mu = mu;
#ifdef _OPENMP
    c->threads = threads > 0 ? threads : omp_get_max_threads();
#else
    c->threads = 1;
#endif
    c->mask = (unsigned char*)malloc((size_t)c->n);
    memcpy(c->mask, fluid_mask, (size_t)c->n);
    c->nb = orc_support(nx, ny, nz, fluid_mask, mode, NULL);
    c->support = (long long*)malloc(sizeof(long long) * (size_t)(c->nb > 0 ? c->nb : 1));
    orc_support(nx, ny, nz, fluid_mask, mode, c->support);
    c->green = (double*)malloc(sizeof(double) * 6 * (size_t)c->n);
    orc_green_tensor(nx, ny, nz, h, mu, p_radius, c->green, c->threads);
    c->spec = (double*)malloc(sizeof(double) * 6 * (size_t)c->n);
    c->spec_u = (double*)malloc(sizeof(double) * 6 * (size_t)c->n);
    c->full_f = (double*)malloc(sizeof(double) * 3 * (size_t)c->n);
    c->full_u = (double*)malloc(sizeof(double) * 3 * (size_t)c->n);
    c->cin = (double*)malloc(sizeof(double) * 3 * (size_t)(c->nb > 0 ? c->nb : 1));
    c->cout = (double*)malloc(sizeof(double) * 3 * (size_t)(c->nb > 0 ? c->nb : 1));
    return c;
}

void orc_destroy(orc_ctx* c) {
    if (!c) return;
    free(c->mask);
    free(c->support);
    free(c->green);
    free(c->spec);
    free(c->spec_u);
    free(c->full_f);
    free(c->full_u);
    free(c->cin);
    free(c->cout);
    free(c);
}

long long orc_nb(const orc_ctx* c) { return c->nb; }

void orc_get_support(const orc_ctx* c, long long* out) {
    memcpy(out, c->support, sizeof(long long) * (size_t)c->nb);
}

void orc_get_green(const orc_ctx* c, double* g6) {
    memcpy(g6, c->green, sizeof(double) * 6 * (size_t)c->n);
}

/* GreenOperator::apply (GreenOperator.cpp:54-93) with the FFTW backend's
 * contract (FFTWBackend.cpp:301-420): per component, real -> complex, forward
 * 3-D DFT (dims nz, ny, nx), 3x3 real-symmetric multiply, backward DFT,
 * keep real part times 1/N. */
void orc_green_apply(orc_ctx* c, const double* f, double* u) {
    const long n = c->n;
    for (int comp = 0; comp < 3; ++comp) {
        double* s = c->spec + 2 * comp * n;
        const double* src = f + comp * n;
#pragma omp parallel for num_threads(c->threads)
        for (long i = 0; i < n; ++i) {
            s[2 * i] = src[i];
            s[2 * i + 1] = 0.0;
        }
        cfft_exec_3d(c->nz, c->ny, c->nx, s, -1, c->threads);
    }
    const double* gxx = c->green;
    const double* gxy = c->green + n;
    const double* gxz = c->green + 2 * n;
    const double* gyy = c->green + 3 * n;
    const double* gyz = c->green + 4 * n;
    const double* gzz = c->green + 5 * n;
    const double* fx = c->spec;
    const double* fy = c->spec + 2 * n;
    const double* fz = c->spec + 4 * n;
    double* ux = c->spec_u;
    double* uy = c->spec_u + 2 * n;
    double* uz = c->spec_u + 4 * n;
#pragma omp parallel for num_threads(c->threads)
    for (long i = 0; i < n; ++i) {
        for (int part = 0; part < 2; ++part) {
            const double ax = fx[2 * i + part], ay = fy[2 * i + part], az = fz[2 * i + part];
            ux[2 * i + part] = gxx[i] * ax + gxy[i] * ay + gxz[i] * az;
            uy[2 * i + part] = gxy[i] * ax + gyy[i] * ay + gyz[i] * az;
            uz[2 * i + part] = gxz[i] * ax + gyz[i] * ay + gzz[i] * az;
        }
    }
    const double inv_n = 1.0 / (double)n;
    for (int comp = 0; comp < 3; ++comp) {
        double* s = c->spec_u + 2 * comp * n;
        cfft_exec_3d(c->nz, c->ny, c->nx, s, +1, c->threads);
        double* dst = u + comp * n;
#pragma omp parallel for num_threads(c->threads)
        for (long i = 0; i < n; ++i) dst[i] = s[2 * i] * inv_n;
    }
}

/* TrialForceField::subtract_mean (TrialForceField.cpp:66-80). */
static void subtract_mean(double* v, long long nb) {
    if (nb == 0) return;
    double sx = 0, sy = 0, sz = 0;
    for (long long i = 0; i < nb; ++i) {
        sx += v[3 * i];
        sy += v[3 * i + 1];
        sz += v[3 * i + 2];
    }
    const double inv = 1.0 / (double)nb;
    const double mx = sx * inv, my = sy * inv, mz = sz * inv;
    for (long long i = 0; i < nb; ++i) {
        v[3 * i] -= mx;
        v[3 * i + 1] -= my;
        v[3 * i + 2] -= mz;
    }
}

/* VariationalOperator::apply (VariationalOperator.cpp:19-41). */
void orc_operator_apply(orc_ctx* c, const double* x, double* y) {
    const long n = c->n;
    const long long nb = c->nb;
    memcpy(c->cin, x, sizeof(double) * 3 * (size_t)nb);
    subtract_mean(c->cin, nb);
    memset(c->full_f, 0, sizeof(double) * 3 * (size_t)n);
    for (long long s = 0; s < nb; ++s) { /* scatter_to_full (TrialForceField.cpp:97-110) */
        const long v = (long)c->support[s];
        c->full_f[v] = c->cin[3 * s];
        c->full_f[n + v] = c->cin[3 * s + 1];
        c->full_f[2 * n + v] = c->cin[3 * s + 2];
    }
    orc_green_apply(c, c->full_f, c->full_u);
    for (long long s = 0; s < nb; ++s) { /* gather_from_full (:112-125) */
        const long v = (long)c->support[s];
        c->cout[3 * s] = c->full_u[v];
        c->cout[3 * s + 1] = c->full_u[n + v];
        c->cout[3 * s + 2] = c->full_u[2 * n + v];
    }
    subtract_mean(c->cout, nb);
    memcpy(y, c->cout, sizeof(double) * 3 * (size_t)nb);
}

/* VariationalRHS::build (VariationalRHS.cpp:15-31). */
void orc_build_rhs(orc_ctx* c, const double grad[3], double* b) {
    const long n = c->n;
    orc_background_force(c->nx, c->ny, c->nz, c->mask, c->support, c->nb, grad, c->full_f);
    orc_green_apply(c, c->full_f, c->full_u);
    for (long long s = 0; s < c->nb; ++s) {
        const long v = (long)c->support[s];
        b[3 * s] = c->full_u[v];
        b[3 * s + 1] = c->full_u[n + v];
        b[3 * s + 2] = c->full_u[2 * n + v];
    }
    subtract_mean(b, c->nb);
    for (long long i = 0; i < 3 * c->nb; ++i) b[i] = -b[i];
}

/* ---- MINRES (src/solver/MinresSolver.cpp:46-218) ------------------------- */

static double vdot(const double* a, const double* b, long m) {
    double s = 0.0;
    for (long i = 0; i < m; ++i) s += a[i] * b[i];
    return s;
}

static double vnorm(const double* a, long m) {
    const double d = vdot(a, a, m);
    return sqrt(d > 0.0 ? d : 0.0);
}

int orc_minres(orc_ctx* c, const double* rhs, const double* x0, double tol, long long maxit,
               double* xout, double* hist, long long* iters, double* final_rel, int* converged) {
    const long m = 3 * (long)c->nb;
    const size_t bytes = sizeof(double) * (size_t)(m > 0 ? m : 1);
    double* x = (double*)calloc(1, bytes);
    double* v_old = (double*)calloc(1, bytes);
    double* v = (double*)calloc(1, bytes);
    double* z = (double*)calloc(1, bytes);
    double* w_prev = (double*)calloc(1, bytes);
    double* w = (double*)calloc(1, bytes);
    double* w_next = (double*)calloc(1, bytes);
    int nh = 0;
    *iters = 0;
    *converged = 0;
    if (x0) memcpy(x, x0, bytes);

    const double rhs_raw_norm = vnorm(rhs, m);
    if (rhs_raw_norm == 0.0) { /* :76-82 */
        *converged = 1;
        *final_rel = 0.0;
        if (hist) hist[nh] = 0.0;
        ++nh;
        memcpy(xout, x, sizeof(double) * (size_t)m);
        goto done;
    }
    {
        const double rhs_norm = rhs_raw_norm > DBL_MIN ? rhs_raw_norm : DBL_MIN;
        orc_operator_apply(c, x, z); /* r0 = b - A x0 (:87-90) */
        for (long i = 0; i < m; ++i) z[i] = rhs[i] - z[i];
        const double beta1 = vnorm(z, m);
        const double rel0 = beta1 / rhs_norm;
        if (hist) hist[nh] = rel0;
        ++nh;
        *final_rel = rel0;
        if (rel0 <= tol || beta1 == 0.0) {
            *converged = 1;
            memcpy(xout, x, sizeof(double) * (size_t)m);
            goto done;
        }
        for (long i = 0; i < m; ++i) v[i] = z[i] / beta1;
        double beta = beta1;
        double cs_old = -1.0, sn_old = 0.0, cs = -1.0, sn = 0.0;
        double phi_bar = beta1;
        const double eps_b = 1e-14; /* kBreakdownEps (:120) */
        for (long long k = 0; k < maxit; ++k) {
            orc_operator_apply(c, v, z);
            const double alpha = vdot(v, z, m);
            for (long i = 0; i < m; ++i) z[i] -= alpha * v[i] + beta * v_old[i];
            const double beta_new = vnorm(z, m);
            memcpy(v_old, v, sizeof(double) * (size_t)m);
            if (beta_new > eps_b) {
                for (long i = 0; i < m; ++i) v[i] = z[i] / beta_new;
            } else {
                memset(v, 0, sizeof(double) * (size_t)m);
            }
            const double eps = sn_old * beta;
            const double delta_raw = -cs_old * beta;
            const double delta = cs * delta_raw + sn * alpha;
            const double phi = sn * delta_raw - cs * alpha;
            const double rho = hypot(phi, beta_new);
            double cs_new = 1.0, sn_new = 0.0;
            if (rho > eps_b) {
                cs_new = phi / rho;
                sn_new = beta_new / rho;
                for (long i = 0; i < m; ++i)
                    w_next[i] = (v_old[i] - eps * w_prev[i] - delta * w[i]) / rho;
            } else {
                memset(w_next, 0, sizeof(double) * (size_t)m);
            }
            const double step = cs_new * phi_bar;
            for (long i = 0; i < m; ++i) x[i] += step * w_next[i];
            phi_bar *= sn_new;
            double* t = w_prev;
            w_prev = w;
            w = w_next;
            w_next = t;
            cs_old = cs;
            sn_old = sn;
            cs = cs_new;
            sn = sn_new;
            beta = beta_new;
            const double rel_res = fabs(phi_bar) / rhs_norm;
            if (hist) hist[nh] = rel_res;
            ++nh;
            *final_rel = rel_res;
            *iters = k + 1;
            if (rel_res <= tol) {
                *converged = 1;
                break;
            }
            if (beta_new < eps_b) {
                *converged = rel_res <= tol;
                break;
            }
        }
        if (!*converged) *converged = *final_rel <= tol;
        memcpy(xout, x, sizeof(double) * (size_t)m);
    }
done:
    free(x);
    free(v_old);
    free(v);
    free(z);
    free(w_prev);
    free(w);
    free(w_next);
    return nh;
}

/* ---- recovery (src/bignonnet/VelocityRecovery.cpp:12-51) ----------------- */

void orc_recover(orc_ctx* c, const double grad[3], const double* xin, double* v_soa,
                 double avg[3]) {
    const long n = c->n;
    const long long nb = c->nb;
    memcpy(c->cin, xin, sizeof(double) * 3 * (size_t)nb);
    subtract_mean(c->cin, nb);
    /* f = f0 + scatter(fx) (:23-27) */
    orc_background_force(c->nx, c->ny, c->nz, c->mask, c->support, nb, grad, c->full_f);
    for (long long s = 0; s < nb; ++s) {
        const long v = (long)c->support[s];
        c->full_f[v] += 1.0 * c->cin[3 * s];
        c->full_f[n + v] += 1.0 * c->cin[3 * s + 1];
        c->full_f[2 * n + v] += 1.0 * c->cin[3 * s + 2];
    }
    orc_green_apply(c, c->full_f, c->full_u);
    /* V' = -mean_B(U) (:33-44) */
    double m[3] = {0, 0, 0};
    if (nb > 0) {
        for (long long s = 0; s < nb; ++s) {
            const long v = (long)c->support[s];
            m[0] += c->full_u[v];
            m[1] += c->full_u[n + v];
            m[2] += c->full_u[2 * n + v];
        }
        const double inv = 1.0 / (double)nb;
        m[0] *= inv;
        m[1] *= inv;
        m[2] *= inv;
    }
    double a[3] = {0, 0, 0};
    for (int comp = 0; comp < 3; ++comp) {
        double* u = c->full_u + comp * n;
        const double vp = -m[comp];
        for (long i = 0; i < n; ++i) {
            u[i] += vp;
            a[comp] += u[i];
        }
        a[comp] *= 1.0 / (double)n; /* mean_over_all (Field3D.hpp:75-90) */
    }
    if (v_soa) memcpy(v_soa, c->full_u, sizeof(double) * 3 * (size_t)n);
    avg[0] = a[0];
    avg[1] = a[1];
    avg[2] = a[2];
}

/* solve_one_direction x 3 + K assembly (PermeabilityRunner.cpp:173-242,
 * :772-777; PermeabilityTensor.cpp:11-18): K[row][col] = mu * <v_row>^(col). */
int orc_solve_permeability(orc_ctx* c, double tol, long long maxit, double K[9],
                           long long iters[3]) {
    const long m = 3 * (long)c->nb;
    double* b = (double*)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
    double* x = (double*)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
    for (int col = 0; col < 3; ++col) {
        double grad[3] = {0, 0, 0};
        grad[col] = 1.0;
        orc_build_rhs(c, grad, b);
        long long it = 0;
        double rel = 0;
        int conv = 0;
        orc_minres(c, b, NULL, tol, maxit, x, NULL, &it, &rel, &conv);
        double avg[3];
        orc_recover(c, grad, x, NULL, avg);
        for (int row = 0; row < 3; ++row) K[row * 3 + col] = -(-c->mu * avg[row]);
        if (iters) iters[col] = it;
    }
    free(b);
    free(x);
    return 0;
}

/* ---- Brinkman (src/brinkman/FluidBrinkman.cpp:282-507) ------------------- */

int orc_brinkman_solve(int nx, int ny, int nz, const unsigned int* ids, unsigned int fluid_id,
                       double fluid_mu, double solid_penalty, double relaxation, double tolerance,
                       int max_iterations, const double force[3], double* ux_out,
                       double* uy_out, double* uz_out, double* p_out, double U[3],
                       int* iterations, double* residual, int* converged, double* porosity,
                       double* mean_mu) {
    const long n = (long)nx * ny * nz;
    /* resolvePhaseMask without phase tags (:98-116) + buildCoefficientFields (:152-191) */
    long fluid_count = 0;
    long solid_count = 0;
    double visc_sum = 0.0;
    double* alpha = (double*)malloc(sizeof(double) * (size_t)n);
    double* visc = (double*)malloc(sizeof(double) * (size_t)n);
    for (long i = 0; i < n; ++i) {
        if (ids[i] == fluid_id) {
            alpha[i] = 0.0;
            visc[i] = fluid_mu;
            ++fluid_count;
            visc_sum += fluid_mu;
        } else {
            alpha[i] = solid_penalty;
            visc[i] = 1.0;
            ++solid_count;
        }
    }
    *porosity = n > 0 ? (double)fluid_count / (double)n : 0.0;
    *mean_mu = fluid_count > 0 ? visc_sum / (double)fluid_count : 1.0;
    if (fluid_count == 0 || solid_count == 0) {
        free(alpha);
        free(visc);
        return -1;
    }
    double* ux = (double*)calloc((size_t)n, sizeof(double));
    double* uy = (double*)calloc((size_t)n, sizeof(double));
    double* uz = (double*)calloc((size_t)n, sizeof(double));
    double* pr = (double*)calloc((size_t)n, sizeof(double));
    double* sx = (double*)calloc((size_t)n, sizeof(double));
    double* sy = (double*)calloc((size_t)n, sizeof(double));
    double* sz = (double*)calloc((size_t)n, sizeof(double));
    double* div = (double*)calloc((size_t)n, sizeof(double));
    double* phi = (double*)calloc((size_t)n, sizeof(double));
    double* phin = (double*)calloc((size_t)n, sizeof(double));
    const long sxy = (long)nx * ny;
    int status = 0;
    *converged = 0;
    *iterations = 0;
    *residual = 0.0;
#define IDX(x, y, z) ((long)(z) * sxy + (long)(y) * nx + (long)(x))
    for (int iter = 0; iter < max_iterations; ++iter) {
        double div_l2 = 0.0;
        /* momentum relaxed Jacobi (:313-369) */
        for (int z = 0; z < nz; ++z) {
            const int zm = (z + nz - 1) % nz, zp = (z + 1) % nz;
            for (int y = 0; y < ny; ++y) {
                const int ym = (y + ny - 1) % ny, yp = (y + 1) % ny;
                for (int x = 0; x < nx; ++x) {
                    const int xm = (x + nx - 1) % nx, xp = (x + 1) % nx;
                    const long id = IDX(x, y, z);
                    const long ixm = IDX(xm, y, z), ixp = IDX(xp, y, z);
                    const long iym = IDX(x, ym, z), iyp = IDX(x, yp, z);
                    const long izm = IDX(x, y, zm), izp = IDX(x, y, zp);
                    const double mu = visc[id];
                    const double al = alpha[id];
                    const double lx = ux[ixm] + ux[ixp] + ux[iym] + ux[iyp] + ux[izm] + ux[izp];
                    const double ly = uy[ixm] + uy[ixp] + uy[iym] + uy[iyp] + uy[izm] + uy[izp];
                    const double lz = uz[ixm] + uz[ixp] + uz[iym] + uz[iyp] + uz[izm] + uz[izp];
                    const double dpdx = 0.5 * (pr[ixp] - pr[ixm]);
                    const double dpdy = 0.5 * (pr[iyp] - pr[iym]);
                    const double dpdz = 0.5 * (pr[izp] - pr[izm]);
                    const double denom = al + 6.0 * mu;
                    const double jx = (force[0] - dpdx + mu * lx) / denom;
                    const double jy = (force[1] - dpdy + mu * ly) / denom;
                    const double jz = (force[2] - dpdz + mu * lz) / denom;
                    sx[id] = relaxation * jx + (1.0 - relaxation) * ux[id];
                    sy[id] = relaxation * jy + (1.0 - relaxation) * uy[id];
                    sz[id] = relaxation * jz + (1.0 - relaxation) * uz[id];
                }
            }
        }
        /* divergence (:371-400) */
        for (int z = 0; z < nz; ++z) {
            const int zm = (z + nz - 1) % nz, zp = (z + 1) % nz;
            for (int y = 0; y < ny; ++y) {
                const int ym = (y + ny - 1) % ny, yp = (y + 1) % ny;
                for (int x = 0; x < nx; ++x) {
                    const int xm = (x + nx - 1) % nx, xp = (x + 1) % nx;
                    const double d = 0.5 * (sx[IDX(xp, y, z)] - sx[IDX(xm, y, z)]) +
                                     0.5 * (sy[IDX(x, yp, z)] - sy[IDX(x, ym, z)]) +
                                     0.5 * (sz[IDX(x, y, zp)] - sz[IDX(x, y, zm)]);
                    div[IDX(x, y, z)] = d;
                    div_l2 += d * d;
                }
            }
        }
        /* 35 pressure Jacobi sweeps from phi = 0 (:402-433) */
        memset(phi, 0, sizeof(double) * (size_t)n);
        for (int k = 0; k < 35; ++k) {
            for (int z = 0; z < nz; ++z) {
                const int zm = (z + nz - 1) % nz, zp = (z + 1) % nz;
                for (int y = 0; y < ny; ++y) {
                    const int ym = (y + ny - 1) % ny, yp = (y + 1) % ny;
                    for (int x = 0; x < nx; ++x) {
                        const int xm = (x + nx - 1) % nx, xp = (x + 1) % nx;
                        const double nbr = phi[IDX(xm, y, z)] + phi[IDX(xp, y, z)] +
                                           phi[IDX(x, ym, z)] + phi[IDX(x, yp, z)] +
                                           phi[IDX(x, y, zm)] + phi[IDX(x, y, zp)];
                        phin[IDX(x, y, z)] = (nbr - div[IDX(x, y, z)]) / 6.0;
                    }
                }
            }
            double* t = phi;
            phi = phin;
            phin = t;
        }
        /* projection (:435-466) */
        for (int z = 0; z < nz; ++z) {
            const int zm = (z + nz - 1) % nz, zp = (z + 1) % nz;
            for (int y = 0; y < ny; ++y) {
                const int ym = (y + ny - 1) % ny, yp = (y + 1) % ny;
                for (int x = 0; x < nx; ++x) {
                    const int xm = (x + nx - 1) % nx, xp = (x + 1) % nx;
                    const long id = IDX(x, y, z);
                    const double gx = 0.5 * (phi[IDX(xp, y, z)] - phi[IDX(xm, y, z)]);
                    const double gy = 0.5 * (phi[IDX(x, yp, z)] - phi[IDX(x, ym, z)]);
                    const double gz = 0.5 * (phi[IDX(x, y, zp)] - phi[IDX(x, y, zm)]);
                    ux[id] = sx[id] - gx;
                    uy[id] = sy[id] - gy;
                    uz[id] = sz[id] - gz;
                    pr[id] += phi[id];
                }
            }
        }
        *iterations = iter + 1;
        *residual = sqrt(div_l2 / (double)n); /* :469 */
        if (!isfinite(*residual)) { /* :473-477 */
            status = -1;
            break;
        }
        if (*residual < tolerance) { /* :494-497 */
            *converged = 1;
            break;
        }
    }
#undef IDX
    /* computeSuperficialVelocity (:233-258) */
    double su[3] = {0, 0, 0};
    for (long i = 0; i < n; ++i) {
        su[0] += ux[i];
        su[1] += uy[i];
        su[2] += uz[i];
    }
    U[0] = su[0] / (double)n;
    U[1] = su[1] / (double)n;
    U[2] = su[2] / (double)n;
    if (ux_out) memcpy(ux_out, ux, sizeof(double) * (size_t)n);
    if (uy_out) memcpy(uy_out, uy, sizeof(double) * (size_t)n);
    if (uz_out) memcpy(uz_out, uz, sizeof(double) * (size_t)n);
    if (p_out) memcpy(p_out, pr, sizeof(double) * (size_t)n);
    free(alpha);
    free(visc);
    free(ux);
    free(uy);
    free(uz);
    free(pr);
    free(sx);
    free(sy);
    free(sz);
    free(div);
    free(phi);
    free(phin);
    if (status == 0 && !(isfinite(U[0]) && isfinite(U[1]) && isfinite(U[2]))) status = -1;
    return status;
}
