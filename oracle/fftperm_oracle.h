/*
 * fftperm_oracle.h -- plain-C, FP64 restatement of the reference's
 * permeability hot path.  TEST INFRASTRUCTURE ONLY: it is the checker the
 * GPU path is compared against (tests/, the smoke check, and bench.py's CPU
 * baseline leg).  No product code links it.
 *
 * Conventions (all follow the reference):
 *   - grid flat index (k*ny + j)*nx + i, x fastest  (src/core/Grid3D.hpp:41-43)
 *   - fluid mask: nonzero = fluid                   (src/geometry/BinaryMedium.cpp:9-11)
 *   - vector fields: three contiguous blocks x|y|z of N values (SoA,
 *     src/core/Field3D.hpp:16-113)
 *   - compact support vectors: value[3*local + comp]
 *     (src/bignonnet/TrialForceField.cpp:16-40)
 *   - Green tensor components ordered xx, xy, xz, yy, yz, zz
 *     (src/bignonnet/GreenOperator.cpp:194-204)
 */
#ifndef FFTPERM_ORACLE_H
#define FFTPERM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Support set.  mode 0 = interface (solid voxels with a fluid voxel among the
 * 26 periodic neighbours), 1 = all solid voxels.  Returns N_B and writes the
 * ascending flat indices to out when out != NULL. */
long long orc_support(int nx, int ny, int nz, const unsigned char* fluid_mask, int mode,
                      long long* out);

/* Background force f0 (3 x N SoA) for a macroscopic gradient. */
void orc_background_force(int nx, int ny, int nz, const unsigned char* fluid_mask,
                          const long long* support, long long nb, const double grad[3],
                          double* f0_soa);

/* Energy-consistent Green tensor on the full C2C spectrum (6 x N). */
void orc_green_tensor(int nx, int ny, int nz, double h, double mu, int p_radius, double* g6,
                      int threads);

typedef struct orc_ctx orc_ctx;

orc_ctx* orc_create(int nx, int ny, int nz, double h, double mu, int p_radius,
                    const unsigned char* fluid_mask, int mode, int threads);
void orc_destroy(orc_ctx* c);
long long orc_nb(const orc_ctx* c);
void orc_get_support(const orc_ctx* c, long long* out);
/* The Green tensor the context uses (6 x N). */
void orc_get_green(const orc_ctx* c, double* g6);

/* u = G * f on full-grid SoA fields. */
void orc_green_apply(orc_ctx* c, const double* f_soa, double* u_soa);
/* y = A x on compact vectors of length 3*N_B. */
void orc_operator_apply(orc_ctx* c, const double* x, double* y);
/* b = -P_B gather(G * f0(grad)). */
void orc_build_rhs(orc_ctx* c, const double grad[3], double* b);
/* MINRES; returns the number of residual-history entries written to hist
 * (hist may be NULL, otherwise it must hold maxit + 1 values). */
int orc_minres(orc_ctx* c, const double* b, const double* x0, double tol, long long maxit,
               double* x, double* hist, long long* iters, double* final_rel, int* converged);
/* Velocity recovery; v_soa (3 x N) may be NULL.  avg = domain average. */
void orc_recover(orc_ctx* c, const double grad[3], const double* x, double* v_soa,
                 double avg[3]);
/* Three unit load cases -> row-major K (Darcy sign). */
int orc_solve_permeability(orc_ctx* c, double tol, long long maxit, double K[9],
                           long long iters[3]);

/* Brinkman penalisation iteration of the reference (FluidBrinkman.cpp).
 * ids: material id per voxel; voxels with id == fluid_id are fluid with
 * viscosity fluid_mu, every other id is solid with penalty solid_penalty and
 * viscosity 1.  ux, uy, uz, p (N each) may be NULL.  Returns 0, or -1 when the
 * residual becomes non-finite or the geometry has no fluid or no solid. */
int orc_brinkman_solve(int nx, int ny, int nz, const unsigned int* ids, unsigned int fluid_id,
                       double fluid_mu, double solid_penalty, double relaxation, double tolerance,
                       int max_iterations, const double force[3], double* ux, double* uy,
                       double* uz, double* p, double U[3], int* iterations, double* residual,
                       int* converged, double* porosity, double* mean_mu);

#ifdef __cplusplus
}
#endif

#endif
