/*
 * fftperm.h -- C ABI of the GB300 permeability hot path.
 *
 * One handle = one periodic voxel grid (nx, ny, nz, voxel size h, viscosity
 * mu, alias radius p_radius) with all of its state resident on the current
 * CUDA device.  Host pointers in, host pointers out; status codes instead of
 * exceptions; no C++ or torch types.  A handle is not thread-safe: use one
 * handle per host thread (the reference builds one FFT backend + Green
 * operator per load case, src/app/PermeabilityRunner.cpp:186-203).
 *
 * Conventions (the reference's):
 *   flat index (k*ny + j)*nx + i, x fastest         src/core/Grid3D.hpp:41-43
 *   fluid mask: nonzero = fluid                      src/geometry/BinaryMedium.cpp:9-11
 *   full-grid vector fields: x|y|z blocks of N      src/core/Field3D.hpp:16-113
 *   compact support vectors: v[3*local + comp]      src/bignonnet/TrialForceField.cpp:16-40
 *   K row-major, K[row*3 + col]                      src/post/PermeabilityTensor.cpp:11-18
 *
 * Error behaviour: the reference throws std::invalid_argument on size or
 * argument errors and std::runtime_error on state errors; here those become
 * FP_ERR_INVALID and FP_ERR_STATE, and fp_last_error() returns the message.
 */
#ifndef FFTPERM_H
#define FFTPERM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fp_problem* fp_handle;

enum fp_status {
    FP_OK = 0,
    FP_ERR_INVALID = 1,     /* invalid argument (reference: std::invalid_argument) */
    FP_ERR_STATE = 2,       /* call out of order (reference: std::runtime_error)   */
    FP_ERR_CUDA = 3,        /* CUDA runtime error                                   */
    FP_ERR_UNSUPPORTED = 4, /* grid edge not a product of 2, 3, 5                   */
    FP_ERR_NOMEM = 5,       /* device allocation failed                             */
    FP_ERR_NONFINITE = 6    /* a non-finite value appeared (Brinkman instability)   */
};

enum fp_precision {
    FP_PREC_FP64 = 0, /* FFT, Green multiply, scatter/gather in FP64 */
    FP_PREC_MIXED = 1 /* FFT, Green multiply, scatter/gather in FP32; Lanczos and sums in FP64 */
};

enum fp_support_mode {
    FP_SUPPORT_INTERFACE = 0, /* SupportMode::InterfaceOnly, src/core/Types.hpp:25-28 */
    FP_SUPPORT_FULLSOLID = 1  /* SupportMode::FullSolid */
};

typedef struct fp_solver_stats {
    int64_t iterations;        /* SolverResult::iterations        (src/solver/SolverResult.hpp:10-16) */
    double final_rel_residual; /* SolverResult::final_rel_residual */
    int32_t converged;         /* SolverResult::converged          */
    int32_t refinements;       /* mixed precision: outer refinement steps taken */
    double seconds;            /* wall time of the call            */
} fp_solver_stats;

/* Replaces the GreenOperator constructor + IFFTBackend::initialize
 * (src/bignonnet/GreenOperator.cpp:27-52, src/fft/FFTWBackend.cpp:185-299):
 * plans the FFTs and precomputes the energy-consistent Green tensor. */
int fp_create(int nx, int ny, int nz, double voxel_size, double mu, int p_radius, int precision,
              fp_handle* out);
int fp_destroy(fp_handle h);
const char* fp_last_error(fp_handle h);
/* The CUDA stream (cudaStream_t) every call of this handle runs on, so a
 * caller can time device-pointer calls with events on that stream. */
void* fp_stream(fp_handle h);
/* Wait for all work queued on the handle's stream. */
int fp_synchronize(fp_handle h);
/* Number of CUDA kernels this library has launched in the process so far
 * (every handle, device and stream).  A diagnostic with no counterpart in the
 * reference: the difference across a region counts the kernels it queued. */
long long fp_kernel_launch_count(void);
/* A diagnostic with no counterpart in the reference: the FP64 FMA throughput
 * of the current device in TFLOP/s (2 flops per FMA), measured with a kernel
 * of independent FMA chains on the legacy default stream; *ms receives the
 * time of one launch.  Either output may be NULL. */
int fp_measure_fp64_rate(double* tflops, double* ms);
/* Precision of later applies/solves (FP_PREC_*). */
int fp_set_precision(fp_handle h, int precision);

/* BinaryMedium + ForceSupport (src/geometry/BinaryMedium.cpp:5-8,
 * src/bignonnet/ForceSupport.cpp:9-25, src/geometry/InterfaceVoxels.cpp:7-43).
 * fluid_mask has N bytes.  *nb_out receives N_B (may be NULL). */
int fp_set_geometry(fp_handle h, const uint8_t* fluid_mask, int support_mode, int64_t* nb_out);
/* VoxelIO::load_fgeo + BinaryMedium + ForceSupport (src/io/VoxelIO.cpp:89-159):
 * reads the reference's binary .fgeo file (magic "FGEO", version 1, value
 * type 1 = u32 or 2 = u16, 2 reserved bytes, nx ny nz as little-endian u64,
 * then one id per voxel, x fastest), streams the ids to the device in chunks
 * and forms the fluid mask there (id == fluid_id), then the support set as
 * fp_set_geometry.  The file's dimensions must be the handle's. */
int fp_load_fgeo(fp_handle h, const char* path, uint32_t fluid_id, int support_mode, int64_t* nb_out);
/* ForceSupport::active_voxels (src/bignonnet/ForceSupport.hpp:22): N_B ascending flat indices. */
int fp_get_support(fp_handle h, int64_t* out);
/* Symmetrised Green tensor on the half spectrum, 6 blocks (xx xy xz yy yz zz)
 * of (nx/2+1)*ny*nz values laid out [kz][ky][kx]: (G(k) + G(-k))/2 with G of
 * src/bignonnet/GreenOperator.cpp:95-178. */
int fp_get_green(fp_handle h, double* g6);

/* IFFTBackend::forward (src/fft/IFFTBackend.hpp:18-19, FFTWBackend.cpp:301-362)
 * in R2C form: the unnormalised forward 3-D DFT of each component of a real
 * SoA field (3*N doubles), returned as the half spectrum kx in [0, nx/2]:
 * 3 blocks of (nx/2+1)*ny*nz interleaved (re, im) doubles laid out
 * [kz][ky][kx].  The other half is the complex conjugate (real input). */
int fp_fft_forward(fp_handle h, const double* real_soa, double* half_spectrum);
/* IFFTBackend::inverse (src/fft/IFFTBackend.hpp:21-22, FFTWBackend.cpp:364-420)
 * in C2R form: real part of the inverse DFT times 1/N.  The input half
 * spectrum stands for the Hermitian part (X(k) + conj X(-k))/2 of a full
 * spectrum X, whose inverse has exactly the real part the reference keeps. */
int fp_fft_inverse(fp_handle h, const double* half_spectrum, double* real_soa);
/* GreenOperator::apply (src/bignonnet/GreenOperator.cpp:54-65), i.e. the
 * IFFTBackend forward + spectral Green multiply + inverse chain, on full-grid
 * SoA fields of 3*N doubles. */
int fp_green_apply(fp_handle h, const double* force_soa, double* velocity_soa);
/* BackgroundForce::build (src/bignonnet/BackgroundForce.cpp:14-60), 3*N doubles. */
int fp_background_force(fp_handle h, const double grad[3], double* f0_soa);
/* VariationalOperator::apply, the ILinearOperator of the method
 * (src/bignonnet/VariationalOperator.cpp:19-41): y = A x, 3*N_B doubles. */
int fp_operator_apply(fp_handle h, const double* x, double* y);
/* The same with device pointers on the handle's stream (inputs resident in
 * HBM), 16-byte aligned (FP_ERR_INVALID otherwise). */
int fp_operator_apply_device(fp_handle h, const double* d_x, double* d_y);
/* VariationalRHS::build (src/bignonnet/VariationalRHS.cpp:15-31). */
int fp_build_rhs(fp_handle h, const double grad[3], double* b);
/* MinresSolver::solve (src/solver/MinresSolver.cpp:46-218).  x0 may be NULL
 * (zero start).  hist (may be NULL) receives the residual history, at most
 * maxit + 1 values; stats->iterations + 1 of them are written. */
int fp_minres(fp_handle h, const double* b, const double* x0, double tol, int64_t maxit,
              double* x, double* hist, fp_solver_stats* stats);
/* VelocityRecovery::recover + average_over_domain
 * (src/bignonnet/VelocityRecovery.cpp:12-51).  v_soa (3*N, may be NULL)
 * receives the velocity field, avg its domain average. */
int fp_recover(fp_handle h, const double grad[3], const double* x, double* v_soa, double avg[3]);
/* One load case, the body of solve_one_direction
 * (src/app/PermeabilityRunner.cpp:173-242): RHS, MINRES from x0 (NULL = zero),
 * recovery, domain-averaged velocity.  x_out (3*N_B, may be NULL) receives the
 * converged interface forces. */
int fp_solve_load_case(fp_handle h, const double grad[3], const double* x0, double tol,
                       int64_t maxit, double avg[3], double* x_out, fp_solver_stats* stats);
/* Three unit load cases and the K assembly of PermeabilityRunner::run
 * (src/app/PermeabilityRunner.cpp:700-777): K[row*3+col] = mu <v_row>^(col). */
int fp_solve_permeability(fp_handle h, double tol, int64_t maxit, double K[9],
                          fp_solver_stats stats[3]);

/* No counterpart in the reference.  The Green-operator apply of fp_green_apply
 * for callers that must not allocate device memory themselves, for example
 * code running inside another framework's memory manager (which owns the
 * device heap) or a latency-critical loop that cannot accept the device-wide
 * synchronisation cudaMalloc/cudaFree may bring.  The caller passes device
 * pointers to the input force field and the output field (3*N doubles each,
 * SoA) and a cudaStream_t (NULL = the legacy default stream); the work is
 * queued on that stream and the call returns without waiting.  FP64.
 * All working memory is one fixed, file-scope device array of about 14 MB,
 * so the grid is limited to N <= 262144 voxels (e.g. 64^3), rs*ny*nz <=
 * 139264 (rs = nx/2+1 rounded up to even) and ny*nz <= 16384; larger grids
 * return FP_ERR_INVALID.  The array is
 * shared by all calls: calls that overlap on the GPU race and must be
 * serialised by the caller.  The first call on a device resolves the array's
 * address; make that first call before any stream capture.  The address stays
 * cached for the process, so do not call this entry on a device after
 * resetting it.  Every call recomputes the twiddles and the Green table (the
 * full alias sum per point) before the transforms. */
int fp_green_apply_noalloc(int nx, int ny, int nz, double voxel_size, double mu, int p_radius,
                           const double* d_force_soa, double* d_velocity_soa, void* stream);

/* fp_recover followed by the reference's .fvel file of the recovered field
 * (write_velocity_field_binary, src/app/PermeabilityRunner.cpp:109-159): the
 * field is formed on the device and leaves it in chunks straight into the
 * file; driving = grad.  x: 3*N_B compact interface forces (host). */
int fp_recover_fvel(fp_handle h, const char* path, const double grad[3], const double* x,
                    double porosity, double viscosity);
/* The reference's .fvel velocity file (write_velocity_field_binary,
 * src/app/PermeabilityRunner.cpp:109-159) from SoA host fields of N doubles
 * each (for example the field of fp_recover).  FP_ERR_INVALID when the file
 * cannot be written. */
int fp_write_fvel(const char* path, int nx, int ny, int nz, double porosity, double viscosity,
                  const double driving[3], const double* vx, const double* vy, const double* vz);

/* ---- batches and tuning (no reference counterpart) --------------------------- */

/* Times the operator apply of this handle for each y/z-pass tiling (kx
 * columns per CTA in {4, 8, 16, 32}, TMA-fed or register-fed) and each
 * inverse-x variant (bulk-copy pipelined or one tile per CTA), x-pass
 * rows per CTA (no cap, 4, 2) and, for FP32 register-fed y/z passes, a
 * 168-register variant, and keeps the fastest; the choice is cached per (grid, precision) for the process and
 * applied to later fp_autotune calls on the same grid without timing.
 * Tiling changes the schedule and the grouping of partial sums (results equal
 * to rounding).  Outputs may be NULL. */
int fp_autotune(fp_handle h, int* tile, int* tma_off, int* x_bulk, int* x_rows, int* lowreg,
                double* apply_ms);
/* A diagnostic with no counterpart in the reference: the mean CUDA-event
 * time (ms) of `reps` back-to-back operator applies as MINRES runs them (the
 * five FFT passes with the scatter and gather fused, on the handle's compact
 * vectors, current precision and tiling), after one warm-up apply. */
int fp_time_apply(fp_handle h, int reps, double* ms);
/* Sets a tiling directly (for example one fp_autotune reported earlier):
 * tile in {0 = default, 2, 4, 8, 16, 32}, tma_off != 0 for the register-fed
 * y/z passes, x_bulk != 0 for the bulk-copy inverse x pass, x_rows > 0 caps
 * the grid rows per CTA of the x passes (0: no cap), lowreg != 0 selects the
 * FP32 register-fed y/z kernels capped at 168 registers per thread. */
int fp_set_tiling(fp_handle h, int tile, int tma_off, int x_bulk, int x_rows, int lowreg);

/* Permeability tensors of `count` independent microstructures (the reference
 * runs PermeabilityRunner once per geometry).  Problem i has grid dims[3i..3i+2]
 * = (nx, ny, nz), fluid mask masks[i] (nz*ny*nx bytes, x fastest) and voxel
 * size voxel_sizes[i] (NULL: 1).  `concurrency` host threads each solve one
 * problem at a time on its own handle and stream, largest grids first, so
 * the problems overlap on the GPU.  autotune != 0 tunes each distinct grid
 * once first (fp_autotune).  K receives 9 doubles per problem (row-major, as
 * fp_solve_permeability), stats 3 per problem (may be NULL), status one code
 * per problem (may be NULL).  Returns the first failing problem's code;
 * message: fp_batch_last_error(). */
int fp_batch_solve_permeability(int count, const int* dims, const uint8_t* const* masks,
                                const double* voxel_sizes, double mu, int p_radius, int precision,
                                int support_mode, double tol, int64_t maxit, int concurrency,
                                int autotune, double* K, fp_solver_stats* stats, int* status);
/* The same batch cut into groups of up to max_group problems of one grid and
 * voxel size, each solved with fp_group_solve_permeability (max_group = 1 is
 * fp_batch_solve_permeability). */
int fp_batch_solve_grouped(int count, const int* dims, const uint8_t* const* masks,
                           const double* voxel_sizes, double mu, int p_radius, int precision,
                           int support_mode, double tol, int64_t maxit, int concurrency, int autotune,
                           int max_group, double* K, fp_solver_stats* stats, int* status);
const char* fp_batch_last_error(void);

/* K of several problems of one grid (same dimensions, precision, reliable
 * interval and FFT tiling; FP_ERR_INVALID otherwise) solved together: the three load cases in turn, each as one
 * lockstep MINRES over the members with one kernel launch per FFT pass and
 * per vector kernel for all of them (no reference counterpart: the reference
 * runs PermeabilityRunner::run once per geometry, src/app/PermeabilityRunner.cpp:451).
 * Every member computes exactly what fp_solve_permeability computes for it.
 * Members run on handles[0]'s stream for the duration.  When a member's grid
 * has no specialised passes the members are solved one after another.
 * K: count x 9 (row-major per member); stats: count x 3 or NULL. */
int fp_group_solve_permeability(int count, fp_handle* handles, double tol, int64_t maxit, double* K,
                                fp_solver_stats* stats);

/* fp_solve_permeability with the three load cases as one block (3-RHS): two
 * sibling solves on the same support borrow h's Green tables, and the three
 * load cases iterate in lockstep as a group (one launch per pass for the
 * three fields; their z passes read one Green table, tile by tile at the
 * same time).  Same K and statistics as fp_solve_permeability (each load
 * case computes exactly what it computes alone); when h's grid has no
 * specialised passes it is fp_solve_permeability.  Extra device memory: two
 * sets of Krylov vectors and spectral buffers. */
int fp_solve_permeability_block(fp_handle h, double tol, int64_t maxit, double K[9],
                                fp_solver_stats stats[3]);

/* ---- learned warm start kernels (no reference counterpart) ------------------- */
/* Building blocks of the warm-start network, all device pointers, queued on
 * `stream` (cudaStream_t, NULL = legacy default).  Activations are
 * channels-last BF16 [voxel][channel] over `total` voxels (samples stacked,
 * each nx*ny*nz, x fastest); weights BF16 [27 taps][cout][cin], tap =
 * (dz+1)*9 + (dy+1)*3 + (dx+1) times `dilation`, periodic.  The MINRES
 * initial guess they produce enters through fp_solve_load_case's x0, the
 * reference's MinresSolver::solve initial_guess (src/solver/MinresSolver.hpp:23).
 *
 * fp_nn_conv: y = conv(x) (+ bias, ReLU) for sign +1; for sign -1 and the
 *   per-tap transposed weights [27][cin_fwd][cout_fwd], the data gradient.
 *   cin % 16 == 0; cout in {8, 16, 32, 64}; FP32 and/or BF16 output.
 * fp_nn_wgrad: dW FP32 [27][cout][cin] from dy and x; `partial` is scratch of
 *   ceil(total/chunk) * 27 * round_up(cout, 16) * cin floats, chunk % 16 == 0.
 * fp_nn_bias_grad: db[o] = sum_v dy[v][o].
 * fp_nn_relu_back: BF16 dpre[v][0..cpad) = dpost * (post > 0), zero-padded.
 * fp_nn_adam: one Adam step on FP32 masters, refreshing the BF16 forward and
 *   transposed weights.
 * fp_nn_loss: per-sample relative squared error of the predicted force on
 *   the support after per-component mean removal, and its gradient. */
int fp_nn_conv(int nx, int ny, int nz, int64_t total, int dilation, int sign, const void* in_bf16,
               int cin, const void* w_bf16, const float* bias, int cout, int relu, float* out_f32,
               void* out_bf16, void* stream);
/* fp_nn_conv on the fifth-generation tensor cores (tcgen05.mma, accumulator
 * in tensor memory): the same arguments and results, cin % 16 == 0 and
 * cin <= 128, cout in {16, 32, 64, 128}.  A bounded wait that gives up sets
 * a flag that fp_nn_tc_error reads (and clears with reset != 0). */
int fp_nn_conv_tc(int nx, int ny, int nz, int64_t total, int dilation, int sign,
                  const void* in_bf16, int cin, const void* w_bf16, const float* bias, int cout,
                  int relu, float* out_f32, void* out_bf16, void* stream);
int fp_nn_tc_error(int* flag, int reset);
int fp_nn_wgrad(int nx, int ny, int nz, int64_t total, int dilation, const void* dy_bf16, int cout,
                const void* x_bf16, int cin, int64_t chunk, float* partial, float* dw, void* stream);
/* The multi-level pieces of the U-Net (fine grid nx, ny, nz even; the coarse
 * grid is half of it along each axis; BF16 or FP32 channels-last tensors of
 * `samples` stacked cells):
 * fp_nn_pool2: coarse = mean of the 8 children;
 * fp_nn_pool2_back: dfine += dcoarse(parent) / 8;
 * fp_nn_up2_add: out = act(coarse(parent) + skip), act = ReLU when relu;
 * fp_nn_up2_add_back: with d = dout masked where post <= 0 (post may be
 *   NULL: no mask), dskip = d and dcoarse = sum of d over the 8 children;
 * fp_nn_wgrad_cc: fp_nn_wgrad on the CUDA cores for any cout, cin that are
 *   multiples of 16; `partial` holds ceil(total/chunk) * 27 * cout * cin floats. */
int fp_nn_pool2(int nx, int ny, int nz, int samples, int c, const void* in_bf16, void* out_bf16,
                void* stream);
int fp_nn_pool2_back(int nx, int ny, int nz, int samples, int c, const float* dcoarse, float* dfine,
                     void* stream);
int fp_nn_up2_add(int nx, int ny, int nz, int samples, int c, const void* coarse_bf16,
                  const void* skip_bf16, int relu, void* out_bf16, void* stream);
int fp_nn_up2_add_back(int nx, int ny, int nz, int samples, int c, const float* dout,
                       const void* post_bf16, float* dskip, float* dcoarse, void* stream);
int fp_nn_wgrad_cc(int nx, int ny, int nz, int64_t total, int dilation, const void* dy_bf16, int cout,
                   const void* x_bf16, int cin, int64_t chunk, float* partial, float* dw, void* stream);
int fp_nn_bias_grad(const void* dy_bf16, int64_t total, int cout, float* db, void* stream);
int fp_nn_relu_back(const float* dpost, const void* post_bf16, int64_t total, int c, int cpad,
                    void* out_bf16, void* stream);
int fp_nn_adam(float* w, float* m1, float* m2, const float* g, int64_t count, float lr, float b1,
               float b2, float eps, float c1, float c2, int cout, int cin, void* wf_bf16,
               void* wt_bf16, void* stream);
int fp_nn_loss(const float* pred, int cstride, const float* tgt, const uint8_t* support, int64_t n,
               int samples, const float* tnorm, float* stats, float* dpred, float* loss,
               void* stream);

/* ---- Brinkman penalisation (src/brinkman/FluidBrinkman.cpp) ---------------- */

typedef struct fp_brinkman_stats {
    int32_t iterations; /* SolveDiagnostics::iterations (include/brinkman/FluidBrinkman.hpp:16-21) */
    int32_t converged;  /* SolveDiagnostics::converged */
    double residual;    /* SolveDiagnostics::residual: sqrt(sum div(u*)^2 / N) */
    double porosity;    /* SolveResult::porosity */
    double viscosity;   /* SolveResult::viscosity (mean fluid viscosity) */
    double seconds;     /* SolveDiagnostics::elapsedSeconds */
} fp_brinkman_stats;

/* common::fluid::solveBrinkman (include/brinkman/FluidBrinkman.hpp:45-49,
 * src/brinkman/FluidBrinkman.cpp:282-507): the reference's relaxed-Jacobi
 * momentum + 35-sweep pressure projection, FP64, from rest.  ids holds one
 * material id per voxel; ids == fluid_id is fluid of viscosity fluid_mu, any
 * other id is solid (penalty solid_penalty, viscosity 1), as the reference
 * resolves phases without phase tags.  ux, uy, uz, p (N doubles each) may be
 * NULL.  U receives the superficial velocity.  Returns FP_ERR_NONFINITE when
 * the residual becomes non-finite (the reference throws) and FP_ERR_STATE
 * when the medium has no fluid or no solid voxel.  Messages:
 * fp_brinkman_last_error(). */
int fp_brinkman_solve(int nx, int ny, int nz, const uint32_t* ids, uint32_t fluid_id,
                      double fluid_mu, double solid_penalty, double relaxation, double tolerance,
                      int max_iterations, const double force[3], double* ux, double* uy,
                      double* uz, double* p, double U[3], fp_brinkman_stats* stats);
/* common::fluid::computePermeabilityTensor (src/brinkman/FluidBrinkman.cpp:509-553):
 * three solves with force = forcing * e_j; K[i*3+j] = mu U_i / f_j * h^2. */
int fp_brinkman_permeability(int nx, int ny, int nz, const uint32_t* ids, uint32_t fluid_id,
                             double fluid_mu, double solid_penalty, double relaxation,
                             double tolerance, int max_iterations, double forcing,
                             double voxel_size, double K[9], fp_brinkman_stats stats[3]);
const char* fp_brinkman_last_error(void);

/* The same Brinkman problem solved to the discrete fixed point of the
 * reference's equations, (alpha + 6 mu) u - mu sum_nbr u + grad_c p = f and
 * div_c u = 0 (the state where FluidBrinkman.cpp:313-369 and :402-466 are at
 * rest), by an FFT-preconditioned projected conjugate gradient, FP64.  The
 * reference iteration converges like iter^-1.2 toward that point and stalls
 * far above tolerances such as 1e-8; this entry reaches them.  No reference
 * counterpart as a function: it replaces solveBrinkman where the caller wants
 * the converged field.  Arguments as fp_brinkman_solve without relaxation;
 * tolerance bounds the projected momentum residual |P(f - A u)| / |P f|
 * (stats->residual).  p receives the pressure with zero mean on the modes
 * grad_c cannot see.  Needs fluid_mu == 1 (the solid's viscosity): other
 * values return FP_ERR_UNSUPPORTED. */
int fp_brinkman_fft_solve(int nx, int ny, int nz, const uint32_t* ids, uint32_t fluid_id,
                          double fluid_mu, double solid_penalty, double tolerance,
                          int max_iterations, const double force[3], double* ux, double* uy,
                          double* uz, double* p, double U[3], fp_brinkman_stats* stats);
/* computePermeabilityTensor (src/brinkman/FluidBrinkman.cpp:509-553) on
 * fp_brinkman_fft_solve: one device set-up, three load cases. */
int fp_brinkman_fft_permeability(int nx, int ny, int nz, const uint32_t* ids, uint32_t fluid_id,
                                 double fluid_mu, double solid_penalty, double tolerance,
                                 int max_iterations, double forcing, double voxel_size,
                                 double K[9], fp_brinkman_stats stats[3]);

#ifdef __cplusplus
}
#endif

#endif
