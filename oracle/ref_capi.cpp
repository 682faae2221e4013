// ref_capi.cpp -- C entry points over the reference's OWN classes, compiled
// together with the unmodified reference sources into oracle/_ref/ by
// oracle/Makefile.  TEST INFRASTRUCTURE ONLY: it exists so that the tests and
// the golden-fixture script can run the reference's code path on the same
// inputs as the GPU path and the C restatement.  Nothing here is shipped.
//
// Each function drives the reference objects exactly the way the reference's
// own driver does (src/app/PermeabilityRunner.cpp:173-242, solve_one_direction)
// or the reference's own tests do (tests/*.cpp).  All arrays are flat,
// x-fastest (src/core/Grid3D.hpp:41-43); vector fields are three contiguous
// component blocks (SoA, src/core/Field3D.hpp:16-113); compact support vectors
// are [3*local + comp] (src/bignonnet/TrialForceField.cpp:16-40).
#include <array>
#include <cstdint>
#include <cstring>
#include <exception>
#include <memory>
#include <vector>

#include "bignonnet/BackgroundForce.hpp"
#include "bignonnet/ForceSupport.hpp"
#include "bignonnet/GreenDiscretization.hpp"
#include "bignonnet/GreenOperator.hpp"
#include "bignonnet/VariationalOperator.hpp"
#include "bignonnet/VariationalRHS.hpp"
#include "bignonnet/VelocityRecovery.hpp"
#include "brinkman/FluidBrinkman.hpp"
#include "fft/FFTWBackend.hpp"
#include "geometry/BinaryMedium.hpp"
#include "geometry/InterfaceVoxels.hpp"
#include "post/PermeabilityTensor.hpp"
#include "solver/MinresSolver.hpp"

using namespace permeability;

namespace {

static_assert(sizeof(Scalar) == sizeof(double), "oracle/_ref must be built with FFT_METHOD_PRECISION_DOUBLE");

Grid3D make_grid(int nx, int ny, int nz, double h) {
    return Grid3D(static_cast<std::size_t>(nx), static_cast<std::size_t>(ny),
                  static_cast<std::size_t>(nz), h, h, h);
}

BinaryMedium make_medium(const Grid3D& g, const unsigned char* fluid_mask) {
    std::vector<unsigned char> m(fluid_mask, fluid_mask + g.total_size());
    return BinaryMedium(g, std::move(m));
}

SupportMode support_mode(int mode) {
    return mode == 1 ? SupportMode::FullSolid : SupportMode::InterfaceOnly;
}

void to_soa(const VectorField3D& f, double* out) {
    const std::size_t n = f.size();
    for (std::size_t i = 0; i < n; ++i) {
        out[i] = f.x()[i];
        out[n + i] = f.y()[i];
        out[2 * n + i] = f.z()[i];
    }
}

void from_soa(const double* in, VectorField3D& f) {
    const std::size_t n = f.size();
    for (std::size_t i = 0; i < n; ++i) {
        f.x()[i] = in[i];
        f.y()[i] = in[n + i];
        f.z()[i] = in[2 * n + i];
    }
}

struct RefCtx {
    Grid3D grid;
    BinaryMedium medium;
    ForceSupport support;
    FFTWBackend fft;
    GreenOperator green;
    BackgroundForce bg;
    VariationalRHS rhs;
    VariationalOperator op;
    VelocityRecovery recovery;

    RefCtx(int nx, int ny, int nz, double h, double mu, int p_radius,
           const unsigned char* mask, int mode, int threads)
        : grid(make_grid(nx, ny, nz, h)),
          medium(make_medium(grid, mask)),
          support(medium, support_mode(mode)),
          fft(),
          green(grid, GreenDiscretization{GreenDiscretizationType::EnergyConsistent}, mu, fft,
                threads, p_radius),
          bg(medium, support),
          rhs(support, green, bg),
          op(support, green),
          recovery(support, green, bg) {}
};

}  // namespace

extern "C" {

// InterfaceVoxels / ForceSupport (src/bignonnet/ForceSupport.cpp:9-25).
// Returns N_B; writes the ascending flat indices to out when out != nullptr.
long long ref_support(int nx, int ny, int nz, const unsigned char* fluid_mask, int mode,
                      long long* out) {
    try {
        const Grid3D g = make_grid(nx, ny, nz, 1.0);
        const BinaryMedium medium = make_medium(g, fluid_mask);
        const ForceSupport support(medium, support_mode(mode));
        if (out) {
            for (std::size_t i = 0; i < support.num_active_voxels(); ++i)
                out[i] = static_cast<long long>(support.active_voxels()[i]);
        }
        return static_cast<long long>(support.num_active_voxels());
    } catch (const std::exception&) {
        return -1;
    }
}

// BackgroundForce::build (src/bignonnet/BackgroundForce.cpp:14-60).
int ref_background_force(int nx, int ny, int nz, const unsigned char* fluid_mask, int mode,
                         const double grad[3], double* f0_soa) {
    try {
        const Grid3D g = make_grid(nx, ny, nz, 1.0);
        const BinaryMedium medium = make_medium(g, fluid_mask);
        const ForceSupport support(medium, support_mode(mode));
        const BackgroundForce bg(medium, support);
        to_soa(bg.build(Real3{grad[0], grad[1], grad[2]}), f0_soa);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// GreenOperator::precompute_energy_consistent_tensor (src/bignonnet/GreenOperator.cpp:95-178),
// read back through tensor_components (xx, xy, xz, yy, yz, zz), 6 blocks of N.
int ref_green_tensor(int nx, int ny, int nz, double h, double mu, int p_radius, double* g6) {
    try {
        const Grid3D g = make_grid(nx, ny, nz, h);
        FFTWBackend fft;
        GreenOperator green(g, GreenDiscretization{GreenDiscretizationType::EnergyConsistent}, mu,
                            fft, 1, p_radius);
        const std::size_t n = g.total_size();
        for (std::size_t i = 0; i < n; ++i) {
            const auto t = green.tensor_components(i);
            for (int c = 0; c < 6; ++c) g6[c * n + i] = t[c];
        }
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// GreenOperator::apply (src/bignonnet/GreenOperator.cpp:54-65) on a full-grid SoA field.
int ref_green_apply(int nx, int ny, int nz, double h, double mu, int p_radius, int threads,
                    const double* f_soa, double* u_soa) {
    try {
        const Grid3D g = make_grid(nx, ny, nz, h);
        FFTWBackend fft;
        GreenOperator green(g, GreenDiscretization{GreenDiscretizationType::EnergyConsistent}, mu,
                            fft, threads, p_radius);
        VectorField3D f(g), u(g);
        from_soa(f_soa, f);
        green.apply(f, u);
        to_soa(u, u_soa);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

void* ref_ctx_create(int nx, int ny, int nz, double h, double mu, int p_radius,
                     const unsigned char* fluid_mask, int mode, int threads) {
    try {
        return new RefCtx(nx, ny, nz, h, mu, p_radius, fluid_mask, mode, threads);
    } catch (const std::exception&) {
        return nullptr;
    }
}

void ref_ctx_destroy(void* ctx) { delete static_cast<RefCtx*>(ctx); }

long long ref_ctx_nb(void* ctx) {
    return static_cast<long long>(static_cast<RefCtx*>(ctx)->support.num_active_voxels());
}

// VariationalOperator::apply (src/bignonnet/VariationalOperator.cpp:19-41).
int ref_operator_apply(void* ctx, const double* x, double* y) {
    try {
        RefCtx* c = static_cast<RefCtx*>(ctx);
        const std::size_t n = c->op.size();
        std::vector<Scalar> in(x, x + n), out;
        c->op.apply(in, out);
        std::memcpy(y, out.data(), n * sizeof(double));
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// VariationalRHS::build (src/bignonnet/VariationalRHS.cpp:15-31).
int ref_build_rhs(void* ctx, const double grad[3], double* b) {
    try {
        RefCtx* c = static_cast<RefCtx*>(ctx);
        const std::vector<Scalar> v = c->rhs.build(Real3{grad[0], grad[1], grad[2]});
        std::memcpy(b, v.data(), v.size() * sizeof(double));
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// MinresSolver::solve (src/solver/MinresSolver.cpp:46-218).  hist receives
// residual_history (at most maxit + 1 entries).
int ref_minres(void* ctx, const double* b, const double* x0, double tol, long long maxit,
               double* x, double* hist, long long* iters, double* final_rel, int* converged) {
    try {
        RefCtx* c = static_cast<RefCtx*>(ctx);
        const std::size_t n = c->op.size();
        const std::vector<Scalar> rhs(b, b + n);
        std::vector<Scalar> guess;
        if (x0) guess.assign(x0, x0 + n);
        const MinresSolver solver(tol, static_cast<std::size_t>(maxit));
        const SolverResult r = solver.solve(c->op, rhs, guess);
        std::memcpy(x, r.solution.data(), n * sizeof(double));
        if (hist) {
            for (std::size_t i = 0; i < r.residual_history.size(); ++i) hist[i] = r.residual_history[i];
        }
        *iters = static_cast<long long>(r.iterations);
        *final_rel = r.final_rel_residual;
        *converged = r.converged ? 1 : 0;
        return static_cast<int>(r.residual_history.size());
    } catch (const std::exception&) {
        return -1;
    }
}

// VelocityRecovery::recover + average_over_domain (src/bignonnet/VelocityRecovery.cpp:12-51).
int ref_recover(void* ctx, const double grad[3], const double* x, double* v_soa, double avg[3]) {
    try {
        RefCtx* c = static_cast<RefCtx*>(ctx);
        const std::size_t n = c->op.size();
        const std::vector<Scalar> xs(x, x + n);
        const VectorField3D v = c->recovery.recover(Real3{grad[0], grad[1], grad[2]}, xs);
        if (v_soa) to_soa(v, v_soa);
        const Real3 a = c->recovery.average_over_domain(v);
        avg[0] = a[0];
        avg[1] = a[1];
        avg[2] = a[2];
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// The body of solve_one_direction (src/app/PermeabilityRunner.cpp:205-234):
// RHS, zero-start MINRES, recovery, domain average.
int ref_solve_load_case(void* ctx, const double grad[3], double tol, long long maxit,
                        double avg[3], long long* iters, double* final_rel, int* converged) {
    try {
        RefCtx* c = static_cast<RefCtx*>(ctx);
        const Real3 g{grad[0], grad[1], grad[2]};
        const std::vector<Scalar> b = c->rhs.build(g);
        const MinresSolver solver(tol, static_cast<std::size_t>(maxit));
        const SolverResult r = solver.solve(c->op, b, {});
        const VectorField3D v = c->recovery.recover(g, r.solution);
        const Real3 a = c->recovery.average_over_domain(v);
        avg[0] = a[0];
        avg[1] = a[1];
        avg[2] = a[2];
        *iters = static_cast<long long>(r.iterations);
        *final_rel = r.final_rel_residual;
        *converged = r.converged ? 1 : 0;
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// K assembly (src/app/PermeabilityRunner.cpp:772-777, src/post/PermeabilityTensor.cpp:11-18)
// for unit gradients along x, y, z.  K is row-major.
int ref_solve_permeability(void* ctx, double mu, double tol, long long maxit, double K[9],
                           long long iters[3]) {
    try {
        PermeabilityTensor kt;
        for (int col = 0; col < 3; ++col) {
            double grad[3] = {0.0, 0.0, 0.0};
            grad[col] = 1.0;
            double avg[3];
            long long it = 0;
            double rel = 0.0;
            int conv = 0;
            if (ref_solve_load_case(ctx, grad, tol, maxit, avg, &it, &rel, &conv) != 0) return -1;
            const Real3 colK{-mu * avg[0], -mu * avg[1], -mu * avg[2]};
            kt.set_column(static_cast<std::size_t>(col), colK);
            if (iters) iters[col] = it;
        }
        const auto d = kt.data();
        for (int i = 0; i < 9; ++i) K[i] = d[static_cast<std::size_t>(i)];
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// common::fluid::solveBrinkman (src/brinkman/FluidBrinkman.cpp:282-507) with a
// material database holding one fluid id of viscosity fluid_mu, as
// run_brinkman builds it when no material file is given
// (src/app/PermeabilityRunner.cpp:261-282).  Velocity components are written
// when the pointers are non-null.
int ref_brinkman_solve(int nx, int ny, int nz, const unsigned int* ids, unsigned int fluid_id,
                       double fluid_mu, double solid_penalty, double relaxation, double tolerance,
                       int max_iterations, double voxel_size, const double force[3], double* ux,
                       double* uy, double* uz, double U[3], int* iterations, double* residual,
                       int* converged) {
    try {
        common::AppConfig cfg;
        cfg.fluid.fluidMaterialId = fluid_id;
        cfg.fluid.solidPenalty = solid_penalty;
        cfg.fluid.relaxation = relaxation;
        cfg.fluid.tolerance = tolerance;
        cfg.fluid.maxIterations = max_iterations;
        cfg.fluid.voxelSize = voxel_size;
        cfg.fluid.progressInterval = 0;
        common::Geometry geo;
        geo.nx = static_cast<std::size_t>(nx);
        geo.ny = static_cast<std::size_t>(ny);
        geo.nz = static_cast<std::size_t>(nz);
        geo.materialIds.assign(ids, ids + geo.voxelCount());
        common::MaterialDatabase db;
        common::MaterialProperties props;
        props.values["viscosity"] = fluid_mu;
        db.insert(fluid_id, std::move(props));
        const std::array<double, 3> f{force[0], force[1], force[2]};
        const common::fluid::SolveResult r = common::fluid::solveBrinkman(cfg, geo, db, f);
        const std::size_t n = geo.voxelCount();
        if (ux) std::memcpy(ux, r.velocity.ux.data(), n * sizeof(double));
        if (uy) std::memcpy(uy, r.velocity.uy.data(), n * sizeof(double));
        if (uz) std::memcpy(uz, r.velocity.uz.data(), n * sizeof(double));
        U[0] = r.superficialVelocity[0];
        U[1] = r.superficialVelocity[1];
        U[2] = r.superficialVelocity[2];
        *iterations = r.diagnostics.iterations;
        *residual = r.diagnostics.residual;
        *converged = r.diagnostics.converged ? 1 : 0;
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

}  // extern "C"
