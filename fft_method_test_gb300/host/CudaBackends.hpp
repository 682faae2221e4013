// CudaBackends.hpp -- drop-in implementations of the reference's C++
// interfaces on top of the C ABI of include/fftperm.h.
//
// These classes are compiled INSIDE the reference's tree (they include its
// headers: fft/IFFTBackend.hpp, solver/ILinearOperator.hpp, ...) and link
// libfftperm.so:
//   * CudaFFTBackend : IFFTBackend  -- registered by create_fft_backend for
//     ComputeBackend::GPU (src/fft/FFTBackendFactory.cpp:23-30), so the
//     reference's GreenOperator runs its FFTs on the GPU unchanged.
//   * CudaVariationalOperator : ILinearOperator -- replaces
//     VariationalOperator (src/bignonnet/VariationalOperator.cpp:19-41); its
//     apply is the fused GPU pipeline, so the reference's MinresSolver can
//     drive it.
//   * cuda_solve_one_direction -- the device-resident fast path replacing the
//     body of solve_one_direction (src/app/PermeabilityRunner.cpp:173-242):
//     RHS, MINRES and recovery stay on the GPU; returns the reference's
//     SolverResult and the domain-averaged velocity.
// C-ABI status codes are rethrown as the reference's exception types:
// FP_ERR_INVALID -> std::invalid_argument, everything else ->
// std::runtime_error.
#pragma once

#include <cstddef>
#include <string>
#include <vector>

#include "core/Field3D.hpp"
#include "core/Grid3D.hpp"
#include "core/Types.hpp"
#include "fft/IFFTBackend.hpp"
#include "fftperm.h"
#include "geometry/BinaryMedium.hpp"
#include "solver/ILinearOperator.hpp"
#include "solver/SolverResult.hpp"

namespace permeability {

// Throws the reference's exception type for a non-OK status.
void fp_throw_if_error(fp_handle h, int status);

class CudaFFTBackend final : public IFFTBackend {
public:
    CudaFFTBackend() = default;
    ~CudaFFTBackend() override;
    CudaFFTBackend(const CudaFFTBackend&) = delete;
    CudaFFTBackend& operator=(const CudaFFTBackend&) = delete;

    void initialize(const Grid3D& grid, int thread_count) override;
    void forward(const VectorField3D& real_in, ComplexVectorField3D& complex_out) override;
    void inverse(const ComplexVectorField3D& complex_in, VectorField3D& real_out) override;
    [[nodiscard]] double normalization_factor() const noexcept override { return inv_n_; }
    [[nodiscard]] const Grid3D& grid() const noexcept override { return grid_; }
    [[nodiscard]] std::string device_info() const override;

private:
    fp_handle h_ = nullptr;
    Grid3D grid_{1, 1, 1};
    double inv_n_ = 1.0;
    std::vector<double> real_;  // 3 x N SoA staging
    std::vector<double> half_;  // 3 x (nx/2+1) ny nz complex staging
};

class CudaVariationalOperator final : public ILinearOperator {
public:
    // precision: FP_PREC_FP64 or FP_PREC_MIXED.
    CudaVariationalOperator(const BinaryMedium& medium, SupportMode mode, Scalar viscosity,
                            int p_radius, int precision = FP_PREC_FP64);
    ~CudaVariationalOperator() override;
    CudaVariationalOperator(const CudaVariationalOperator&) = delete;
    CudaVariationalOperator& operator=(const CudaVariationalOperator&) = delete;

    [[nodiscard]] std::size_t size() const override { return 3 * nb_; }
    void apply(const std::vector<Scalar>& in, std::vector<Scalar>& out) const override;

    [[nodiscard]] fp_handle handle() const noexcept { return h_; }
    [[nodiscard]] std::size_t num_active_voxels() const noexcept { return nb_; }
    [[nodiscard]] Scalar viscosity() const noexcept { return mu_; }

private:
    fp_handle h_ = nullptr;
    std::size_t nb_ = 0;
    Scalar mu_ = 1;
    mutable std::vector<double> in_, out_;
};

struct CudaDirectionResult {
    SolverResult solve_result;
    Real3 avg_velocity{};
    double elapsed_seconds = 0.0;
};

// Device-resident solve of one load case (RHS, MINRES from zero, recovery).
CudaDirectionResult cuda_solve_one_direction(CudaVariationalOperator& op, const Real3& grad,
                                             Scalar tolerance, std::size_t max_iterations);

}  // namespace permeability
