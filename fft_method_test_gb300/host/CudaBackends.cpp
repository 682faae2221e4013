// CudaBackends.cpp -- see CudaBackends.hpp.
#include "CudaBackends.hpp"

#include <stdexcept>

namespace permeability {

void fp_throw_if_error(fp_handle h, int status) {
    if (status == FP_OK) return;
    const std::string msg = h ? fp_last_error(h) : "fftperm: invalid handle";
    if (status == FP_ERR_INVALID) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

// ---------------------------------------------------------------------------
// CudaFFTBackend
// ---------------------------------------------------------------------------

CudaFFTBackend::~CudaFFTBackend() {
    if (h_) fp_destroy(h_);
}

void CudaFFTBackend::initialize(const Grid3D& grid, int thread_count) {
    (void)thread_count;
    if (h_) {
        fp_destroy(h_);
        h_ = nullptr;
    }
    grid_ = grid;
    inv_n_ = 1.0 / static_cast<double>(grid.total_size());
    // Viscosity and alias radius do not matter for the plain transforms.
    const int st = fp_create(static_cast<int>(grid.nx()), static_cast<int>(grid.ny()),
                             static_cast<int>(grid.nz()), static_cast<double>(grid.hx()), 1.0, 0,
                             FP_PREC_FP64, &h_);
    fp_throw_if_error(h_, st);
    real_.assign(3 * grid.total_size(), 0.0);
    half_.assign(2 * 3 * (grid.nx() / 2 + 1) * grid.ny() * grid.nz(), 0.0);
}

void CudaFFTBackend::forward(const VectorField3D& real_in, ComplexVectorField3D& complex_out) {
    if (!h_) throw std::runtime_error("CudaFFTBackend must be initialized before forward transform");
    if (real_in.size() != complex_out.size() || real_in.size() != grid_.total_size())
        throw std::invalid_argument("CudaFFTBackend::forward grid size mismatch");
    const std::size_t n = grid_.total_size();
    for (std::size_t i = 0; i < n; ++i) {
        real_[i] = static_cast<double>(real_in.x()[i]);
        real_[n + i] = static_cast<double>(real_in.y()[i]);
        real_[2 * n + i] = static_cast<double>(real_in.z()[i]);
    }
    fp_throw_if_error(h_, fp_fft_forward(h_, real_.data(), half_.data()));
    // expand the half spectrum by Hermitian symmetry X(-k) = conj X(k)
    const std::size_t nx = grid_.nx(), ny = grid_.ny(), nz = grid_.nz(), nxh = nx / 2 + 1;
    const std::size_t nh = nxh * ny * nz;
    Array3D<ScalarComplex>* dst[3] = {&complex_out.x(), &complex_out.y(), &complex_out.z()};
    for (int c = 0; c < 3; ++c) {
        const double* hc = half_.data() + 2 * c * nh;
        Array3D<ScalarComplex>& d = *dst[c];
        for (std::size_t k = 0; k < nz; ++k)
            for (std::size_t j = 0; j < ny; ++j)
                for (std::size_t i = 0; i < nx; ++i) {
                    double re, im;
                    if (i < nxh) {
                        const std::size_t q = (k * ny + j) * nxh + i;
                        re = hc[2 * q];
                        im = hc[2 * q + 1];
                    } else {
                        const std::size_t q =
                            (((nz - k) % nz) * ny + (ny - j) % ny) * nxh + (nx - i);
                        re = hc[2 * q];
                        im = -hc[2 * q + 1];
                    }
                    d[grid_.flat_index(i, j, k)] =
                        ScalarComplex(static_cast<Scalar>(re), static_cast<Scalar>(im));
                }
    }
}

void CudaFFTBackend::inverse(const ComplexVectorField3D& complex_in, VectorField3D& real_out) {
    if (!h_) throw std::runtime_error("CudaFFTBackend must be initialized before inverse transform");
    if (real_out.size() != complex_in.size() || real_out.size() != grid_.total_size())
        throw std::invalid_argument("CudaFFTBackend::inverse grid size mismatch");
    // Re(IFFT X) = C2R of the Hermitian part (X(k) + conj X(-k)) / 2
    const std::size_t nx = grid_.nx(), ny = grid_.ny(), nz = grid_.nz(), nxh = nx / 2 + 1;
    const std::size_t nh = nxh * ny * nz;
    const Array3D<ScalarComplex>* src[3] = {&complex_in.x(), &complex_in.y(), &complex_in.z()};
    for (int c = 0; c < 3; ++c) {
        double* hc = half_.data() + 2 * c * nh;
        const Array3D<ScalarComplex>& s = *src[c];
        for (std::size_t k = 0; k < nz; ++k)
            for (std::size_t j = 0; j < ny; ++j)
                for (std::size_t i = 0; i < nxh; ++i) {
                    const ScalarComplex a = s[grid_.flat_index(i, j, k)];
                    const ScalarComplex b = s[grid_.flat_index((nx - i) % nx, (ny - j) % ny,
                                                               (nz - k) % nz)];
                    const std::size_t q = (k * ny + j) * nxh + i;
                    hc[2 * q] = 0.5 * (static_cast<double>(a.real()) + static_cast<double>(b.real()));
                    hc[2 * q + 1] =
                        0.5 * (static_cast<double>(a.imag()) - static_cast<double>(b.imag()));
                }
    }
    fp_throw_if_error(h_, fp_fft_inverse(h_, half_.data(), real_.data()));
    const std::size_t n = grid_.total_size();
    for (std::size_t i = 0; i < n; ++i) {
        real_out.x()[i] = static_cast<Scalar>(real_[i]);
        real_out.y()[i] = static_cast<Scalar>(real_[n + i]);
        real_out.z()[i] = static_cast<Scalar>(real_[2 * n + i]);
    }
}

std::string CudaFFTBackend::device_info() const { return "CUDA sm_103a (libfftperm)"; }

// ---------------------------------------------------------------------------
// CudaVariationalOperator
// ---------------------------------------------------------------------------

CudaVariationalOperator::CudaVariationalOperator(const BinaryMedium& medium, SupportMode mode,
                                                 Scalar viscosity, int p_radius, int precision)
    : mu_(viscosity) {
    const Grid3D& g = medium.grid();
    int st = fp_create(static_cast<int>(g.nx()), static_cast<int>(g.ny()), static_cast<int>(g.nz()),
                       static_cast<double>(g.hx()), static_cast<double>(viscosity), p_radius,
                       precision, &h_);
    fp_throw_if_error(h_, st);
    int64_t nb = 0;
    st = fp_set_geometry(h_, medium.mask().data(),
                         mode == SupportMode::FullSolid ? FP_SUPPORT_FULLSOLID : FP_SUPPORT_INTERFACE,
                         &nb);
    fp_throw_if_error(h_, st);
    nb_ = static_cast<std::size_t>(nb);
    in_.resize(3 * nb_);
    out_.resize(3 * nb_);
}

CudaVariationalOperator::~CudaVariationalOperator() {
    if (h_) fp_destroy(h_);
}

void CudaVariationalOperator::apply(const std::vector<Scalar>& in, std::vector<Scalar>& out) const {
    if (in.size() != size()) throw std::invalid_argument("VariationalOperator::apply input size mismatch");
    for (std::size_t i = 0; i < in.size(); ++i) in_[i] = static_cast<double>(in[i]);
    fp_throw_if_error(h_, fp_operator_apply(h_, in_.data(), out_.data()));
    out.resize(size());
    for (std::size_t i = 0; i < out.size(); ++i) out[i] = static_cast<Scalar>(out_[i]);
}

CudaDirectionResult cuda_solve_one_direction(CudaVariationalOperator& op, const Real3& grad,
                                             Scalar tolerance, std::size_t max_iterations) {
    if (tolerance <= Scalar(0)) throw std::invalid_argument("MinresSolver tolerance must be positive");
    const double g[3] = {static_cast<double>(grad[0]), static_cast<double>(grad[1]),
                         static_cast<double>(grad[2])};
    double avg[3] = {0.0, 0.0, 0.0};
    std::vector<double> x(op.size());
    fp_solver_stats st{};
    fp_throw_if_error(op.handle(),
                      fp_solve_load_case(op.handle(), g, nullptr, static_cast<double>(tolerance),
                                         static_cast<int64_t>(max_iterations), avg, x.data(), &st));
    CudaDirectionResult r;
    r.solve_result.solution.assign(x.begin(), x.end());
    r.solve_result.converged = st.converged != 0;
    r.solve_result.iterations = static_cast<std::size_t>(st.iterations);
    r.solve_result.final_rel_residual = static_cast<Scalar>(st.final_rel_residual);
    r.avg_velocity = Real3{static_cast<Scalar>(avg[0]), static_cast<Scalar>(avg[1]),
                           static_cast<Scalar>(avg[2])};
    r.elapsed_seconds = st.seconds;
    return r;
}

}  // namespace permeability
