// internal.h -- device-resident state of one permeability problem and the
// host-side launchers of the CUDA kernels.  Not part of the public C ABI
// (include/fftperm.h).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/fftperm.h"
#include "fft_engine.cuh"

namespace fp {


enum Precision { kFP64 = 0, kMixed = 1 };

struct AxisPlan {
    FftPlanDev dev{};
    double2* tw64 = nullptr;
    float2* tw32 = nullptr;
};

// Build a plan for length n (factors 2, 3, 5 only); returns false otherwise.
// Twiddle tables are stream-ordered allocations on the handle's stream.
bool make_axis_plan(int n, AxisPlan& p, std::string& err, cudaStream_t stream);
void free_axis_plan(AxisPlan& p, cudaStream_t stream);

// MINRES scalar state on the device (all FP64).  Layout is private.
struct MinresScalars {
    double tol;
    double rhs_norm;
    double beta;      // beta_k
    double beta_new;  // beta_{k+1}
    double alpha;
    double cs_old, sn_old, cs, sn;
    double phi_bar;
    double rel_res;
    // coefficients of the current iteration's vector update
    double eps, delta, rho, step, inv_beta_new;
    double vsum[3];  // component sums of the current Lanczos vector v
    double zmean[3];
    long long it;     // completed iterations
    long long maxit;
    int done;
    int converged;
    int breakdown;
    int pad;
};

// Cached TMA descriptor of the spectral field for one pass and precision.
struct TmaCache {
    bool valid = false;
    int t = 0;    // kx columns per tile
    int box = 0;  // rows per box along the transform axis
    CUtensorMap map;
};

// One instantiated CUDA graph of `count` MINRES iterations starting at buffer
// rotation phase `phase` (iteration index mod 6).
struct MinresGraph {
    cudaGraphExec_t exec = nullptr;
    int phase = 0;
    int count = 0;
    long long kernels = 0;  // kernel nodes, for the launch counter
};

struct Problem {
    int nx = 0, ny = 0, nz = 0;
    long long n = 0;      // voxels
    int nxh = 0;          // nx/2 + 1
    long long rs = 0;     // row stride of spectral fields and Green tables: nxh rounded up to a multiple of 4
    long long nh = 0;     // half spectrum points stored: rs * ny * nz
    long long nrows = 0;  // ny * nz
    double h = 1.0, mu = 1.0;
    int p_radius = 2;
    int precision = kFP64;
    cudaStream_t stream = nullptr;
    int sm_count = 0;
    int tile_yz = 0;  // kx columns per CTA of the y and z passes (0 = default)
    // mixed precision: true-residual check every this many iterations (40:
    // measured 2 % faster than 20 at 256^3 with the same iteration counts)
    int reliable_interval = 40;
    // mixed precision: a refinement segment ends when the recurrence estimate
    // falls below this fraction of the segment's true residual (0.95: 2 %
    // fewer iterations than 0.85 at 256^3, K as close to the CPU oracle's;
    // 0.7 took more)
    double ahead_factor = 0.95;
    // mixed precision: a segment also ends when its true residual is below
    // this fraction of tol (then the FP64 residual decides)
    double segment_tol_factor = 1.0;

    AxisPlan px, py, pz;

    // geometry
    uint8_t* d_mask = nullptr;
    int* d_support = nullptr;    // ascending flat indices (N_B)
    int* d_row_ptr = nullptr;    // nrows + 1
    int* d_row_cnt = nullptr;    // scratch: per-row counts
    long long nb = 0;
    long long nf = 0;            // fluid voxels
    int support_mode = 0;
    bool has_geometry = false;

    // Green tensor on the half spectrum, symmetrised: 6 x nh (xx xy xz yy yz zz)
    double* d_green64 = nullptr;
    float* d_green32 = nullptr;

    // spectral work field: 3 x nh complex (double2 or float2)
    void* d_spec = nullptr;

    // dense real fields for full-grid entry points (3 x n), allocated lazily
    double* d_dense_in = nullptr;
    double* d_dense_out = nullptr;

    // compact vectors (3 * nb doubles)
    double* d_cin = nullptr;
    double* d_cout = nullptr;
    double* d_b = nullptr;
    double* d_x = nullptr;
    double* d_z = nullptr;
    double* d_r0 = nullptr;    // mixed mode: the refinement segment's FP64 residual
    double* d_corr = nullptr;  // mixed mode: the segment's start point
    double* d_v[3] = {nullptr, nullptr, nullptr};
    double* d_w[2] = {nullptr, nullptr};

    // reductions
    double* d_partials = nullptr;  // partial sums (kMaxPartials * 8)
    double* d_red = nullptr;       // small result slots
    MinresScalars* d_sc = nullptr;
    MinresScalars* h_sc = nullptr;  // pinned mirror
    double* d_hist = nullptr;       // residual history (maxit + 1)
    long long hist_cap = 0;

    // TMA-fed y and z passes: [precision 0 = FP64, 1 = FP32]
    TmaCache tma_y[2], tma_z[2];
    // specialised z pass: tensor maps of the spectral field and the Green
    // table [precision 0 = FP64, 1 = FP32], keyed by the table's address
    CUtensorMap fz_spec_map[2], fz_green_map[2];
    const void* fz_green_ptr[2] = {nullptr, nullptr};
    bool fz_valid[2] = {false, false};
    // MINRES iteration chunks replayed as CUDA graphs (FFTPERM_NO_GRAPHS=1: off).
    // Captured pointers and kernels depend on the geometry, the precision and
    // the tiling: every change of those releases the graphs.
    bool use_graphs = true;
    MinresGraph graphs[6];
    long long queued = 0;  // iterations queued since minres_start (buffer rotation)
    bool tma_off = false;      // FFTPERM_NO_TMA=1 selects the register-fed passes
    bool fast_off = false;     // FFTPERM_NO_FAST=1: the generic passes for every edge
    bool x_bulk = true;        // inverse x pass fed by bulk copies (tuned)
    int x_rows = 0;            // cap on grid rows per CTA of the x passes (0 = none; tuned)
    bool yz_lowreg = false;    // FP32 register-fed y/z passes capped at 168 registers (tuned)
    int* d_err = nullptr;      // device error flag (a bounded wait gave up)

    std::string err;
};

constexpr int kMaxPartials = 8192;
// d_red slot (in doubles) holding the block-count tickets of the fused MINRES
// vector kernels (two unsigned ints, zero between launches)
constexpr int kTicketSlot = 56;

// ---- setup kernels (kernels_setup.cu) ----
// Inputs of the Green-table kernel: per-axis tables of sinc(pi m / n) and
// q = 2 pi m / L for m = k + p n, p = -P-1 .. P (nw = 2P + 2 entries per k).
struct GreenArgs {
    int nx, ny, nz, nxh, nw, pr;
    long long rs;  // row stride of the table (>= nxh; padding entries are zero)
    double mu;
    const double* sx;  // [nx][nw]
    const double* qx;
    const double* sy;
    const double* qy;
    const double* sz;
    const double* qz;
    double* g64;
    float* g32;
    long long nh;
};
cudaError_t launch_green_kernel(const GreenArgs& a, cudaStream_t stream);
// Radix plan of one axis without twiddles (no allocation); false when n does
// not factor into 2, 3 and 5 or exceeds the supported maximum.
bool fill_plan_radices(int n, FftPlanDev& d);
cudaError_t launch_support(Problem& P);
// mask[i] = (ids[i] == fluid_id) for `count` material ids of 2 or 4 bytes
cudaError_t launch_ids_to_mask(const void* ids, int id_bytes, long long count, uint32_t fluid_id,
                               uint8_t* mask, cudaStream_t stream);
// The .fvel header (io.cu): "FVEL", version 1, dims, porosity, viscosity,
// driving gradient; false when it cannot be written.
bool write_fvel_header(void* file, int nx, int ny, int nz, double porosity, double viscosity,
                       const double driving[3]);
// Computes the Green table into g64 and/or g32 (either may be null).
cudaError_t launch_green(Problem& P, double* g64, float* g32);

// Tensor maps of the specialised z pass (kernels_fft.cu): the spectral field
// as [3][nz][ny][2*nxh] reals with boxes {2*tx, 1, nz, 1} and the Green table
// as [6][nz][ny][nxh] with boxes {tx, 1, nz, 1}.  false when TMA is
// unavailable or the layout does not qualify.
bool fast_maps(Problem& P, bool dbl, int tx, const CUtensorMap** spec, const CUtensorMap** green);

// ---- operator passes (kernels_fft.cu) ----
// Source of the forward x pass.
enum XSource {
    kSrcCompact = 0,   // scatter compact (3*nb AoS) minus mean
    kSrcDense = 1,     // dense SoA field (3 x n)
    kSrcF0 = 2,        // background force f0 only
    kSrcF0Compact = 3  // f0 plus scattered compact vector minus mean
};
// Destination of the inverse x pass.
enum XDest {
    kDstCompact = 0,  // gather to compact (raw, not mean-removed) + partial sums
    kDstDense = 1     // dense SoA field (3 x n) + partial sums over all voxels
};

// Which part of the pipeline launch_apply runs.
enum Stage {
    kStageFull = 0,     // forward x, y, z + Green + inverse z, y, x
    kStageForward = 1,  // forward x, y, z only: the half spectrum is left in d_spec
    kStageInverse = 2   // inverse z, y, x of the half spectrum in d_spec
};

struct ApplyArgs {
    const double* src = nullptr;     // compact or dense source
    const double* src_sum = nullptr; // device: component sums of the compact source (3), or null
    double f0_fluid[3] = {0, 0, 0};  // f0 coefficient on fluid voxels (per component)
    double f0_support[3] = {0, 0, 0};
    double* dst = nullptr;           // compact or dense destination
    const double* dot_with = nullptr;  // optional compact vector v: partial dot(v, dst)
    int src_kind = kSrcCompact;
    int dst_kind = kDstCompact;
    const int* skip = nullptr;       // device flag: when nonzero every pass returns at once
    int precision = -1;              // kFP64 / kMixed; -1 = the problem's default
    int stage = kStageFull;
};

// Runs the five passes (forward x, y, z + Green + inverse z, inverse y,
// inverse x).  Writes per-CTA partial sums of the destination into
// P.d_partials as [blocks][4] = {sum_x, sum_y, sum_z, dot}; returns the number
// of partial rows in *nparts.
cudaError_t launch_apply(Problem& P, const ApplyArgs& a, int* nparts);

// ---- groups of problems of one grid (kernels_minres.cu, group.cu) ----
// One member's pointers for one MINRES iteration of a group: the group
// kernels read tab[member] and run the same arithmetic as the single ones.
struct IterArgs {
    MinresScalars* sc;
    double* partials;  // the apply's partial rows in, the vector kernels' out
    int nparts;        // partial rows the apply wrote
    int nblk;          // vector-kernel blocks of this member
    double inv_nb;
    long long nb;
    double* z;
    const double* v;
    const double* v_old;
    double* v_new;
    double* w_prev;
    const double* w;
    double* x;
    unsigned int* tickets;  // [0] z update, [1] v/w update
    double* hist;
};
// Arguments of the next iteration of P (the buffer rotation at P.queued, which
// it advances) and the apply it starts with.
cudaError_t iteration_args(Problem& P, IterArgs* t, ApplyArgs* aa);
// alpha, z update (+ Givens step), v/w/x update (+ iteration end) of
// `members` problems, one launch each; max_blocks = the largest nblk.
cudaError_t group_iteration_tail(cudaStream_t s, const IterArgs* d_tab, int members, int max_blocks);

// Device tables of a group's lockstep iterations (group.cu).
struct GroupTables;
cudaError_t group_tables_create(GroupTables** out, int members, int iters);
void group_tables_destroy(GroupTables* t);
// true when P can be a group member (its applies run the specialised passes)
bool group_supported(Problem& P);
// `count` MINRES iterations of members m[0..members) in lockstep: per
// iteration five pass launches and three vector-kernel launches for all of
// them.  The members share grid, precision, tiling and stream (m[0]'s).
cudaError_t group_iterations(Problem* const* m, int members, int count, GroupTables* t);

// ---- vector kernels (kernels_minres.cu) ----
cudaError_t launch_sum3(Problem& P, const double* v, long long nb, double* out3);
// Reduce [nparts][4] partials into out4 (deterministic, one block).
cudaError_t launch_reduce4(Problem& P, int nparts, double* out4);
// r0_precision: operator precision of r0 = b - A x0 (-1: the problem's own)
cudaError_t minres_start(Problem& P, const double* b, const double* x0, double tol,
                         long long maxit, int r0_precision = -1);
cudaError_t minres_iteration(Problem& P);
cudaError_t minres_iterations(Problem& P, int count);
void release_graphs(Problem& P);
cudaError_t launch_sub_mean(Problem& P, double* v, const double* sums, double scale);
// out4[3] = |b - ax|^2
cudaError_t launch_resnorm(Problem& P, const double* b, const double* ax, double* out4);
// out = a x + b y over the 3 nb compact entries
cudaError_t launch_axpby(Problem& P, double* out, double a, const double* x, double b,
                         const double* y);
cudaError_t launch_gather_sum(Problem& P, const double* u_dense, double* out4);
cudaError_t launch_add_const3(Problem& P, double* u_dense, const double* add3);
cudaError_t launch_background_force(Problem& P, const double cf[3], const double cs[3],
                                    double* f0);

// ---- handles (capi.cu) ----
// fp_create's body: plans, stream and work buffers; the Green tables only when
// with_green.  On failure *out still holds the handle with its error message.
int create_handle(int nx, int ny, int nz, double voxel_size, double mu, int p_radius,
                  int precision, bool with_green, fp_handle* out);

}  // namespace fp

// The opaque handle of include/fftperm.h.
struct fp_problem {
    fp::Problem P;
};
