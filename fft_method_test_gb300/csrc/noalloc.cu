// noalloc.cu -- fp_green_apply_noalloc: the Green-operator apply on caller
// device buffers, with every piece of working memory in one file-scope
// __device__ array instead of cudaMalloc.
//
// Who needs it: code that may not allocate device memory itself.  Examples:
// a caller living inside another framework's memory manager, which owns the
// device heap and forbids raw cudaMalloc; or a latency-critical loop that
// cannot accept the implicit device-wide synchronisation cudaMalloc/cudaFree
// may incur.  Such a caller hands in device pointers for the input and output
// fields and gets the work queued on its own stream; nothing is allocated.
//
// Limits: N = nx*ny*nz <= kNoAllocMaxVoxels (262144, e.g. 64^3),
// rs*ny*nz <= kNoAllocMaxHalf (139264) with rs = nx/2+1 rounded up to even,
// ny*nz <= kNoAllocMaxRows (16384),
// every edge a product of 2, 3 and 5 and <= 640.  Larger grids are rejected
// with FP_ERR_INVALID; use fp_create / fp_green_apply for them.
//
// The scratch array is shared by every call in the process and keeps the last
// call's contents.  Nothing in it needs to start at zero: every call rewrites
// the twiddles, the alias tables, the Green table, the spectral field and the
// partial sums it reads.  Calls that overlap on the GPU (two streams, or two
// host threads) race on it; callers must serialise them.
//
// Set-up: the first call on a device, with that device current, resolves the
// array's device address with cudaGetSymbolAddress (host code cannot use the
// array's name as a device address).  That first call should come before any
// stream capture on the device.  The address is cached per device for the
// life of the process: a caller that resets a device (cudaDeviceReset) must
// not call this entry on that device afterwards, because the cached address
// belongs to the destroyed context.
//
// Cost: nothing is cached between calls, so every call recomputes the
// twiddles and the whole Green table, each point of which sums the full
// (2P+2)^3 alias window, before the transforms.  At 64^3 with P = 2 that is
// a few times the cost of the transforms themselves.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/fftperm.h"
#include "internal.h"

namespace fp {
namespace {

constexpr long long kNoAllocMaxVoxels = 262144;
constexpr long long kNoAllocMaxHalf = 139264;  // 34 * 64 * 64
constexpr long long kNoAllocMaxRows = 16384;
constexpr int kNoAllocMaxEdge = 640;
constexpr int kNoAllocMaxNw = 2 * 8 + 2;  // alias radius P <= 8

// byte offsets inside the scratch array (each 256-byte aligned)
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffSpec = 0;
constexpr size_t kOffGreen = align256(kOffSpec + sizeof(double2) * 3 * kNoAllocMaxHalf);
constexpr size_t kOffPart = align256(kOffGreen + sizeof(double) * 6 * kNoAllocMaxHalf);
constexpr size_t kOffTw64 = align256(kOffPart + sizeof(double) * 4 * (kNoAllocMaxRows + 64));
constexpr size_t kOffTw32 = align256(kOffTw64 + sizeof(double2) * 3 * kNoAllocMaxEdge);
constexpr size_t kOffTab = align256(kOffTw32 + sizeof(float2) * 3 * kNoAllocMaxEdge);
constexpr size_t kScratchBytes =
    align256(kOffTab + sizeof(double) * 6 * kNoAllocMaxEdge * kNoAllocMaxNw);

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
void* g_addr[64] = {nullptr};

// twiddles exp(-2 pi i j / n) of the three axes
__global__ void k_noalloc_twiddles(int nx, int ny, int nz, double2* tw64, float2* tw32) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int ns[3] = {nx, ny, nz};
    for (int a = 0; a < 3; ++a) {
        if (j < ns[a]) {
            double s, c;
            sincospi(2.0 * (double)j / (double)ns[a], &s, &c);
            tw64[a * kNoAllocMaxEdge + j] = make_double2(c, -s);
            tw32[a * kNoAllocMaxEdge + j] = make_float2((float)c, (float)-s);
        }
    }
}

// per-axis sinc(pi m / n) and q = 2 pi m / L, m = k + p n, p = -P-1 .. P
__global__ void k_noalloc_tables(int nx, int ny, int nz, double h, int pr, double* tab) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int nw = 2 * pr + 2;
    const int ns[3] = {nx, ny, nz};
    const double kPi = 3.14159265358979323846;
    for (int a = 0; a < 3; ++a) {
        if (k >= ns[a]) continue;
        const double L = h * (double)ns[a];
        double* s = tab + (size_t)(2 * a) * kNoAllocMaxEdge * kNoAllocMaxNw;
        double* q = tab + (size_t)(2 * a + 1) * kNoAllocMaxEdge * kNoAllocMaxNw;
        for (int i = 0; i < nw; ++i) {
            const long long m = (long long)k + (long long)(i - pr - 1) * ns[a];
            const double x = kPi * (double)m / (double)ns[a];
            s[(size_t)k * nw + i] = fabs(x) < 1e-12 ? 1.0 : sin(x) / x;
            q[(size_t)k * nw + i] = (2.0 * kPi * (double)m) / L;
        }
    }
}

int scratch_address(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return FP_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return FP_ERR_CUDA;
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return FP_OK;
}

}  // namespace
}  // namespace fp

extern "C" int fp_green_apply_noalloc(int nx, int ny, int nz, double voxel_size, double mu,
                                      int p_radius, const double* d_force_soa,
                                      double* d_velocity_soa, void* stream) {
    using namespace fp;
    if (nx <= 0 || ny <= 0 || nz <= 0 || !d_force_soa || !d_velocity_soa) return FP_ERR_INVALID;
    if (!(mu > 0.0) || !(voxel_size > 0.0)) return FP_ERR_INVALID;
    const long long n = (long long)nx * ny * nz;
    const long long nrows = (long long)ny * nz;
    const long long rs = ((long long)(nx / 2 + 1) + 1) & ~1LL;
    const long long nh = rs * nrows;
    const int pr = p_radius < 0 ? 0 : p_radius;
    if (n > kNoAllocMaxVoxels || nh > kNoAllocMaxHalf || nrows > kNoAllocMaxRows || nx > kNoAllocMaxEdge ||
        ny > kNoAllocMaxEdge || nz > kNoAllocMaxEdge || 2 * pr + 2 > kNoAllocMaxNw)
        return FP_ERR_INVALID;  // beyond the fixed scratch array: use fp_green_apply
    Problem P;
    if (!fill_plan_radices(nx, P.px.dev) || !fill_plan_radices(ny, P.py.dev) ||
        !fill_plan_radices(nz, P.pz.dev))
        return FP_ERR_UNSUPPORTED;
    void* base = nullptr;
    int rc = scratch_address(&base);
    if (rc != FP_OK) return rc;
    unsigned char* sb = static_cast<unsigned char*>(base);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&P.sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return FP_ERR_CUDA;

    double2* tw64 = reinterpret_cast<double2*>(sb + kOffTw64);
    float2* tw32 = reinterpret_cast<float2*>(sb + kOffTw32);
    double* tab = reinterpret_cast<double*>(sb + kOffTab);
    FftPlanDev* plans[3] = {&P.px.dev, &P.py.dev, &P.pz.dev};
    for (int a = 0; a < 3; ++a) {
        plans[a]->tw64 = tw64 + a * kNoAllocMaxEdge;
        plans[a]->tw32 = tw32 + a * kNoAllocMaxEdge;
    }
    const int maxe = nx > ny ? (nx > nz ? nx : nz) : (ny > nz ? ny : nz);
    FP_LAUNCHED(); k_noalloc_twiddles<<<(maxe + 127) / 128, 128, 0, s>>>(nx, ny, nz, tw64, tw32);
    FP_LAUNCHED(); k_noalloc_tables<<<(maxe + 127) / 128, 128, 0, s>>>(nx, ny, nz, voxel_size, pr, tab);

    P.nx = nx;
    P.ny = ny;
    P.nz = nz;
    P.n = n;
    P.nxh = nx / 2 + 1;
    P.nrows = nrows;
    P.rs = rs;
    P.nh = nh;
    P.h = voxel_size;
    P.mu = mu;
    P.p_radius = pr;
    P.precision = kFP64;
    P.tma_off = true;  // the register-fed passes: no descriptor or error flag to allocate
    P.stream = s;
    P.d_spec = sb + kOffSpec;
    P.d_green64 = reinterpret_cast<double*>(sb + kOffGreen);
    P.d_partials = reinterpret_cast<double*>(sb + kOffPart);

    GreenArgs g{};
    g.nx = nx;
    g.ny = ny;
    g.nz = nz;
    g.nxh = P.nxh;
    g.rs = rs;
    g.nw = 2 * pr + 2;
    g.pr = pr;
    g.mu = mu;
    const size_t plane = (size_t)kNoAllocMaxEdge * kNoAllocMaxNw;
    g.sx = tab;
    g.qx = tab + plane;
    g.sy = tab + 2 * plane;
    g.qy = tab + 3 * plane;
    g.sz = tab + 4 * plane;
    g.qz = tab + 5 * plane;
    g.g64 = P.d_green64;
    g.g32 = nullptr;
    g.nh = nh;
    if (launch_green_kernel(g, s) != cudaSuccess) return FP_ERR_CUDA;

    ApplyArgs a;
    a.src = d_force_soa;
    a.dst = d_velocity_soa;
    a.src_kind = kSrcDense;
    a.dst_kind = kDstDense;
    a.precision = kFP64;
    int nparts = 0;
    if (launch_apply(P, a, &nparts) != cudaSuccess) return FP_ERR_CUDA;
    return FP_OK;
}
