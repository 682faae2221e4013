// fft_fast.cuh -- the five apply passes specialised at compile time for the
// cubic grid edges 32, 48, 64, 80, 96, 128, 160 and 256, for compact-vector
// operator applies (scatter in, gather out).  The generic engine of
// fft_passes.cuh serves every other edge, source and destination.
//
// Each line of length N = R1 * R2 is transformed by TPL threads (TPL divides
// R1 and R2) with the four-step decomposition, one vector component per
// thread:
//
//   x[R2*i + a]  (i < R1, a < R2)
//   stage A  threads owning a: DFT-R1 over i, times W_N^(S a k) -> Y[k][a]
//   stage B  threads owning k: DFT-R2 over a                     -> X[k + R1*m]
//
// The inverse runs the same two stages with the radices swapped (R2 first).
// Only the Y exchange between the stages (and the natural-order exchange
// around the Green multiply) goes through shared memory; every stage reads
// or writes HBM directly where its owner pattern is the natural one.
//
// Passes (kernels below):
//   k_fx_fwd   scatter of the compact vector (minus its mean) into real
//              x-lines, two real lines per complex FFT, half spectrum out
//   k_fcol_y   y pass, one component per CTA slice, TX kx columns per CTA
//   k_fz       z pass: forward, 3x3 Green multiply, inverse, all three
//              components in one CTA; persistent CTAs with a two-stage TMA
//              pipeline (cp.async.bulk.tensor boxes of the spectral and Green
//              tiles of the next (kx, ky) tile load while the current one is
//              transformed)
//   k_fx_inv   C2R x lines, gather to the support, 1/N scale, per-CTA partial
//              sums (component sums and the dot with a given vector);
//              persistent CTAs, the next tile's half-spectrum rows arriving
//              by cp.async while the current tile is transformed
//
// Shared-memory line strides are chosen so that the half-warp (FP32) or
// quarter-warp (FP64) of every exchange touches distinct banks.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "common.cuh"
#include "fft_engine.cuh"
#include "internal.h"
#include "tma.cuh"

namespace fp {
namespace fast {

// N = R1 * R2 with R1 >= R2; TPL threads per line (TPL divides R1 and R2:
// R2 for the powers of two, 4 for the edges with a factor 3 or 5).
template <int N>
struct Split;
template <>
struct Split<32> {
    static constexpr int R1 = 8, R2 = 4, TPL = 4;
};
template <>
struct Split<48> {
    static constexpr int R1 = 12, R2 = 4, TPL = 4;
};
template <>
struct Split<64> {
    static constexpr int R1 = 8, R2 = 8, TPL = 8;
};
template <>
struct Split<80> {
    static constexpr int R1 = 20, R2 = 4, TPL = 4;
};
template <>
struct Split<96> {
    static constexpr int R1 = 12, R2 = 8, TPL = 4;
};
template <>
struct Split<128> {
    static constexpr int R1 = 16, R2 = 8, TPL = 8;
};
template <>
struct Split<160> {
    static constexpr int R1 = 20, R2 = 8, TPL = 4;
};
template <>
struct Split<256> {
    static constexpr int R1 = 16, R2 = 16, TPL = 16;
};

// ---- small DFTs in natural order -------------------------------------------

template <int P, int Q, int S, typename T2>
__device__ __forceinline__ void dft_pfa(T2 (&v)[P * Q]);

// Natural-order DFT of R values (S = -1 forward, +1 backward) with the
// radix kernels of fft_engine.cuh (2, 3, 4, 5, 8, 16); 12 = 4 x 3 and
// 20 = 4 x 5 by the prime-factor algorithm.
template <int R, int S, typename T2>
__device__ __forceinline__ void dft_nat(T2 (&v)[R]) {
    if constexpr (R == 12) {
        dft_pfa<4, 3, S>(v);
    } else if constexpr (R == 20) {
        dft_pfa<4, 5, S>(v);
    } else {
        T2 t[R];
#pragma unroll
        for (int i = 0; i < R; ++i) t[i] = v[i];
        dft_r<R, S>(t);
#pragma unroll
        for (int k = 0; k < R; ++k) v[k] = t[out_slot<R>(k)];
    }
}

// Prime-factor (Good-Thomas) DFT of R = P * Q values, P and Q coprime: input
// n = (Q n1 + P n2) mod R goes to a[n1][n2], length-Q DFTs along n2, then
// length-P DFTs along n1, and output k is a[k mod P][k mod Q].  No twiddles
// (Chinese-remainder index maps).
template <int P, int Q, int S, typename T2>
__device__ __forceinline__ void dft_pfa(T2 (&v)[P * Q]) {
    constexpr int R = P * Q;
    T2 a[P][Q];
#pragma unroll
    for (int n1 = 0; n1 < P; ++n1)
#pragma unroll
        for (int n2 = 0; n2 < Q; ++n2) a[n1][n2] = v[(Q * n1 + P * n2) % R];
#pragma unroll
    for (int n1 = 0; n1 < P; ++n1) dft_nat<Q, S>(a[n1]);
#pragma unroll
    for (int n2 = 0; n2 < Q; ++n2) {
        T2 c[P];
#pragma unroll
        for (int n1 = 0; n1 < P; ++n1) c[n1] = a[n1][n2];
        dft_nat<P, S>(c);
#pragma unroll
        for (int n1 = 0; n1 < P; ++n1) a[n1][n2] = c[n1];
    }
#pragma unroll
    for (int k = 0; k < R; ++k) v[k] = a[k % P][k % Q];
}

// twiddle W_N^(S e) from the table tw[j] = exp(-2 pi i j / N), 0 <= e < N
template <int S, typename T2>
__device__ __forceinline__ T2 twiddle(const T2* __restrict__ tw, int e) {
    T2 w = __ldg(tw + e);
    if (S > 0) w.y = -w.y;
    return w;
}

// ---- line strides ------------------------------------------------------------

// Positions used in a line: the natural N plus the Y layout k*(RB+1) + a of
// either direction (RB = R2 forward, R1 inverse).
template <int N>
__host__ __device__ constexpr int line_span() {
    return N + Split<N>::R1;
}

// Column passes (thread = column + TX * (owner + TPL * comp)): one
// shared-memory wavefront serves G = 128 / sizeof(complex) threads (a
// half-warp in FP32, a quarter-warp in FP64), TX columns x G / TX
// consecutive owners; every exchange steps owners by an odd number of
// elements, so a line stride of G / TX modulo G keeps them in distinct banks.
template <int N, typename T, int TX>
__host__ __device__ constexpr int col_ld() {
    constexpr int G = 128 / (2 * (int)sizeof(T));
    return ((line_span<N>() + G - 1) / G) * G + (G / TX) % G;
}

// x passes (thread = owner + TPL * line): the lines of one half-warp (FP32)
// or quarter-warp (FP64) must fall in distinct banks, so for a power-of-two
// TPL below the group size G the stride is TPL mod G.
template <int N, typename T>
__host__ __device__ constexpr int x_ld() {
    constexpr int G = sizeof(T) == 4 ? 16 : 8;
    constexpr int tpl = Split<N>::TPL;
    constexpr int base = ((line_span<N>() + G - 1) / G) * G;
    return tpl < G ? base + tpl : base;
}

// ---- barriers -------------------------------------------------------------------

// the whole CTA
struct CtaBarrier {
    __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
// the `count` threads (a multiple of 32) of one named barrier `id` (1..15)
struct GroupBarrier {
    int id, count;
    __device__ __forceinline__ void operator()() const {
        asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
    }
};

template <class B>
__device__ __forceinline__ B make_group_barrier(int id, int count);
template <>
__device__ __forceinline__ GroupBarrier make_group_barrier<GroupBarrier>(int id, int count) {
    return GroupBarrier{id, count};
}
template <>
__device__ __forceinline__ CtaBarrier make_group_barrier<CtaBarrier>(int, int) {
    return CtaBarrier{};
}

// ---- four-step stages --------------------------------------------------------

// Stage A for owners a = t + TPL*j (j < RB/TPL): loads RA values through
// load(pos) (pos = RB*i + a), DFT-RA, twiddle W_N^(S a k), stores Y[k][a] at
// line[k*(RB+1) + a].  With SYNC, bar() runs between the loads and the
// stores (the loads read the same lines).
template <int RA, int RB, int S, int TPL, bool SYNC, typename T2, class Load,
          class Bar = CtaBarrier>
__device__ __forceinline__ void stage_a(T2* line, int t, bool active, const T2* __restrict__ tw,
                                        Load& load, Bar bar = Bar{}) {
    static_assert(RB % TPL == 0, "owners per thread");
    constexpr int J = RB / TPL;
    T2 v[J][RA];
#pragma unroll
    for (int j = 0; j < J; ++j)
#pragma unroll
        for (int i = 0; i < RA; ++i) v[j][i] = active ? load(RB * i + t + TPL * j) : T2{};
    if (SYNC) bar();
    if (active) {
#pragma unroll
        for (int j = 0; j < J; ++j) {
            const int a = t + TPL * j;
            dft_nat<RA, S>(v[j]);
#pragma unroll
            for (int k = 0; k < RA; ++k) {
                T2 y = v[j][k];
                if (k > 0) y = cmul(y, twiddle<S>(tw, a * k));  // a * k < N
                line[k * (RB + 1) + a] = y;
            }
        }
    }
}

// Stage B for owners k = t + TPL*j (j < RA/TPL): loads Y[k][a] (a < RB),
// DFT-RB, hands X[k + RA*m] to store(pos, value).  With SYNC, bar() runs
// between the loads and the stores.
template <int RA, int RB, int S, int TPL, bool SYNC, typename T2, class Store,
          class Bar = CtaBarrier>
__device__ __forceinline__ void stage_b(const T2* line, int t, bool active, Store& store,
                                        Bar bar = Bar{}) {
    static_assert(RA % TPL == 0, "owners per thread");
    constexpr int J = RA / TPL;
    T2 u[J][RB];
#pragma unroll
    for (int j = 0; j < J; ++j)
#pragma unroll
        for (int a = 0; a < RB; ++a)
            u[j][a] = active ? line[(t + TPL * j) * (RB + 1) + a] : T2{};
    if (SYNC) bar();
    if (active) {
#pragma unroll
        for (int j = 0; j < J; ++j) {
            const int k = t + TPL * j;
            dft_nat<RB, S>(u[j]);
#pragma unroll
            for (int m = 0; m < RB; ++m) store(k + RA * m, u[j][m]);
        }
    }
}

// ---- kernel arguments ----------------------------------------------------------

struct FastArgs {
    int nx, ny, nz, nxh;
    long long rs, nh, nrows, n, plane;
    const float2* tw32x;
    const float2* tw32y;
    const float2* tw32z;
    const double2* tw64x;
    const double2* tw64y;
    const double2* tw64z;
    void* spec;
    const void* green;
    int* err;  // z pass: a bounded TMA wait gave up
    // x passes
    int rows;       // grid rows per tile (even)
    long long ntiles;
    const int* support;
    const int* row_ptr;
    const double* src;
    const double* src_sum;
    double inv_nb;
    double* dst;
    const double* dot_with;
    double scale;
    double* partials;
    const int* skip;
    // A group of problems of one grid in one launch per pass: when set, the
    // kernels (GROUP = true) take their member's arguments from group[p], p =
    // blockIdx.y (x and z passes) or blockIdx.z / 3 (y pass), and the z pass
    // its tensor maps from group_maps[2p] (spectral) and [2p + 1] (Green).
    const FastArgs* group;
    const CUtensorMap* group_maps;
    // members of a group whose z pass shares one Green table (group_maps[1]):
    // k_fz_shared loads each Green tile once for all of them (0 = not shared)
    int share;
};

template <typename T>
__device__ __forceinline__ const c_t<T>* tw_of(const FastArgs& a, int axis);
template <>
__device__ __forceinline__ const float2* tw_of<float>(const FastArgs& a, int axis) {
    return axis == 0 ? a.tw32x : (axis == 1 ? a.tw32y : a.tw32z);
}
template <>
__device__ __forceinline__ const double2* tw_of<double>(const FastArgs& a, int axis) {
    return axis == 0 ? a.tw64x : (axis == 1 ? a.tw64y : a.tw64z);
}

// threads of the x passes for `rows` grid rows per tile: 3*rows/2 complex
// lines of TPL threads, rounded up to whole warps
template <int N>
__host__ __device__ constexpr int x_threads(int rows) {
    return ((3 * rows / 2 * Split<N>::TPL + 31) / 32) * 32;
}

// ---- cp.async (global -> shared, completion by group) ---------------------------

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                     static_cast<uint32_t>(__cvta_generic_to_shared(smem))),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(PENDING) : "memory");
}

// ---- P1: scatter + R2C x -------------------------------------------------------

// complex lines per tile of the x passes at most (3 * rows / 2, rows <= 32)
constexpr int kMaxXLines = 48;

// two neighbouring complex values to 16-byte aligned global memory
__device__ __forceinline__ void store_pair(float2* p, float2 a, float2 b) {
    *reinterpret_cast<float4*>(p) = make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ void store_pair(double2* p, double2 a, double2 b) {
    p[0] = a;
    p[1] = b;
}

template <typename T, int N, bool GROUP>
__global__ void __launch_bounds__(384) k_fx_fwd(const __grid_constant__ FastArgs a0) {
    // a group member's arguments are copied out of the table once: read
    // through a reference they would be reloaded after every global store
    const FastArgs ag = GROUP ? a0.group[blockIdx.y] : FastArgs{};
    const FastArgs& a = GROUP ? ag : a0;
    if (a.skip && *a.skip) return;
    using T2 = c_t<T>;
    constexpr int R1 = Split<N>::R1, R2 = Split<N>::R2, TPL = Split<N>::TPL;
    constexpr int LD = x_ld<N, T>();
    constexpr int NH = N / 2 + 1;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ long long dst_a[kMaxXLines], dst_b[kMaxXLines];
    T2* lines = reinterpret_cast<T2*>(smem_raw);
    const int RB = a.rows;
    const int nq = 3 * RB / 2;
    const int tid = threadIdx.x;
    const int nthr = blockDim.x;
    const int q = tid / TPL;
    const int t = tid - q * TPL;
    const T2* tw = tw_of<T>(a, 0);
    T2* spec = reinterpret_cast<T2*>(a.spec);
    const T mean[3] = {a.src_sum ? (T)(a.src_sum[0] * a.inv_nb) : (T)0,
                       a.src_sum ? (T)(a.src_sum[1] * a.inv_nb) : (T)0,
                       a.src_sum ? (T)(a.src_sum[2] * a.inv_nb) : (T)0};
    for (long long tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
        const long long r0 = tile * RB;
        const int rows = (int)min((long long)RB, a.nrows - r0);
        const int nreal = 3 * rows;
        const int nqa = (nreal + 1) / 2;
        // 1) zero the lines
        for (int i = tid; i < nq * LD; i += nthr) lines[i] = T2{};
        __syncthreads();
        // 2) scatter the compact vector minus its mean (support voxels only)
        {
            const int s0 = a.row_ptr[r0];
            const int s1 = a.row_ptr[r0 + rows];
            for (int s = s0 + tid; s < s1; s += nthr) {
                const int idx = a.support[s];
                const int row = idx / N;
                const int x = idx - row * N;
                const int rl = row - (int)r0;
                const double c0 = a.src[3LL * s], c1 = a.src[3LL * s + 1], c2 = a.src[3LL * s + 2];
                const T v3[3] = {(T)c0 - mean[0], (T)c1 - mean[1], (T)c2 - mean[2]};
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const int L = 3 * rl + c;
                    T2* p = &lines[(L >> 1) * LD + x];
                    if (L & 1) p->y = v3[c]; else p->x = v3[c];
                }
            }
        }
        __syncthreads();
        // 3) forward FFT of every complex line (stage A reads the natural line,
        //    stage B leaves X in registers, written back in natural order)
        const bool act = q < nqa;
        T2* my = lines + (act ? q : 0) * LD;
        {
            auto ld_nat = [&](int pos) { return my[pos]; };
            stage_a<R1, R2, -1, TPL, true>(my, t, act, tw, ld_nat);
            __syncthreads();
            auto st_nat = [&](int pos, T2 v) { my[pos] = v; };
            stage_b<R1, R2, -1, TPL, true>(my, t, act, st_nat);
        }
        __syncthreads();
        // 4) separate the two real spectra of each complex line, store the half
        //    spectra, two neighbouring kx per thread (one 16-byte store for
        //    FP32; rs is a multiple of 4, so every even kx is 16-byte aligned;
        //    kx = N/2 + 1 lands in the row padding)
        if (tid < nqa) {
            const int La = 2 * tid, rla = La / 3, ca = La - 3 * rla;
            dst_a[tid] = ca * a.nh + (r0 + rla) * a.rs;
            const int Lb = La + 1, rlb = Lb / 3, cb = Lb - 3 * rlb;
            dst_b[tid] = Lb < nreal ? cb * a.nh + (r0 + rlb) * a.rs : -1;
        }
        __syncthreads();
        constexpr int NP = (NH + 1) / 2;
        for (int it = tid; it < nqa * NP; it += nthr) {
            const int qq = it / NP;
            const int k = 2 * (it - qq * NP);
            const T2* ln = lines + qq * LD;
            T2 A[2], B[2];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int kk = k + e;
                const T2 zk = ln[kk];
                const T2 zn = ln[kk == 0 ? 0 : N - kk];
                const T h = (T)0.5;
                A[e] = cmk<T2>(h * (zk.x + zn.x), h * (zk.y - zn.y));
                B[e] = cmk<T2>(h * (zk.y + zn.y), h * (zn.x - zk.x));
            }
            store_pair(spec + dst_a[qq] + k, A[0], A[1]);
            if (dst_b[qq] >= 0) store_pair(spec + dst_b[qq] + k, B[0], B[1]);
        }
        __syncthreads();
    }
}

// ---- P5: C2R x + gather + partial sums -------------------------------------------

// Persistent CTAs walk tiles of `rows` grid rows.  The three component blocks
// of a tile are contiguous rows of the half spectrum; cp.async brings the next
// tile's rows into the other of two shared-memory stages while the current
// tile is transformed.  Stage A of the inverse transform builds the complex
// lines Z = A + iB of two real lines straight from the raw Hermitian half
// spectra ([comp][row][rs], as copied); after a barrier the padded lines
// overwrite the same stage.  stage_bytes covers the larger of the two layouts.
template <typename T, int N, bool GROUP>
__global__ void __launch_bounds__(384) k_fx_inv(const __grid_constant__ FastArgs a0, int stage_bytes) {
    const FastArgs ag = GROUP ? a0.group[blockIdx.y] : FastArgs{};
    const FastArgs& a = GROUP ? ag : a0;
    if (a.skip && *a.skip) return;
    using T2 = c_t<T>;
    constexpr int R1 = Split<N>::R1, R2 = Split<N>::R2, TPL = Split<N>::TPL;
    constexpr int LD = x_ld<N, T>();
    constexpr int NH = N / 2 + 1;
    constexpr int SPC = 16 / sizeof(T2);  // elements per 16-byte copy
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ double red[4 * 32];
    const int RB = a.rows;
    const int tid = threadIdx.x;
    const int nthr = blockDim.x;
    const int q = tid / TPL;
    const int t = tid - q * TPL;
    const T2* tw = tw_of<T>(a, 0);
    const T2* spec = reinterpret_cast<const T2*>(a.spec);
    const T scale = (T)a.scale;
    const long long rs = a.rs;
    T acc[4] = {(T)0, (T)0, (T)0, (T)0};

    auto issue = [&](long long tile, int st) {
        T2* raw = reinterpret_cast<T2*>(smem_raw + st * (size_t)stage_bytes);
        const long long r0 = tile * RB;
        const int rows = (int)min((long long)RB, a.nrows - r0);
        const int per_comp = (int)(rows * rs / SPC);  // rs is a multiple of 4: whole copies
        for (int i = tid; i < 3 * per_comp; i += nthr) {
            const int cc = i / per_comp;
            const int j = i - cc * per_comp;
            cp_async16(raw + (size_t)cc * RB * rs + (size_t)j * SPC,
                       spec + cc * a.nh + r0 * rs + (long long)j * SPC);
        }
        cp_async_commit();
    };

    long long tile = blockIdx.x;
    if (tile < a.ntiles) issue(tile, 0);
    for (int it = 0; tile < a.ntiles; tile += gridDim.x, ++it) {
        const int st = it & 1;
        const long long next = tile + gridDim.x;
        if (next < a.ntiles) {
            issue(next, st ^ 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const T2* raw = reinterpret_cast<const T2*>(smem_raw + st * (size_t)stage_bytes);
        T2* lines = reinterpret_cast<T2*>(smem_raw + st * (size_t)stage_bytes);
        const long long r0 = tile * RB;
        const int rows = (int)min((long long)RB, a.nrows - r0);
        const int nreal = 3 * rows;
        const int nqa = (nreal + 1) / 2;
        const bool act = q < nqa;
        T2* my = lines + (act ? q : 0) * LD;
        {
            // complex line q carries real lines 2q (A) and 2q + 1 (B)
            const int La = 2 * q, rla = La / 3, ca = La - 3 * rla;
            const int Lb = La + 1, rlb = Lb / 3, cb = Lb - 3 * rlb;
            const T2* ra = raw + ((size_t)ca * RB + rla) * rs;
            const T2* rb = raw + ((size_t)cb * RB + rlb) * rs;
            const bool hasb = Lb < nreal;
            auto ld_herm = [&](int k) {
                const bool lo = k < NH;
                const int kk = lo ? k : N - k;
                T2 A = ra[kk];
                T2 B = hasb ? rb[kk] : T2{};
                if (kk == 0 || 2 * kk == N) {  // DC and Nyquist are real
                    A.y = (T)0;
                    B.y = (T)0;
                }
                if (!lo) {  // Z[k] = conj(A[N-k]) + i conj(B[N-k])
                    A.y = -A.y;
                    B.y = -B.y;
                }
                return cmk<T2>(A.x - B.y, A.y + B.x);
            };
            stage_a<R2, R1, +1, TPL, true>(my, t, act, tw, ld_herm);
        }
        __syncthreads();
        {
            auto st_nat = [&](int pos, T2 v) { my[pos] = v; };
            stage_b<R2, R1, +1, TPL, true>(my, t, act, st_nat);
        }
        __syncthreads();
        // gather to the support with the 1/N scale, partial sums
        {
            const int s0 = a.row_ptr[r0];
            const int s1 = a.row_ptr[r0 + rows];
            for (int s = s0 + tid; s < s1; s += nthr) {
                const int idx = a.support[s];
                const int row = idx / N;
                const int x = idx - row * N;
                const int rl = row - (int)r0;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const int L = 3 * rl + c;
                    const T2 zv = lines[(L >> 1) * LD + x];
                    const T val = ((L & 1) ? zv.y : zv.x) * scale;
                    a.dst[3LL * s + c] = (double)val;
                    acc[c] += val;
                    if (a.dot_with) acc[3] += (T)a.dot_with[3LL * s + c] * val;
                }
            }
        }
        __syncthreads();  // this stage is refilled by the issue of iteration it + 1
    }
    double accd[4] = {(double)acc[0], (double)acc[1], (double)acc[2], (double)acc[3]};
    double out[4];
    block_sum<4>(accd, red, out);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < 4; ++i) a.partials[4LL * blockIdx.x + i] = out[i];
    }
}

// ---- P2 / P4: y pass -------------------------------------------------------------

// One CTA: TX kx columns of one z plane for one component (blockIdx.z, or
// blockIdx.z mod 3 of member blockIdx.z / 3 in a group).
template <typename T, int N, int S, int TX, bool GROUP>
__global__ void __launch_bounds__(TX * Split<N>::TPL) k_fcol_y(const __grid_constant__ FastArgs a0) {
    const FastArgs ag = GROUP ? a0.group[blockIdx.z / 3] : FastArgs{};
    const FastArgs& a = GROUP ? ag : a0;
    const int comp = GROUP ? (int)(blockIdx.z % 3) : (int)blockIdx.z;
    if (a.skip && *a.skip) return;
    using T2 = c_t<T>;
    constexpr int R1 = Split<N>::R1, R2 = Split<N>::R2, TPL = Split<N>::TPL;
    constexpr int LD = col_ld<N, T, TX>();
    __shared__ __align__(16) T2 lines[TX * LD];
    const int c = threadIdx.x % TX;
    const int t = threadIdx.x / TX;
    const int k0 = blockIdx.x * TX;
    const bool act = k0 + c < a.nxh;
    const T2* tw = tw_of<T>(a, 1);
    T2* base = reinterpret_cast<T2*>(a.spec) + comp * a.nh + (long long)blockIdx.y * N * a.rs +
               k0 + (act ? c : 0);
    const long long es = a.rs;
    T2* my = lines + c * LD;
    auto ld_g = [&](int pos) { return base[pos * es]; };
    auto st_g = [&](int pos, T2 v) { base[pos * es] = v; };
    if (S < 0) {
        stage_a<R1, R2, -1, TPL, false>(my, t, act, tw, ld_g);
        __syncthreads();
        stage_b<R1, R2, -1, TPL, false>(my, t, act, st_g);
    } else {
        stage_a<R2, R1, +1, TPL, false>(my, t, act, tw, ld_g);
        __syncthreads();
        stage_b<R2, R1, +1, TPL, false>(my, t, act, st_g);
    }
}

// ---- P3: z forward + Green + z inverse -------------------------------------------

// Component stride (elements) of the spectral tile in shared memory: the
// padded lines of one component, rounded up so that each component block
// starts 128-byte aligned (a TMA destination) and the blocks never overlap.
template <typename T, int N, int TX>
__host__ __device__ constexpr int comp_stride() {
    return (int)(((size_t)TX * col_ld<N, T, TX>() * 2 * sizeof(T) + 127) / 128 * 128 /
                 (2 * sizeof(T)));
}

// Shared memory of one pipeline stage of the z pass: the spectral tile (per
// component first raw [kz][TX] as the TMA box lands, then the padded lines
// [TX][LD] in the same block) and the Green tile [6][kz][TX].
template <typename T, int N, int TX>
__host__ __device__ constexpr size_t z_green_offset() {
    return (size_t)3 * comp_stride<T, N, TX>() * 2 * sizeof(T);
}
template <typename T, int N, int TX>
__host__ __device__ constexpr size_t z_stage_bytes() {
    return (z_green_offset<T, N, TX>() + (size_t)6 * N * TX * sizeof(T) + 127) & ~size_t(127);
}

// Persistent CTAs walk the (kx tile, ky) tiles; thread = column + TX *
// (owner + TPL * comp).  One thread has the TMA engine bring the spectral
// tile (three boxes of {2 TX reals, 1, nz}) and the Green tile (six boxes of
// {TX, 1, nz}) into a stage, completing on that stage's mbarrier; boxes past
// the last kx column read zeros.  With two stages the tiles of iteration
// i + 1 load while tile i is transformed (one CTA per SM); with one stage the
// next tile loads after the current one is done, and three CTAs per SM (at
// most 112 registers per thread) overlap one another instead.  The phases
// that touch one component only synchronise that component's threads (named
// barrier 1 + comp); the Green multiply reads all three.  Waits are bounded:
// on a timeout the CTA raises a.err and returns.
template <typename T, int N, int TX, int STAGES, bool GROUP>
__global__ void __launch_bounds__(3 * TX * Split<N>::TPL, STAGES == 1 ? 3 : 1)
    k_fz(const __grid_constant__ CUtensorMap spec_map, const __grid_constant__ CUtensorMap green_map,
         const __grid_constant__ FastArgs a0) {
    // (the few fields read per tile are read through the table: a copy would
    // hold them in registers across the kernel)
    const FastArgs& a = GROUP ? a0.group[blockIdx.y] : a0;
    const CUtensorMap* smap = GROUP ? &a0.group_maps[2 * blockIdx.y] : &spec_map;
    const CUtensorMap* gmap = GROUP ? &a0.group_maps[2 * blockIdx.y + 1] : &green_map;
    if (a.skip && *a.skip) return;
    using T2 = c_t<T>;
    constexpr int R1 = Split<N>::R1, R2 = Split<N>::R2, TPL = Split<N>::TPL;
    constexpr int LD = col_ld<N, T, TX>();
    constexpr int CS = comp_stride<T, N, TX>();
    constexpr size_t STAGE = z_stage_bytes<T, N, TX>();
    constexpr size_t GOFF = z_green_offset<T, N, TX>();
    constexpr uint32_t TILE_BYTES = (uint32_t)(3 * N * TX * sizeof(T2) + 6 * N * TX * sizeof(T));
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);
    unsigned char* stage0 = smem_raw + 128;
    const int c = threadIdx.x % TX;
    const int t = (threadIdx.x / TX) % TPL;
    const int comp = threadIdx.x / (TX * TPL);
    // a named barrier per component needs whole warps per component
    using GBar = typename std::conditional<(TX * TPL) % 32 == 0, GroupBarrier, CtaBarrier>::type;
    GBar gbar = make_group_barrier<GBar>(1 + comp, TX * TPL);
    const int ntx = (a.nxh + TX - 1) / TX;
    const long long ntiles = (long long)ntx * a.ny;
    const T2* tw = tw_of<T>(a, 2);
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
        if (GROUP) {
            fence_tensormap_acquire(smap);
            fence_tensormap_acquire(gmap);
        }
    }
    __syncthreads();

    auto issue = [&](long long tile, int st) {
        unsigned char* base = stage0 + st * STAGE;
        const int k0 = (int)(tile % ntx) * TX;
        const int ky = (int)(tile / ntx);
        mbar_arrive_expect_tx(&bars[st], TILE_BYTES);
        for (int cc = 0; cc < 3; ++cc)
            tma_load_4d(base + (size_t)cc * CS * sizeof(T2), smap, 2 * k0, ky, 0, cc, &bars[st]);
        for (int gc = 0; gc < 6; ++gc)
            tma_load_4d(base + GOFF + (size_t)gc * N * TX * sizeof(T), gmap, k0, ky, 0, gc, &bars[st]);
    };

    long long tile = blockIdx.x;
    if (threadIdx.x == 0 && tile < ntiles) issue(tile, 0);
    for (int i = 0; tile < ntiles; tile += gridDim.x, ++i) {
        const int st = STAGES == 2 ? (i & 1) : 0;
        const long long next = tile + gridDim.x;
        if (STAGES == 2) {
            if (threadIdx.x == 0 && next < ntiles) {
                fence_proxy_async_smem();
                issue(next, st ^ 1);
            }
            if (!tma_pipeline_wait<T2>(bars, i, st, next < ntiles, a.err)) return;
        } else {
            const bool ok = mbar_wait_bounded(&bars[0], (uint32_t)(i & 1));
            if (__syncthreads_or(!ok)) {
                if (threadIdx.x == 0) atomicExch(a.err, 1);
                return;
            }
        }
        T2* blk = reinterpret_cast<T2*>(stage0 + st * STAGE);
        const T* gsm = reinterpret_cast<const T*>(stage0 + st * STAGE + GOFF);
        const int k0 = (int)(tile % ntx) * TX;
        const long long ky = tile / ntx;
        const bool act = k0 + c < a.nxh;
        T2* my = blk + comp * CS + c * LD;  // padded line in this component's block
        // forward stage A from the raw box; Y into the lines after the group barrier
        {
            const T2* rc = blk + comp * CS + c;
            auto ld_raw = [&](int pos) { return rc[pos * TX]; };
            stage_a<R1, R2, -1, TPL, true>(my, t, act, tw, ld_raw, gbar);
        }
        gbar();
        {
            auto st_nat = [&](int pos, T2 v) { my[pos] = v; };
            stage_b<R1, R2, -1, TPL, true>(my, t, act, st_nat, gbar);
        }
        __syncthreads();
        // Green multiply while loading the inverse stage A (owner k1 = same owner)
        {
            const T2* lx = blk + 0 * CS + c * LD;
            const T2* ly = blk + 1 * CS + c * LD;
            const T2* lz = blk + 2 * CS + c * LD;
            // row `comp` of the symmetric tensor (xx xy xz yy yz zz)
            const int g0 = comp == 0 ? 0 : (comp == 1 ? 1 : 2);
            const int g1 = comp == 0 ? 1 : (comp == 1 ? 3 : 4);
            const int g2 = comp == 0 ? 2 : (comp == 1 ? 4 : 5);
            auto ld_green = [&](int pos) {
                const T2 X = lx[pos], Y = ly[pos], Z = lz[pos];
                const T a0 = gsm[((size_t)g0 * N + pos) * TX + c];
                const T a1 = gsm[((size_t)g1 * N + pos) * TX + c];
                const T a2 = gsm[((size_t)g2 * N + pos) * TX + c];
                return cmk<T2>(a0 * X.x + a1 * Y.x + a2 * Z.x, a0 * X.y + a1 * Y.y + a2 * Z.y);
            };
            stage_a<R2, R1, +1, TPL, true>(my, t, act, tw, ld_green);  // CTA barrier
        }
        gbar();
        {
            T2* base = reinterpret_cast<T2*>(a.spec) + comp * a.nh + ky * a.rs + k0 + (act ? c : 0);
            const long long es = a.plane;
            auto st_g = [&](int pos, T2 v) { base[pos * es] = v; };
            stage_b<R2, R1, +1, TPL, false>(my, t, act, st_g);
        }
        __syncthreads();  // this stage is refilled by the next issue
        if (STAGES == 1 && threadIdx.x == 0 && next < ntiles) {
            fence_proxy_async_smem();
            issue(next, 0);
        }
    }
}

// The z pass of a group whose members share one Green table (the three load
// cases of one cell, or cells of one grid and Green parameters): each CTA
// walks its (kx, ky) tiles and, per tile, the members one after another as
// pipeline items (tile, member).  The spectral boxes of item i + 1 load into
// the other stage while item i is transformed, as in k_fz; the Green tile is
// loaded once per tile, with the tile's first item, into one of two Green
// buffers (tile parity) and serves all members.  Per tile the HBM reads are
// G spectral tiles and one Green tile instead of G of each (the byte model
// of a G-field block apply).  A member whose solve is done is transformed
// all the same (its spectrum is scratch that the next fresh apply rewrites).
// Waits are bounded: on a timeout member 0's error flag is raised.
template <typename T, int N, int TX>
__global__ void __launch_bounds__(3 * TX * Split<N>::TPL, sizeof(T) == 4 ? 2 : 1)
    k_fz_shared(const __grid_constant__ FastArgs a0) {
    using T2 = c_t<T>;
    constexpr int R1 = Split<N>::R1, R2 = Split<N>::R2, TPL = Split<N>::TPL;
    constexpr int LD = col_ld<N, T, TX>();
    constexpr int CS = comp_stride<T, N, TX>();
    constexpr size_t SPEC = z_green_offset<T, N, TX>();  // one spectral stage (128-byte multiple)
    constexpr size_t GREEN = ((size_t)6 * N * TX * sizeof(T) + 127) & ~size_t(127);
    constexpr uint32_t SPEC_BYTES = (uint32_t)(3 * N * TX * sizeof(T2));
    constexpr uint32_t GREEN_BYTES = (uint32_t)(6 * N * TX * sizeof(T));
    static_assert(128 + 2 * SPEC + 2 * GREEN <= 128 + 2 * z_stage_bytes<T, N, TX>(), "shared memory");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);
    unsigned char* spec0 = smem_raw + 128;
    unsigned char* green0 = spec0 + 2 * SPEC;
    const int G = a0.share;
    int* err = a0.group[0].err;
    const int c = threadIdx.x % TX;
    const int t = (threadIdx.x / TX) % TPL;
    const int comp = threadIdx.x / (TX * TPL);
    using GBar = typename std::conditional<(TX * TPL) % 32 == 0, GroupBarrier, CtaBarrier>::type;
    GBar gbar = make_group_barrier<GBar>(1 + comp, TX * TPL);
    const int ntx = (a0.nxh + TX - 1) / TX;
    const long long ntiles = (long long)ntx * a0.ny;
    const T2* tw = tw_of<T>(a0, 2);
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
        fence_tensormap_acquire(&a0.group_maps[1]);
        for (int m = 0; m < G; ++m) fence_tensormap_acquire(&a0.group_maps[2 * m]);
    }
    __syncthreads();
    const long long my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int nitems = (int)(my_tiles * G);

    auto issue = [&](int i) {
        const int st = i & 1;
        const int m = i % G;
        const long long tile = blockIdx.x + (long long)(i / G) * gridDim.x;
        const int k0 = (int)(tile % ntx) * TX;
        const int ky = (int)(tile / ntx);
        unsigned char* sb = spec0 + st * SPEC;
        mbar_arrive_expect_tx(&bars[st], SPEC_BYTES + (m == 0 ? GREEN_BYTES : 0u));
        for (int cc = 0; cc < 3; ++cc)
            tma_load_4d(sb + (size_t)cc * CS * sizeof(T2), &a0.group_maps[2 * m], 2 * k0, ky, 0, cc,
                        &bars[st]);
        if (m == 0) {
            unsigned char* gb = green0 + ((i / G) & 1) * GREEN;
            for (int gc = 0; gc < 6; ++gc)
                tma_load_4d(gb + (size_t)gc * N * TX * sizeof(T), &a0.group_maps[1], k0, ky, 0, gc,
                            &bars[st]);
        }
    };

    if (threadIdx.x == 0 && nitems > 0) issue(0);
    for (int i = 0; i < nitems; ++i) {
        const int st = i & 1;
        if (threadIdx.x == 0 && i + 1 < nitems) {
            fence_proxy_async_smem();
            issue(i + 1);
        }
        if (!tma_pipeline_wait<T2>(bars, i, st, i + 1 < nitems, err)) return;
        const int m = i % G;
        const long long tile = blockIdx.x + (long long)(i / G) * gridDim.x;
        T2* blk = reinterpret_cast<T2*>(spec0 + st * SPEC);
        const T* gsm = reinterpret_cast<const T*>(green0 + ((i / G) & 1) * GREEN);
        const int k0 = (int)(tile % ntx) * TX;
        const long long ky = tile / ntx;
        const bool act = k0 + c < a0.nxh;
        T2* my = blk + comp * CS + c * LD;
        {
            const T2* rc = blk + comp * CS + c;
            auto ld_raw = [&](int pos) { return rc[pos * TX]; };
            stage_a<R1, R2, -1, TPL, true>(my, t, act, tw, ld_raw, gbar);
        }
        gbar();
        {
            auto st_nat = [&](int pos, T2 v) { my[pos] = v; };
            stage_b<R1, R2, -1, TPL, true>(my, t, act, st_nat, gbar);
        }
        __syncthreads();
        {
            const T2* lx = blk + 0 * CS + c * LD;
            const T2* ly = blk + 1 * CS + c * LD;
            const T2* lz = blk + 2 * CS + c * LD;
            const int g0 = comp == 0 ? 0 : (comp == 1 ? 1 : 2);
            const int g1 = comp == 0 ? 1 : (comp == 1 ? 3 : 4);
            const int g2 = comp == 0 ? 2 : (comp == 1 ? 4 : 5);
            auto ld_green = [&](int pos) {
                const T2 X = lx[pos], Y = ly[pos], Z = lz[pos];
                const T a0g = gsm[((size_t)g0 * N + pos) * TX + c];
                const T a1g = gsm[((size_t)g1 * N + pos) * TX + c];
                const T a2g = gsm[((size_t)g2 * N + pos) * TX + c];
                return cmk<T2>(a0g * X.x + a1g * Y.x + a2g * Z.x, a0g * X.y + a1g * Y.y + a2g * Z.y);
            };
            stage_a<R2, R1, +1, TPL, true>(my, t, act, tw, ld_green);  // CTA barrier
        }
        gbar();
        {
            T2* base = reinterpret_cast<T2*>(a0.group[m].spec) + comp * a0.nh + ky * a0.rs + k0 +
                       (act ? c : 0);
            const long long es = a0.plane;
            auto st_g = [&](int pos, T2 v) { base[pos * es] = v; };
            stage_b<R2, R1, +1, TPL, false>(my, t, act, st_g);
        }
        __syncthreads();  // this stage and, after the tile's last member, this Green buffer are refilled
    }
}


}  // namespace fast

// Runs the five passes with the specialised kernels when the grid, the
// precision and the source/destination allow it; returns false (nothing
// launched) otherwise.  Defined in fast_dispatch.cu.
bool fast_apply_supported(const Problem& P, int precision, int src_kind, int dst_kind, int stage);
cudaError_t fast_apply(Problem& P, int precision, const ApplyArgs& aa, int* nparts);

// Group applies (one launch per pass for several problems of one grid and
// tiling).  fast_member_args fills one member's kernel arguments, its two
// tensor maps (spectral, Green) and the launch geometry the members of a
// group must share (kGroupGeometry values); fast_apply_group launches the five
// passes over `members` members whose arguments and maps the caller copied to
// device memory (d_args[members], d_maps[2 * members], 64-byte aligned).
// shared_green: every member's Green map is member 0's (k_fz_shared).
constexpr int kGroupGeometry = 12;
cudaError_t fast_member_args(Problem& P, int precision, const ApplyArgs& aa, fast::FastArgs* args,
                             CUtensorMap* maps, long long* geometry);
cudaError_t fast_apply_group(Problem& P0, int precision, int members, const fast::FastArgs* d_args,
                             const CUtensorMap* d_maps, bool shared_green, int* nparts);

}  // namespace fp

// ---- launch runners (fast32.cu / fast64.cu) -------------------------------------

namespace fp {
namespace fast {

// kx columns per CTA of the y pass (64-byte row segments) and per tile of the
// z pass (32-byte spectral rows, 16-byte FP32 Green rows: two CTAs per SM)
template <typename T>
constexpr int col_tx() {
    return sizeof(T) == 4 ? 8 : 4;
}
template <typename T>
constexpr int z_tx() {
    return 4;
}

// grid edges with specialised kernels
#define FP_FAST_EDGES(CALL) CALL(32) CALL(48) CALL(64) CALL(80) CALL(96) CALL(128) CALL(160) CALL(256)

inline bool edge_supported(int n) {
#define FP_CASE(N) if (n == N) return true;
    FP_FAST_EDGES(FP_CASE)
#undef FP_CASE
    return false;
}

// grid rows per tile of the x passes: about 192 threads per CTA, 96 where
// the lines are long and served by 4 threads (shared memory)
inline int x_rows_for(int n) {
    switch (n) {
        case 32: return 32;
        case 48: return 32;
        case 64: return 16;
        case 80: return 32;
        case 96: return 16;
        case 128: return 16;
        case 160: return 16;
        default: return 8;
    }
}
inline int x_tpl(int n) {
#define FP_CASE(N) if (n == N) return Split<N>::TPL;
    FP_FAST_EDGES(FP_CASE)
#undef FP_CASE
    return 0;
}
template <typename T>
int x_ld_rt(int n) {
#define FP_CASE(N) if (n == N) return x_ld<N, T>();
    FP_FAST_EDGES(FP_CASE)
#undef FP_CASE
    return 0;
}

// dynamic shared memory of the z pass: mbarriers + its pipeline stages
template <typename T>
size_t z_smem_rt(int n, int stages) {
    constexpr int TX = z_tx<T>();
#define FP_CASE(N) if (n == N) return 128 + stages * z_stage_bytes<T, N, TX>();
    FP_FAST_EDGES(FP_CASE)
#undef FP_CASE
    return 0;
}

// Launch runners of one edge, defined in fast_runners.cuh and instantiated
// per precision and edge group (fast32.cu, fast64.cu: powers of two;
// fast32n.cu, fast64n.cu: 48, 80, 96, 160) so that they build in parallel.
// A set a.group selects the group kernels; the grid then carries the member
// index (grid.y for the x and z passes, grid.z = 3 x members for the y pass).
template <typename T, int N>
struct Passes {
    static cudaError_t xfwd(const FastArgs& a, dim3 grid, int threads, size_t smem, cudaStream_t s);
    static cudaError_t xinv(const FastArgs& a, int stage_bytes, dim3 grid, int threads, size_t smem,
                            cudaStream_t s);
    static cudaError_t y(int dir, const FastArgs& a, dim3 grid, cudaStream_t s);
    static cudaError_t z(int stages, const CUtensorMap& spec_map, const CUtensorMap& green_map,
                         const FastArgs& a, dim3 grid, size_t smem, cudaStream_t s);
    // the group z pass with one shared Green table (a.share members)
    static cudaError_t z_shared(const FastArgs& a, int grid, size_t smem, cudaStream_t s);
    // blocks resident per SM at this shared-memory size
    static int z_per_sm(int stages, size_t smem);
    static int x_per_sm(bool inverse, int threads, size_t smem);
};

template <typename T>
cudaError_t run_xfwd(int n, const FastArgs& a, dim3 grid, int threads, size_t smem, cudaStream_t s);
template <typename T>
cudaError_t run_xinv(int n, const FastArgs& a, int stage_bytes, dim3 grid, int threads, size_t smem,
                     cudaStream_t s);
template <typename T>
cudaError_t run_y(int n, int dir, const FastArgs& a, dim3 grid, cudaStream_t s);
template <typename T>
cudaError_t run_z(int n, int stages, const CUtensorMap& spec_map, const CUtensorMap& green_map,
                  const FastArgs& a, dim3 grid, size_t smem, cudaStream_t s);
template <typename T>
cudaError_t run_z_shared(int n, const FastArgs& a, int grid, size_t smem, cudaStream_t s);
// blocks of the z kernel resident per SM at this shared-memory size
template <typename T>
int z_blocks_per_sm(int n, int stages, size_t smem);

// blocks of the x kernels resident per SM at this shared-memory size
template <typename T>
int x_blocks_per_sm(int n, bool inverse, int threads, size_t smem);

}  // namespace fast
}  // namespace fp
