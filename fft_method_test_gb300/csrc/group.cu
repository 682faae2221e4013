// group.cu -- lockstep MINRES iterations of several problems of one grid: one
// launch per pass and per vector kernel for the whole group.
//
// Each member keeps its own buffers, scalars and partial sums; per iteration
// the host writes one table entry per member (the specialised passes'
// arguments and the vector kernels' pointers at that member's buffer
// rotation), and the group kernels (fft_fast.cuh GROUP = true, k_*_g in
// kernels_minres.cu) take their member from blockIdx.  A member whose solve
// is done returns at the top of every kernel through its own stop flag.  The
// x passes keep each member's own grid and the vector kernels its own block
// count, so every member computes exactly what it computes alone.  When all
// members share one Green table (same grid, voxel size, viscosity and alias
// radius), the z pass is k_fz_shared, which loads each Green tile once for
// all members (and transforms a done member's stale spectrum, which nothing
// reads, rather than skip it).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "fft_fast.cuh"
#include "internal.h"

namespace fp {

struct GroupTables {
    int members = 0, iters = 0;
    fast::FastArgs* d_fast = nullptr;  // [iters][members]
    IterArgs* d_iter = nullptr;        // [iters][members]
    CUtensorMap* d_maps = nullptr;     // [members][2]
    fast::FastArgs* h_fast = nullptr;  // pinned staging of the same
    IterArgs* h_iter = nullptr;
    CUtensorMap* h_maps = nullptr;
};

cudaError_t group_tables_create(GroupTables** out, int members, int iters) {
    *out = nullptr;
    if (members < 1 || iters < 1) return cudaErrorInvalidValue;
    GroupTables* t = new GroupTables;
    t->members = members;
    t->iters = iters;
    const size_t nf = (size_t)members * iters;
    DeviceMemGuard mem_guard;
    cudaError_t e = cudaMalloc(&t->d_fast, nf * sizeof(fast::FastArgs));
    if (e == cudaSuccess) e = cudaMalloc(&t->d_iter, nf * sizeof(IterArgs));
    if (e == cudaSuccess) e = cudaMalloc(&t->d_maps, 2 * (size_t)members * sizeof(CUtensorMap));
    if (e == cudaSuccess) e = cudaMallocHost(&t->h_fast, nf * sizeof(fast::FastArgs));
    if (e == cudaSuccess) e = cudaMallocHost(&t->h_iter, nf * sizeof(IterArgs));
    if (e == cudaSuccess) e = cudaMallocHost(&t->h_maps, 2 * (size_t)members * sizeof(CUtensorMap));
    if (e != cudaSuccess) {
        group_tables_destroy(t);
        return e;
    }
    *out = t;
    return cudaSuccess;
}

void group_tables_destroy(GroupTables* t) {
    if (!t) return;
    DeviceMemGuard mem_guard;
    cudaFree(t->d_fast);
    cudaFree(t->d_iter);
    cudaFree(t->d_maps);
    cudaFreeHost(t->h_fast);
    cudaFreeHost(t->h_iter);
    cudaFreeHost(t->h_maps);
    delete t;
}

bool group_supported(Problem& P) {
    ApplyArgs aa;
    return fast_apply_supported(P, P.precision, aa.src_kind, aa.dst_kind, aa.stage);
}

cudaError_t group_iterations(Problem* const* m, int members, int count, GroupTables* t) {
    if (members < 1 || count < 1 || !t || members > t->members || count > t->iters)
        return cudaErrorInvalidValue;
    Problem& P0 = *m[0];
    cudaStream_t s = P0.stream;
    const int prec = P0.precision;
    // the staging buffers of the previous call must have been copied
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    // each member's fixed arguments, its two tensor maps, and the launch
    // geometry all members must share
    std::vector<fast::FastArgs> base((size_t)members);
    long long geom0[kGroupGeometry];
    for (int p = 0; p < members; ++p) {
        Problem& P = *m[p];
        if (P.stream != s || P.precision != prec) return cudaErrorInvalidValue;
        long long g[kGroupGeometry];
        ApplyArgs aa;
        e = fast_member_args(P, prec, aa, &base[(size_t)p], &t->h_maps[2 * p], g);
        if (e != cudaSuccess) return e;
        if (p == 0)
            std::memcpy(geom0, g, sizeof(g));
        else if (std::memcmp(geom0, g, sizeof(g)) != 0)
            return cudaErrorInvalidValue;
    }
    // The Green table depends only on the grid, voxel size, viscosity and
    // alias radius: members that share them all read member 0's table, and
    // when all of them do, the z pass (k_fz_shared) loads each Green tile
    // once for the whole group.
    bool shared_green = true;
    for (int p = 1; p < members; ++p) {
        const Problem& P = *m[p];
        if (P.h == P0.h && P.mu == P0.mu && P.p_radius == P0.p_radius) {
            base[(size_t)p].green = base[0].green;
            t->h_maps[2 * p + 1] = t->h_maps[1];
        } else {
            shared_green = false;
        }
    }
    const int nparts = (int)geom0[7];  // partial rows of the inverse x pass
    int max_blocks = 1;
    for (int i = 0; i < count; ++i) {
        for (int p = 0; p < members; ++p) {
            IterArgs ia;
            ApplyArgs aa;
            iteration_args(*m[p], &ia, &aa);
            ia.nparts = nparts;
            fast::FastArgs fa = base[(size_t)p];
            fa.src = aa.src;
            fa.src_sum = aa.src_sum;
            fa.dst = aa.dst;
            fa.dot_with = aa.dot_with;
            fa.skip = aa.skip;
            t->h_fast[(size_t)i * members + p] = fa;
            t->h_iter[(size_t)i * members + p] = ia;
            max_blocks = std::max(max_blocks, ia.nblk);
        }
    }
    const size_t nf = (size_t)count * members;
    if ((e = cudaMemcpyAsync(t->d_maps, t->h_maps, 2 * (size_t)members * sizeof(CUtensorMap),
                             cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(t->d_fast, t->h_fast, nf * sizeof(fast::FastArgs), cudaMemcpyHostToDevice, s)) !=
        cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(t->d_iter, t->h_iter, nf * sizeof(IterArgs), cudaMemcpyHostToDevice, s)) !=
        cudaSuccess)
        return e;
    for (int i = 0; i < count; ++i) {
        int np = 0;
        e = fast_apply_group(P0, prec, members, t->d_fast + (size_t)i * members, t->d_maps, shared_green,
                             &np);
        if (e != cudaSuccess) return e;
        e = group_iteration_tail(s, t->d_iter + (size_t)i * members, members, max_blocks);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace fp
