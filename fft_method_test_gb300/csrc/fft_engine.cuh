// fft_engine.cuh -- register-resident Stockham FFT of lines on one CTA.
//
// Stage s with radix R of the Stockham auto-sort formulation reads element
// j + r*(n/R) (r < R), multiplies by exp(SIGN*2*pi*i*(j mod Ns)*r/(Ns*R)),
// does a length-R DFT in registers and writes element
// (j/Ns)*Ns*R + (j mod Ns) + r*Ns, with Ns the product of the earlier radices.
//
// A line of length n is served by tpl = ceil(n / Rmax) threads, Rmax the
// largest radix of the plan (FP32 plans use radices up to 16, FP64 plans up
// to 8: the FP64 register budget), so a thread owns at most ceil(Rmax/R)
// butterflies of a radix-R stage.  Each thread may carry NL lines (the three
// vector components) with the same butterfly indices, which multiplies the
// independent memory operations in flight per thread.
//
// The first stage can read its inputs straight from global memory and the
// last stage can write straight to global memory (functors src/dst); only the
// exchanges between stages go through shared memory.  Shared-memory lines are
// padded (one slot every 16 FP32 / 8 FP64 elements) so that the stride-R
// writes of the early stages do not pile onto one bank.
//
// Radices: 16, 8, 4, 2, 3, 5 (lengths must factor into 2, 3 and 5).
#pragma once

#include "common.cuh"

namespace fp {

constexpr int kMaxStages = 16;

struct FftPlanDev {
    int n;
    int nstage32;
    int tpl32;
    int radix32[kMaxStages];  // FP32 stages (radix up to 16)
    int nstage64;
    int tpl64;
    int radix64[kMaxStages];  // FP64 stages (radix up to 8)
    const double2* tw64;      // exp(-2 pi i j / n), j < n
    const float2* tw32;
};

template <typename T2>
struct Prec;
template <>
struct Prec<float2> {
    static constexpr int MAXR = 16;
    static constexpr int PADSH = 4;
};
template <>
struct Prec<double2> {
    static constexpr int MAXR = 8;
    static constexpr int PADSH = 3;
};

template <typename T2>
__device__ __forceinline__ int pidx(int i) {
    return i + (i >> Prec<T2>::PADSH);
}

// padded, odd line stride (elements) of a shared-memory line of length n
__host__ __device__ __forceinline__ int line_stride(int n, int padsh) {
    const int l = n + ((n - 1) >> padsh) + 1;
    return l | 1;
}

// Line stride for the passes whose threads run over columns first (y, z:
// thread = column + t * position).  One shared-memory wavefront of 8-byte
// (16-byte) accesses serves B = 16 (8) threads: min(t, B) columns times B/t
// neighbouring positions of each line.  An odd stride separates the columns
// when t >= B; for t < B a stride congruent to B/t modulo B puts the B/t
// positions of every column in banks of their own.
__host__ __device__ __forceinline__ int column_line_stride(int n, int padsh, int t, int elem) {
    int ld = line_stride(n, padsh);
    const int B = 128 / elem;
    if (t >= B) return ld;
    const int target = (B / t) % B;
    while (ld % B != target) ++ld;
    return ld;
}

template <typename T2>
__device__ __forceinline__ const T2* plan_tw(const FftPlanDev& p);
template <>
__device__ __forceinline__ const double2* plan_tw<double2>(const FftPlanDev& p) {
    return p.tw64;
}
template <>
__device__ __forceinline__ const float2* plan_tw<float2>(const FftPlanDev& p) {
    return p.tw32;
}
template <typename T2>
__device__ __forceinline__ int plan_nstage(const FftPlanDev& p) {
    return sizeof(T2) == 16 ? p.nstage64 : p.nstage32;
}
template <typename T2>
__device__ __forceinline__ int plan_tpl(const FftPlanDev& p) {
    return sizeof(T2) == 16 ? p.tpl64 : p.tpl32;
}
template <typename T2>
__device__ __forceinline__ int plan_radix(const FftPlanDev& p, int s) {
    return sizeof(T2) == 16 ? p.radix64[s] : p.radix32[s];
}

// ---- small DFT kernels (SIGN = -1 forward, +1 backward) ---------------------

template <int S, typename T2>
__device__ __forceinline__ void dft2(T2& a, T2& b) {
    const T2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <int S, typename T2>
__device__ __forceinline__ void dft4(T2& x0, T2& x1, T2& x2, T2& x3) {
    const T2 s02 = cadd(x0, x2), d02 = csub(x0, x2);
    const T2 s13 = cadd(x1, x3), d13 = cmul_si<S>(csub(x1, x3));
    x0 = cadd(s02, s13);
    x2 = csub(s02, s13);
    x1 = cadd(d02, d13);
    x3 = csub(d02, d13);
}

template <int S, typename T2>
__device__ __forceinline__ void dft3(T2& x0, T2& x1, T2& x2) {
    using T = decltype(T2::x);
    const T kS3 = (T)0.86602540378443864676;  // sin(2 pi / 3)
    const T2 t1 = cadd(x1, x2);
    const T2 t2 = cmk<T2>(x0.x - (T)0.5 * t1.x, x0.y - (T)0.5 * t1.y);
    const T2 d = csub(x1, x2);
    const T2 t3 = cmul_si<S>(cmk<T2>(kS3 * d.x, kS3 * d.y));
    x0 = cadd(x0, t1);
    x1 = cadd(t2, t3);
    x2 = csub(t2, t3);
}

template <int S, typename T2>
__device__ __forceinline__ void dft5(T2& x0, T2& x1, T2& x2, T2& x3, T2& x4) {
    using T = decltype(T2::x);
    const T c1 = (T)0.30901699437494742410;   // cos(2 pi / 5)
    const T c2 = (T)-0.80901699437494742410;  // cos(4 pi / 5)
    const T s1 = (T)0.95105651629515357212;   // sin(2 pi / 5)
    const T s2 = (T)0.58778525229247312917;   // sin(4 pi / 5)
    const T2 p14 = cadd(x1, x4), m14 = csub(x1, x4);
    const T2 p23 = cadd(x2, x3), m23 = csub(x2, x3);
    const T2 a1 = cmk<T2>(x0.x + c1 * p14.x + c2 * p23.x, x0.y + c1 * p14.y + c2 * p23.y);
    const T2 a2 = cmk<T2>(x0.x + c2 * p14.x + c1 * p23.x, x0.y + c2 * p14.y + c1 * p23.y);
    const T2 b1 = cmul_si<S>(cmk<T2>(s1 * m14.x + s2 * m23.x, s1 * m14.y + s2 * m23.y));
    const T2 b2 = cmul_si<S>(cmk<T2>(s2 * m14.x - s1 * m23.x, s2 * m14.y - s1 * m23.y));
    x0 = cadd(x0, cadd(p14, p23));
    x1 = cadd(a1, b1);
    x4 = csub(a1, b1);
    x2 = cadd(a2, b2);
    x3 = csub(a2, b2);
}

// multiply by exp(S * i * pi / 4) and exp(S * 3 i pi / 4)
template <int S, typename T2>
__device__ __forceinline__ T2 mul_w8_1(T2 a) {
    using T = decltype(T2::x);
    const T c = (T)0.70710678118654752440;
    return S < 0 ? cmk<T2>(c * (a.x + a.y), c * (a.y - a.x)) : cmk<T2>(c * (a.x - a.y), c * (a.y + a.x));
}
template <int S, typename T2>
__device__ __forceinline__ T2 mul_w8_3(T2 a) {
    using T = decltype(T2::x);
    const T c = (T)0.70710678118654752440;
    return S < 0 ? cmk<T2>(c * (a.y - a.x), -c * (a.x + a.y)) : cmk<T2>(-c * (a.x + a.y), c * (a.x - a.y));
}

// DFT8 as 2 x 4: y[2q] = DFT4(x_r + x_{r+4})[q], y[2q+1] = DFT4((x_r - x_{r+4}) W8^r)[q].
// y[k] is left in register out_slot<8>(k).
template <int S, typename T2>
__device__ __forceinline__ void dft8(T2 (&v)[8]) {
#pragma unroll
    for (int r = 0; r < 4; ++r) dft2<S>(v[r], v[r + 4]);
    v[5] = mul_w8_1<S>(v[5]);
    v[6] = cmul_si<S>(v[6]);
    v[7] = mul_w8_3<S>(v[7]);
    dft4<S>(v[0], v[1], v[2], v[3]);
    dft4<S>(v[4], v[5], v[6], v[7]);
}

template <int S, typename T2>
__device__ __forceinline__ T2 mul_const(T2 a, decltype(T2::x) c, decltype(T2::x) s) {
    // a * (c + i*S*s)
    const decltype(T2::x) ss = S < 0 ? -s : s;
    return cmk<T2>(a.x * c - a.y * ss, a.x * ss + a.y * c);
}

// DFT16 as 4 x 4: r = 4a + b, k = c + 4d.  y[c + 4d] is left in v[4c + d].
template <int S, typename T2>
__device__ __forceinline__ void dft16(T2 (&v)[16]) {
    using T = decltype(T2::x);
    const T c8 = (T)0.92387953251128675613;   // cos(pi/8)
    const T s8 = (T)0.38268343236508977173;   // sin(pi/8)
    const T h = (T)0.70710678118654752440;
#pragma unroll
    for (int b = 0; b < 4; ++b) dft4<S>(v[b], v[4 + b], v[8 + b], v[12 + b]);
    // t_b[c] lives in v[4c + b]; multiply by W16^(b*c)
    v[5] = mul_const<S>(v[5], c8, s8);     // W^1
    v[6] = mul_const<S>(v[6], h, h);       // W^2
    v[7] = mul_const<S>(v[7], s8, c8);     // W^3
    v[9] = mul_const<S>(v[9], h, h);       // W^2
    v[10] = cmul_si<S>(v[10]);             // W^4
    v[11] = mul_const<S>(v[11], -h, h);    // W^6
    v[13] = mul_const<S>(v[13], s8, c8);   // W^3
    v[14] = mul_const<S>(v[14], -h, h);    // W^6
    v[15] = mul_const<S>(v[15], -c8, -s8); // W^9
#pragma unroll
    for (int c = 0; c < 4; ++c) dft4<S>(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);
}

// register holding output k of dft_r<R>
template <int R>
__device__ __forceinline__ constexpr int out_slot(int k) {
    return R == 16 ? (k % 4) * 4 + k / 4 : (R == 8 ? (k % 2) * 4 + k / 2 : k);
}

template <int R, int S, typename T2>
__device__ __forceinline__ void dft_r(T2 (&v)[R]) {
    if constexpr (R == 2) {
        dft2<S>(v[0], v[1]);
    } else if constexpr (R == 3) {
        dft3<S>(v[0], v[1], v[2]);
    } else if constexpr (R == 4) {
        dft4<S>(v[0], v[1], v[2], v[3]);
    } else if constexpr (R == 5) {
        dft5<S>(v[0], v[1], v[2], v[3], v[4]);
    } else if constexpr (R == 8) {
        dft8<S>(v);
    } else {
        static_assert(R == 16, "unsupported radix");
        dft16<S>(v);
    }
}

// ---------------------------------------------------------------------------
// stages
// ---------------------------------------------------------------------------

// Stage input/output modes: shared-memory lines, a functor (global memory),
// or a functor that reads shared memory the stage's own output overwrites
// (a barrier separates the loads from the stores).
enum { kIoSmem = 0, kIoFunc = 1, kIoFuncSmem = 2 };

template <typename T2, int R>
struct StageRegs {
    static constexpr int KM = (Prec<T2>::MAXR + R - 1) / R;
};

// Register arrays are zero-filled before the guarded loads: with elements
// that are only conditionally written the compiler keeps them alive around
// the runtime stage loop, which multiplies register demand by the number of
// radix cases and spills.
template <int NL, int KM, int R, typename T2>
__device__ __forceinline__ void zero_regs(T2 (&v)[NL][KM][R]) {
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
        for (int k = 0; k < KM; ++k)
#pragma unroll
            for (int r = 0; r < R; ++r) v[l][k][r] = T2{};
}

// Load the butterflies of one stage into registers.
template <int R, int IN, int NL, typename T2, class Src>
__device__ __forceinline__ void stage_load(T2 (&v)[NL][StageRegs<T2, R>::KM][R], T2* const* sl,
                                           int n, int lane, int tpl, bool active, Src& src) {
    constexpr int KM = StageRegs<T2, R>::KM;
    const int m = n / R;
    if (!active) return;
#pragma unroll
    for (int kk = 0; kk < KM; ++kk) {
        const int j = lane + kk * tpl;
        if (j < m) {
#pragma unroll
            for (int l = 0; l < NL; ++l)
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    if constexpr (IN == kIoSmem) {
                        v[l][kk][r] = sl[l][pidx<T2>(j + r * m)];
                    } else {
                        v[l][kk][r] = src(l, j + r * m);
                    }
                }
        }
    }
}

// Twiddle + DFT of the loaded butterflies (outputs left in out_slot order).
template <int R, int S, int NL, typename T2>
__device__ __forceinline__ void stage_compute(T2 (&v)[NL][StageRegs<T2, R>::KM][R], int n, int ns,
                                              int lane, int tpl, bool active,
                                              const T2* __restrict__ tw) {
    constexpr int KM = StageRegs<T2, R>::KM;
    const int m = n / R;
    if (!active) return;
    const int step = n / (ns * R);
#pragma unroll
    for (int kk = 0; kk < KM; ++kk) {
        const int j = lane + kk * tpl;
        if (j < m) {
            const int k = j % ns;
            if (k != 0) {
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    T2 w = tw[k * r * step];
                    if (S > 0) w.y = -w.y;
#pragma unroll
                    for (int l = 0; l < NL; ++l) v[l][kk][r] = cmul(v[l][kk][r], w);
                }
            }
#pragma unroll
            for (int l = 0; l < NL; ++l) dft_r<R, S>(v[l][kk]);
        }
    }
}

// Store the outputs of one stage.
template <int R, int OUT, int NL, typename T2, class Dst>
__device__ __forceinline__ void stage_store(T2 (&v)[NL][StageRegs<T2, R>::KM][R], T2* const* sl,
                                            int n, int ns, int lane, int tpl, bool active, Dst& dst) {
    constexpr int KM = StageRegs<T2, R>::KM;
    const int m = n / R;
    if (!active) return;
#pragma unroll
    for (int kk = 0; kk < KM; ++kk) {
        const int j = lane + kk * tpl;
        if (j < m) {
            const int k = j % ns;
            const int base = (j - k) * R + k;
#pragma unroll
            for (int l = 0; l < NL; ++l)
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    if constexpr (OUT == kIoSmem) {
                        sl[l][pidx<T2>(base + r * ns)] = v[l][kk][out_slot<R>(r)];
                    } else {
                        dst(l, base + r * ns, v[l][kk][out_slot<R>(r)]);
                    }
                }
        }
    }
}

// One complete stage.  When IN != kIoSmem the caller guarantees that the
// shared-memory lines may be overwritten on entry; the stage ends with a
// barrier whenever its outputs go to shared memory.
template <int R, int S, int IN, int OUT, int NL, typename T2, class Src, class Dst>
__device__ __forceinline__ void fft_stage(T2* const* sl, int n, int ns, int lane, int tpl,
                                          bool active, const T2* __restrict__ tw, Src& src,
                                          Dst& dst) {
    T2 v[NL][StageRegs<T2, R>::KM][R];
    zero_regs(v);
    stage_load<R, IN, NL>(v, sl, n, lane, tpl, active, src);
    if ((IN == kIoSmem || IN == kIoFuncSmem) && OUT == kIoSmem) __syncthreads();
    stage_compute<R, S, NL>(v, n, ns, lane, tpl, active, tw);
    stage_store<R, OUT, NL>(v, sl, n, ns, lane, tpl, active, dst);
    if (OUT == kIoSmem) __syncthreads();
}

template <int S, int IN, int OUT, int NL, typename T2, class Src, class Dst>
__device__ __forceinline__ void fft_stage_rt(int R, T2* const* sl, int n, int ns, int lane,
                                             int tpl, bool active, const T2* __restrict__ tw,
                                             Src& src, Dst& dst) {
    switch (R) {
        case 16:
            if constexpr (Prec<T2>::MAXR >= 16)
                fft_stage<16, S, IN, OUT, NL>(sl, n, ns, lane, tpl, active, tw, src, dst);
            break;
        case 8: fft_stage<8, S, IN, OUT, NL>(sl, n, ns, lane, tpl, active, tw, src, dst); break;
        case 4: fft_stage<4, S, IN, OUT, NL>(sl, n, ns, lane, tpl, active, tw, src, dst); break;
        case 2: fft_stage<2, S, IN, OUT, NL>(sl, n, ns, lane, tpl, active, tw, src, dst); break;
        case 3: fft_stage<3, S, IN, OUT, NL>(sl, n, ns, lane, tpl, active, tw, src, dst); break;
        default: fft_stage<5, S, IN, OUT, NL>(sl, n, ns, lane, tpl, active, tw, src, dst); break;
    }
}

template <typename T2>
struct NoSrc {
    __device__ __forceinline__ T2 operator()(int, int) const { return T2{}; }
};
template <typename T2>
struct NoDst {
    __device__ __forceinline__ void operator()(int, int, T2) const {}
};

// Full FFT of NL lines per thread.  IN/OUT select whether the first stage
// reads through src(l, i) and the last stage writes through dst(l, i, v)
// (kIoFunc) or both use the shared-memory lines sl[l] (kIoSmem).  reverse
// runs the stages in reverse radix order.
template <int S, int IN, int OUT, int NL, typename T2, class Src, class Dst>
__device__ __forceinline__ void fft_lines(T2* const* sl, const FftPlanDev& p, int lane, bool active,
                                          bool reverse, Src src, Dst dst) {
    const T2* tw = plan_tw<T2>(p);
    const int nst = plan_nstage<T2>(p);
    const int tpl = plan_tpl<T2>(p);
    const int n = p.n;
    NoSrc<T2> nsrc;
    NoDst<T2> ndst;
    if (nst == 0) {  // n == 1: the transform is the identity
        if (active && lane == 0) {
            for (int l = 0; l < NL; ++l) {
                T2 v;
                if constexpr (IN != kIoSmem) v = src(l, 0); else v = sl[l][0];
                if constexpr (OUT == kIoFunc) dst(l, 0, v); else sl[l][0] = v;
            }
        }
        if (OUT == kIoSmem) __syncthreads();
        return;
    }
    int ns = 1;
    for (int s = 0; s < nst; ++s) {
        const int R = plan_radix<T2>(p, reverse ? nst - 1 - s : s);
        const bool first = s == 0, last = s == nst - 1;
        if (first && last) {
            fft_stage_rt<S, IN, OUT, NL>(R, sl, n, ns, lane, tpl, active, tw, src, dst);
        } else if (first) {
            fft_stage_rt<S, IN, kIoSmem, NL>(R, sl, n, ns, lane, tpl, active, tw, src, ndst);
        } else if (last) {
            fft_stage_rt<S, kIoSmem, OUT, NL>(R, sl, n, ns, lane, tpl, active, tw, nsrc, dst);
        } else {
            fft_stage_rt<S, kIoSmem, kIoSmem, NL>(R, sl, n, ns, lane, tpl, active, tw, nsrc, ndst);
        }
        ns *= R;
    }
}

}  // namespace fp
