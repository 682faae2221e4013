// fft_engine.cuh -- in-place Stockham FFT of lines held in shared memory.
//
// A CTA holds several lines of length n in shared memory; each line is served
// by tpl = ceil(n/8) threads.  One radix-R stage of the Stockham auto-sort
// formulation reads element j + r*(n/R) (r < R), multiplies by the twiddle
// exp(SIGN*2*pi*i*(j mod Ns)*r/(Ns*R)), does a length-R DFT in registers and
// writes element (j/Ns)*Ns*R + (j mod Ns) + r*Ns.  Every thread first loads
// all of its butterflies into registers, the CTA synchronises, and then the
// results are written back into the same line, so one buffer suffices.
// Radices: 16, 8, 4, 2, 3, 5 (lengths must factor into 2, 3 and 5).  With
// tpl = ceil(n/8) a thread owns at most ceil(8/R) butterflies of a stage.
#pragma once

#include "common.cuh"

namespace fp {

constexpr int kMaxStages = 16;

struct FftPlanDev {
    int n;
    int nstage;
    int tpl;  // threads per line
    int radix[kMaxStages];    // FP32 stages (radix up to 16)
    int nstage64;
    int radix64[kMaxStages];  // FP64 stages (radix up to 8: register budget)
    const double2* tw64;  // exp(-2 pi i j / n), j < n
    const float2* tw32;
};

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

template <int S, typename T2>
__device__ __forceinline__ void dft8(T2 (&v)[8]) {
    T2 a0 = cadd(v[0], v[4]), a1 = cadd(v[1], v[5]), a2 = cadd(v[2], v[6]), a3 = cadd(v[3], v[7]);
    T2 b0 = csub(v[0], v[4]), b1 = csub(v[1], v[5]), b2 = csub(v[2], v[6]), b3 = csub(v[3], v[7]);
    b1 = mul_w8_1<S>(b1);
    b2 = cmul_si<S>(b2);
    b3 = mul_w8_3<S>(b3);
    dft4<S>(a0, a1, a2, a3);
    dft4<S>(b0, b1, b2, b3);
    v[0] = a0; v[2] = a1; v[4] = a2; v[6] = a3;
    v[1] = b0; v[3] = b1; v[5] = b2; v[7] = b3;
}

template <int S, typename T2>
__device__ __forceinline__ T2 mul_const(T2 a, decltype(T2::x) c, decltype(T2::x) s) {
    // a * (c + i*S*s)
    const decltype(T2::x) ss = S < 0 ? -s : s;
    return cmk<T2>(a.x * c - a.y * ss, a.x * ss + a.y * c);
}

// DFT16 as 4 x 4: r = 4a + b, k = c + 4d.  The result y[c + 4d] is left in
// register v[4c + d]; out_slot<16>() maps output index -> register.
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

// register holding output r of dft_r<R>
template <int R>
__device__ __forceinline__ constexpr int out_slot(int r) {
    return R == 16 ? (r % 4) * 4 + r / 4 : r;
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

// One Stockham stage on one line (line == nullptr: idle thread that only
// takes part in the barriers).
template <int R, int S, typename T2>
__device__ __forceinline__ void fft_stage(T2* line, int n, int ns, int lane, int tpl,
                                          const T2* __restrict__ tw) {
    constexpr int KM = (R >= 8) ? 1 : (8 + R - 1) / R;
    const int m = n / R;
    T2 v[KM][R];
    if (line) {
#pragma unroll
        for (int kk = 0; kk < KM; ++kk) {
            const int j = lane + kk * tpl;
            if (j < m) {
#pragma unroll
                for (int r = 0; r < R; ++r) v[kk][r] = line[j + r * m];
            }
        }
    }
    __syncthreads();
    if (line) {
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
                        v[kk][r] = cmul(v[kk][r], w);
                    }
                }
                dft_r<R, S>(v[kk]);
                const int base = (j - k) * R + k;
#pragma unroll
                for (int r = 0; r < R; ++r) line[base + r * ns] = v[kk][out_slot<R>(r)];
            }
        }
    }
    __syncthreads();
}

// Full in-place FFT of the line owned by this thread (lane < tpl).
template <int S, typename T2>
__device__ __forceinline__ void fft_line(T2* line, const FftPlanDev& p, int lane) {
    const T2* tw = plan_tw<T2>(p);
    constexpr bool dbl = sizeof(T2) == 16;
    const int nst = dbl ? p.nstage64 : p.nstage;
    const int* rad = dbl ? p.radix64 : p.radix;
    int ns = 1;
    for (int s = 0; s < nst; ++s) {
        const int R = rad[s];
        switch (R) {
            case 16:
                if constexpr (!dbl) fft_stage<16, S>(line, p.n, ns, lane, p.tpl, tw);
                break;
            case 8: fft_stage<8, S>(line, p.n, ns, lane, p.tpl, tw); break;
            case 4: fft_stage<4, S>(line, p.n, ns, lane, p.tpl, tw); break;
            case 2: fft_stage<2, S>(line, p.n, ns, lane, p.tpl, tw); break;
            case 3: fft_stage<3, S>(line, p.n, ns, lane, p.tpl, tw); break;
            default: fft_stage<5, S>(line, p.n, ns, lane, p.tpl, tw); break;
        }
        ns *= R;
    }
}

}  // namespace fp
