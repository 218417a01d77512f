// fft_comp.cuh -- compensated FP32 arithmetic for the directional passes:
// small DFTs (sizes 1, 2, 4, 8, 16) on double-float complex values.
//
// A value is hi + lo, both float2 (re, im).  Every addition keeps its exact
// rounding error (Knuth's TwoSum, six operations) and every product by a
// double-word constant its exact error (the FMA residual a*b - RN(a*b));
// those errors, and the lo parts of the inputs, travel through the rest of
// the transform as a second, linear FP32 computation.  The lo parts are about
// 2^-24 of the hi parts, so their own rounding is about 2^-48 of the value:
// the transform is accurate to near-FP64 level on FP32 instructions, and the
// only FP32 rounding left in a pass is the store of the field.
//
// This matters where the time stepping amplifies round-off: at the 256^3
// quantum-turbulence workload (coeffD = -0.0354, dt = 2.5e-3) the modes with
// |coeffD| |k|^2 dt near pi grow by about 2.7x per 25 steps (the split-step
// resonance), and the rounding noise of plain FP32 FFTs is the seed that they
// grow from.
//
// All operations are packed f32x2 instructions (add/sub/mul/fma.rn.f32x2),
// one instruction per complex component pair, written as inline PTX so the
// compiler can neither contract nor reassociate them (the error terms rely on
// the exact IEEE round-to-nearest results).
#pragma once
#include <cuda_runtime.h>
#include "fft_core.cuh"

namespace gpss {

struct cdf {
    float2 h, l;
};

__device__ __forceinline__ unsigned long long pk(float2 a)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}
__device__ __forceinline__ float2 upk(unsigned long long r)
{
    float2 a;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
    return a;
}

__device__ __forceinline__ float2 p_add(float2 a, float2 b)
{
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)));
    return upk(d);
}
__device__ __forceinline__ float2 p_sub(float2 a, float2 b)
{
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)));
    return upk(d);
}
__device__ __forceinline__ float2 p_mul(float2 a, float2 b)
{
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)));
    return upk(d);
}
__device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c)
{
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)), "l"(pk(c)));
    return upk(d);
}
__device__ __forceinline__ float2 p_neg(float2 a) { return make_float2(-a.x, -a.y); }

// s + e == a + b exactly (per component)
__device__ __forceinline__ void two_sum(float2 a, float2 b, float2 &s, float2 &e)
{
    s = p_add(a, b);
    const float2 bb = p_sub(s, a);
    e = p_add(p_sub(a, p_sub(s, bb)), p_sub(b, bb));
}
// s + e == a - b exactly
__device__ __forceinline__ void two_diff(float2 a, float2 b, float2 &s, float2 &e)
{
    s = p_sub(a, b);
    const float2 bb = p_sub(s, a);  // ~ -b
    e = p_sub(p_sub(a, p_sub(s, bb)), p_add(b, bb));
}

__device__ __forceinline__ cdf c_of(float2 h) { return cdf{h, make_float2(0.f, 0.f)}; }
// hi + lo rounded once to FP32
__device__ __forceinline__ float2 c_round(const cdf &a) { return p_add(a.h, a.l); }

__device__ __forceinline__ cdf cdf_add(const cdf &a, const cdf &b)
{
    cdf r;
    float2 e;
    two_sum(a.h, b.h, r.h, e);
    r.l = p_add(p_add(a.l, b.l), e);
    return r;
}
__device__ __forceinline__ cdf cdf_sub(const cdf &a, const cdf &b)
{
    cdf r;
    float2 e;
    two_diff(a.h, b.h, r.h, e);
    r.l = p_add(p_sub(a.l, b.l), e);
    return r;
}
// exact sum / difference of two FP32 values (the first butterfly level of a
// transform whose inputs are the stored field)
__device__ __forceinline__ cdf cdf_add0(float2 a, float2 b)
{
    cdf r;
    two_sum(a, b, r.h, r.l);
    return r;
}
__device__ __forceinline__ cdf cdf_sub0(float2 a, float2 b)
{
    cdf r;
    two_diff(a, b, r.h, r.l);
    return r;
}

// multiply by DIR*i (exact)
template <int DIR> __device__ __forceinline__ cdf cdf_muli(const cdf &a)
{
    if (DIR < 0) return cdf{make_float2(a.h.y, -a.h.x), make_float2(a.l.y, -a.l.x)};
    return cdf{make_float2(-a.h.y, a.h.x), make_float2(-a.l.y, a.l.x)};
}
__device__ __forceinline__ cdf cdf_neg(const cdf &a) { return cdf{p_neg(a.h), p_neg(a.l)}; }

// a * s for a real FP32 scalar s (exact product error kept)
__device__ __forceinline__ cdf cdf_scale(const cdf &a, float s)
{
    const float2 ss = make_float2(s, s);
    cdf r;
    r.h = p_mul(a.h, ss);
    const float2 e = p_fma(a.h, ss, p_neg(r.h));
    r.l = p_fma(a.l, ss, e);
    return r;
}
// a * (hi + lo) for a real double-word constant
__device__ __forceinline__ cdf cdf_rmul2(const cdf &a, float hi, float lo)
{
    const float2 H = make_float2(hi, hi), L = make_float2(lo, lo);
    cdf r;
    r.h = p_mul(a.h, H);
    const float2 e = p_fma(a.h, H, p_neg(r.h));
    r.l = p_fma(a.h, L, p_fma(a.l, H, e));
    return r;
}

// a * (bh + bl), b a double-word complex constant:
//   re = ax bx - ay by, im = ax by + ay bx as packed pairs
//   (ax, ax)*(bx, by) + (ay, ay)*(-by, bx)
__device__ __forceinline__ cdf cdf_cmul2(const cdf &a, float2 bh, float2 bl)
{
    const float2 X = make_float2(a.h.x, a.h.x), Y = make_float2(a.h.y, a.h.y);
    const float2 b2 = make_float2(-bh.y, bh.x), bl2 = make_float2(-bl.y, bl.x);
    const float2 p1 = p_mul(X, bh), p2 = p_mul(Y, b2);
    const float2 e1 = p_fma(X, bh, p_neg(p1)), e2 = p_fma(Y, b2, p_neg(p2));
    cdf r;
    float2 es;
    two_sum(p1, p2, r.h, es);
    float2 l = p_add(p_add(e1, e2), es);
    l = p_fma(X, bl, l);
    l = p_fma(Y, bl2, l);
    l = p_fma(make_float2(a.l.x, a.l.x), bh, l);
    l = p_fma(make_float2(a.l.y, a.l.y), b2, l);
    r.l = l;
    return r;
}
// a * conj(bh + bl)
__device__ __forceinline__ cdf cdf_cmulc2(const cdf &a, float2 bh, float2 bl)
{
    return cdf_cmul2(a, make_float2(bh.x, -bh.y), make_float2(bl.x, -bl.y));
}

// multiply by w16^m = exp(DIR * 2 pi i m / 16) for a compile-time m
template <int M, int DIR> __device__ __forceinline__ cdf cdf_mulw16(const cdf &a)
{
    using K = DftConst<float>;
    constexpr int m = ((M % 16) + 16) % 16;
    if constexpr (m == 0) return a;
    else if constexpr (m == 4) return cdf_muli<DIR>(a);
    else if constexpr (m == 8) return cdf_neg(a);
    else if constexpr (m == 12) return cdf_muli<-DIR>(a);
    else if constexpr (m % 2 == 0) {
        // odd multiple of pi/4: value = (sc + i ss) / sqrt2 with sc, ss = +-1
        constexpr int q = m / 2;
        constexpr float sc = (q == 1 || q == 7) ? 1.f : -1.f;
        constexpr float ss = ((q == 1 || q == 3) ? 1.f : -1.f) * (float)DIR;
        // (sc ax - ss ay, ss ax + sc ay) = (sc, ss) ax + (-ss, sc) ay, exact signs
        const cdf A{make_float2(sc * a.h.x, ss * a.h.x), make_float2(sc * a.l.x, ss * a.l.x)};
        const cdf B{make_float2(-ss * a.h.y, sc * a.h.y), make_float2(-ss * a.l.y, sc * a.l.y)};
        return cdf_rmul2(cdf_add(A, B), K::Hh, K::Hl);
    } else {
        constexpr int ci = (m == 1 || m == 15) ? 1 : (m == 3 || m == 13) ? 2 : (m == 5 || m == 11) ? -2 : -1;
        constexpr int si = (m == 1 || m == 7) ? 2 : (m == 3 || m == 5) ? 1 : (m == 9 || m == 15) ? -2 : -1;
        const float crh = (ci == 1 || ci == -1) ? (ci > 0 ? K::C1h : -K::C1h) : (ci > 0 ? K::S1h : -K::S1h);
        const float crl = (ci == 1 || ci == -1) ? (ci > 0 ? K::C1l : -K::C1l) : (ci > 0 ? K::S1l : -K::S1l);
        const float srh = (si == 2 || si == -2) ? (si > 0 ? K::S1h : -K::S1h) : (si > 0 ? K::C1h : -K::C1h);
        const float srl = (si == 2 || si == -2) ? (si > 0 ? K::S1l : -K::S1l) : (si > 0 ? K::C1l : -K::C1l);
        return cdf_cmul2(a, make_float2(crh, (float)DIR * srh), make_float2(crl, (float)DIR * srl));
    }
}

template <int DIR> __device__ __forceinline__ void cdf_dft2(cdf &a0, cdf &a1)
{
    const cdf t = a0;
    a0 = cdf_add(t, a1);
    a1 = cdf_sub(t, a1);
}

template <int DIR> __device__ __forceinline__ void cdf_dft4(cdf &a0, cdf &a1, cdf &a2, cdf &a3)
{
    const cdf s02 = cdf_add(a0, a2), d02 = cdf_sub(a0, a2);
    const cdf s13 = cdf_add(a1, a3), t = cdf_muli<DIR>(cdf_sub(a1, a3));
    a0 = cdf_add(s02, s13);
    a2 = cdf_sub(s02, s13);
    a1 = cdf_add(d02, t);
    a3 = cdf_sub(d02, t);
}
// the same on FP32 inputs (lo parts zero)
template <int DIR> __device__ __forceinline__ void cdf_dft4_0(float2 x0, float2 x1, float2 x2, float2 x3, cdf &a0,
                                                          cdf &a1, cdf &a2, cdf &a3)
{
    const cdf s02 = cdf_add0(x0, x2), d02 = cdf_sub0(x0, x2);
    const cdf s13 = cdf_add0(x1, x3), t = cdf_muli<DIR>(cdf_sub0(x1, x3));
    a0 = cdf_add(s02, s13);
    a2 = cdf_sub(s02, s13);
    a1 = cdf_add(d02, t);
    a3 = cdf_sub(d02, t);
}

// the 16-point transform after its first radix-4 level: b[j1 + 4 k1] holds
// the inner DFT4 over j2 of x[j1 + 4 j2]; twiddles, outer DFT4s, natural order
template <int DIR> __device__ __forceinline__ void cdf_dft16_tail(cdf *a)
{
    a[5] = cdf_mulw16<1, DIR>(a[5]);
    a[9] = cdf_mulw16<2, DIR>(a[9]);
    a[13] = cdf_mulw16<3, DIR>(a[13]);
    a[6] = cdf_mulw16<2, DIR>(a[6]);
    a[10] = cdf_mulw16<4, DIR>(a[10]);
    a[14] = cdf_mulw16<6, DIR>(a[14]);
    a[7] = cdf_mulw16<3, DIR>(a[7]);
    a[11] = cdf_mulw16<6, DIR>(a[11]);
    a[15] = cdf_mulw16<9, DIR>(a[15]);
    cdf o[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) {
        cdf u0 = a[4 * k1 + 0], u1 = a[4 * k1 + 1], u2 = a[4 * k1 + 2], u3 = a[4 * k1 + 3];
        cdf_dft4<DIR>(u0, u1, u2, u3);
        o[k1] = u0;
        o[k1 + 4] = u1;
        o[k1 + 8] = u2;
        o[k1 + 12] = u3;
    }
#pragma unroll
    for (int i = 0; i < 16; i++) a[i] = o[i];
}

template <int DIR> __device__ __forceinline__ void cdf_dft8_tail(cdf *a)
{
    a[3] = cdf_mulw16<2, DIR>(a[3]);
    a[5] = cdf_mulw16<4, DIR>(a[5]);
    a[7] = cdf_mulw16<6, DIR>(a[7]);
    cdf o[8];
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) {
        cdf u0 = a[2 * k1], u1 = a[2 * k1 + 1];
        cdf_dft2<DIR>(u0, u1);
        o[k1] = u0;
        o[k1 + 4] = u1;
    }
#pragma unroll
    for (int i = 0; i < 8; i++) a[i] = o[i];
}

// In-place natural-order DFT of size N (1, 2, 4, 8, 16) on double-float values.
template <int N, int DIR> __device__ __forceinline__ void cdf_dft(cdf *a)
{
    if constexpr (N == 2) {
        cdf_dft2<DIR>(a[0], a[1]);
    } else if constexpr (N == 4) {
        cdf_dft4<DIR>(a[0], a[1], a[2], a[3]);
    } else if constexpr (N == 8) {
        cdf_dft4<DIR>(a[0], a[2], a[4], a[6]);
        cdf_dft4<DIR>(a[1], a[3], a[5], a[7]);
        cdf_dft8_tail<DIR>(a);
    } else if constexpr (N == 16) {
        cdf_dft4<DIR>(a[0], a[4], a[8], a[12]);
        cdf_dft4<DIR>(a[1], a[5], a[9], a[13]);
        cdf_dft4<DIR>(a[2], a[6], a[10], a[14]);
        cdf_dft4<DIR>(a[3], a[7], a[11], a[15]);
        cdf_dft16_tail<DIR>(a);
    }
}

// The same transform of FP32 inputs x[0..N) into double-float outputs a[0..N)
// (the first level needs no lo parts).
template <int N, int DIR> __device__ __forceinline__ void cdf_dft_from(const float2 *x, cdf *a)
{
    if constexpr (N == 1) {
        a[0] = c_of(x[0]);
    } else if constexpr (N == 2) {
        a[0] = cdf_add0(x[0], x[1]);
        a[1] = cdf_sub0(x[0], x[1]);
    } else if constexpr (N == 4) {
        cdf_dft4_0<DIR>(x[0], x[1], x[2], x[3], a[0], a[1], a[2], a[3]);
    } else if constexpr (N == 8) {
        cdf_dft4_0<DIR>(x[0], x[2], x[4], x[6], a[0], a[2], a[4], a[6]);
        cdf_dft4_0<DIR>(x[1], x[3], x[5], x[7], a[1], a[3], a[5], a[7]);
        cdf_dft8_tail<DIR>(a);
    } else if constexpr (N == 16) {
        cdf_dft4_0<DIR>(x[0], x[4], x[8], x[12], a[0], a[4], a[8], a[12]);
        cdf_dft4_0<DIR>(x[1], x[5], x[9], x[13], a[1], a[5], a[9], a[13]);
        cdf_dft4_0<DIR>(x[2], x[6], x[10], x[14], a[2], a[6], a[10], a[14]);
        cdf_dft4_0<DIR>(x[3], x[7], x[11], x[15], a[3], a[7], a[11], a[15]);
        cdf_dft16_tail<DIR>(a);
    }
}

}  // namespace gpss
