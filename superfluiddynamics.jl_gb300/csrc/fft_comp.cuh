// fft_comp.cuh -- compensated FP32 arithmetic for the directional passes:
// small DFTs (sizes 2, 4, 8, 16) on two-float complex values whose high part
// lives on a power-of-two grid.
//
// A value is h + l (both float2: re, im).  Within one transform stage a
// thread picks a quantum q (a power of two, 2^-17 of a bound of the stage's
// input magnitudes) and keeps every h an integer multiple of q with
// |h| < 2^22 q.  Then:
//   * the sum of two h is exact (a multiple of q below 2^24 q), so a complex
//     add is two FP32 adds, h + h and l + l;
//   * a product h * c by a double-word constant c_hi + c_lo is split into
//     its rounding to the grid, fma(h, c_hi, C) - C with C = 1.5 * 2^23 q
//     (one rounding of the exact product), and the exact residual
//     fma(h, c_hi, -that), which goes to l together with h * c_lo + l * c_hi;
//   * l only collects residuals of size ~q, so its own FP32 rounding is
//     ~2^-24 q: about 2^-41 of the stage's largest input, far below FP32.
// A stage's values grow at most 16 sqrt(2) (< 32) times its input bound
// (one DFT-16 and unit-modulus twiddles; the kinetic phase factors include
// 1/n), which is the headroom 2^22 q = 2^5 * 2^E above a bound 2^E of the
// input.  Between stages (through shared memory) each thread re-grids the
// values it gathers on its own quantum: h' = RN_q'(h), l' = l + (h - h'),
// exact except for the l add.
//
// Cost per complex operation in packed f32x2 instructions: add 2, product by
// a double-word constant 12, entering the grid 3; against 8 / 16 for
// double-float arithmetic with TwoSum additions.
//
// This matters where the time stepping amplifies round-off: at the 256^3
// quantum-turbulence workload (coeffD = -0.0354, dt = 2.5e-3) the modes with
// |coeffD| |k|^2 dt near pi grow by about 2.7x per 25 steps (the split-step
// resonance), and the rounding noise of plain FP32 FFTs is the seed that
// they grow from.
//
// All operations are packed f32x2 instructions (add/sub/mul/fma.rn.f32x2)
// written as inline PTX, so the compiler can neither contract nor
// reassociate them ((x + C) - C must round x to the grid).
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
// (x, y) -> (y, x): register renaming or moves, no arithmetic
__device__ __forceinline__ float2 p_swap(float2 a) { return make_float2(a.y, a.x); }
// -x by a flip of the sign bit on the integer ALU.  GB300 runs packed f32x2
// and scalar FP32 instructions on the same FMA pipes, and a stream that mixes
// them issues at ~75 % of the rate of either kind alone (measured), so the
// compensated code keeps scalar FP32 instructions out: a sign that differs
// between the two lanes is either a packed multiply-add by a +-1 pair or,
// for run-time table constants, this integer xor (which co-issues).
__device__ __forceinline__ float negx(float a)
{
    unsigned u = __float_as_uint(a);
    asm("xor.b32 %0, %0, 0x80000000;" : "+r"(u));
    return __uint_as_float(u);
}
// a + DIR * i * b (S = (-DIR, DIR)) or a - DIR * i * b (S = (DIR, -DIR)) as
// one packed fma of the lane-swapped b by the sign pair: exact products by
// +-1, one rounding of the sum (exact for two values on one grid)
template <int SX, int SY> __device__ __forceinline__ float2 p_addrot(float2 a, float2 b)
{
    return p_fma(p_swap(b), make_float2((float)SX, (float)SY), a);
}

// ---------------------------------------------------------------- the grid --
// C = 1.5 * 2^23 * q (both lanes) for the quantum q = 2^(E - 17), E the
// exponent with m < 2^E.  q is kept a normal number (m below 2^-109 uses the
// smallest such grid; those values then ride in l at FP32 precision) and C
// finite.
__device__ __forceinline__ float2 grid_for(float m)
{
    int e = (int)((__float_as_uint(m) >> 23) & 0xffu);  // m in [2^(e-127), 2^(e-126))
    e = e < 17 ? 17 : (e > 247 ? 247 : e);
    const float C = __uint_as_float(((unsigned)(e + 7) << 23) | 0x400000u);
    return make_float2(C, C);
}

// bound of |re|, |im| over NV values (ALU min/max; the inputs of one stage)
template <int NV> __device__ __forceinline__ float absmax(const float2 *x)
{
    float m = 0.f;
#pragma unroll
    for (int i = 0; i < NV; i++) m = fmaxf(m, fmaxf(fabsf(x[i].x), fabsf(x[i].y)));
    return m;
}
template <int NV> __device__ __forceinline__ float absmax(const cdf *x)
{
    float mh = 0.f, ml = 0.f;
#pragma unroll
    for (int i = 0; i < NV; i++) {
        mh = fmaxf(mh, fmaxf(fabsf(x[i].h.x), fabsf(x[i].h.y)));
        ml = fmaxf(ml, fmaxf(fabsf(x[i].l.x), fabsf(x[i].l.y)));
    }
    return mh + ml;
}

// FP32 x onto the grid: h = RN_q(x), l = x - h (exact)
__device__ __forceinline__ cdf g_from(float2 x, float2 C)
{
    const float2 h = p_sub(p_add(x, C), C);
    return cdf{h, p_sub(x, h)};
}
// FP32 x times an FP32 scale s onto the grid: h = RN_q(x s), l = x s - h
// (the exact residual, one FP32 rounding of a value below q)
__device__ __forceinline__ cdf g_from_scaled(float2 x, float2 s, float2 C)
{
    const float2 h = p_sub(p_fma(x, s, C), C);
    return cdf{h, p_fma(x, s, p_neg(h))};
}
// a value from another thread's grid onto this one
__device__ __forceinline__ cdf g_regrid(const cdf &a, float2 C)
{
    const float2 h = p_sub(p_add(a.h, C), C);
    return cdf{h, p_add(a.l, p_sub(a.h, h))};
}
// h + l rounded once to FP32
__device__ __forceinline__ float2 c_round(const cdf &a) { return p_add(a.h, a.l); }

__device__ __forceinline__ cdf g_add(const cdf &a, const cdf &b) { return cdf{p_add(a.h, b.h), p_add(a.l, b.l)}; }
__device__ __forceinline__ cdf g_sub(const cdf &a, const cdf &b) { return cdf{p_sub(a.h, b.h), p_sub(a.l, b.l)}; }

// multiply by DIR*i (exact): (x, y) -> (-DIR y, DIR x), one packed multiply
// of the swapped lanes by a sign pair per part
template <int DIR> __device__ __forceinline__ cdf g_muli(const cdf &a)
{
    const float2 S = make_float2((float)-DIR, (float)DIR);
    return cdf{p_mul(p_swap(a.h), S), p_mul(p_swap(a.l), S)};
}
// a + DIR*i*b and a - DIR*i*b (exact on the grid)
template <int DIR> __device__ __forceinline__ cdf g_addi(const cdf &a, const cdf &b)
{
    return cdf{p_addrot<-DIR, DIR>(a.h, b.h), p_addrot<-DIR, DIR>(a.l, b.l)};
}
template <int DIR> __device__ __forceinline__ cdf g_subi(const cdf &a, const cdf &b)
{
    return cdf{p_addrot<DIR, -DIR>(a.h, b.h), p_addrot<DIR, -DIR>(a.l, b.l)};
}
__device__ __forceinline__ cdf g_neg(const cdf &a) { return cdf{p_neg(a.h), p_neg(a.l)}; }

// a * (hi + lo) for a real double-word constant
__device__ __forceinline__ cdf g_rmul2(const cdf &a, float hi, float lo, float2 C)
{
    const float2 H = make_float2(hi, hi), L = make_float2(lo, lo);
    const float2 h = p_sub(p_fma(a.h, H, C), C);
    const float2 r = p_fma(a.h, H, p_neg(h));
    return cdf{h, p_fma(a.h, L, p_fma(a.l, H, r))};
}

// a * (bh + bl), b a double-word complex constant, as packed pairs:
//   (re, im) = (ax, ax) * (bx, by) + (ay, ay) * (-by, bx)
// each of the two packed products is gridded with its exact residual;
// b2, bl2 are the rotated pairs (-by, bx) of bh, bl
__device__ __forceinline__ cdf g_cmul2r(const cdf &a, float2 bh, float2 b2, float2 bl, float2 bl2, float2 C)
{
    const float2 X = make_float2(a.h.x, a.h.x), Y = make_float2(a.h.y, a.h.y);
    const float2 u = p_sub(p_fma(X, bh, C), C);
    const float2 v = p_sub(p_fma(Y, b2, C), C);
    // the low parts in two independent chains (2% faster at 256^3 than one
    // chain; residual forms without the negated operands were 5% slower)
    float2 l1 = p_fma(X, bl, p_fma(X, bh, p_neg(u)));
    float2 l2 = p_fma(Y, bl2, p_fma(Y, b2, p_neg(v)));
    l1 = p_fma(make_float2(a.l.x, a.l.x), bh, l1);
    l2 = p_fma(make_float2(a.l.y, a.l.y), b2, l2);
    return cdf{p_add(u, v), p_add(l1, l2)};
}
// a * (bh + bl) for a run-time constant (a table entry): the one-lane signs
// of the rotated pairs on the integer ALU
__device__ __forceinline__ cdf g_cmul2(const cdf &a, float2 bh, float2 bl, float2 C)
{
    return g_cmul2r(a, bh, make_float2(negx(bh.y), bh.x), bl, make_float2(negx(bl.y), bl.x), C);
}
// a * conj(bh + bl) for a run-time constant: conj(b) = (bx, -by), rotated (by, bx)
__device__ __forceinline__ cdf g_cmulc2(const cdf &a, float2 bh, float2 bl, float2 C)
{
    return g_cmul2r(a, make_float2(bh.x, negx(bh.y)), p_swap(bh), make_float2(bl.x, negx(bl.y)), p_swap(bl), C);
}
// a * (bh + bl) for a compile-time constant: (re, im) = a (c, c) + swap(a) (-s, s)
// -- the constant pairs are immediates, so the data needs one lane swap per
// part instead of two lane broadcasts
__device__ __forceinline__ cdf g_cmul2k(const cdf &a, float2 bh, float2 bl, float2 C)
{
    const float2 c = make_float2(bh.x, bh.x), s = make_float2(-bh.y, bh.y);
    const float2 cl = make_float2(bl.x, bl.x), sl = make_float2(-bl.y, bl.y);
    const float2 sh = p_swap(a.h);
    const float2 u = p_sub(p_fma(a.h, c, C), C);
    const float2 v = p_sub(p_fma(sh, s, C), C);
    float2 l1 = p_fma(a.h, cl, p_fma(a.h, c, p_neg(u)));
    float2 l2 = p_fma(sh, sl, p_fma(sh, s, p_neg(v)));
    l1 = p_fma(a.l, c, l1);
    l2 = p_fma(p_swap(a.l), s, l2);
    return cdf{p_add(u, v), p_add(l1, l2)};
}

// multiply by w16^m = exp(DIR * 2 pi i m / 16) for a compile-time m
template <int M, int DIR> __device__ __forceinline__ cdf g_mulw16(const cdf &a, float2 C)
{
    using K = DftConst<float>;
    constexpr int m = ((M % 16) + 16) % 16;
    if constexpr (m == 0) return a;
    else if constexpr (m == 4) return g_muli<DIR>(a);
    else if constexpr (m == 8) return g_neg(a);
    else if constexpr (m == 12) return g_muli<-DIR>(a);
    else if constexpr (m % 2 == 0) {
        // odd multiple of pi/4: value = (sc + i ss) / sqrt2 with sc, ss = +-1.
        // a (sc + i ss) = sc (a + i (ss/sc) a): one exact packed fma of the
        // swapped lanes by a sign pair, then the product by sc sqrt(1/2)
        constexpr int q = m / 2;
        constexpr int sc = (q == 1 || q == 7) ? 1 : -1;
        constexpr int ss = ((q == 1 || q == 3) ? 1 : -1) * DIR;
        constexpr int r = ss * sc;  // a + i r a = (x - r y, y + r x)
        const cdf t{p_addrot<-r, r>(a.h, a.h), p_addrot<-r, r>(a.l, a.l)};
        return g_rmul2(t, (float)sc * K::Hh, (float)sc * K::Hl, C);
    } else {
        constexpr int ci = (m == 1 || m == 15) ? 1 : (m == 3 || m == 13) ? 2 : (m == 5 || m == 11) ? -2 : -1;
        constexpr int si = (m == 1 || m == 7) ? 2 : (m == 3 || m == 5) ? 1 : (m == 9 || m == 15) ? -2 : -1;
        const float crh = (ci == 1 || ci == -1) ? (ci > 0 ? K::C1h : -K::C1h) : (ci > 0 ? K::S1h : -K::S1h);
        const float crl = (ci == 1 || ci == -1) ? (ci > 0 ? K::C1l : -K::C1l) : (ci > 0 ? K::S1l : -K::S1l);
        const float srh = (si == 2 || si == -2) ? (si > 0 ? K::S1h : -K::S1h) : (si > 0 ? K::C1h : -K::C1h);
        const float srl = (si == 2 || si == -2) ? (si > 0 ? K::S1l : -K::S1l) : (si > 0 ? K::C1l : -K::C1l);
        return g_cmul2k(a, make_float2(crh, (float)DIR * srh), make_float2(crl, (float)DIR * srl), C);
    }
}

template <int DIR> __device__ __forceinline__ void g_dft2(cdf &a0, cdf &a1)
{
    const cdf t = a0;
    a0 = g_add(t, a1);
    a1 = g_sub(t, a1);
}

template <int DIR> __device__ __forceinline__ void g_dft4(cdf &a0, cdf &a1, cdf &a2, cdf &a3)
{
    const cdf s02 = g_add(a0, a2), d02 = g_sub(a0, a2);
    const cdf s13 = g_add(a1, a3), d13 = g_sub(a1, a3);
    a0 = g_add(s02, s13);
    a2 = g_sub(s02, s13);
    a1 = g_addi<DIR>(d02, d13);
    a3 = g_subi<DIR>(d02, d13);
}
// the same with a2 still to be multiplied by DIR*i (the twiddle w16^4 of the
// 16-point tail, folded into the butterfly)
template <int DIR> __device__ __forceinline__ void g_dft4_i2(cdf &a0, cdf &a1, cdf &a2, cdf &a3)
{
    const cdf s02 = g_addi<DIR>(a0, a2), d02 = g_subi<DIR>(a0, a2);
    const cdf s13 = g_add(a1, a3), d13 = g_sub(a1, a3);
    a0 = g_add(s02, s13);
    a2 = g_sub(s02, s13);
    a1 = g_addi<DIR>(d02, d13);
    a3 = g_subi<DIR>(d02, d13);
}

// the 16-point transform after its first radix-4 level: b[j1 + 4 k1] holds
// the inner DFT4 over j2 of x[j1 + 4 j2]; twiddles, outer DFT4s, natural order
template <int DIR> __device__ __forceinline__ void g_dft16_tail(cdf *a, float2 C)
{
    a[5] = g_mulw16<1, DIR>(a[5], C);
    a[9] = g_mulw16<2, DIR>(a[9], C);
    a[13] = g_mulw16<3, DIR>(a[13], C);
    a[6] = g_mulw16<2, DIR>(a[6], C);
    a[14] = g_mulw16<6, DIR>(a[14], C);
    a[7] = g_mulw16<3, DIR>(a[7], C);
    a[11] = g_mulw16<6, DIR>(a[11], C);
    a[15] = g_mulw16<9, DIR>(a[15], C);
    cdf o[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) {
        cdf u0 = a[4 * k1 + 0], u1 = a[4 * k1 + 1], u2 = a[4 * k1 + 2], u3 = a[4 * k1 + 3];
        if (k1 == 2) g_dft4_i2<DIR>(u0, u1, u2, u3);  // a[10] carries w16^4 = DIR*i
        else g_dft4<DIR>(u0, u1, u2, u3);
        o[k1] = u0;
        o[k1 + 4] = u1;
        o[k1 + 8] = u2;
        o[k1 + 12] = u3;
    }
#pragma unroll
    for (int i = 0; i < 16; i++) a[i] = o[i];
}

template <int DIR> __device__ __forceinline__ void g_dft8_tail(cdf *a, float2 C)
{
    a[3] = g_mulw16<2, DIR>(a[3], C);
    a[7] = g_mulw16<6, DIR>(a[7], C);
    cdf o[8];
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) {
        const cdf u0 = a[2 * k1], u1 = a[2 * k1 + 1];
        if (k1 == 2) {  // a[5] carries w16^4 = DIR*i
            o[k1] = g_addi<DIR>(u0, u1);
            o[k1 + 4] = g_subi<DIR>(u0, u1);
        } else {
            o[k1] = g_add(u0, u1);
            o[k1 + 4] = g_sub(u0, u1);
        }
    }
#pragma unroll
    for (int i = 0; i < 8; i++) a[i] = o[i];
}

// In-place natural-order DFT of size N (1, 2, 4, 8, 16) on gridded values
// (every h a multiple of the quantum of C).
template <int N, int DIR> __device__ __forceinline__ void g_dft(cdf *a, float2 C)
{
    if constexpr (N == 2) {
        g_dft2<DIR>(a[0], a[1]);
    } else if constexpr (N == 4) {
        g_dft4<DIR>(a[0], a[1], a[2], a[3]);
    } else if constexpr (N == 8) {
        g_dft4<DIR>(a[0], a[2], a[4], a[6]);
        g_dft4<DIR>(a[1], a[3], a[5], a[7]);
        g_dft8_tail<DIR>(a, C);
    } else if constexpr (N == 16) {
        g_dft4<DIR>(a[0], a[4], a[8], a[12]);
        g_dft4<DIR>(a[1], a[5], a[9], a[13]);
        g_dft4<DIR>(a[2], a[6], a[10], a[14]);
        g_dft4<DIR>(a[3], a[7], a[11], a[15]);
        g_dft16_tail<DIR>(a, C);
    }
}

}  // namespace gpss
