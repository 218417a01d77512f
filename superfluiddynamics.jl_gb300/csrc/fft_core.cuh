// fft_core.cuh -- register-resident small DFTs (sizes 2, 4, 8, 16) for the
// directional split-step passes.
//
// Sign convention follows FFTW / AbstractFFTs, which the reference calls
// through plan_fft (src/Discretization/Plans.jl:847-848): the forward
// transform uses exp(-2 pi i jk/n) and is unnormalised; the backward one uses
// exp(+2 pi i jk/n).  DIR = -1 forward, DIR = +1 backward.
//
// Every routine takes its input in natural order in a[0..N) and leaves the
// output in natural frequency order in a[0..N).  With full unrolling the
// reordering is register renaming only.
#pragma once
#include <cuda_runtime.h>

namespace gpss {

template <typename T> struct vec2_of;
template <> struct vec2_of<float> { using type = float2; };
template <> struct vec2_of<double> { using type = double2; };
template <typename T> using vec2 = typename vec2_of<T>::type;

template <typename V> __device__ __forceinline__ V mk(decltype(V::x) x, decltype(V::x) y)
{
    V r; r.x = x; r.y = y; return r;
}
template <typename V> __device__ __forceinline__ V cadd(V a, V b) { return mk<V>(a.x + b.x, a.y + b.y); }
template <typename V> __device__ __forceinline__ V csub(V a, V b) { return mk<V>(a.x - b.x, a.y - b.y); }
// FP32: a complex add or subtract is one packed f32x2 instruction (sm_100
// and later), with the same round-to-nearest result per component as two
// scalar operations.
#ifndef GPSS_PACKED_F32
#define GPSS_PACKED_F32 1
#endif
#if GPSS_PACKED_F32
__device__ __forceinline__ unsigned long long pack_f2(float2 a)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}
__device__ __forceinline__ float2 unpack_f2(unsigned long long r)
{
    float2 a;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
    return a;
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b)
{
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pack_f2(a)), "l"(pack_f2(b)));
    return unpack_f2(d);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b)
{
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pack_f2(a)), "l"(pack_f2(b)));
    return unpack_f2(d);
}
// a * b + c and a * b lane by lane (one rounding each, as the scalar fma and mul)
__device__ __forceinline__ float2 pfma_f2(float2 a, float2 b, float2 c)
{
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(pack_f2(a)), "l"(pack_f2(b)), "l"(pack_f2(c)));
    return unpack_f2(d);
}
__device__ __forceinline__ float2 pmul_f2(float2 a, float2 b)
{
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pack_f2(a)), "l"(pack_f2(b)));
    return unpack_f2(d);
}
__device__ __forceinline__ float2 swap_f2(float2 a) { return make_float2(a.y, a.x); }
#endif
// FP32 DFT-4 butterflies and the w16^2k twiddles in packed form: a sign that
// differs between the lanes is a packed multiply-add of the lane-swapped
// value by a +-1 pair (exact products), rounding exactly as the scalar
// expressions it replaces (256^3 plain z pass 67.8 -> 67.1 us; the plain
// passes are not bound by their FMA pipes, and packed double-word constant
// products measured no faster than the scalar ones kept below)
#ifndef GPSS_PACKED_DFT
#define GPSS_PACKED_DFT GPSS_PACKED_F32
#endif
// a * b
template <typename V> __device__ __forceinline__ V cmul(V a, V b)
{
    return mk<V>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename V> __device__ __forceinline__ V cmulc(V a, V b)
{
    return mk<V>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename V> __device__ __forceinline__ V cscale(V a, decltype(V::x) s) { return mk<V>(a.x * s, a.y * s); }

// multiply by DIR*i: forward (DIR=-1) gives -i*a, backward +i*a
template <int DIR, typename V> __device__ __forceinline__ V mul_i(V a)
{
    if (DIR < 0) return mk<V>(a.y, -a.x);
    return mk<V>(-a.y, a.x);
}

// Constants of the 16-point DFT as double-word pairs (hi + lo): cos(pi/8),
// sin(pi/8), sqrt(1/2).  Multiplying by hi and adding the product with lo
// leaves only the random rounding of the arithmetic; a rounded constant alone
// would add the same relative error to the same frequency at every pass, an
// error that a split-step run accumulates over thousands of passes.
template <typename T> struct DftConst;
template <> struct DftConst<float> {
    static constexpr float C1h = 0.9238795042037964f, C1l = 2.830748968563057e-08f;
    static constexpr float S1h = 0.3826834261417389f, S1l = 6.2233507236442165e-09f;
    static constexpr float Hh = 0.7071067690849304f, Hl = 1.2101617485882343e-08f;
};
template <> struct DftConst<double> {
    static constexpr double C1h = 0.9238795325112867, C1l = 1.7645047084336677e-17;
    static constexpr double S1h = 0.3826834323650898, S1l = -1.0050772696461588e-17;
    static constexpr double Hh = 0.7071067811865476, Hl = -4.833646656726457e-17;
};

// a * (bh + bl), b given as a double-word complex constant
template <typename V> __device__ __forceinline__ V cmul2(V a, V bh, V bl)
{
    using T = decltype(V::x);
    const T lx = fma(a.x, bl.x, -a.y * bl.y);
    const T ly = fma(a.x, bl.y, a.y * bl.x);
    return mk<V>(fma(a.x, bh.x, fma(-a.y, bh.y, lx)), fma(a.x, bh.y, fma(a.y, bh.x, ly)));
}
// a * conj(bh + bl)
template <typename V> __device__ __forceinline__ V cmulc2(V a, V bh, V bl)
{
    using T = decltype(V::x);
    const T lx = fma(a.x, bl.x, a.y * bl.y);
    const T ly = fma(a.y, bl.x, -a.x * bl.y);
    return mk<V>(fma(a.x, bh.x, fma(a.y, bh.y, lx)), fma(a.y, bh.x, fma(-a.x, bh.y, ly)));
}
// t * (hi + lo) for a real double-word constant
template <typename T> __device__ __forceinline__ T rmul2(T t, T hi, T lo) { return fma(t, hi, t * lo); }

// Multiply by w16^m = exp(DIR * 2 pi i m / 16) for a compile-time m.
template <int M, int DIR, typename V> __device__ __forceinline__ V mul_w16(V a)
{
    using T = decltype(V::x);
    using K = DftConst<T>;
    constexpr int m = ((M % 16) + 16) % 16;
    constexpr bool packed = GPSS_PACKED_DFT && sizeof(T) == 4;
    if constexpr (m == 0) return a;
    else if constexpr (m == 4 && packed) return pmul_f2(swap_f2(a), make_float2((float)-DIR, (float)DIR));
    else if constexpr (m == 4) return mul_i<DIR>(a);
    else if constexpr (m == 8) return mk<V>(-a.x, -a.y);
    else if constexpr (m == 12 && packed) return pmul_f2(swap_f2(a), make_float2((float)DIR, (float)-DIR));
    else if constexpr (m == 12) return mul_i<-DIR>(a);
    else if constexpr (m % 2 == 0) {
        // odd multiple of pi/4: value = (sc + i ss) / sqrt2 with sc, ss = +-1
        constexpr int q = m / 2;  // 1, 3, 5, 7
        constexpr int sc = (q == 1 || q == 7) ? 1 : -1;
        constexpr int ss = ((q == 1 || q == 3) ? 1 : -1) * DIR;
        if constexpr (packed) {
            // (sc x - ss y, ss x + sc y) = sc (x - r y, y + r x), r = ss sc: one
            // exact packed fma of the swapped lanes by a sign pair, the sign sc
            // folded into sqrt(1/2)
            constexpr int r = ss * sc;
            const float2 t = pfma_f2(swap_f2(a), make_float2((float)-r, (float)r), a);
            const float hh = (float)sc * K::Hh, hl = (float)sc * K::Hl;
            return pfma_f2(t, make_float2(hh, hh), pmul_f2(t, make_float2(hl, hl)));
        } else {
            // (a.x + i a.y)(sc + i ss) = (sc a.x - ss a.y) + i (ss a.x + sc a.y)
            const T re = sc * a.x - ss * a.y;
            const T im = ss * a.x + sc * a.y;
            return mk<V>(rmul2(re, K::Hh, K::Hl), rmul2(im, K::Hh, K::Hl));
        }
    } else {
        // odd multiple of pi/8: cos/sin are +-C1 / +-S1
        constexpr int ci = (m == 1 || m == 15) ? 1 : (m == 3 || m == 13) ? 2 : (m == 5 || m == 11) ? -2 : -1;
        constexpr int si = (m == 1 || m == 7) ? 2 : (m == 3 || m == 5) ? 1 : (m == 9 || m == 15) ? -2 : -1;
        // ci/si: +-1 selects C1, +-2 selects S1 (cos(2 pi m/16), sin(2 pi m/16))
        const T crh = (ci == 1 || ci == -1) ? (T)(ci > 0 ? K::C1h : -K::C1h) : (T)(ci > 0 ? K::S1h : -K::S1h);
        const T crl = (ci == 1 || ci == -1) ? (T)(ci > 0 ? K::C1l : -K::C1l) : (T)(ci > 0 ? K::S1l : -K::S1l);
        const T srh = (si == 2 || si == -2) ? (T)(si > 0 ? K::S1h : -K::S1h) : (T)(si > 0 ? K::C1h : -K::C1h);
        const T srl = (si == 2 || si == -2) ? (T)(si > 0 ? K::S1l : -K::S1l) : (T)(si > 0 ? K::C1l : -K::C1l);
        return cmul2(a, mk<V>(crh, (T)DIR * srh), mk<V>(crl, (T)DIR * srl));
    }
}

template <int DIR, typename V> __device__ __forceinline__ void dft2(V &a0, V &a1)
{
    V t = a0;
    a0 = cadd(t, a1);
    a1 = csub(t, a1);
}

template <int DIR, typename V> __device__ __forceinline__ void dft4(V &a0, V &a1, V &a2, V &a3)
{
    V s02 = cadd(a0, a2), d02 = csub(a0, a2);
    V s13 = cadd(a1, a3), t = csub(a1, a3);
    a0 = cadd(s02, s13);
    a2 = csub(s02, s13);
    // a1 = d02 + DIR i t, a3 = d02 - DIR i t: per component, or (FP32) one
    // packed fma each of the lane-swapped t by a sign pair
    if constexpr (GPSS_PACKED_DFT && sizeof(decltype(V::x)) == 4) {
        const float2 ts = make_float2(t.y, t.x);
        a1 = pfma_f2(ts, make_float2((float)-DIR, (float)DIR), d02);
        a3 = pfma_f2(ts, make_float2((float)DIR, (float)-DIR), d02);
    } else if (DIR < 0) {
        a1 = mk<V>(d02.x + t.y, d02.y - t.x);
        a3 = mk<V>(d02.x - t.y, d02.y + t.x);
    } else {
        a1 = mk<V>(d02.x - t.y, d02.y + t.x);
        a3 = mk<V>(d02.x + t.y, d02.y - t.x);
    }
}

// In-place natural-order DFT of size N (1, 2, 4, 8, 16) on a[0..N).
template <int N, int DIR, typename V> __device__ __forceinline__ void dft(V *a)
{
    if constexpr (N == 1) {
    } else if constexpr (N == 2) {
        dft2<DIR>(a[0], a[1]);
    } else if constexpr (N == 4) {
        dft4<DIR>(a[0], a[1], a[2], a[3]);
    } else if constexpr (N == 8) {
        // j = j1 + 2 j2 ; k = k1 + 4 k2
        // inner DFT4 over j2 for j1 = 0, 1
        dft4<DIR>(a[0], a[2], a[4], a[6]);  // -> b[0][k1] at a[0],a[2],a[4],a[6]
        dft4<DIR>(a[1], a[3], a[5], a[7]);  // -> b[1][k1] at a[1],a[3],a[5],a[7]
        // twiddle w8^(j1 k1) = w16^(2 j1 k1) on j1 = 1
        a[3] = mul_w16<2, DIR>(a[3]);
        a[5] = mul_w16<4, DIR>(a[5]);
        a[7] = mul_w16<6, DIR>(a[7]);
        // outer DFT2 over j1 for each k1: X[k1 + 4 k2]
        V o[8];
#pragma unroll
        for (int k1 = 0; k1 < 4; k1++) {
            V u0 = a[2 * k1], u1 = a[2 * k1 + 1];
            dft2<DIR>(u0, u1);
            o[k1] = u0;
            o[k1 + 4] = u1;
        }
#pragma unroll
        for (int i = 0; i < 8; i++) a[i] = o[i];
    } else if constexpr (N == 16) {
        // j = j1 + 4 j2 ; k = k1 + 4 k2
        dft4<DIR>(a[0], a[4], a[8], a[12]);   // j1 = 0 -> b[0][k1] at a[0 + 4 k1]
        dft4<DIR>(a[1], a[5], a[9], a[13]);   // j1 = 1
        dft4<DIR>(a[2], a[6], a[10], a[14]);  // j1 = 2
        dft4<DIR>(a[3], a[7], a[11], a[15]);  // j1 = 3
        // twiddle w16^(j1 k1): element b[j1][k1] sits at a[j1 + 4 k1]
        a[5] = mul_w16<1, DIR>(a[5]);
        a[9] = mul_w16<2, DIR>(a[9]);
        a[13] = mul_w16<3, DIR>(a[13]);
        a[6] = mul_w16<2, DIR>(a[6]);
        a[10] = mul_w16<4, DIR>(a[10]);
        a[14] = mul_w16<6, DIR>(a[14]);
        a[7] = mul_w16<3, DIR>(a[7]);
        a[11] = mul_w16<6, DIR>(a[11]);
        a[15] = mul_w16<9, DIR>(a[15]);
        // outer DFT4 over j1 for each k1 -> X[k1 + 4 k2]
        V o[16];
#pragma unroll
        for (int k1 = 0; k1 < 4; k1++) {
            V u0 = a[4 * k1 + 0], u1 = a[4 * k1 + 1], u2 = a[4 * k1 + 2], u3 = a[4 * k1 + 3];
            dft4<DIR>(u0, u1, u2, u3);
            o[k1] = u0;
            o[k1 + 4] = u1;
            o[k1 + 8] = u2;
            o[k1 + 12] = u3;
        }
#pragma unroll
        for (int i = 0; i < 16; i++) a[i] = o[i];
    }
}

}  // namespace gpss
