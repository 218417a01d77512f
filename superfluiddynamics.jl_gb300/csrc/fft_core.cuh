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

// Multiply by w16^m = exp(DIR * 2 pi i m / 16) for a compile-time m.
template <int M, int DIR, typename V> __device__ __forceinline__ V mul_w16(V a)
{
    using T = decltype(V::x);
    constexpr int m = ((M % 16) + 16) % 16;
    const T C1 = (T)0.92387953251128675613;  // cos(pi/8)
    const T S1 = (T)0.38268343236508977173;  // sin(pi/8)
    const T H = (T)0.70710678118654752440;   // sqrt(1/2)
    // angle = DIR * 2 pi m / 16 ; value = cos(angle) + i sin(angle)
    if constexpr (m == 0) return a;
    else if constexpr (m == 4) return mul_i<DIR>(a);
    else if constexpr (m == 8) return mk<V>(-a.x, -a.y);
    else if constexpr (m == 12) return mul_i<-DIR>(a);
    else if constexpr (m % 2 == 0) {
        // odd multiple of pi/4: (+-1 +- i)/sqrt2
        constexpr int q = m / 2;  // 1, 3, 5, 7
        const T cr = (q == 1 || q == 7) ? H : -H;
        const T si = (q == 1 || q == 3) ? (T)DIR * H : -(T)DIR * H;
        return mk<V>((a.x * cr - a.y * si), (a.x * si + a.y * cr));
    } else {
        // odd multiple of pi/8
        T cr, sr;  // cos, sin of 2 pi m/16 (positive orientation)
        if constexpr (m == 1) { cr = C1; sr = S1; }
        else if constexpr (m == 3) { cr = S1; sr = C1; }
        else if constexpr (m == 5) { cr = -S1; sr = C1; }
        else if constexpr (m == 7) { cr = -C1; sr = S1; }
        else if constexpr (m == 9) { cr = -C1; sr = -S1; }
        else if constexpr (m == 11) { cr = -S1; sr = -C1; }
        else if constexpr (m == 13) { cr = S1; sr = -C1; }
        else { cr = C1; sr = -S1; }  // 15
        const T si = (T)DIR * sr;
        return mk<V>(a.x * cr - a.y * si, a.x * si + a.y * cr);
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
    V s13 = cadd(a1, a3), d13 = mul_i<DIR>(csub(a1, a3));
    a0 = cadd(s02, s13);
    a2 = csub(s02, s13);
    a1 = cadd(d02, d13);
    a3 = csub(d02, d13);
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
