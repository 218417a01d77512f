// nl_phase.cuh -- the nonlinear/potential flow of the split step,
// src/NumModels/GrossPitaevskii/splitting.jl:205-209:
//     psi <- exp(-i (V + beta |psi|^2) dt) psi              (real time)
//     psi <- exp(-(V + beta |psi|^2) dt) psi                 (imaginary time)
//
// FP64 fields use the expression as written, in FP64.
//
// FP32 fields: GB300 runs FP64 arithmetic at a small fraction of its FP32
// rate, so instead of FP64 the phase argument theta = (V + beta|psi|^2) dt is
// formed in double-float arithmetic (an unevaluated sum of two floats,
// ~48-bit significand; Dekker's two-product and Knuth's two-sum via FMA),
// reduced modulo pi/2 with a three-term Cody-Waite split of pi/2, and only
// the reduced |f| <= pi/4 is rounded to one float.  sin f and cos f then come
// from their Taylor series (degree 9 and 10: truncation below 3e-9 relative
// on |f| <= pi/4, under half an FP32 ulp) and the quadrant.  The error of the
// reduced argument is about one float ulp of f, whatever the size of theta.
// Cells with |theta| <= 0.78 take a short path without reduction (below).
#pragma once
#include <cuda_runtime.h>
#include "fft_core.cuh"

namespace gpss {

// pi/2 = PIO2_A + PIO2_B + PIO2_C (floats; residual ~1e-23)
#define GPSS_PIO2_A 1.5707963705062866f
#define GPSS_PIO2_B (-4.371138828673793e-08f)
#define GPSS_PIO2_C (-1.7151245100058819e-15f)
#define GPSS_TWO_OVER_PI 0.6366197466850281f

struct DF { float hi, lo; };

// sin f and cos f for |f| <= pi/4 from the Taylor series
//   sin f = f - f^3/3! + f^5/5! - f^7/7! + f^9/9!
//   cos f = 1 - f^2/2! + f^4/4! - f^6/6! + f^8/8! - f^10/10!
// evaluated by Horner's rule in f^2.
__device__ __forceinline__ void sincos_reduced(float f, float *s, float *c)
{
    const float z = f * f;
    float ps = fmaf(z, 1.0f / 362880.0f, -1.0f / 5040.0f);
    ps = fmaf(z, ps, 1.0f / 120.0f);
    ps = fmaf(z, ps, -1.0f / 6.0f);
    *s = fmaf(f * z, ps, f);
    float pc = fmaf(z, -1.0f / 3628800.0f, 1.0f / 40320.0f);
    pc = fmaf(z, pc, -1.0f / 720.0f);
    pc = fmaf(z, pc, 1.0f / 24.0f);
    pc = fmaf(z, pc, -0.5f);
    *c = fmaf(z, pc, 1.0f);
}

__device__ __forceinline__ DF two_prod(float a, float b)
{
    float p = a * b;
    return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ DF two_sum(float a, float b)
{
    float s = a + b;
    float bb = s - a;
    float e = (a - (s - bb)) + (b - bb);
    return {s, e};
}

// Constants of one NL application, split once per thread.
template <typename T> struct NLConst;
template <> struct NLConst<double> {
    double beta, dt;
    __device__ __forceinline__ NLConst(double b, double d) : beta(b), dt(d) {}
};
// beta, dt and beta*dt as float pairs hi + lo.  Formed on the host for the
// pass kernels: GB300 executes FP64 at a small fraction of its FP32 rate, and
// a dozen FP64 operations per thread took a quarter of the FP64 pipe in a
// 256^3 pass.
struct NLSplit {
    float bh, bl, dh, dl, bdh, bdl;
};
__host__ __device__ inline NLSplit nl_split(double b, double d)
{
    NLSplit s;
    s.bh = (float)b; s.bl = (float)(b - (double)s.bh);
    s.dh = (float)d; s.dl = (float)(d - (double)s.dh);
    const double bd = b * d;
    s.bdh = (float)bd; s.bdl = (float)(bd - (double)s.bdh);
    return s;
}
template <> struct NLConst<float> {
    float bh, bl, dh, dl, bf, df, bdh, bdl;
    __device__ __forceinline__ NLConst(const NLSplit &s)
        : bh(s.bh), bl(s.bl), dh(s.dh), dl(s.dl), bf(s.bh), df(s.dh), bdh(s.bdh), bdl(s.bdl) {}
    __device__ __forceinline__ NLConst(double b, double d) : NLConst(nl_split(b, d)) {}
};
// the NL constants of a pass kernel: FP32 from the host-made split, FP64 as is
template <typename T> __device__ __forceinline__ NLConst<T> nl_const(const NLSplit &s, double b, double d);
template <> __device__ __forceinline__ NLConst<float> nl_const<float>(const NLSplit &s, double, double)
{
    return NLConst<float>(s);
}
template <> __device__ __forceinline__ NLConst<double> nl_const<double>(const NLSplit &, double b, double d)
{
    return NLConst<double>(b, d);
}

// Short path of the FP32 real-time factor, taken by every cell whose
// |theta| <= NL_SHORT_MAX < pi/4 (no reduction needed): theta from one-float
// rho with the constants beta*dt and dt kept as float pairs, so that their
// rounding adds no systematic phase drift; the error of theta is a few float
// ulps of theta itself, below 2e-7 absolute.
#define NL_SHORT_MAX 0.78f
__device__ __forceinline__ float nl_theta_short(float2 v, float Vv, const NLConst<float> &c)
{
    const float rho = fmaf(v.x, v.x, v.y * v.y);
    float th = fmaf(rho, c.bdh, rho * c.bdl);
    if (Vv != 0.0f) th = fmaf(Vv, c.dh, fmaf(Vv, c.dl, th));
    return th;
}
// For |theta| <= NL_TINY_MAX shorter series suffice: sin to degree 5 and cos
// to degree 6 truncate below 8e-10 relative there.
#define NL_TINY_MAX 0.125f
__device__ __forceinline__ float2 nl_factor_tiny(float th)
{
    const float z = th * th;
    const float sf = fmaf(th * z, fmaf(z, 1.0f / 120.0f, -1.0f / 6.0f), th);
    const float cf = fmaf(z, fmaf(z, fmaf(z, -1.0f / 720.0f, 1.0f / 24.0f), -0.5f), 1.0f);
    return make_float2(cf, -sf);
}
// For |theta| <= NL_MICRO_MAX: sin to degree 3 and cos to degree 4, truncation
// below 8e-9 absolute (a fifteenth of an FP32 ulp of the unit factor)
#define NL_MICRO_MAX 0.0625f
__device__ __forceinline__ float2 nl_factor_micro(float th)
{
    const float z = th * th;
    const float sf = fmaf(th * z, -1.0f / 6.0f, th);
    const float cf = fmaf(z, fmaf(z, 1.0f / 24.0f, -0.5f), 1.0f);
    return make_float2(cf, -sf);
}
// exp(-i theta) for |theta| <= NL_TINY_MAX: the micro series where
// |theta| <= NL_MICRO_MAX, else the tiny one, bitwise; branch-free (the two
// share their Horner steps but the innermost, picked by a select), so the
// cells of a warp do not diverge
__device__ __forceinline__ float2 nl_factor_tiny_cell(float th)
{
    const bool micro = fabsf(th) <= NL_MICRO_MAX;
    const float z = th * th;
    const float ps = micro ? -1.0f / 6.0f : fmaf(z, 1.0f / 120.0f, -1.0f / 6.0f);
    const float sf = fmaf(th * z, ps, th);
    const float pc = micro ? 1.0f / 24.0f : fmaf(z, -1.0f / 720.0f, 1.0f / 24.0f);
    const float cf = fmaf(z, fmaf(z, pc, -0.5f), 1.0f);
    return make_float2(cf, -sf);
}
// exp(-i theta) for |theta| <= NL_SHORT_MAX, by the series of its size class
__device__ __forceinline__ float2 nl_factor_short(float th)
{
    if (fabsf(th) <= NL_TINY_MAX) return nl_factor_tiny_cell(th);
    float sf, cf;
    sincos_reduced(th, &sf, &cf);
    return make_float2(cf, -sf);
}
// A bound on |nl_theta_short| over every cell with |psi|^2 <= rmax and
// |V| <= vmax, with a margin far above its rounding: a warp whose bound is
// <= NL_MICRO_MAX (NL_TINY_MAX, NL_SHORT_MAX) may call nl_factor_micro
// (nl_factor_tiny_cell, nl_factor_short) directly and still produce exactly
// what nl_factor gives cell by cell.
__device__ __forceinline__ float nl_theta_bound(float rmax, float vmax, const NLConst<float> &c)
{
    return (fabsf(c.bdh) * rmax + fabsf(c.dh) * vmax) * 1.001f;
}

// The factor f = exp(-i theta) (real time) or exp(-theta) (imaginary time,
// returned as (f, 0)) of one cell; the step is psi <- f psi (nl_rotate).  The
// discrete adjoint recomputes the same factor, so forward and backward agree
// to the bit.
__device__ __forceinline__ double2 nl_factor(double2 v, double Vv, const NLConst<double> &c, bool imag)
{
    const double rho = v.x * v.x + v.y * v.y;          // abs2
    const double r = Vv + c.beta * rho;
    if (!imag) {
        const double t = -r * c.dt;
        double s, co;
        sincos(t, &s, &co);
        return make_double2(co, s);
    }
    return make_double2(exp(-r * c.dt), 0.0);
}

template <typename V> __device__ __forceinline__ V nl_rotate(V f, V v)
{
    return mk<V>(f.x * v.x - f.y * v.y, f.x * v.y + f.y * v.x);
}

__device__ __forceinline__ double2 nl_apply(double2 v, double Vv, const NLConst<double> &c, bool imag)
{
    const double2 f = nl_factor(v, Vv, c, imag);
    if (imag) return make_double2(f.x * v.x, f.x * v.y);
    return nl_rotate(f, v);
}

__device__ __forceinline__ float2 nl_factor(float2 v, float Vv, const NLConst<float> &c, bool imag)
{
    if (imag) {
        const float rho = fmaf(v.x, v.x, v.y * v.y);
        return make_float2(expf(-fmaf(c.bf, rho, Vv) * c.df), 0.0f);
    }
    {
        const float th = nl_theta_short(v, Vv, c);
        if (fabsf(th) <= NL_SHORT_MAX) return nl_factor_short(th);
    }
    // rho = x^2 + y^2 in double-float
    DF px = two_prod(v.x, v.x), py = two_prod(v.y, v.y);
    DF rho = two_sum(px.hi, py.hi);
    rho.lo += px.lo + py.lo;
    // q = beta * rho
    DF q = two_prod(c.bh, rho.hi);
    q.lo += c.bh * rho.lo + c.bl * rho.hi;
    // s = V + q
    DF s = two_sum(Vv, q.hi);
    s.lo += q.lo;
    // theta = s * dt
    DF th = two_prod(s.hi, c.dh);
    th.lo += s.hi * c.dl + s.lo * c.dh;
    // reduce theta modulo pi/2 (the first FMA is exact: both terms are
    // multiples of the ulp of PIO2_A and the result is below 1 in magnitude)
    const float k = rintf(th.hi * GPSS_TWO_OVER_PI);
    const float r1 = fmaf(-k, GPSS_PIO2_A, th.hi);
    float corr = fmaf(-k, GPSS_PIO2_B, th.lo);
    corr = fmaf(-k, GPSS_PIO2_C, corr);
    const float f = r1 + corr;
    float sf, cf;
    sincos_reduced(f, &sf, &cf);
    // sin/cos of theta from the quadrant q = k mod 4
    const int quad = ((int)k) & 3;
    float st = (quad & 1) ? cf : sf;
    float ct = (quad & 1) ? sf : cf;
    if (quad == 1 || quad == 2) ct = -ct;
    if (quad >= 2) st = -st;
    return make_float2(ct, -st);  // exp(-i theta)
}

__device__ __forceinline__ float2 nl_apply(float2 v, float Vv, const NLConst<float> &c, bool imag)
{
    const float2 f = nl_factor(v, Vv, c, imag);
    if (imag) return make_float2(f.x * v.x, f.x * v.y);
    return nl_rotate(f, v);
}

// The FP32 real-time step of one cell as an out-of-line call, for the pass
// kernels' fallback when a warp's cells do not all take the short path: the
// double-float evaluation's temporaries then do not count against the
// registers of the kernel's common path.
static __device__ __noinline__ float2 nl_apply_real_cell(float2 v, float Vv, NLConst<float> c)
{
    return nl_apply(v, Vv, c, false);
}

}  // namespace gpss
