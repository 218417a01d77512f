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
// reduced modulo 2 pi with a three-term Cody-Waite split of 2 pi, and only
// the reduced |r| <= pi is rounded to one float for sincosf.  The error of the
// reduced argument is therefore about one float ulp of r, independent of how
// large theta is.
#pragma once
#include <cuda_runtime.h>
#include "fft_core.cuh"

namespace gpss {

// 2 pi = PI2_A + PI2_B + PI2_C (floats; residual ~4e-23)
#define GPSS_PI2_A 6.2831854820251465f
#define GPSS_PI2_B (-1.7484555314695172e-07f)
#define GPSS_PI2_C (-6.8604980400235275e-15f)
#define GPSS_INV_PI2 0.15915493667125702f

struct DF { float hi, lo; };

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
template <> struct NLConst<float> {
    float bh, bl, dh, dl, bf, df;
    __device__ __forceinline__ NLConst(double b, double d)
    {
        bh = (float)b; bl = (float)(b - (double)bh);
        dh = (float)d; dl = (float)(d - (double)dh);
        bf = bh; df = dh;
    }
};

__device__ __forceinline__ double2 nl_apply(double2 v, double Vv, const NLConst<double> &c, bool imag)
{
    const double rho = v.x * v.x + v.y * v.y;          // abs2
    const double r = Vv + c.beta * rho;
    if (!imag) {
        const double t = -r * c.dt;
        double s, co;
        sincos(t, &s, &co);
        return make_double2(co * v.x - s * v.y, co * v.y + s * v.x);
    }
    const double f = exp(-r * c.dt);
    return make_double2(f * v.x, f * v.y);
}

__device__ __forceinline__ float2 nl_apply(float2 v, float Vv, const NLConst<float> &c, bool imag)
{
    if (imag) {
        const float rho = fmaf(v.x, v.x, v.y * v.y);
        const float f = expf(-fmaf(c.bf, rho, Vv) * c.df);
        return make_float2(f * v.x, f * v.y);
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
    // reduce theta modulo 2 pi (the first FMA is exact)
    const float k = rintf(th.hi * GPSS_INV_PI2);
    const float r1 = fmaf(-k, GPSS_PI2_A, th.hi);
    float corr = fmaf(-k, GPSS_PI2_B, th.lo);
    corr = fmaf(-k, GPSS_PI2_C, corr);
    const float red = r1 + corr;
    float sn, cs;
    sincosf(-red, &sn, &cs);
    return make_float2(cs * v.x - sn * v.y, cs * v.y + sn * v.x);
}

}  // namespace gpss
