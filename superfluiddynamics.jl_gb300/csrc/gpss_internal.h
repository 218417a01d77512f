// gpss_internal.h -- declarations shared by the translation units of libgpss.
#pragma once
#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>
#include "pass_kernel.cuh"
#include "pass_generic.cuh"

namespace gpss {

// ---- host-side tables shared by the context, the batch and the no-alloc path

// (cos, sin) of 2 pi k / n in long double, reduced to the first octant so
// that the symmetric values are exact.
inline void unit_root(int64_t k, int64_t n, long double *cs, long double *sn)
{
    const long double half_pi = 1.570796326794896619231321691639751442L;
    k %= n;
    if (k < 0) k += n;
    const int64_t q = (4 * k) / n, r4 = 4 * k - q * n;
    long double cc, ss;
    if (2 * r4 <= n) {
        const long double a = half_pi * (long double)r4 / (long double)n;
        cc = cosl(a); ss = sinl(a);
    } else {
        const long double a = half_pi * (long double)(n - r4) / (long double)n;
        cc = sinl(a); ss = cosl(a);
    }
    switch (q) {
    case 0: *cs = cc; *sn = ss; break;
    case 1: *cs = -ss; *sn = cc; break;
    case 2: *cs = -cc; *sn = -ss; break;
    default: *cs = ss; *sn = -cc; break;
    }
}

// The twiddles w_n^{r k1} = exp(-2 pi i r k1 / n) of a line of n cells in the
// pass kernel's two orders: row 0 at m = k1*N2 + r (stage A), row 1 at
// m = r*N1 + k1 (stage B), N1 = min(n, 16), N2 = n / N1.
inline void twiddle_rows(int64_t n, std::vector<long double> &re, std::vector<long double> &im)
{
    const int64_t N1 = n <= 16 ? n : 16, N2 = n / N1;
    re.assign((size_t)(2 * n), 0.0L);
    im.assign((size_t)(2 * n), 0.0L);
    for (int64_t k1 = 0; k1 < N1; k1++)
        for (int64_t r = 0; r < N2; r++) {
            long double cs, sn;
            unit_root(r * k1, n, &cs, &sn);
            re[(size_t)(k1 * N2 + r)] = cs;
            im[(size_t)(k1 * N2 + r)] = -sn;
            re[(size_t)(n + r * N1 + k1)] = cs;
            im[(size_t)(n + r * N1 + k1)] = -sn;
        }
}

// Complex values in rows of n (long double) as double-word pairs of the field
// precision: per row hi[n] then lo[n], hi + lo = value.
template <typename T>
std::vector<vec2<T>> dw_split(const std::vector<long double> &re, const std::vector<long double> &im, int64_t n)
{
    const int64_t rows = (int64_t)re.size() / n;
    std::vector<vec2<T>> out((size_t)(2 * n * rows));
    for (int64_t r = 0; r < rows; r++)
        for (int64_t k = 0; k < n; k++) {
            const size_t i = (size_t)(r * n + k);
            const T hr = (T)re[i], hi = (T)im[i];
            vec2<T> h, l;
            h.x = hr;
            h.y = hi;
            l.x = (T)(re[i] - (long double)hr);
            l.y = (T)(im[i] - (long double)hi);
            out[(size_t)(r * 2 * n + k)] = h;
            out[(size_t)(r * 2 * n + n + k)] = l;
        }
    return out;
}

// pass launchers (pass_f32.cu / pass_f64.cu)
cudaError_t launch_pass_f32(int mode, bool xl, int n, const PassArgs<float> &a, int blocks,
                            cudaStream_t s);
cudaError_t launch_pass_f64(int mode, bool xl, int n, const PassArgs<double> &a, int blocks,
                            cudaStream_t s);
int pass_lines_per_cta_f32(int n, bool xl);
int pass_lines_per_cta_f64(int n, bool xl);
// pipelined fused pass (n in {64, 128, 256}; tiles of 4096/n lines)
cudaError_t launch_pipe_f32(bool xl, int n, const PassArgs<float> &a, int ntiles, cudaStream_t s);
cudaError_t launch_pipe_f64(bool xl, int n, const PassArgs<double> &a, int ntiles, cudaStream_t s);

// the generic-length pass (pass_gen.cu)
cudaError_t launch_gen_f32(int mode, const PassArgs<float> &a, const GenPlan &p, cudaStream_t s);
cudaError_t launch_gen_f64(int mode, const PassArgs<double> &a, const GenPlan &p, cudaStream_t s);

template <typename T> struct PassLauncher;
template <> struct PassLauncher<float> {
    static cudaError_t launch(int mode, bool xl, int n, const PassArgs<float> &a, int blocks,
                              cudaStream_t s) { return launch_pass_f32(mode, xl, n, a, blocks, s); }
    static int lines(int n, bool xl) { return pass_lines_per_cta_f32(n, xl); }
    static cudaError_t pipe(bool xl, int n, const PassArgs<float> &a, int ntiles, cudaStream_t s)
    {
        return launch_pipe_f32(xl, n, a, ntiles, s);
    }
    static cudaError_t gen(int mode, const PassArgs<float> &a, const GenPlan &p, cudaStream_t s)
    {
        return launch_gen_f32(mode, a, p, s);
    }
};
template <> struct PassLauncher<double> {
    static cudaError_t launch(int mode, bool xl, int n, const PassArgs<double> &a, int blocks,
                              cudaStream_t s) { return launch_pass_f64(mode, xl, n, a, blocks, s); }
    static int lines(int n, bool xl) { return pass_lines_per_cta_f64(n, xl); }
    static cudaError_t pipe(bool xl, int n, const PassArgs<double> &a, int ntiles, cudaStream_t s)
    {
        return launch_pipe_f64(xl, n, a, ntiles, s);
    }
    static cudaError_t gen(int mode, const PassArgs<double> &a, const GenPlan &p, cudaStream_t s)
    {
        return launch_gen_f64(mode, a, p, s);
    }
};

// Lines per tile of the generic pass: as many as fit about 96 KB of shared
// memory (two buffers), at most 16 (FP32) / 8 (FP64) -- 128-byte rows of
// adjacent columns for the y/z passes.
inline int gen_tile_lines(int n, int precision_bytes)
{
    const size_t per_line = 2 * (size_t)n * 2 * (size_t)precision_bytes;
    int W = (int)((96u * 1024u) / per_line);
    const int cap = precision_bytes == 4 ? 16 : 8;
    if (W > cap) W = cap;
    return W < 1 ? 1 : W;
}

// Is a line of n cells taken by the register kernel (a power of two up to
// 256)?  Otherwise the generic pass runs it.
inline bool reg_line(int64_t n) { return n >= 2 && n <= 256 && (n & (n - 1)) == 0; }

// pointwise kernels (pointwise.cu)
cudaError_t launch_f64_to_f32(const double *in, float *out, int64_t count, cudaStream_t s);
cudaError_t launch_f32_to_f64(const float *in, double *out, int64_t count, cudaStream_t s);
template <typename T>
cudaError_t launch_mul_phase(vec2<T> *data, const vec2<T> *phase, int64_t prow, int axis,
                             const int64_t *n, int64_t total, cudaStream_t s);
template <typename T>
cudaError_t launch_nl(vec2<T> *psi, const T *V, double beta, double dt, int imag, int64_t total,
                      cudaStream_t s);
template <typename T>
cudaError_t launch_scale(vec2<T> *psi, const double *scale, int64_t total, cudaStream_t s);
// implicit schemes (implicit.cu); the scheme numbers are the GPSS_IMPLICIT_* of gpss.h
enum {
    IM_SCHEME_BE = 0, IM_SCHEME_BE_NOPRE = 1, IM_SCHEME_CN = 2, IM_SCHEME_CN_QN = 3, IM_SCHEME_CN_T = 4,
    IM_SCHEME_CN_QN_T = 5
};
template <typename T>
cudaError_t im_prep_be(const vec2<T> *phi, const T *V, double beta, double dt, int scheme, vec2<T> *M, T *Anl,
                       vec2<T> *b, int64_t total, cudaStream_t s);
template <typename T>
cudaError_t im_prep_cn(const vec2<T> *phi, const vec2<T> *phi1, const T *V, double beta, double dt, int scheme,
                       vec2<T> *psim, T *Anl, vec2<T> *Anl2, vec2<T> *M, int64_t total, cudaStream_t s);
template <typename T>
cudaError_t im_rhs_cn(const vec2<T> *phi, const vec2<T> *phi1, const vec2<T> *psim, const vec2<T> *lap, const T *V,
                      double beta, double dt, int tsch, vec2<T> *b, int64_t total, cudaStream_t s);
template <typename T>
cudaError_t im_op(const vec2<T> *x, const vec2<T> *lap, int scheme, double dt, const vec2<T> *M, const T *Anl,
                  const vec2<T> *Anl2, const vec2<T> *b, int precond, vec2<T> *out, int64_t total, cudaStream_t s);
template <typename T>
cudaError_t im_dot2(const vec2<T> *a1, const vec2<T> *b1, const vec2<T> *a2, const vec2<T> *b2, int64_t total,
                    double *partials, double *out, cudaStream_t s);
template <typename T>
cudaError_t im_axmy(vec2<T> *out, const vec2<T> *x, double alpha, const vec2<T> *y, int64_t total, cudaStream_t s);

// The scalars of one BiCGStab solve (krylov.jl:1-67), kept on the device so
// that iterations run without a host round trip: the dot products are
// finished on the device, one thread forms alpha, omega, beta and the
// stopping test from them in FP64 (the same operations, in the same order, as
// the reference), and the vector updates read them from here.  Once `done`
// is set (converged, out of iterations, or a non-finite residual) every later
// update of the same solve is a no-op, so the host may issue iterations in
// chunks and read this back once per chunk.
struct KrylovDev {
    double normb, rr2, alpha, omega, beta;
    int done, niter, nonfinite, it;
};
cudaError_t kry_init(KrylovDev *K, const double *dots, cudaStream_t s);
cudaError_t kry_alpha(KrylovDev *K, const double *dots, cudaStream_t s);
cudaError_t kry_omega(KrylovDev *K, const double *dots, cudaStream_t s);
cudaError_t kry_check(KrylovDev *K, const double *dots, double tol, int nkrylov, cudaStream_t s);
// s = r - alpha Ap;  phi = (phi + alpha p) + omega s, r = s - omega As;  p = r + beta (p - omega Ap)
template <typename T>
cudaError_t im_axmy_k(vec2<T> *out, const vec2<T> *x, const vec2<T> *y, const KrylovDev *K, int64_t total,
                      cudaStream_t s);
template <typename T>
cudaError_t im_update_k(vec2<T> *phi, const vec2<T> *p, const vec2<T> *sv, const vec2<T> *As, vec2<T> *r,
                        const KrylovDev *K, int64_t total, cudaStream_t s);
template <typename T>
cudaError_t im_pdir_k(vec2<T> *p, const vec2<T> *r, const vec2<T> *Ap, const KrylovDev *K, int64_t total,
                      cudaStream_t s);
template <typename T>
cudaError_t im_mfield(vec2<T> *out, const vec2<T> *M, const vec2<T> *x, int64_t total, cudaStream_t s);

// explicit Runge-Kutta helpers (pointwise.cu)
template <typename T>
cudaError_t launch_nl_term(const vec2<T> *q, const T *V, double beta, vec2<T> *t, int64_t total, cudaStream_t s);
template <typename T>
cudaError_t launch_rk_combine(const vec2<T> *k, const vec2<T> *t, const vec2<T> *psi0, vec2<T> *acc, vec2<T> *out,
                              int acc_mode, double acc_w, double cf, int from_acc, int64_t total, cudaStream_t s);

// discrete adjoint (adjoint.cu)
// z[0..1] = dV * sum conj(a) b; partials needs 2 * 152 * 8 doubles
template <typename T>
cudaError_t launch_overlap(const vec2<T> *a, const vec2<T> *b, int64_t total, double *partials, double dV,
                           double *z, cudaStream_t s);
template <typename T>
cudaError_t launch_seed(vec2<T> *g, const vec2<T> *target, const double *z, double dV, int64_t total,
                        cudaStream_t s);
template <typename T>
cudaError_t launch_nl_adjoint(vec2<T> *g, const vec2<T> *psi_in, const T *V, double *dLdV, double beta, double dt,
                              int64_t total, cudaStream_t s);
}  // namespace gpss
