// implicit.cu -- pointwise kernels of the implicit imaginary-/real-time
// schemes (src/NumModels/GrossPitaevskii/backward-euler.jl, crank-nicolson.jl)
// and of their BiCGStab solver (src/NumModels/krylov.jl:1-67).  lapRot comes
// from the fused directional passes (the host chains them); everything else of
// a Krylov iteration is here.
#include "gpss_internal.h"
#include "pdl.cuh"

namespace gpss {

static int im_grid(int64_t count)
{
    int64_t b = (count + 255) / 256;
    const int64_t cap = 152 * 8;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

#define GRID_LOOP(e, total) \
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (total); e += (int64_t)gridDim.x * blockDim.x)

// ---- setup of a time step / Newton iteration

// BackwardEuler:          M = 1 / (1/dt + V + beta|phi|^2),  b = M phi / dt
// BackwardEulerNoPrecond: Anl = V + beta|phi|^2,             b = phi / dt
template <typename T>
__global__ void k_im_prep_be(const vec2<T> *__restrict__ phi, const T *__restrict__ V, double beta, double idt,
                             double dt, int scheme, vec2<T> *__restrict__ M, T *__restrict__ Anl,
                             vec2<T> *__restrict__ b, int64_t total)
{
    pdl_enter();
    GRID_LOOP(e, total) {
        const vec2<T> p = phi[e];
        const T vv = V ? V[e] : (T)0;
        const T a2 = p.x * p.x + p.y * p.y;
        if (scheme == IM_SCHEME_BE) {
            const T m = (T)1.0 / ((T)idt + vv + (T)beta * a2);
            M[e] = mk<vec2<T>>(m, (T)0);
            b[e] = mk<vec2<T>>(m * p.x / (T)dt, m * p.y / (T)dt);
        } else {
            Anl[e] = vv + (T)beta * a2;
            b[e] = mk<vec2<T>>(p.x / (T)dt, p.y / (T)dt);
        }
    }
}

// Crank-Nicolson schemes, one Newton iteration: psi = (phi1 + phi)/2,
// Anl = V + (2 or 3) beta|psi|^2, Anl2 = beta psi^2,
// M = 1 / (1/dt + d) (stationary) or 1 / (i/dt - d) (T schemes), d = (V + 3 beta|psi|^2)/2
template <typename T>
__global__ void k_im_prep_cn(const vec2<T> *__restrict__ phi, const vec2<T> *__restrict__ phi1,
                             const T *__restrict__ V, double beta, double idt, int scheme,
                             vec2<T> *__restrict__ psim, T *__restrict__ Anl, vec2<T> *__restrict__ Anl2,
                             vec2<T> *__restrict__ M, int64_t total)
{
    pdl_enter();
    const bool newton = scheme == IM_SCHEME_CN || scheme == IM_SCHEME_CN_T;
    const bool tsch = scheme == IM_SCHEME_CN_T || scheme == IM_SCHEME_CN_QN_T;
    const T bt = (T)beta;
    GRID_LOOP(e, total) {
        const vec2<T> a = phi1[e], p = phi[e];
        const vec2<T> q = mk<vec2<T>>((T)0.5 * (a.x + p.x), (T)0.5 * (a.y + p.y));
        psim[e] = q;
        const T vv = V ? V[e] : (T)0;
        const T a2 = q.x * q.x + q.y * q.y;
        Anl[e] = vv + (newton ? (T)2 : (T)3) * bt * a2;
        const T qr = bt * q.x, qi = bt * q.y;
        Anl2[e] = mk<vec2<T>>(qr * q.x - qi * q.y, qr * q.y + qi * q.x);
        const T d = (vv + (T)3 * bt * a2) * (T)0.5;
        if (!tsch) {
            M[e] = mk<vec2<T>>((T)1.0 / ((T)idt + d), (T)0);
        } else {
            const T zr = -d, zi = (T)idt, den = zr * zr + zi * zi;
            M[e] = mk<vec2<T>>(zr / den, -zi / den);
        }
    }
}

// b = (1/dt)(phi1 - phi) + f psi - lap     (stationary)
//   = (i/dt)(phi1 - phi) - f psi + lap     (T schemes),   f = V + beta|psi|^2, lap = lapRot(psi)
template <typename T>
__global__ void k_im_rhs_cn(const vec2<T> *__restrict__ phi, const vec2<T> *__restrict__ phi1,
                            const vec2<T> *__restrict__ psim, const vec2<T> *__restrict__ lap,
                            const T *__restrict__ V, double beta, double idt, int tsch, vec2<T> *__restrict__ b,
                            int64_t total)
{
    pdl_enter();
    GRID_LOOP(e, total) {
        const vec2<T> q = psim[e], L = lap[e], a = phi1[e], p = phi[e];
        const T f = (V ? V[e] : (T)0) + (T)beta * (q.x * q.x + q.y * q.y);
        const T dr = a.x - p.x, di = a.y - p.y, id = (T)idt;
        if (!tsch)
            b[e] = mk<vec2<T>>((id * dr + f * q.x) - L.x, (id * di + f * q.y) - L.y);
        else
            b[e] = mk<vec2<T>>((-(id * di) - f * q.x) + L.x, (id * dr - f * q.y) + L.y);
    }
}

// out = prodA(x) given lap = lapRot(x) (backward-euler.jl:87-90, 179-189;
// crank-nicolson.jl:112-114, 234-236, 356-359, 478-481); bsub: out = b - prodA(x);
// precond: out = M * out
template <typename T>
__global__ void k_im_op(const vec2<T> *__restrict__ x, const vec2<T> *__restrict__ lap, int scheme, double idt,
                        const vec2<T> *__restrict__ M, const T *__restrict__ Anl, const vec2<T> *__restrict__ Anl2,
                        const vec2<T> *__restrict__ b, int precond, vec2<T> *__restrict__ out, int64_t total)
{
    pdl_enter();
    const T id = (T)idt, h = (T)0.5;
    GRID_LOOP(e, total) {
        const vec2<T> v = x[e], L = lap[e];
        T ox, oy;
        switch (scheme) {
        case IM_SCHEME_BE: {
            const T m = M[e].x;
            ox = v.x - m * L.x; oy = v.y - m * L.y;
            break;
        }
        case IM_SCHEME_BE_NOPRE: {
            const T a = id + Anl[e];
            ox = a * v.x - L.x; oy = a * v.y - L.y;
            break;
        }
        case IM_SCHEME_CN: {
            const T a = id + Anl[e];
            const vec2<T> q = Anl2[e];
            const T hx = h * q.x, hy = h * q.y;
            ox = (a * v.x + (hx * v.x + hy * v.y)) - h * L.x;
            oy = (a * v.y + (hy * v.x - hx * v.y)) - h * L.y;
            break;
        }
        case IM_SCHEME_CN_QN: {
            const T a = id + Anl[e] * h;
            ox = a * v.x - h * L.x; oy = a * v.y - h * L.y;
            break;
        }
        case IM_SCHEME_CN_T: {
            const T ar = -h * Anl[e];
            const vec2<T> q = Anl2[e];
            const T hx = h * q.x, hy = h * q.y;
            ox = ((ar * v.x - id * v.y) - (hx * v.x + hy * v.y)) + h * L.x;
            oy = ((ar * v.y + id * v.x) - (hy * v.x - hx * v.y)) + h * L.y;
            break;
        }
        default: {  // IM_SCHEME_CN_QN_T
            const T ar = -(Anl[e] * h);
            ox = (ar * v.x - id * v.y) + h * L.x;
            oy = (ar * v.y + id * v.x) + h * L.y;
            break;
        }
        }
        if (b) {
            const vec2<T> bb = b[e];
            ox = bb.x - ox; oy = bb.y - oy;
        }
        if (precond) {
            const vec2<T> m = M[e];
            const T tx = m.x * ox - m.y * oy, ty = m.x * oy + m.y * ox;
            ox = tx; oy = ty;
        }
        out[e] = mk<vec2<T>>(ox, oy);
    }
}

// ---- BiCGStab vector operations (krylov.jl)

// partials[2 * block + {0, 1}] = per-CTA sums of Re(a1 conj b1), Re(a2 conj b2) in FP64
template <typename T>
__global__ void k_im_dot2(const vec2<T> *__restrict__ a1, const vec2<T> *__restrict__ b1,
                          const vec2<T> *__restrict__ a2, const vec2<T> *__restrict__ b2, int64_t total,
                          double *__restrict__ partials)
{
    pdl_enter();
    __shared__ double s1[256], s2[256];
    double x1 = 0.0, x2 = 0.0;
    GRID_LOOP(e, total) {
        const vec2<T> p = a1[e], q = b1[e];
        x1 += (double)p.x * (double)q.x + (double)p.y * (double)q.y;
        if (a2) {
            const vec2<T> u = a2[e], w = b2[e];
            x2 += (double)u.x * (double)w.x + (double)u.y * (double)w.y;
        }
    }
    s1[threadIdx.x] = x1;
    s2[threadIdx.x] = x2;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            s1[threadIdx.x] += s1[threadIdx.x + o];
            s2[threadIdx.x] += s2[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = s1[0];
        partials[2 * blockIdx.x + 1] = s2[0];
    }
}

// out[0..1] = the sums of the partials (fixed order), one CTA
__global__ void k_im_dot_finish(const double *__restrict__ partials, int nblocks, double *__restrict__ out)
{
    pdl_enter();
    __shared__ double s1[256], s2[256];
    double x1 = 0.0, x2 = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
        x1 += partials[2 * i];
        x2 += partials[2 * i + 1];
    }
    s1[threadIdx.x] = x1;
    s2[threadIdx.x] = x2;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            s1[threadIdx.x] += s1[threadIdx.x + o];
            s2[threadIdx.x] += s2[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = s1[0];
        out[1] = s2[0];
    }
}

// out = x - alpha y
template <typename T>
__global__ void k_im_axmy(vec2<T> *__restrict__ out, const vec2<T> *__restrict__ x, double alpha,
                          const vec2<T> *__restrict__ y, int64_t total)
{
    pdl_enter();
    const T a = (T)alpha;
    GRID_LOOP(e, total) {
        const vec2<T> u = x[e], w = y[e];
        out[e] = mk<vec2<T>>(u.x - a * w.x, u.y - a * w.y);
    }
}

// ---- the solve's scalars on the device (one thread each; KrylovDev)

// normb = sqrt(b.b) (or |M b|), a fresh solve
__global__ void k_kry_init(KrylovDev *K, const double *__restrict__ dots)
{
    pdl_enter();
    K->normb = sqrt(dots[0]);
    K->rr2 = K->alpha = K->omega = K->beta = 0.0;
    K->done = K->niter = K->nonfinite = K->it = 0;
}
// iteration it: rr2 = r.r2, alpha = rr2 / (Ap.r2)
__global__ void k_kry_alpha(KrylovDev *K, const double *__restrict__ dots)
{
    pdl_enter();
    if (K->done) return;
    K->it += 1;
    K->rr2 = dots[0];
    K->alpha = dots[0] / dots[1];
}
// omega = (As.s) / (As.As)
__global__ void k_kry_omega(KrylovDev *K, const double *__restrict__ dots)
{
    pdl_enter();
    if (K->done) return;
    K->omega = dots[0] / dots[1];
}
// the stopping test on |r| / normb, then niter = it and beta = (r.r2) / rr2 *
// alpha / omega; the last allowed iteration ends the solve
__global__ void k_kry_check(KrylovDev *K, const double *__restrict__ dots, double tol, int nkrylov)
{
    pdl_enter();
    if (K->done) return;
    const double rr = dots[0];
    if (!isfinite(rr)) {
        K->nonfinite = 1;
        K->done = 1;
        return;
    }
    if (sqrt(rr) / K->normb < tol) {
        K->done = 1;
        return;
    }
    K->niter = K->it;
    K->beta = dots[1] / K->rr2 * K->alpha / K->omega;
    if (K->it >= nkrylov) K->done = 1;
}

// s = r - alpha Ap (alpha from the device)
template <typename T>
__global__ void k_im_axmy_k(vec2<T> *__restrict__ out, const vec2<T> *__restrict__ x, const vec2<T> *__restrict__ y,
                            const KrylovDev *__restrict__ K, int64_t total)
{
    pdl_enter();
    if (K->done) return;
    const T a = (T)K->alpha;
    GRID_LOOP(e, total) {
        const vec2<T> u = x[e], w = y[e];
        out[e] = mk<vec2<T>>(u.x - a * w.x, u.y - a * w.y);
    }
}

// phi = (phi + alpha p) + omega s;  r = s - omega As
template <typename T>
__global__ void k_im_update_k(vec2<T> *__restrict__ phi, const vec2<T> *__restrict__ p,
                              const vec2<T> *__restrict__ s, const vec2<T> *__restrict__ As, vec2<T> *__restrict__ r,
                              const KrylovDev *__restrict__ K, int64_t total)
{
    pdl_enter();
    if (K->done) return;
    const T a = (T)K->alpha, w = (T)K->omega;
    GRID_LOOP(e, total) {
        const vec2<T> f = phi[e], pp = p[e], ss = s[e], aa = As[e];
        phi[e] = mk<vec2<T>>((f.x + a * pp.x) + w * ss.x, (f.y + a * pp.y) + w * ss.y);
        r[e] = mk<vec2<T>>(ss.x - w * aa.x, ss.y - w * aa.y);
    }
}

// p = r + beta (p - omega Ap)
template <typename T>
__global__ void k_im_pdir_k(vec2<T> *__restrict__ p, const vec2<T> *__restrict__ r, const vec2<T> *__restrict__ Ap,
                            const KrylovDev *__restrict__ K, int64_t total)
{
    pdl_enter();
    if (K->done) return;
    const T bt = (T)K->beta, w = (T)K->omega;
    GRID_LOOP(e, total) {
        const vec2<T> pp = p[e], rr = r[e], aa = Ap[e];
        const T qx = pp.x - w * aa.x, qy = pp.y - w * aa.y;
        p[e] = mk<vec2<T>>(rr.x + bt * qx, rr.y + bt * qy);
    }
}

// out = M x (the preconditioner applied to a vector)
template <typename T>
__global__ void k_im_mfield(vec2<T> *__restrict__ out, const vec2<T> *__restrict__ M, const vec2<T> *__restrict__ x,
                            int64_t total)
{
    pdl_enter();
    GRID_LOOP(e, total) {
        const vec2<T> m = M[e], v = x[e];
        out[e] = mk<vec2<T>>(m.x * v.x - m.y * v.y, m.x * v.y + m.y * v.x);
    }
}

// ---- host launchers

template <typename T>
cudaError_t im_mfield(vec2<T> *out, const vec2<T> *M, const vec2<T> *x, int64_t total, cudaStream_t s)
{
    launch_pdl(k_im_mfield<T>, dim3(im_grid(total)), dim3(256), 0, s, out, M, x, total);
    return cudaGetLastError();
}

template <typename T>
cudaError_t im_prep_be(const vec2<T> *phi, const T *V, double beta, double dt, int scheme, vec2<T> *M, T *Anl,
                       vec2<T> *b, int64_t total, cudaStream_t s)
{
    launch_pdl(k_im_prep_be<T>, dim3(im_grid(total)), dim3(256), 0, s,
               phi, V, beta, 1.0 / dt, dt, scheme, M, Anl, b, total);
    return cudaGetLastError();
}

template <typename T>
cudaError_t im_prep_cn(const vec2<T> *phi, const vec2<T> *phi1, const T *V, double beta, double dt, int scheme,
                       vec2<T> *psim, T *Anl, vec2<T> *Anl2, vec2<T> *M, int64_t total, cudaStream_t s)
{
    launch_pdl(k_im_prep_cn<T>, dim3(im_grid(total)), dim3(256), 0, s,
               phi, phi1, V, beta, 1.0 / dt, scheme, psim, Anl, Anl2, M, total);
    return cudaGetLastError();
}

template <typename T>
cudaError_t im_rhs_cn(const vec2<T> *phi, const vec2<T> *phi1, const vec2<T> *psim, const vec2<T> *lap, const T *V,
                      double beta, double dt, int tsch, vec2<T> *b, int64_t total, cudaStream_t s)
{
    launch_pdl(k_im_rhs_cn<T>, dim3(im_grid(total)), dim3(256), 0, s,
               phi, phi1, psim, lap, V, beta, 1.0 / dt, tsch, b, total);
    return cudaGetLastError();
}

template <typename T>
cudaError_t im_op(const vec2<T> *x, const vec2<T> *lap, int scheme, double dt, const vec2<T> *M, const T *Anl,
                  const vec2<T> *Anl2, const vec2<T> *b, int precond, vec2<T> *out, int64_t total, cudaStream_t s)
{
    launch_pdl(k_im_op<T>, dim3(im_grid(total)), dim3(256), 0, s,
               x, lap, scheme, 1.0 / dt, M, Anl, Anl2, b, precond, out, total);
    return cudaGetLastError();
}

template <typename T>
cudaError_t im_dot2(const vec2<T> *a1, const vec2<T> *b1, const vec2<T> *a2, const vec2<T> *b2, int64_t total,
                    double *partials, double *out, cudaStream_t s)
{
    const int g = im_grid(total);
    launch_pdl(k_im_dot2<T>, dim3(g), dim3(256), 0, s, a1, b1, a2, b2, total, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    launch_pdl(k_im_dot_finish, dim3(1), dim3(256), 0, s, partials, g, out);
    return cudaGetLastError();
}

template <typename T>
cudaError_t im_axmy(vec2<T> *out, const vec2<T> *x, double alpha, const vec2<T> *y, int64_t total, cudaStream_t s)
{
    launch_pdl(k_im_axmy<T>, dim3(im_grid(total)), dim3(256), 0, s, out, x, alpha, y, total);
    return cudaGetLastError();
}

cudaError_t kry_init(KrylovDev *K, const double *dots, cudaStream_t s)
{
    launch_pdl(k_kry_init, dim3(1), dim3(1), 0, s, K, dots);
    return cudaGetLastError();
}
cudaError_t kry_alpha(KrylovDev *K, const double *dots, cudaStream_t s)
{
    launch_pdl(k_kry_alpha, dim3(1), dim3(1), 0, s, K, dots);
    return cudaGetLastError();
}
cudaError_t kry_omega(KrylovDev *K, const double *dots, cudaStream_t s)
{
    launch_pdl(k_kry_omega, dim3(1), dim3(1), 0, s, K, dots);
    return cudaGetLastError();
}
cudaError_t kry_check(KrylovDev *K, const double *dots, double tol, int nkrylov, cudaStream_t s)
{
    launch_pdl(k_kry_check, dim3(1), dim3(1), 0, s, K, dots, tol, nkrylov);
    return cudaGetLastError();
}

template <typename T>
cudaError_t im_axmy_k(vec2<T> *out, const vec2<T> *x, const vec2<T> *y, const KrylovDev *K, int64_t total,
                      cudaStream_t s)
{
    launch_pdl(k_im_axmy_k<T>, dim3(im_grid(total)), dim3(256), 0, s, out, x, y, K, total);
    return cudaGetLastError();
}

template <typename T>
cudaError_t im_update_k(vec2<T> *phi, const vec2<T> *p, const vec2<T> *sv, const vec2<T> *As, vec2<T> *r,
                        const KrylovDev *K, int64_t total, cudaStream_t s)
{
    launch_pdl(k_im_update_k<T>, dim3(im_grid(total)), dim3(256), 0, s, phi, p, sv, As, r, K, total);
    return cudaGetLastError();
}

template <typename T>
cudaError_t im_pdir_k(vec2<T> *p, const vec2<T> *r, const vec2<T> *Ap, const KrylovDev *K, int64_t total,
                      cudaStream_t s)
{
    launch_pdl(k_im_pdir_k<T>, dim3(im_grid(total)), dim3(256), 0, s, p, r, Ap, K, total);
    return cudaGetLastError();
}

#define GPSS_IM_INST(T)                                                                                             \
    template cudaError_t im_prep_be<T>(const vec2<T> *, const T *, double, double, int, vec2<T> *, T *, vec2<T> *,  \
                                       int64_t, cudaStream_t);                                                      \
    template cudaError_t im_prep_cn<T>(const vec2<T> *, const vec2<T> *, const T *, double, double, int, vec2<T> *, \
                                       T *, vec2<T> *, vec2<T> *, int64_t, cudaStream_t);                           \
    template cudaError_t im_rhs_cn<T>(const vec2<T> *, const vec2<T> *, const vec2<T> *, const vec2<T> *,           \
                                      const T *, double, double, int, vec2<T> *, int64_t, cudaStream_t);            \
    template cudaError_t im_op<T>(const vec2<T> *, const vec2<T> *, int, double, const vec2<T> *, const T *,        \
                                  const vec2<T> *, const vec2<T> *, int, vec2<T> *, int64_t, cudaStream_t);        \
    template cudaError_t im_dot2<T>(const vec2<T> *, const vec2<T> *, const vec2<T> *, const vec2<T> *, int64_t,    \
                                    double *, double *, cudaStream_t);                                              \
    template cudaError_t im_axmy<T>(vec2<T> *, const vec2<T> *, double, const vec2<T> *, int64_t, cudaStream_t);    \
    template cudaError_t im_axmy_k<T>(vec2<T> *, const vec2<T> *, const vec2<T> *, const KrylovDev *, int64_t,      \
                                      cudaStream_t);                                                                \
    template cudaError_t im_update_k<T>(vec2<T> *, const vec2<T> *, const vec2<T> *, const vec2<T> *, vec2<T> *,    \
                                        const KrylovDev *, int64_t, cudaStream_t);                                  \
    template cudaError_t im_pdir_k<T>(vec2<T> *, const vec2<T> *, const vec2<T> *, const KrylovDev *, int64_t,      \
                                      cudaStream_t);                                                                \
    template cudaError_t im_mfield<T>(vec2<T> *, const vec2<T> *, const vec2<T> *, int64_t, cudaStream_t);
GPSS_IM_INST(float)
GPSS_IM_INST(double)

}  // namespace gpss
