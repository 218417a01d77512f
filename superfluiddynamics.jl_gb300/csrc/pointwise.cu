// pointwise.cu -- element-wise kernels: precision conversion at the host
// boundary, the plain-form phase multiply and nonlinear step, and the
// scaling that applies a renormalisation factor left on the device.
#include "gpss_internal.h"
#include "pdl.cuh"

namespace gpss {

static int grid_for(int64_t count, int threads)
{
    int64_t b = (count + threads - 1) / threads;
    const int64_t cap = 152 * 16;  // 16 CTAs of 256 threads per SM, grid-stride beyond
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

__global__ void k_f64_to_f32(const double *__restrict__ in, float *__restrict__ out, int64_t count)
{
    pdl_enter();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

__global__ void k_f32_to_f64(const float *__restrict__ in, double *__restrict__ out, int64_t count)
{
    pdl_enter();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

cudaError_t launch_f64_to_f32(const double *in, float *out, int64_t count, cudaStream_t s)
{
    launch_pdl(k_f64_to_f32, dim3(grid_for(count, 256)), dim3(256), 0, s, in, out, count);
    return cudaGetLastError();
}

cudaError_t launch_f32_to_f64(const float *in, double *out, int64_t count, cudaStream_t s)
{
    launch_pdl(k_f32_to_f64, dim3(grid_for(count, 256)), dim3(256), 0, s, in, out, count);
    return cudaGetLastError();
}

// Plain form: psi_hat(k, row) *= phase(k, row) on a natural-order spectrum
// along `axis` (the broadcasts of splitting.jl:167/172/190/195/200).  Table
// rows are hi[n] then lo[n] (double-word factors); row `row` starts at row*prow.
template <typename T>
__global__ void k_mul_phase(vec2<T> *__restrict__ data, const vec2<T> *__restrict__ phase,
                            int64_t prow, int axis, int64_t nx, int64_t ny, int64_t nk, int64_t total)
{
    pdl_enter();
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t k, row;
        if (axis == 0) { k = e % nx; row = (e / nx) % ny; }
        else if (axis == 1) { k = (e / nx) % ny; row = e % nx; }
        else { k = e / (nx * ny); row = 0; }
        const vec2<T> *p = phase + row * prow;
        data[e] = cmul2(data[e], p[k], p[nk + k]);
    }
}

template <typename T>
cudaError_t launch_mul_phase(vec2<T> *data, const vec2<T> *phase, int64_t prow, int axis,
                             const int64_t *n, int64_t total, cudaStream_t s)
{
    launch_pdl(k_mul_phase<T>, dim3(grid_for(total, 256)), dim3(256), 0, s,
               data, phase, prow, axis, n[0], n[1], n[axis],
                                                        total);
    return cudaGetLastError();
}

// Plain form: solveNL! (splitting.jl:205-209) as its own sweep.
template <typename T>
__global__ void k_nl(vec2<T> *__restrict__ psi, const T *__restrict__ V, double beta, double dt,
                     int imag, int64_t total)
{
    pdl_enter();
    const NLConst<T> c(beta, dt);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const T vv = V ? V[e] : (T)0;
        psi[e] = nl_apply(psi[e], vv, c, imag != 0);
    }
}

template <typename T>
cudaError_t launch_nl(vec2<T> *psi, const T *V, double beta, double dt, int imag, int64_t total,
                      cudaStream_t s)
{
    launch_pdl(k_nl<T>, dim3(grid_for(total, 256)), dim3(256), 0, s, psi, V, beta, dt, imag, total);
    return cudaGetLastError();
}

template <typename T>
__global__ void k_scale(vec2<T> *__restrict__ psi, const double *__restrict__ scale, int64_t total)
{
    pdl_enter();
    const T s = (T)(*scale);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x)
        psi[e] = cscale(psi[e], s);
}

template <typename T>
cudaError_t launch_scale(vec2<T> *psi, const double *scale, int64_t total, cudaStream_t s)
{
    launch_pdl(k_scale<T>, dim3(grid_for(total, 256)), dim3(256), 0, s, psi, scale, total);
    return cudaGetLastError();
}

// ---- explicit Runge-Kutta (NumModelGPRK, explicit-rk.jl:96-166) ----

// t = (V + beta |q|^2) q, the nonlinear term of gp_rhs! (explicit-rk.jl:100-106)
template <typename T>
__global__ void k_nl_term(const vec2<T> *__restrict__ q, const T *__restrict__ V, T beta, vec2<T> *__restrict__ t,
                          int64_t total)
{
    pdl_enter();
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const vec2<T> v = q[e];
        const T f = (V ? V[e] : (T)0) + beta * (v.x * v.x + v.y * v.y);
        t[e] = mk<vec2<T>>(f * v.x, f * v.y);
    }
}

template <typename T>
cudaError_t launch_nl_term(const vec2<T> *q, const T *V, double beta, vec2<T> *t, int64_t total, cudaStream_t s)
{
    launch_pdl(k_nl_term<T>, dim3(grid_for(total, 256)), dim3(256), 0, s, q, V, (T)beta, t, total);
    return cudaGetLastError();
}

// One RK stage from k = lapRot(q) and t = the (filtered) nonlinear term:
//   kk = i (k - t)                                  (gp_rhs!)
//   acc_mode 1: acc = kk; 2: acc = acc + acc_w kk   (k1 + 2k2 + 2k3 + k4, left to right)
//   out = psi0 + cf acc  (from_acc)  or  psi0 + cf kk
template <typename T>
__global__ void k_rk_combine(const vec2<T> *__restrict__ k, const vec2<T> *__restrict__ t, const vec2<T> *psi0,
                             vec2<T> *acc, vec2<T> *out, int acc_mode, T acc_w, T cf, int from_acc, int64_t total)
{
    pdl_enter();
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const vec2<T> a = k[e], b = t[e];
        const vec2<T> kk = mk<vec2<T>>(-(a.y - b.y), a.x - b.x);
        vec2<T> s = kk;
        if (acc_mode == 1) {
            acc[e] = kk;
        } else if (acc_mode == 2) {
            const vec2<T> p = acc[e];
            s = mk<vec2<T>>(p.x + acc_w * kk.x, p.y + acc_w * kk.y);
            acc[e] = s;
        }
        const vec2<T> base = psi0[e];
        const vec2<T> d = from_acc ? s : kk;
        out[e] = mk<vec2<T>>(base.x + cf * d.x, base.y + cf * d.y);
    }
}

template <typename T>
cudaError_t launch_rk_combine(const vec2<T> *k, const vec2<T> *t, const vec2<T> *psi0, vec2<T> *acc, vec2<T> *out,
                              int acc_mode, double acc_w, double cf, int from_acc, int64_t total, cudaStream_t s)
{
    launch_pdl(k_rk_combine<T>, dim3(grid_for(total, 256)), dim3(256), 0, s,
               k, t, psi0, acc, out, acc_mode, (T)acc_w, (T)cf, from_acc, total);
    return cudaGetLastError();
}

template cudaError_t launch_nl_term<float>(const vec2<float> *, const float *, double, vec2<float> *, int64_t,
                                           cudaStream_t);
template cudaError_t launch_nl_term<double>(const vec2<double> *, const double *, double, vec2<double> *, int64_t,
                                            cudaStream_t);
template cudaError_t launch_rk_combine<float>(const vec2<float> *, const vec2<float> *, const vec2<float> *,
                                              vec2<float> *, vec2<float> *, int, double, double, int, int64_t,
                                              cudaStream_t);
template cudaError_t launch_rk_combine<double>(const vec2<double> *, const vec2<double> *, const vec2<double> *,
                                               vec2<double> *, vec2<double> *, int, double, double, int, int64_t,
                                               cudaStream_t);

template cudaError_t launch_mul_phase<float>(vec2<float> *, const vec2<float> *, int64_t, int,
                                             const int64_t *, int64_t, cudaStream_t);
template cudaError_t launch_mul_phase<double>(vec2<double> *, const vec2<double> *, int64_t, int,
                                              const int64_t *, int64_t, cudaStream_t);
template cudaError_t launch_nl<float>(vec2<float> *, const float *, double, double, int, int64_t,
                                      cudaStream_t);
template cudaError_t launch_nl<double>(vec2<double> *, const double *, double, double, int, int64_t,
                                       cudaStream_t);
template cudaError_t launch_scale<float>(vec2<float> *, const double *, int64_t, cudaStream_t);
template cudaError_t launch_scale<double>(vec2<double> *, const double *, int64_t, cudaStream_t);

}  // namespace gpss
