// adjoint.cu -- pointwise kernels of the discrete adjoint of the Strang step
// (an extension; the reference has no gradient path).
//
// Conventions: for a real loss L of a complex field psi the adjoint field is
// g = 2 dL/d conj(psi) (Wirtinger), so dL = Re sum conj(g) dpsi.  A linear
// stage psi_out = A psi_in propagates g_in = A^H g_out.  The nonlinear stage
// psi_out = f psi_in, f = exp(-i theta), theta = (V + beta |psi_in|^2) dt,
// propagates
//     g_in = conj(f) g + 2 beta dt Im(conj(g) psi_out) psi_in,
//     dL/dV += dt Im(conj(g) psi_out)          (per cell, accumulated in FP64).
#include "gpss_internal.h"
#include "pdl.cuh"

namespace gpss {

static int grid_for(int64_t count, int threads)
{
    int64_t b = (count + threads - 1) / threads;
    const int64_t cap = 152 * 8;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

// per-CTA FP64 partials of sum conj(a) b  ->  partials[2*blockIdx.x + {0,1}]
template <typename T>
__global__ void k_overlap(const vec2<T> *__restrict__ a, const vec2<T> *__restrict__ b, int64_t total,
                          double *__restrict__ partials)
{
    pdl_enter();
    __shared__ double sr[256], si[256];
    double re = 0.0, im = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const double ax = a[e].x, ay = a[e].y, bx = b[e].x, by = b[e].y;
        re += ax * bx + ay * by;
        im += ax * by - ay * bx;
    }
    sr[threadIdx.x] = re;
    si[threadIdx.x] = im;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            sr[threadIdx.x] += sr[threadIdx.x + o];
            si[threadIdx.x] += si[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = sr[0];
        partials[2 * blockIdx.x + 1] = si[0];
    }
}

// z = dV * sum of the partials (fixed order), one CTA
__global__ void k_overlap_finish(const double *__restrict__ partials, int nblocks, double dV, double *__restrict__ z)
{
    pdl_enter();
    __shared__ double sr[256], si[256];
    double re = 0.0, im = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
        re += partials[2 * i];
        im += partials[2 * i + 1];
    }
    sr[threadIdx.x] = re;
    si[threadIdx.x] = im;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            sr[threadIdx.x] += sr[threadIdx.x + o];
            si[threadIdx.x] += si[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        z[0] = sr[0] * dV;
        z[1] = si[0] * dV;
    }
}

template <typename T>
cudaError_t launch_overlap(const vec2<T> *a, const vec2<T> *b, int64_t total, double *partials, double dV,
                           double *z, cudaStream_t s)
{
    const int blocks = grid_for(total, 256);
    launch_pdl(k_overlap<T>, dim3(blocks), dim3(256), 0, s, a, b, total, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    launch_pdl(k_overlap_finish, dim3(1), dim3(256), 0, s, partials, blocks, dV, z);
    return cudaGetLastError();
}

// g = -2 z target dV  (the adjoint of L = 1 - |z|^2 at the final field)
template <typename T>
__global__ void k_seed(vec2<T> *__restrict__ g, const vec2<T> *__restrict__ target, const double *__restrict__ z,
                       double dV, int64_t total)
{
    pdl_enter();
    const double zr = -2.0 * dV * z[0], zi = -2.0 * dV * z[1];
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const double tx = target[e].x, ty = target[e].y;
        g[e] = mk<vec2<T>>((T)(zr * tx - zi * ty), (T)(zr * ty + zi * tx));
    }
}

template <typename T>
cudaError_t launch_seed(vec2<T> *g, const vec2<T> *target, const double *z, double dV, int64_t total,
                        cudaStream_t s)
{
    launch_pdl(k_seed<T>, dim3(grid_for(total, 256)), dim3(256), 0, s, g, target, z, dV, total);
    return cudaGetLastError();
}

// adjoint of the nonlinear stage at one step (see the file comment)
template <typename T>
__global__ void k_nl_adjoint(vec2<T> *__restrict__ g, const vec2<T> *__restrict__ psi_in, const T *__restrict__ V,
                             double *__restrict__ dLdV, double beta, double dt, int64_t total)
{
    pdl_enter();
    const NLConst<T> c(beta, dt);
    const T two_beta_dt = (T)(2.0 * beta * dt);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const vec2<T> pin = psi_in[e];
        const T vv = V ? V[e] : (T)0;
        const vec2<T> f = nl_factor(pin, vv, c, false);
        const vec2<T> pout = nl_rotate(f, pin);
        const vec2<T> ge = g[e];
        const T im = ge.x * pout.y - ge.y * pout.x;  // Im(conj(g) psi_out)
        dLdV[e] += dt * (double)im;
        const vec2<T> rot = cmulc(ge, f);            // conj(f) g
        g[e] = mk<vec2<T>>(rot.x + two_beta_dt * im * pin.x, rot.y + two_beta_dt * im * pin.y);
    }
}

template <typename T>
cudaError_t launch_nl_adjoint(vec2<T> *g, const vec2<T> *psi_in, const T *V, double *dLdV, double beta, double dt,
                              int64_t total, cudaStream_t s)
{
    launch_pdl(k_nl_adjoint<T>, dim3(grid_for(total, 256)), dim3(256), 0, s, g, psi_in, V, dLdV, beta, dt, total);
    return cudaGetLastError();
}

template cudaError_t launch_overlap<float>(const vec2<float> *, const vec2<float> *, int64_t, double *, double,
                                           double *, cudaStream_t);
template cudaError_t launch_overlap<double>(const vec2<double> *, const vec2<double> *, int64_t, double *, double,
                                            double *, cudaStream_t);
template cudaError_t launch_seed<float>(vec2<float> *, const vec2<float> *, const double *, double, int64_t,
                                        cudaStream_t);
template cudaError_t launch_seed<double>(vec2<double> *, const vec2<double> *, const double *, double, int64_t,
                                         cudaStream_t);
template cudaError_t launch_nl_adjoint<float>(vec2<float> *, const vec2<float> *, const float *, double *, double,
                                              double, int64_t, cudaStream_t);
template cudaError_t launch_nl_adjoint<double>(vec2<double> *, const vec2<double> *, const double *, double *,
                                               double, double, int64_t, cudaStream_t);

}  // namespace gpss
