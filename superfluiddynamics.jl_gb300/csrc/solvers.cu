// solvers.cu -- gpss_rk_step (explicit Runge-Kutta, NumModelGPRK) and
// gpss_implicit_step (backward Euler and Crank-Nicolson with BiCGStab) on the
// fused multiplier passes and the pointwise kernels of pointwise.cu and implicit.cu.
#include "ctx.cuh"

// ------------------------------------------------ explicit Runge-Kutta ----
// timeStep!(::NumModelGPRK), explicit-rk.jl:135-166.  Every stage evaluates
// gp_rhs! (:96-107): lapRot(q) as one fused pass per axis with the axis's
// multiplier table (the x and y tables carry the rotation term per row),
// accumulated across axes; the nonlinear term (V + beta|q|^2) q, 2/3-filtered
// through the full transform (FWD passes, mask, INV passes) when filter is
// "product"; then i (lapRot - N) goes straight into the stage state and the
// running k1 + 2k2 + 2k3 + k4 sum.

// largest kept |kk| along the last axis for every inner position, from the
// reference's Float64 test (xi_x^2 + xi_y^2 [+ xi_z^2]) < xi_max
static int rk_mask_table(gpss_ctx *c)
{
    if (c->rk_lim) return GPSS_OK;
    double xmax = 0.0;
    for (int a = 0; a < c->ndim; a++) {
        double m = 0.0;
        for (int64_t k = 0; k < c->n[a]; k++) {
            const double x = xi_of(c, a, k);
            if (x * x > m) m = x * x;
        }
        if (a == 0 || m < xmax) xmax = m;
    }
    xmax = (4.0 / 9.0) * xmax;  // Plans.jl:529-532
    const int last = c->ndim - 1;
    const int64_t inner = c->total / c->n[last], nl = c->n[last];
    std::vector<int> lim((size_t)inner);
    for (int64_t j = 0; j < inner; j++) {
        const int64_t ix = j % c->n[0], iy = (j / c->n[0]) % c->n[1];
        double sxy = xi_of(c, 0, ix) * xi_of(c, 0, ix);
        if (c->ndim == 3) sxy = sxy + xi_of(c, 1, iy) * xi_of(c, 1, iy);
        int best = -1;
        for (int64_t kk = 0; kk <= nl / 2; kk++) {
            const double z = (double)kk * xi_mult(c, last);
            if (sxy + z * z < xmax) best = (int)kk;
            else break;  // the test is monotone in |kk|
        }
        lim[(size_t)j] = best;
    }
    GPSS_TRY(dev_alloc(c, (void **)&c->rk_lim, lim.size() * sizeof(int)));
    CUDA_TRY(c, cudaMemcpy(c->rk_lim, lim.data(), lim.size() * sizeof(int), cudaMemcpyHostToDevice));
    return GPSS_OK;
}

// in-place full transform of `f` (mul_all!/ldiv_all!): FWD x, y[, z] or INV z, y, x
// The 2/3 filter (Plans.jl:529-532) of a field: forward transforms along the
// leading axes, then one fused pass along the last axis (transform, keep the
// modes inside the limit, inverse transform), then the inverse transforms
// along the leading axes -- 2 ndim - 1 sweeps instead of 2 ndim + 1.
template <typename T> static int dealias_field(gpss_ctx *c, void *f)
{
    GPSS_TRY(rk_mask_table(c));
    const int last = c->ndim - 1;
    for (int axis = 0; axis < last; axis++) {
        PassArgs<T> a = axis_args<T>(c, axis, f, f);
        GPSS_TRY(launch<T>(c, axis, MODE_FWD, a));
    }
    PassArgs<T> m = axis_args<T>(c, last, f, f);
    m.mask_lim = c->rk_lim;
    GPSS_TRY(launch<T>(c, last, MODE_FUSED, m));
    for (int axis = last - 1; axis >= 0; axis--) {
        PassArgs<T> a = axis_args<T>(c, axis, f, f);
        GPSS_TRY(launch<T>(c, axis, MODE_INV, a));
    }
    return GPSS_OK;
}

// out = lapRot(q) (GrossPitaevskii.jl:12-45) as one fused pass per axis with
// the axis multiplier table, the y/z passes adding into the x result
template <typename T> static int lap_rot_dev(gpss_ctx *c, const void *q, void *out)
{
    for (int axis = 0; axis < c->ndim; axis++) {
        PassArgs<T> a = axis_args<T>(c, axis, q, out);
        const void *ph;
        GPSS_TRY(get_phase(c, axis, 0.0, 2, 1, &ph, &a.prow));
        a.phase = (const vec2<T> *)ph;
        if (axis > 0) a.acc = (const vec2<T> *)out;
        GPSS_TRY(launch<T>(c, axis, MODE_FUSED, a));
    }
    return GPSS_OK;
}

// k = i (lapRot(q) - N(q)) folded into the stage update (launch_rk_combine)
template <typename T>
static int rk_stage(gpss_ctx *c, const void *q, int filter, int acc_mode, double acc_w, double cf, int from_acc,
                    void *out)
{
    void *k = c->rk_buf[1], *t = c->rk_buf[2], *acc = c->rk_buf[3];
    GPSS_TRY(lap_rot_dev<T>(c, q, k));
    cudaError_t e = launch_nl_term<T>((const vec2<T> *)q, c->have_V ? (const T *)c->V : nullptr, c->beta,
                                      (vec2<T> *)t, c->total, c->stream);
    if (e != cudaSuccess) return fail(c, GPSS_ECUDA, "nl_term: %s", cudaGetErrorString(e));
    c->launches++;
    if (filter == 1) GPSS_TRY(dealias_field<T>(c, t));
    e = launch_rk_combine<T>((const vec2<T> *)k, (const vec2<T> *)t, (const vec2<T> *)c->psi, (vec2<T> *)acc,
                             (vec2<T> *)out, acc_mode, acc_w, cf, from_acc, c->total, c->stream);
    if (e != cudaSuccess) return fail(c, GPSS_ECUDA, "rk_combine: %s", cudaGetErrorString(e));
    c->launches++;
    return GPSS_OK;
}

template <typename T> static int rk_step_impl(gpss_ctx *c, int nsteps, int stepper, int filter, double dt)
{
    const size_t fb = (size_t)c->total * sizeof(vec2<T>);
    for (int i = 0; i < 4; i++)
        if (!c->rk_buf[i]) GPSS_TRY(dev_alloc(c, &c->rk_buf[i], fb));
    void *st = c->rk_buf[0];
    const double half = 0.5 * dt, sixth = dt / 6;
    auto one_step = [&]() -> int {
        if (stepper == 1) {
            GPSS_TRY(rk_stage<T>(c, c->psi, filter, 0, 0.0, dt, 0, c->psi));
        } else if (stepper == 2) {
            GPSS_TRY(rk_stage<T>(c, c->psi, filter, 0, 0.0, half, 0, st));
            GPSS_TRY(rk_stage<T>(c, st, filter, 0, 0.0, dt, 0, c->psi));
        } else {
            GPSS_TRY(rk_stage<T>(c, c->psi, filter, 1, 1.0, half, 0, st));
            GPSS_TRY(rk_stage<T>(c, st, filter, 2, 2.0, half, 0, st));
            GPSS_TRY(rk_stage<T>(c, st, filter, 2, 2.0, dt, 0, st));
            GPSS_TRY(rk_stage<T>(c, st, filter, 2, 1.0, sixth, 1, c->psi));
        }
        if (filter == 2) GPSS_TRY(dealias_field<T>(c, c->psi));
        return GPSS_OK;
    };
    int s = 0;
    if (c->total <= kGraphCells) {
        const int chunk = kGraphChunk / 4;
        const std::string key = graph_key("rk", {(double)stepper, (double)filter, dt, (double)chunk});
        for (; s + chunk <= nsteps; s += chunk)
            GPSS_TRY(graph_run(c, key, [&]() -> int {
                for (int i = 0; i < chunk; i++) GPSS_TRY(one_step());
                return GPSS_OK;
            }));
    }
    for (; s < nsteps; s++) GPSS_TRY(one_step());
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return GPSS_OK;
}

// ------------------------------------------- implicit schemes (BE / CN) ----
// timeStep! of NumModelBackwardEuler[NoPrecond] (backward-euler.jl:62-83,
// 155-172) and NumModelCrankNicolson[QuasiNewton][T] (crank-nicolson.jl:62-103,
// 186-225, 308-347, 432-468) with the BiCGStab of krylov.jl.  lapRot is the
// fused multiplier passes; the operators, right-hand sides and vector updates
// are the pointwise kernels of implicit.cu; each Krylov iteration reads back
// its dot products (the scalars and the stopping test are the reference's).

struct ImBufs {
    void *r, *r2, *p, *Ap, *s, *As, *lap, *b, *M, *Anl2, *psim, *phi1, *phiw, *Anl;
    double *partials, *dots;
    KrylovDev *kry;
};

template <typename T> static int im_bufs(gpss_ctx *c, ImBufs &B)
{
    const size_t fb = (size_t)c->total * sizeof(vec2<T>);
    const size_t rb = (size_t)c->total * sizeof(T);
    const size_t pb = sizeof(double) * (2 * 152 * 8 + 2) + sizeof(KrylovDev);
    const size_t need = 13 * fb + rb + pb;
    if (!c->im_buf || c->im_bytes < need) {
        if (c->im_buf) { cudaStreamSynchronize(c->stream); cudaFree(c->im_buf); c->im_buf = nullptr; }
        GPSS_TRY(dev_alloc(c, &c->im_buf, need));
        c->im_bytes = need;
    }
    char *base = static_cast<char *>(c->im_buf);
    void **f[13] = {&B.r, &B.r2, &B.p, &B.Ap, &B.s, &B.As, &B.lap, &B.b, &B.M, &B.Anl2, &B.psim, &B.phi1, &B.phiw};
    for (int i = 0; i < 13; i++) *f[i] = base + (size_t)i * fb;
    B.Anl = base + 13 * fb;
    B.partials = reinterpret_cast<double *>(base + 13 * fb + rb);
    B.dots = B.partials + 2 * 152 * 8;
    B.kry = reinterpret_cast<KrylovDev *>(B.dots + 2);
    return GPSS_OK;
}

#define IM_TRY(call)                                                                   \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) return fail(c, GPSS_ECUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
        c->launches++;                                                                 \
    } while (0)

// two dot products Sum Re(a conj b) (FP64) read back to the host
template <typename T>
static int im_dots(gpss_ctx *c, ImBufs &B, const void *a1, const void *b1, const void *a2, const void *b2,
                   double out[2])
{
    using V = vec2<T>;
    IM_TRY(im_dot2<T>((const V *)a1, (const V *)b1, (const V *)a2, (const V *)b2, c->total, B.partials, B.dots,
                      c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(out, B.dots, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return GPSS_OK;
}

// out = [M] prodA(x) or [M](b - prodA(x))
template <typename T>
static int im_apply(gpss_ctx *c, ImBufs &B, int scheme, double dt, const void *x, bool bsub, int precond, void *out)
{
    using V = vec2<T>;
    GPSS_TRY(lap_rot_dev<T>(c, x, B.lap));
    IM_TRY(im_op<T>((const V *)x, (const V *)B.lap, scheme, dt, (const V *)B.M, (const T *)B.Anl,
                    (const V *)B.Anl2, bsub ? (const V *)B.b : nullptr, precond, (V *)out, c->total, c->stream));
    return GPSS_OK;
}

// krylov! (precond = 0) / krylovPreCond! (precond = 1), krylov.jl:1-67.
// The scalars and the stopping test live on the device (KrylovDev), so the
// host issues iterations in chunks (2, 2, 4, 4, 8, ... up to 16) and reads the
// solve's state back once per chunk; iterations issued past the end of the
// solve leave phi, r and p untouched, so the result and the iteration count
// are those of the reference's loop.
template <typename T>
static int im_krylov(gpss_ctx *c, ImBufs &B, int scheme, double dt, void *phi, int nkrylov, double tol, int precond,
                     int *niter_out)
{
    using V = vec2<T>;
    const size_t fb = (size_t)c->total * sizeof(V);
    const int64_t n = c->total;
    if (precond) {
        IM_TRY(im_mfield<T>((V *)B.s, (const V *)B.M, (const V *)B.b, n, c->stream));
        IM_TRY(im_dot2<T>((const V *)B.s, (const V *)B.s, nullptr, nullptr, n, B.partials, B.dots, c->stream));
    } else {
        IM_TRY(im_dot2<T>((const V *)B.b, (const V *)B.b, nullptr, nullptr, n, B.partials, B.dots, c->stream));
    }
    IM_TRY(kry_init(B.kry, B.dots, c->stream));
    GPSS_TRY(im_apply<T>(c, B, scheme, dt, phi, true, precond, B.r));
    CUDA_TRY(c, cudaMemcpyAsync(B.r2, B.r, fb, cudaMemcpyDeviceToDevice, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(B.p, B.r, fb, cudaMemcpyDeviceToDevice, c->stream));
    KrylovDev h{};
    int issued = 0;
    for (int chunk = 0; issued < nkrylov; chunk++) {
        const int m = std::min(chunk < 6 ? 2 << (chunk / 2) : 16, nkrylov - issued);
        for (int j = 0; j < m; j++) {
            GPSS_TRY(im_apply<T>(c, B, scheme, dt, B.p, false, precond, B.Ap));
            IM_TRY(im_dot2<T>((const V *)B.r, (const V *)B.r2, (const V *)B.Ap, (const V *)B.r2, n, B.partials,
                              B.dots, c->stream));
            IM_TRY(kry_alpha(B.kry, B.dots, c->stream));
            IM_TRY(im_axmy_k<T>((V *)B.s, (const V *)B.r, (const V *)B.Ap, B.kry, n, c->stream));
            GPSS_TRY(im_apply<T>(c, B, scheme, dt, B.s, false, precond, B.As));
            IM_TRY(im_dot2<T>((const V *)B.As, (const V *)B.s, (const V *)B.As, (const V *)B.As, n, B.partials,
                              B.dots, c->stream));
            IM_TRY(kry_omega(B.kry, B.dots, c->stream));
            IM_TRY(im_update_k<T>((V *)phi, (const V *)B.p, (const V *)B.s, (const V *)B.As, (V *)B.r, B.kry, n,
                                  c->stream));
            IM_TRY(im_dot2<T>((const V *)B.r, (const V *)B.r, (const V *)B.r, (const V *)B.r2, n, B.partials,
                              B.dots, c->stream));
            IM_TRY(kry_check(B.kry, B.dots, tol, nkrylov, c->stream));
            IM_TRY(im_pdir_k<T>((V *)B.p, (const V *)B.r, (const V *)B.Ap, B.kry, n, c->stream));
        }
        issued += m;
        CUDA_TRY(c, cudaMemcpyAsync(&h, B.kry, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
        if (h.done) break;
    }
    if (h.nonfinite) return fail(c, GPSS_ENONFINITE, "Krylov solver: non-finite residual");
    *niter_out = h.niter;
    return GPSS_OK;
}


template <typename T>
static int implicit_impl(gpss_ctx *c, int nsteps, int scheme, double dt, int nkrylov, double tol, int nnewton,
                         double tolnewton, int64_t *ktot)
{
    using V = vec2<T>;
    ImBufs B;
    GPSS_TRY(im_bufs<T>(c, B));
    const size_t fb = (size_t)c->total * sizeof(V);
    const T *Vp = c->have_V ? (const T *)c->V : nullptr;
    int64_t total_k = 0;
    for (int st = 0; st < nsteps; st++) {
        int nk = 0;
        if (scheme == IM_SCHEME_BE || scheme == IM_SCHEME_BE_NOPRE) {
            IM_TRY(im_prep_be<T>((const V *)c->psi, Vp, c->beta, dt, scheme, (V *)B.M, (T *)B.Anl, (V *)B.b,
                                 c->total, c->stream));
            GPSS_TRY(im_krylov<T>(c, B, scheme, dt, c->psi, nkrylov, tol, 0, &nk));
            total_k += nk;
            GPSS_TRY(normalize_impl<T>(c));
            continue;
        }
        const int tsch = scheme == IM_SCHEME_CN_T || scheme == IM_SCHEME_CN_QN_T;
        CUDA_TRY(c, cudaMemcpyAsync(B.phi1, c->psi, fb, cudaMemcpyDeviceToDevice, c->stream));
        CUDA_TRY(c, cudaMemsetAsync(B.phiw, 0, fb, c->stream));
        for (int itn = 1; itn <= nnewton; itn++) {
            IM_TRY(im_prep_cn<T>((const V *)c->psi, (const V *)B.phi1, Vp, c->beta, dt, scheme, (V *)B.psim,
                                 (T *)B.Anl, (V *)B.Anl2, (V *)B.M, c->total, c->stream));
            GPSS_TRY(lap_rot_dev<T>(c, B.psim, B.lap));
            IM_TRY(im_rhs_cn<T>((const V *)c->psi, (const V *)B.phi1, (const V *)B.psim, (const V *)B.lap, Vp,
                                c->beta, dt, tsch, (V *)B.b, c->total, c->stream));
            GPSS_TRY(im_krylov<T>(c, B, scheme, dt, B.phiw, nkrylov, tol, 1, &nk));
            total_k += nk;
            IM_TRY(im_axmy<T>((V *)B.phi1, (const V *)B.phi1, 1.0, (const V *)B.phiw, c->total, c->stream));
            double d[2];
            GPSS_TRY(im_dots<T>(c, B, B.phiw, B.phiw, nullptr, nullptr, d));
            if (std::sqrt(d[0]) < tolnewton) break;
        }
        CUDA_TRY(c, cudaMemcpyAsync(c->psi, B.phi1, fb, cudaMemcpyDeviceToDevice, c->stream));
        if (!tsch) GPSS_TRY(normalize_impl<T>(c));
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (ktot) *ktot = total_k;
    return GPSS_OK;
}

extern "C" {

int gpss_rk_step(gpss_ctx *c, int nsteps, int stepper, int filter, double dt)
{
    NvtxRange nvtx_("gpss_rk_step");
    if (!c) return GPSS_EINVAL;
    c->version++;  // the field or the parameters may change
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "gpss_rk_step: no field uploaded");
    if (nsteps < 0) return fail(c, GPSS_EINVAL, "gpss_rk_step: nsteps < 0");
    if (stepper != 1 && stepper != 2 && stepper != 4)
        return fail(c, GPSS_EINVAL, "gpss_rk_step: stepper must be 1, 2 or 4 (got %d)", stepper);
    if (filter < 0 || filter > 2) return fail(c, GPSS_EINVAL, "gpss_rk_step: filter must be 0, 1 or 2");
    if (!std::isfinite(dt)) return fail(c, GPSS_EINVAL, "gpss_rk_step: dt must be finite");
    CUDA_TRY(c, cudaSetDevice(c->device));
    GPSS_TRY(flush_pending(c));
    return c->precision == GPSS_FP32 ? rk_step_impl<float>(c, nsteps, stepper, filter, dt)
                                     : rk_step_impl<double>(c, nsteps, stepper, filter, dt);
}

int gpss_implicit_step(gpss_ctx *c, int nsteps, int scheme, double dt, int nkrylov, double tolkrylov, int nnewton,
                       double tolnewton, int64_t *krylov_iters)
{
    NvtxRange nvtx_("gpss_implicit_step");
    if (!c) return GPSS_EINVAL;
    c->version++;  // the field or the parameters may change
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "gpss_implicit_step: no field uploaded");
    if (nsteps < 0 || nkrylov < 1 || nnewton < 1)
        return fail(c, GPSS_EINVAL, "gpss_implicit_step: need nsteps >= 0, nkrylov >= 1, nnewton >= 1");
    if (scheme < GPSS_IMPLICIT_BE || scheme > GPSS_IMPLICIT_CN_QN_T)
        return fail(c, GPSS_EINVAL, "gpss_implicit_step: unknown scheme %d", scheme);
    if (!(dt > 0.0) || !std::isfinite(dt) || !(tolkrylov > 0.0) || !(tolnewton > 0.0))
        return fail(c, GPSS_EINVAL, "gpss_implicit_step: dt and the tolerances must be positive");
    CUDA_TRY(c, cudaSetDevice(c->device));
    GPSS_TRY(flush_pending(c));
    return c->precision == GPSS_FP32
               ? implicit_impl<float>(c, nsteps, scheme, dt, nkrylov, tolkrylov, nnewton, tolnewton, krylov_iters)
               : implicit_impl<double>(c, nsteps, scheme, dt, nkrylov, tolkrylov, nnewton, tolnewton, krylov_iters);
}

}  // extern "C"
