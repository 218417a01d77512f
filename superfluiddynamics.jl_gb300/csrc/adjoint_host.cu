// adjoint_host.cu -- gpss_adjoint: the discrete adjoint of the Strang step
// (dL/dV and dL/dpsi0 of L = 1 - |<psi_target, psi(T)>|^2), orchestrating the
// fused passes and the pointwise kernels of adjoint.cu.
#include "ctx.cuh"

// ---------------------------------------------------------------- adjoint --
// device buffers of one gpss_adjoint call, released on every exit path
struct DevBufs {
    std::vector<void *> ptrs;
    ~DevBufs()
    {
        for (void *p : ptrs) cudaFree(p);
    }
    int get(gpss_ctx *c, void **p, size_t bytes)
    {
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) {
            *p = nullptr;
            return fail(c, GPSS_ENOMEM, "cudaMalloc(%zu) for the adjoint failed: %s", bytes, cudaGetErrorString(e));
        }
        ptrs.push_back(*p);
        return GPSS_OK;
    }
};

// one Strang step on `buf` as the forward of the adjoint: unmerged half
// steps, no mass lock, so that the recomputed states are bitwise those of
// the forward run
template <typename T> static int strang_on(gpss_ctx *c, void *buf, double dt)
{
    GPSS_TRY(kinetic_fused<T>(c, dt * 0.5, 0, true, dt, 0, false, false, FIN_NONE, buf));
    return kinetic_fused<T>(c, dt * 0.5, 0, false, 0.0, 0, false, false, FIN_NONE, buf);
}

// One kinetic flow L(dtl) as fused passes on `buf` (axis order reversed for
// the adjoint L^H, with dtl < 0).  The last pass may apply the nonlinear flow
// N(dtnl) and store its input in pre_out, or apply the adjoint of N at the
// state adj_pre (accumulating dL/dV into dv).
template <typename T>
static int adj_group(gpss_ctx *c, void *buf, double dtl, bool reverse, bool nl, double dtnl, void *pre_out,
                     const void *adj_pre, double *dv)
{
    for (int step = 0; step < c->ndim; step++) {
        const int axis = reverse ? c->ndim - 1 - step : step;
        PassArgs<T> a = axis_args<T>(c, axis, buf, buf);
        const void *ph;
        GPSS_TRY(get_phase(c, axis, dtl, 0, 1, &ph, &a.prow));
        a.phase = (const vec2<T> *)ph;
        // a compensated FP32 context differentiates with compensated passes
        // (forward, recompute and backward alike, so the recomputed states
        // stay bitwise those of the forward)
        a.comp = sizeof(T) == 4 && (c->flags & GPSS_FLAG_COMPENSATED) != 0;
        if (step == c->ndim - 1 && (nl || adj_pre)) {
            a.V = c->have_V ? (const T *)c->V : nullptr;
            a.nl_beta = c->beta;
            a.nl_dt = dtnl;
            a.nl_split = nl_split(c->beta, dtnl);
            if (nl) {
                a.nl_mode = NL_REAL;
                a.pre_out = (vec2<T> *)pre_out;
            } else {
                a.adj_pre = (const vec2<T> *)adj_pre;
                a.adj_dLdV = dv;
            }
        }
        GPSS_TRY(launch<T>(c, axis, MODE_FUSED, a));
    }
    return GPSS_OK;
}

// The discrete adjoint on the merged Strang sequence (Omega = 0: adjacent
// half kinetic flows compose exactly).  With pre_n the state entering the
// nonlinear stage of step n:
//   pre_0 = L(h) psi_0,  pre_{n+1} = L(dt) N(pre_n),  psi_T = L(h) N(pre_{T-1})
// so the forward is one pass group per step (N fused into its last pass,
// which also stores pre_n at the checkpoints), and the backward is
//   g <- N^H_{pre_{T-1}} L^H(h) g,  g <- N^H_{pre_n} L^H(dt) g (n = T-2..0),
//   dL/dpsi0 = L^H(h) g
// one group per step with N^H fused into its last pass.  Segments of K steps
// are recomputed from their checkpoint into K state buffers (the same
// kernels as the forward, so the states are bitwise the forward's).  The
// recompute of segment s-1 runs on a second stream while the backward sweep
// works through segment s (two sets of state buffers, alternating): a 256^2
// pass fills a few dozen SMs, so the two chains share the GPU.
template <typename T>
static int adjoint_merged(gpss_ctx *c, const double *psi_target, int nsteps, int K, double dt, double *loss,
                          double *dLdV, double *dLdpsi0)
{
    using V = vec2<T>;
    const size_t fb = (size_t)c->total * sizeof(V);
    const int nck = (nsteps + K - 1) / K;
    // psi0, g, tgt, work, states[2][K], ckpt[nck]; dv (doubles); reduction scratch
    const size_t red_bytes = sizeof(double) * (2 * 152 * 8 + 2);
    const size_t need = fb * (size_t)(4 + 2 * K + nck) + (size_t)c->total * sizeof(double) + red_bytes;
    if (!c->side) {
        CUDA_TRY(c, cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
        for (auto &e : c->side_ev) CUDA_TRY(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    if (c->adj_bytes < need) {
        clear_graphs(c);
        if (c->adj_buf) { cudaStreamSynchronize(c->stream); cudaFree(c->adj_buf); c->adj_buf = nullptr; c->adj_bytes = 0; }
        GPSS_TRY(dev_alloc(c, &c->adj_buf, need));
        c->adj_bytes = need;
    }
    char *base = static_cast<char *>(c->adj_buf);
    void *psi0 = base, *g = base + fb, *tgt = base + 2 * fb, *work = base + 3 * fb;
    auto state = [&](int set, int j) { return static_cast<void *>(base + fb * (size_t)(4 + set * K + j)); };
    auto ckpt = [&](int i) { return static_cast<void *>(base + fb * (size_t)(4 + 2 * K + i)); };
    double *dv = reinterpret_cast<double *>(base + fb * (size_t)(4 + 2 * K + nck));
    double *red = dv + c->total;
    double *zdev = red + 2 * 152 * 8;
    const double dV = cell_volume(c), h = dt * 0.5;
    if (c->precision == GPSS_FP64) {
        CUDA_TRY(c, cudaMemcpyAsync(tgt, psi_target, fb, cudaMemcpyHostToDevice, c->stream));
    } else {
        CUDA_TRY(c, cudaMemcpyAsync(c->scratch, psi_target, (size_t)c->total * 16, cudaMemcpyHostToDevice,
                                    c->stream));
        CUDA_TRY(c, launch_f64_to_f32((const double *)c->scratch, (float *)tgt, 2 * c->total, c->stream));
    }
    // everything from here to the outputs is device work with fixed arguments:
    // a repeated call replays it as one CUDA graph
    auto body = [&]() -> int {
        CUDA_TRY(c, cudaMemcpyAsync(psi0, c->psi, fb, cudaMemcpyDeviceToDevice, c->stream));
        CUDA_TRY(c, cudaMemsetAsync(dv, 0, (size_t)c->total * sizeof(double), c->stream));
        // forward: c->psi becomes N(pre_n) after group n; pre_n kept at the checkpoints
        for (int n = 0; n < nsteps; n++)
            GPSS_TRY(adj_group<T>(c, c->psi, n == 0 ? h : dt, false, true, dt, n % K == 0 ? ckpt(n / K) : nullptr,
                                  nullptr, nullptr));
        GPSS_TRY(adj_group<T>(c, c->psi, h, false, false, 0.0, nullptr, nullptr, nullptr));
        // loss and the adjoint of the final field
        CUDA_TRY(c, launch_overlap<T>((const V *)tgt, (const V *)c->psi, c->total, red, dV, zdev, c->stream));
        CUDA_TRY(c, launch_seed<T>((V *)g, (const V *)tgt, zdev, dV, c->total, c->stream));
        c->launches += 3;
        // backward, segment by segment from the last; the recomputes run on
        // the side stream one segment ahead (side_ev: 0 fork, 1 recompute
        // done, 2 backward through a segment done)
        cudaStream_t main = c->stream;
        auto recompute = [&](int seg) -> int {
            const int start = seg * K, end = std::min(start + K, nsteps);
            if (end - start < 2) return GPSS_OK;
            // work = N(pre_start), then pre_{start+j} = L(dt) N(pre_{start+j-1}) into state(j)
            CUDA_TRY(c, cudaMemcpyAsync(work, ckpt(seg), fb, cudaMemcpyDeviceToDevice, c->stream));
            cudaError_t e = launch_nl<T>((V *)work, c->have_V ? (const T *)c->V : nullptr, c->beta, dt, 0,
                                         c->total, c->stream);
            if (e != cudaSuccess) return fail(c, GPSS_ECUDA, "nl: %s", cudaGetErrorString(e));
            c->launches++;
            for (int j = 1; j < end - start; j++)
                GPSS_TRY(adj_group<T>(c, work, dt, false, true, dt, state(seg & 1, j), nullptr, nullptr));
            return GPSS_OK;
        };
        auto on_side = [&](auto fn) -> int {  // issue fn's work on the side stream
            c->stream = c->side;
            const int rc = fn();
            c->stream = main;
            return rc;
        };
        CUDA_TRY(c, cudaEventRecord(c->side_ev[0], main));
        CUDA_TRY(c, cudaStreamWaitEvent(c->side, c->side_ev[0], 0));
        GPSS_TRY(on_side([&] { return recompute(nck - 1); }));
        CUDA_TRY(c, cudaEventRecord(c->side_ev[1], c->side));
        for (int seg = nck - 1; seg >= 0; seg--) {
            const int start = seg * K, end = std::min(start + K, nsteps);
            CUDA_TRY(c, cudaStreamWaitEvent(main, c->side_ev[1], 0));  // segment seg recomputed
            if (seg > 0) {
                // segment seg-1's states reuse the set of segment seg+1, which
                // the backward sweep has finished with (side_ev[2])
                if (seg < nck - 1) CUDA_TRY(c, cudaStreamWaitEvent(c->side, c->side_ev[2], 0));
                GPSS_TRY(on_side([&] { return recompute(seg - 1); }));
                CUDA_TRY(c, cudaEventRecord(c->side_ev[1], c->side));
            }
            for (int n = end - 1; n >= start; n--) {
                const void *pre = n == start ? ckpt(seg) : state(seg & 1, n - start);
                GPSS_TRY(adj_group<T>(c, g, n == nsteps - 1 ? -h : -dt, true, false, dt, nullptr, pre, dv));
            }
            CUDA_TRY(c, cudaEventRecord(c->side_ev[2], main));
        }
        CUDA_TRY(c, cudaStreamWaitEvent(main, c->side_ev[1], 0));  // join the side stream
        GPSS_TRY(adj_group<T>(c, g, -h, true, false, 0.0, nullptr, nullptr, nullptr));
        CUDA_TRY(c, cudaMemcpyAsync(c->psi, psi0, fb, cudaMemcpyDeviceToDevice, c->stream));
        return GPSS_OK;
    };
    GPSS_TRY(graph_run(c, graph_key("adjoint", {(double)nsteps, (double)K, dt, (double)c->have_V}), body));
    double z[2];
    CUDA_TRY(c, cudaMemcpyAsync(z, zdev, sizeof(z), cudaMemcpyDeviceToHost, c->stream));
    // outputs; the context's field is back at the initial state
    if (dLdV) CUDA_TRY(c, cudaMemcpyAsync(dLdV, dv, (size_t)c->total * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (dLdpsi0) {
        if (c->precision == GPSS_FP64) {
            CUDA_TRY(c, cudaMemcpyAsync(dLdpsi0, g, fb, cudaMemcpyDeviceToHost, c->stream));
        } else {
            CUDA_TRY(c, launch_f32_to_f64((const float *)g, (double *)c->scratch, 2 * c->total, c->stream));
            CUDA_TRY(c, cudaMemcpyAsync(dLdpsi0, c->scratch, (size_t)c->total * 16, cudaMemcpyDeviceToHost,
                                        c->stream));
        }
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    *loss = 1.0 - (z[0] * z[0] + z[1] * z[1]);
    if (!std::isfinite(*loss)) return fail(c, GPSS_ENONFINITE, "adjoint: non-finite loss");
    return GPSS_OK;
}

template <typename T>
static int adjoint_impl(gpss_ctx *c, const double *psi_target, int nsteps, int K, double dt, double *loss,
                        double *dLdV, double *dLdpsi0)
{
    if (c->omega == 0.0) return adjoint_merged<T>(c, psi_target, nsteps, K, dt, loss, dLdV, dLdpsi0);
    using V = vec2<T>;
    const size_t fb = (size_t)c->total * sizeof(V);
    const int nck = (nsteps + K - 1) / K;
    DevBufs m;
    void *psi0, *ckpt, *states, *g, *tgt, *work, *dv, *red;
    GPSS_TRY(m.get(c, &psi0, fb));
    GPSS_TRY(m.get(c, &ckpt, fb * (size_t)nck));
    GPSS_TRY(m.get(c, &states, fb * (size_t)K));
    GPSS_TRY(m.get(c, &g, fb));
    GPSS_TRY(m.get(c, &tgt, fb));
    GPSS_TRY(m.get(c, &work, fb));
    GPSS_TRY(m.get(c, &dv, (size_t)c->total * sizeof(double)));
    GPSS_TRY(m.get(c, &red, sizeof(double) * (2 * 152 * 8 + 2)));
    double *zdev = static_cast<double *>(red) + 2 * 152 * 8;
    auto at = [&](void *base, int i) { return static_cast<void *>(static_cast<char *>(base) + fb * (size_t)i); };
    const double dV = cell_volume(c);
    CUDA_TRY(c, cudaMemcpyAsync(psi0, c->psi, fb, cudaMemcpyDeviceToDevice, c->stream));
    CUDA_TRY(c, cudaMemsetAsync(dv, 0, (size_t)c->total * sizeof(double), c->stream));
    // target in the field precision
    if (c->precision == GPSS_FP64) {
        CUDA_TRY(c, cudaMemcpyAsync(tgt, psi_target, fb, cudaMemcpyHostToDevice, c->stream));
    } else {
        CUDA_TRY(c, cudaMemcpyAsync(c->scratch, psi_target, (size_t)c->total * 16, cudaMemcpyHostToDevice,
                                    c->stream));
        CUDA_TRY(c, launch_f64_to_f32((const double *)c->scratch, (float *)tgt, 2 * c->total, c->stream));
    }
    // forward, keeping psi at the start of every segment
    for (int s = 0; s < nsteps; s++) {
        if (s % K == 0)
            CUDA_TRY(c, cudaMemcpyAsync(at(ckpt, s / K), c->psi, fb, cudaMemcpyDeviceToDevice, c->stream));
        GPSS_TRY(strang_on<T>(c, c->psi, dt));
    }
    // loss and the adjoint of the final field
    CUDA_TRY(c, launch_overlap<T>((const V *)tgt, (const V *)c->psi, c->total, (double *)red, dV, zdev, c->stream));
    double z[2];
    CUDA_TRY(c, cudaMemcpyAsync(z, zdev, sizeof(z), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, launch_seed<T>((V *)g, (const V *)tgt, zdev, dV, c->total, c->stream));
    c->launches += 3;
    // backward, segment by segment from the last
    const T *Vp = c->have_V ? (const T *)c->V : nullptr;
    for (int seg = nck - 1; seg >= 0; seg--) {
        const int start = seg * K, end = std::min(start + K, nsteps);
        CUDA_TRY(c, cudaMemcpyAsync(work, at(ckpt, seg), fb, cudaMemcpyDeviceToDevice, c->stream));
        CUDA_TRY(c, cudaMemcpyAsync(at(states, 0), work, fb, cudaMemcpyDeviceToDevice, c->stream));
        for (int j = 1; j < end - start; j++) {
            GPSS_TRY(strang_on<T>(c, work, dt));
            CUDA_TRY(c, cudaMemcpyAsync(at(states, j), work, fb, cudaMemcpyDeviceToDevice, c->stream));
        }
        for (int nstep = end - 1; nstep >= start; nstep--) {
            // second kinetic half step: g <- K^H g (conjugate phases, reverse axis order)
            GPSS_TRY(kinetic_fused<T>(c, -dt * 0.5, 0, false, 0.0, 0, false, false, FIN_NONE, g, true));
            // the state entering the nonlinear stage: K psi_n
            CUDA_TRY(c, cudaMemcpyAsync(work, at(states, nstep - start), fb, cudaMemcpyDeviceToDevice, c->stream));
            GPSS_TRY(kinetic_fused<T>(c, dt * 0.5, 0, false, 0.0, 0, false, false, FIN_NONE, work));
            CUDA_TRY(c, launch_nl_adjoint<T>((V *)g, (const V *)work, Vp, (double *)dv, c->beta, dt, c->total,
                                             c->stream));
            c->launches++;
            // first kinetic half step
            GPSS_TRY(kinetic_fused<T>(c, -dt * 0.5, 0, false, 0.0, 0, false, false, FIN_NONE, g, true));
        }
    }
    // outputs; the context's field goes back to the initial state
    if (dLdV) CUDA_TRY(c, cudaMemcpyAsync(dLdV, dv, (size_t)c->total * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (dLdpsi0) {
        if (c->precision == GPSS_FP64) {
            CUDA_TRY(c, cudaMemcpyAsync(dLdpsi0, g, fb, cudaMemcpyDeviceToHost, c->stream));
        } else {
            CUDA_TRY(c, launch_f32_to_f64((const float *)g, (double *)c->scratch, 2 * c->total, c->stream));
            CUDA_TRY(c, cudaMemcpyAsync(dLdpsi0, c->scratch, (size_t)c->total * 16, cudaMemcpyDeviceToHost,
                                        c->stream));
        }
    }
    CUDA_TRY(c, cudaMemcpyAsync(c->psi, psi0, fb, cudaMemcpyDeviceToDevice, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    *loss = 1.0 - (z[0] * z[0] + z[1] * z[1]);
    if (!std::isfinite(*loss)) return fail(c, GPSS_ENONFINITE, "adjoint: non-finite loss");
    return GPSS_OK;
}

extern "C" {

int gpss_adjoint(gpss_ctx *c, const double *psi_target, int nsteps, int K, double dt, double *loss,
                 double *dLdV, double *dLdpsi0)
{
    NvtxRange nvtx_("gpss_adjoint");
    if (!c) return GPSS_EINVAL;
    c->version++;  // the field or the parameters may change
    if (!psi_target || !loss) return fail(c, GPSS_EINVAL, "gpss_adjoint: null psi_target or loss");
    if (nsteps < 1 || K < 1) return fail(c, GPSS_EINVAL, "gpss_adjoint: need nsteps >= 1 and K >= 1");
    if (!std::isfinite(dt)) return fail(c, GPSS_EINVAL, "dt must be finite");
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "no field uploaded");
    if (any_generic(c))
        return fail(c, GPSS_EINVAL, "gpss_adjoint: every axis must be a power of two of at most 256");
    CUDA_TRY(c, cudaSetDevice(c->device));
    GPSS_TRY(flush_pending(c));
    if (c->precision == GPSS_FP32) return adjoint_impl<float>(c, psi_target, nsteps, K, dt, loss, dLdV, dLdpsi0);
    return adjoint_impl<double>(c, psi_target, nsteps, K, dt, loss, dLdV, dLdpsi0);
}

}  // extern "C"
