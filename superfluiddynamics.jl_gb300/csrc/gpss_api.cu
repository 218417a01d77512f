// gpss_api.cu -- the C ABI of libgpss.so (include/gpss.h): context setup,
// host-built FP64 tables, and the orchestration of the directional passes
// that make up NumModelSplit1 / NumModelSplit2 time steps.
#include <cuda.h>
#include "ctx.cuh"

static thread_local std::string g_create_error;

int gpss::fail(gpss_ctx *c, int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    else g_create_error = buf;
    return code;
}

// Host-side fault injection for tests: with GPSS_FAULT_ALLOC=N in the
// environment, the N-th device allocation of the process fails as if the
// device were out of memory (no GPU fault is involved).
static bool injected_alloc_failure()
{
    static const long target = [] {
        const char *v = std::getenv("GPSS_FAULT_ALLOC");
        return v ? std::atol(v) : 0L;
    }();
    static std::atomic<long> count{0};
    return target > 0 && ++count == target;
}

int gpss::dev_alloc(gpss_ctx *c, void **p, size_t bytes)
{
    if (injected_alloc_failure()) {
        *p = nullptr;
        return fail(c, GPSS_ENOMEM, "cudaMalloc(%zu) failed: injected by GPSS_FAULT_ALLOC", bytes);
    }
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(c, GPSS_ENOMEM, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    }
    c->bytes += (int64_t)bytes;
    return GPSS_OK;
}


// energies from the per-axis sums (slot a holds the sums of the axis-a pass)
static void energies_from_sums(const gpss_ctx *c, const double *h, int point_slot, double *out)
{
    const double *pt = h + point_slot * RQ_COUNT;
    double grad = 0.0;
    for (int a = 0; a < c->ndim; a++) grad += h[a * RQ_COUNT + RQ_KIN];
    // sum Re(i conj(psi) Om (rx + ry)) = -Om (rot_x - rot_y) by Parseval on x and y lines
    const double rotx = h[0 * RQ_COUNT + RQ_ROT];
    const double roty = c->ndim >= 2 ? h[1 * RQ_COUNT + RQ_ROT] : 0.0;
    const double eom = times_cell(c, -c->omega * (rotx - roty));
    const double edel = times_cell(c, -c->cD * grad + pt[RQ_POT]);
    const double ebeta = times_cell(c, 0.5 * c->beta * pt[RQ_INT]);
    out[0] = eom;
    out[1] = edel;
    out[2] = ebeta;
    out[3] = -eom + edel + ebeta;
    out[4] = -eom + edel + ebeta * 2.0;
}

static int read_sums(gpss_ctx *c, double *h)
{
    CUDA_TRY(c, cudaMemcpyAsync(h, c->sums, sizeof(double) * 4 * RQ_COUNT, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return GPSS_OK;
}

template <typename T> static int energy_impl(gpss_ctx *c, double *out, double *mass)
{
    GPSS_TRY(diag_passes<T>(c, true, FIN_NONE));
    double h[4 * RQ_COUNT];
    GPSS_TRY(read_sums(c, h));
    if (!std::isfinite(h[RQ_MASS])) return fail(c, GPSS_ENONFINITE, "field holds NaN/Inf");
    if (out) energies_from_sums(c, h, 0, out);
    if (mass) *mass = times_cell(c, h[RQ_MASS]);
    return GPSS_OK;
}

// One kinetic flow L(dtl) in imaginary time as passes x, y[, z] for the
// merged step below: the first pass reads `in0` and may carry the nonlinear
// prologue (chi = N(dtnl)(c->scale * psi), stored to chi_out when non-null),
// the last pass writes `out_last` and may carry the nonlinear epilogue, the
// inner product with `dot_with` in place of the mass sum, and a finish.
template <typename T>
static int imag_flow(gpss_ctx *c, double dtl, const void *in0, bool pre_nl, void *chi_out, double dtnl,
                     bool nl_last, void *out_last, const void *dot_with, int red_last, int fin_last)
{
    for (int axis = 0; axis < c->ndim; axis++) {
        const bool first = axis == 0, last = axis == c->ndim - 1;
        PassArgs<T> a = axis_args<T>(c, axis, first ? in0 : c->psi, last ? out_last : c->psi);
        const void *ph;
        GPSS_TRY(get_phase(c, axis, dtl, 1, 1, &ph, &a.prow));
        a.phase = (const vec2<T> *)ph;
        if ((first && pre_nl) || (last && nl_last)) {
            a.V = c->have_V ? (const T *)c->V : nullptr;
            a.nl_beta = c->beta;
            a.nl_dt = dtnl;
            a.nl_split = nl_split(c->beta, dtnl);
        }
        if (first && pre_nl) {
            a.nl_pre = 1;
            a.scale = c->scale;
            a.nl_pre_out = (vec2<T> *)chi_out;
        }
        if (last) {
            if (nl_last) a.nl_mode = NL_IMAG;
            a.dot_with = (const vec2<T> *)dot_with;
            a.red |= red_last;
        }
        if (a.red) set_finish<T>(c, a, axis, last ? fin_last : FIN_NONE);
        GPSS_TRY(launch<T>(c, axis, MODE_FUSED, a));
    }
    return GPSS_OK;
}

// Imaginary time, Strang, Omega = 0, fused forms.  With chi_n = N L(dt/2)
// psi_n and the step psi_{n+1} = c_n L(dt/2) chi_n (c_n the unit-mass
// factor of normalize!, Fields.jl:196-200):
//     chi_{n+1} = N(c_n L(dt) chi_n),   c_n^-2 = <chi_n, L(dt) chi_n> dV,
// because L(dt/2) is real, positive and self-adjoint on the spectrum, so
// ||L(dt/2) chi||^2 = <chi, L(dt) chi>.  One kinetic flow per step instead of
// two: chi_n is kept in the scratch buffer for the inner product of the last
// pass, and N with the factor c_n runs as the prologue of the next first
// pass.  The sequence is L(dt/2) N | [L(dt) <.,.> | c N]^(n-1) | L(dt/2) |.|.
template <typename T> static int imag_merged(gpss_ctx *c, int nsteps, double dt)
{
    void *chi = c->scratch;
    GPSS_TRY(imag_flow<T>(c, dt * 0.5, c->psi, false, nullptr, dt, true, chi, nullptr, 0, FIN_NONE));
    auto full = [&](bool first) -> int {
        return imag_flow<T>(c, dt, first ? chi : c->psi, !first, chi, dt, false, c->psi, chi, RED_MASS,
                            FIN_UNITMASS);
    };
    int s = 1;
    if (s < nsteps) {
        GPSS_TRY(full(true));
        s++;
    }
    if (c->total <= kGraphCells) {
        const std::string key = graph_key("imag", {dt, (double)kGraphChunk});
        for (; s + kGraphChunk <= nsteps; s += kGraphChunk)
            GPSS_TRY(graph_run(c, key, [&]() -> int {
                for (int i = 0; i < kGraphChunk; i++) GPSS_TRY(full(false));
                return GPSS_OK;
            }));
    }
    for (; s < nsteps; s++) GPSS_TRY(full(false));
    // the last half step: psi_n = c L(dt/2) chi, c from its own mass
    GPSS_TRY(imag_flow<T>(c, dt * 0.5, nsteps == 1 ? chi : c->psi, nsteps > 1, nullptr, dt, false, c->psi,
                          nullptr, RED_MASS, FIN_UNITMASS));
    return apply_scale<T>(c);
}

// the cached energies of the current field (GPSS_FLAG_ENERGY_CACHE), if any
// Tensor maps for the FEAT_TMA y/z passes of an FP32 3D field: psi as a
// (nx, ny, nz) tensor of 8-byte elements, boxes of W x-adjacent columns by a
// whole line (W = the pass's lines per CTA, which must divide nx).  The
// encoder comes from the driver through the runtime's entry-point query, so
// the library links no driver library.  No map (a plain loads pass) when the
// shapes do not fit or the query fails.
#ifndef GPSS_PASS_TMA
#define GPSS_PASS_TMA 1
#endif
static int make_tensor_maps(gpss_ctx *c)
{
    if (!GPSS_PASS_TMA || c->precision != GPSS_FP32 || c->ndim != 3 || any_generic(c)) return GPSS_OK;
    using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
        cudaGetLastError();
        return GPSS_OK;
    }
    CUtensorMap maps[2];
    std::memset(maps, 0, sizeof(maps));
    const cuuint64_t dims[3] = {(cuuint64_t)c->n[0], (cuuint64_t)c->n[1], (cuuint64_t)c->n[2]};
    const cuuint64_t strides[2] = {(cuuint64_t)c->n[0] * 8, (cuuint64_t)(c->n[0] * c->n[1]) * 8};
    const cuuint32_t estr[3] = {1, 1, 1};
    for (int axis = 1; axis <= 2; axis++) {
        const int64_t n = c->n[axis];
        const int W = PassLauncher<float>::lines((int)n, false);
        if (n < 64 || W < 2 || c->n[0] % W) return GPSS_OK;
        const cuuint32_t box[3] = {(cuuint32_t)W, axis == 1 ? (cuuint32_t)n : 1u, axis == 2 ? (cuuint32_t)n : 1u};
        const CUresult r = reinterpret_cast<EncodeFn>(fn)(
            &maps[axis - 1], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, c->psi, dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return GPSS_OK;
    }
    GPSS_TRY(dev_alloc(c, &c->tmap_dev, sizeof(maps)));
    CUDA_TRY(c, cudaMemcpy(c->tmap_dev, maps, sizeof(maps), cudaMemcpyHostToDevice));
    return GPSS_OK;
}

static bool ecache_fresh(const gpss_ctx *c)
{
    return (c->flags & GPSS_FLAG_ENERGY_CACHE) && c->ecache_version == c->version;
}

// mass_slot >= 0: that sums slot holds the mass of the current field (the
// previous call measured it with the cached energies and nothing has changed
// since), so the FP32 mass lock takes its target from there instead of a
// read-only pass.
template <typename T>
static int step_impl(gpss_ctx *c, int nsteps, int scheme, int imag, double dt, gpss_diag *diag,
                     int mass_slot = -1)
{
    const bool plain = (c->flags & GPSS_FLAG_PLAIN) != 0;
    const bool merge = !plain && !imag && scheme == GPSS_STRANG && c->omega == 0.0 &&
                       !(c->flags & GPSS_FLAG_NOMERGE);
    // FP32 real time: restore the mass of the start of the call after every
    // nonlinear stage (every stage is unitary, so in exact arithmetic the
    // factor is 1; in FP32 it removes the drift that rounding feeds into the
    // global phase through the nonlinear frequency beta |psi|^2)
    const bool lock = !plain && !imag && c->precision == GPSS_FP32 && !(c->flags & GPSS_FLAG_NOMASSLOCK);
    const int red_nl = lock ? RED_MASS : 0;
    const int fin_nl = lock ? FIN_MASSLOCK : FIN_NONE;
    bool diag_done = false;
    // continue the previous call's merged sequence (its pending half flow is
    // folded into this call's first flow), or apply that flow first
    const bool chain = merge && nsteps > 0 && c->pending_h != 0.0;
    if (!chain) GPSS_TRY(flush_pending_t<T>(c));
    if (nsteps == 0) {
        if (diag) {
            diag->steps = 0;
            GPSS_TRY(energy_impl<T>(c, diag->energy, &diag->mass));
            c->ecache_mass_slot = 0;
        }
        return GPSS_OK;
    }
    // the status word: renormalisations and the mass lock report a non-finite
    // mass there, the pipelined pass a wait that gave up
    const bool pipe = (c->flags & GPSS_FLAG_PIPE) != 0;
    if (imag || lock || pipe) {
        CUDA_TRY(c, cudaMemsetAsync(c->status, 0, sizeof(int), c->stream));
    }
    if (lock && !chain) {  // target mass -> diagnostics slot (a chained call keeps the previous target)
        if (mass_slot >= 0) {
            CUDA_TRY(c, cudaMemcpyAsync(c->sums + kDiagSlot * RQ_COUNT + RQ_MASS,
                                        c->sums + mass_slot * RQ_COUNT + RQ_MASS, sizeof(double),
                                        cudaMemcpyDeviceToDevice, c->stream));
        } else {
            GPSS_TRY(diag_passes<T>(c, false, FIN_NONE));
        }
    }
    if (plain) {
        for (int s = 0; s < nsteps; s++) {
            if (scheme == GPSS_STRANG) {
                GPSS_TRY(kinetic_plain<T>(c, dt * 0.5, imag));
                GPSS_TRY(nl_plain<T>(c, dt, imag));
                GPSS_TRY(kinetic_plain<T>(c, dt * 0.5, imag));
            } else {
                GPSS_TRY(kinetic_plain<T>(c, dt, imag));
                GPSS_TRY(nl_plain<T>(c, dt, imag));
            }
            if (imag) {  // normalize! (Fields.jl:196-200)
                GPSS_TRY(diag_passes<T>(c, false, FIN_UNITMASS));
                GPSS_TRY(apply_scale<T>(c));
            }
        }
    } else if (merge) {
        // L(dt/2) N [L(dt) N]^(nsteps-1) L(dt/2): the kinetic flows of
        // consecutive steps commute (Omega = 0) and compose exactly.  A
        // pending flow of the previous call joins the first one.
        const double lead = dt * 0.5 + c->pending_h;
        const bool lead_scale = c->pending_scale;
        drop_pending(c);
        GPSS_TRY(kinetic_fused<T>(c, lead, 0, true, dt, red_nl, false, lead_scale, fin_nl));
        int s = 1;
        if (c->total <= kGraphCells) {
            const std::string key = graph_key("step", {dt, (double)lock, (double)kGraphChunk});
            for (; s + kGraphChunk <= nsteps; s += kGraphChunk)
                GPSS_TRY(graph_run(c, key, [&]() -> int {
                    for (int i = 0; i < kGraphChunk; i++)
                        GPSS_TRY(kinetic_fused<T>(c, dt, 0, true, dt, red_nl, false, lock, fin_nl));
                    return GPSS_OK;
                }));
        }
        for (; s < nsteps; s++)
            GPSS_TRY(kinetic_fused<T>(c, dt, 0, true, dt, red_nl, false, lock, fin_nl));
        // final half step; with diag, the kinetic sums of each axis are exact
        // for the final field (real-time kinetic flows are unitary and commute
        // with the other axes' derivatives when Omega = 0).  Without diag it
        // is left pending for the next call or the next read of the field.
        if (diag) {
            GPSS_TRY(kinetic_fused<T>(c, dt * 0.5, 0, false, 0.0, RED_POINT, true, lock));
            diag_done = true;
        } else {
            c->pending_h = dt * 0.5;
            c->pending_scale = lock;
        }
    } else if (imag && scheme == GPSS_STRANG && c->omega == 0.0 && !(c->flags & GPSS_FLAG_NOMERGE) &&
               !any_generic(c)) {
        GPSS_TRY(imag_merged<T>(c, nsteps, dt));
    } else if (imag) {
        for (int s = 0; s < nsteps; s++) {
            const bool pre = s > 0;
            if (scheme == GPSS_STRANG) {
                GPSS_TRY(kinetic_fused<T>(c, dt * 0.5, 1, true, dt, 0, false, pre));
                GPSS_TRY(kinetic_fused<T>(c, dt * 0.5, 1, false, 0.0, RED_MASS, false, false, FIN_UNITMASS));
            } else {
                GPSS_TRY(kinetic_fused<T>(c, dt, 1, true, dt, RED_MASS, false, pre, FIN_UNITMASS));
            }
        }
        GPSS_TRY(apply_scale<T>(c));
    } else {
        for (int s = 0; s < nsteps; s++) {
            if (scheme == GPSS_STRANG) {
                GPSS_TRY(kinetic_fused<T>(c, dt * 0.5, 0, true, dt, red_nl, false, false, fin_nl));
                if (diag && s == nsteps - 1) {
                    // the last half step measures the energies of the final
                    // field: its pointwise sums (last pass) and the kinetic
                    // sums of every axis the later passes leave unchanged --
                    // all of them when Omega = 0; with rotation the y flow
                    // (phase x xi_y) changes the x spectrum, so the x sums come
                    // from one read-only pass over the final field
                    GPSS_TRY(kinetic_fused<T>(c, dt * 0.5, 0, false, 0.0, RED_POINT, true, lock));
                    if (c->omega != 0.0 && c->ndim >= 2) GPSS_TRY(diag_kin_axis<T>(c, 0));
                    diag_done = true;
                } else {
                    GPSS_TRY(kinetic_fused<T>(c, dt * 0.5, 0, false, 0.0, 0, false, lock));
                }
            } else {
                GPSS_TRY(kinetic_fused<T>(c, dt, 0, true, dt, red_nl, false, lock && s > 0, fin_nl));
            }
        }
    }
    // the status word and (with fused diagnostics) the sums, one synchronisation
    const bool check = imag || lock || pipe, want_sums = diag && diag_done;
    double *h = c->host_stage;
    if (check) CUDA_TRY(c, cudaMemcpyAsync(h + 4 * RQ_COUNT, c->status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    if (want_sums)
        CUDA_TRY(c, cudaMemcpyAsync(h, c->sums, sizeof(double) * 4 * RQ_COUNT, cudaMemcpyDeviceToHost, c->stream));
    if (check || want_sums) CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (check) {
        int st = 0;
        std::memcpy(&st, h + 4 * RQ_COUNT, sizeof(int));
        if (st & 2) return fail(c, GPSS_ETIMEOUT, "a pipelined pass gave up waiting for a tile copy");
        if (st) return fail(c, GPSS_ENONFINITE, "a renormalisation saw a non-finite or zero mass");
    }
    if (diag) {
        diag->steps = nsteps;
        if (diag_done) {
            const int last = c->ndim - 1;
            if (!std::isfinite(h[last * RQ_COUNT + RQ_MASS]))
                return fail(c, GPSS_ENONFINITE, "field holds NaN/Inf");
            energies_from_sums(c, h, last, diag->energy);
            diag->mass = times_cell(c, h[last * RQ_COUNT + RQ_MASS]);
            c->ecache_mass_slot = last;
        } else {
            GPSS_TRY(energy_impl<T>(c, diag->energy, &diag->mass));
            c->ecache_mass_slot = 0;  // diag_passes with the kinetic sums: the mass is in slot 0
        }
    }
    return GPSS_OK;
}



extern "C" {

const char *gpss_version(void) { return GPSS_VERSION_STRING; }

const char *gpss_last_error(const gpss_ctx *ctx)
{
    if (!ctx) return g_create_error.c_str();
    return ctx->err.c_str();
}

void gpss_destroy(gpss_ctx *c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    clear_phases(c);  // and the graphs
    void *ptrs[] = {c->psi, c->scratch, c->V, c->tw[0], c->tw[1], c->tw[2], c->coord_dev[0],
                    c->coord_dev[1], c->coord_dev[2], c->partials, c->sums, c->scale, c->status,
                    c->counter, c->rk_buf[0], c->rk_buf[1], c->rk_buf[2], c->rk_buf[3], c->rk_lim,
                    c->adj_buf, c->im_buf, c->tmap_dev};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    for (auto &e : c->side_ev)
        if (e) cudaEventDestroy(e);
    if (c->side) {
        cudaStreamSynchronize(c->side);
        cudaStreamDestroy(c->side);
    }
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->host_stage) cudaFreeHost(c->host_stage);
    delete c;
}

int gpss_create(gpss_ctx **out, int ndim, const int64_t *n, const double *lo, const double *hi,
                int precision, int flags)
{
    NvtxRange nvtx_("gpss_create");
    if (!out || !n || !lo || !hi) return fail(nullptr, GPSS_EINVAL, "gpss_create: null argument");
    *out = nullptr;
    if (ndim != 2 && ndim != 3) return fail(nullptr, GPSS_EINVAL, "ndim must be 2 or 3 (got %d)", ndim);
    if (precision != GPSS_FP64 && precision != GPSS_FP32)
        return fail(nullptr, GPSS_EINVAL, "precision must be GPSS_FP64 or GPSS_FP32 (got %d)", precision);
    if (flags & ~(GPSS_FLAG_PLAIN | GPSS_FLAG_NOMERGE | GPSS_FLAG_NOMASSLOCK | GPSS_FLAG_PIPE | GPSS_FLAG_ENERGY_CACHE |
                  GPSS_FLAG_COMPENSATED))
        return fail(nullptr, GPSS_EINVAL, "unknown flags 0x%x", flags);
    bool any_gen = false;
    for (int a = 0; a < ndim; a++) {
        GenPlan gp;
        if (!reg_line(n[a]) && !(n[a] >= 2 && n[a] <= GEN_MAX_N && gen_plan_radices((int)n[a], gp)))
            return fail(nullptr, GPSS_EINVAL,
                        "n[%d] = %lld: each axis needs 2 <= n <= %d cells with no prime factor above 31", a,
                        (long long)n[a], GEN_MAX_N);
        any_gen = any_gen || !reg_line(n[a]);
        if (!(hi[a] > lo[a]) || !std::isfinite(lo[a]) || !std::isfinite(hi[a]))
            return fail(nullptr, GPSS_EINVAL, "axis %d: need finite lo < hi", a);
    }
    if (any_gen && (flags & GPSS_FLAG_COMPENSATED))
        return fail(nullptr, GPSS_EINVAL, "GPSS_FLAG_COMPENSATED needs every axis to be a power of two of at most 256");
    gpss_ctx *c = new (std::nothrow) gpss_ctx();
    if (!c) return fail(nullptr, GPSS_ENOMEM, "host allocation failed");
    c->ndim = ndim;
    c->precision = precision;
    c->flags = flags;
    c->total = 1;
    for (int a = 0; a < ndim; a++) {
        c->gen[a] = !reg_line(n[a]);
        if (c->gen[a]) {
            gen_plan_radices((int)n[a], c->gplan[a]);
            c->gplan[a].W = gen_tile_lines((int)n[a], precision == GPSS_FP32 ? 4 : 8);
        }
    }
    for (int a = 0; a < 3; a++) {
        c->n[a] = a < ndim ? n[a] : 1;
        c->lo[a] = a < ndim ? lo[a] : 0.0;
        c->hi[a] = a < ndim ? hi[a] : 1.0;
        c->L[a] = c->hi[a] - c->lo[a];
        c->d[a] = c->L[a] / (double)c->n[a];
        c->total *= c->n[a];
        grid_coords(c->n[a], c->lo[a], c->hi[a], c->coord[a]);
    }
    auto bail = [&](int rc) {
        g_create_error = c->err;
        gpss_destroy(c);
        return rc;
    };
    cudaError_t e = cudaGetDevice(&c->device);
    if (e != cudaSuccess) { fail(c, GPSS_ECUDA, "cudaGetDevice: %s", cudaGetErrorString(e)); return bail(GPSS_ECUDA); }
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { fail(c, GPSS_ECUDA, "cudaStreamCreate: %s", cudaGetErrorString(e)); return bail(GPSS_ECUDA); }
    for (auto &ev : c->ev) {
        e = cudaEventCreate(&ev);
        if (e != cudaSuccess) { fail(c, GPSS_ECUDA, "cudaEventCreate: %s", cudaGetErrorString(e)); return bail(GPSS_ECUDA); }
    }
    int rc;
    if ((rc = dev_alloc(c, &c->psi, (size_t)c->total * cplx_bytes(c)))) return bail(rc);
    if ((rc = dev_alloc(c, &c->scratch, (size_t)c->total * 16))) return bail(rc);
    // twiddles per axis, stage-A layout m = k1*N2 + r: exp(-2 pi i r k1 / n) as hi + lo
    for (int a = 0; a < ndim; a++) {
        const int64_t na = c->n[a];
        std::vector<ldouble> re, im;
        if (c->gen[a]) {
            // generic pass: the roots w_n^k = exp(-2 pi i k / n), k < n
            re.resize((size_t)na);
            im.resize((size_t)na);
            for (int64_t k = 0; k < na; k++) {
                ldouble cs, sn;
                unit_root(k, na, &cs, &sn);
                re[(size_t)k] = cs;
                im[(size_t)k] = -sn;
            }
            if ((rc = upload_dw(c, &c->tw[a], re, im, 1, na))) return bail(rc);
        } else {
            // two rows: stage-A order (k1*N2 + r) and stage-B order (r*N1 + k1)
            twiddle_rows(na, re, im);
            if ((rc = upload_dw(c, &c->tw[a], re, im, 2, na))) return bail(rc);
        }
        if ((rc = dev_alloc(c, (void **)&c->coord_dev[a], sizeof(double) * (size_t)c->n[a]))) return bail(rc);
        e = cudaMemcpy(c->coord_dev[a], c->coord[a].data(), sizeof(double) * (size_t)c->n[a], cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { fail(c, GPSS_ECUDA, "cudaMemcpy: %s", cudaGetErrorString(e)); return bail(GPSS_ECUDA); }
    }
    int maxb = 1;
    for (int a = 0; a < ndim; a++) {
        int b = precision == GPSS_FP32 ? blocks_for<float>(c, a) : blocks_for<double>(c, a);
        if (b > maxb) maxb = b;
    }
    c->max_blocks = maxb;
    if ((rc = dev_alloc(c, (void **)&c->partials, sizeof(double) * RQ_COUNT * (size_t)maxb))) return bail(rc);
    if ((rc = dev_alloc(c, (void **)&c->sums, sizeof(double) * 4 * RQ_COUNT))) return bail(rc);
    if ((rc = dev_alloc(c, (void **)&c->scale, sizeof(double) * 2))) return bail(rc);
    if ((rc = dev_alloc(c, (void **)&c->status, sizeof(int) * 2))) return bail(rc);
    if ((rc = dev_alloc(c, (void **)&c->counter, sizeof(unsigned int) * 2))) return bail(rc);
    if ((rc = make_tensor_maps(c))) return bail(rc);
    e = cudaHostAlloc((void **)&c->host_stage, sizeof(double) * (4 * RQ_COUNT + 1), cudaHostAllocDefault);
    if (e != cudaSuccess) {
        c->host_stage = nullptr;
        fail(c, GPSS_ENOMEM, "cudaHostAlloc: %s", cudaGetErrorString(e));
        return bail(GPSS_ENOMEM);
    }
    e = cudaMemset(c->counter, 0, sizeof(unsigned int) * 2);
    if (e != cudaSuccess) { fail(c, GPSS_ECUDA, "cudaMemset: %s", cudaGetErrorString(e)); return bail(GPSS_ECUDA); }
    const ScaleCell one = {1.0, 1.0f};
    e = cudaMemcpy(c->scale, &one, sizeof(one), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { fail(c, GPSS_ECUDA, "cudaMemcpy: %s", cudaGetErrorString(e)); return bail(GPSS_ECUDA); }
    *out = c;
    return GPSS_OK;
}

int gpss_set_params(gpss_ctx *c, double coeffD, double beta, double omega)
{
    if (!c) return GPSS_EINVAL;
    c->version++;  // the field or the parameters may change
    if (!std::isfinite(coeffD) || !std::isfinite(beta) || !std::isfinite(omega))
        return fail(c, GPSS_EINVAL, "parameters must be finite");
    CUDA_TRY(c, cudaSetDevice(c->device));
    GPSS_TRY(flush_pending(c));  // with the parameters it was computed for
    if (coeffD != c->cD || omega != c->omega) clear_phases(c);
    clear_graphs(c);
    c->cD = coeffD;
    c->beta = beta;
    c->omega = omega;
    return GPSS_OK;
}

int gpss_set_potential(gpss_ctx *c, const double *V)
{
    if (!c) return GPSS_EINVAL;
    c->version++;  // the field or the parameters may change
    CUDA_TRY(c, cudaSetDevice(c->device));
    GPSS_TRY(flush_pending(c));
    clear_graphs(c);
    if (!V) { c->have_V = false; return GPSS_OK; }
    if (!c->V) GPSS_TRY(dev_alloc(c, &c->V, (size_t)c->total * real_bytes(c)));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (c->precision == GPSS_FP64) {
        CUDA_TRY(c, cudaMemcpyAsync(c->V, V, (size_t)c->total * 8, cudaMemcpyHostToDevice, c->stream));
    } else {
        CUDA_TRY(c, cudaMemcpyAsync(c->scratch, V, (size_t)c->total * 8, cudaMemcpyHostToDevice, c->stream));
        CUDA_TRY(c, launch_f64_to_f32((const double *)c->scratch, (float *)c->V, c->total, c->stream));
        c->launches++;
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    c->have_V = true;
    return GPSS_OK;
}

int gpss_upload(gpss_ctx *c, const double *psi)
{
    NvtxRange nvtx_("gpss_upload");
    if (!c) return GPSS_EINVAL;
    c->version++;  // the field or the parameters may change
    if (!psi) return fail(c, GPSS_EINVAL, "gpss_upload: null psi");
    CUDA_TRY(c, cudaSetDevice(c->device));
    drop_pending(c);  // the field is replaced
    if (c->precision == GPSS_FP64) {
        CUDA_TRY(c, cudaMemcpyAsync(c->psi, psi, (size_t)c->total * 16, cudaMemcpyHostToDevice, c->stream));
    } else {
        CUDA_TRY(c, cudaMemcpyAsync(c->scratch, psi, (size_t)c->total * 16, cudaMemcpyHostToDevice, c->stream));
        CUDA_TRY(c, launch_f64_to_f32((const double *)c->scratch, (float *)c->psi, 2 * c->total, c->stream));
        c->launches++;
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    c->have_psi = true;
    return GPSS_OK;
}

int gpss_download(gpss_ctx *c, double *psi)
{
    NvtxRange nvtx_("gpss_download");
    if (!c) return GPSS_EINVAL;
    if (!psi) return fail(c, GPSS_EINVAL, "gpss_download: null psi");
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "no field uploaded");
    CUDA_TRY(c, cudaSetDevice(c->device));
    GPSS_TRY(flush_pending(c));
    if (c->precision == GPSS_FP64) {
        CUDA_TRY(c, cudaMemcpyAsync(psi, c->psi, (size_t)c->total * 16, cudaMemcpyDeviceToHost, c->stream));
    } else {
        CUDA_TRY(c, launch_f32_to_f64((const float *)c->psi, (double *)c->scratch, 2 * c->total, c->stream));
        c->launches++;
        CUDA_TRY(c, cudaMemcpyAsync(psi, c->scratch, (size_t)c->total * 16, cudaMemcpyDeviceToHost, c->stream));
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return GPSS_OK;
}

int gpss_step(gpss_ctx *c, int nsteps, int scheme, int imag, double dt, gpss_diag *diag)
{
    NvtxRange nvtx_("gpss_step");
    if (!c) return GPSS_EINVAL;
    const int mass_slot = ecache_fresh(c) ? c->ecache_mass_slot : -1;  // before the version moves on
    c->version++;  // the field or the parameters may change
    if (nsteps < 0) return fail(c, GPSS_EINVAL, "nsteps must be >= 0");
    if (scheme != GPSS_LIE && scheme != GPSS_STRANG) return fail(c, GPSS_EINVAL, "scheme must be 1 (Lie) or 2 (Strang)");
    if (!std::isfinite(dt)) return fail(c, GPSS_EINVAL, "dt must be finite");
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "no field uploaded");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (nsteps == 0 && !diag) return GPSS_OK;
    // GPSS_FLAG_ENERGY_CACHE: where the final passes can measure the energies
    // at no extra sweep (merged real-time Strang), do so and keep them
    gpss_diag own;
    gpss_diag *d = diag;
    if (!d && (c->flags & GPSS_FLAG_ENERGY_CACHE) && !imag && scheme == GPSS_STRANG &&
        !(c->flags & GPSS_FLAG_PLAIN) && nsteps > 0)
        d = &own;
    const int rc = c->precision == GPSS_FP32 ? step_impl<float>(c, nsteps, scheme, imag, dt, d, mass_slot)
                                             : step_impl<double>(c, nsteps, scheme, imag, dt, d, mass_slot);
    if (rc == GPSS_OK && d) {
        for (int i = 0; i < 5; i++) c->ecache[i] = d->energy[i];
        c->ecache_mass = d->mass;
        c->ecache_version = c->version;
    }
    return rc;
}




int gpss_energy(gpss_ctx *c, double *out)
{
    NvtxRange nvtx_("gpss_energy");
    if (!c || !out) return c ? fail(c, GPSS_EINVAL, "gpss_energy: null out") : GPSS_EINVAL;
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "no field uploaded");
    if (ecache_fresh(c)) {
        for (int i = 0; i < 5; i++) out[i] = c->ecache[i];
        return GPSS_OK;
    }
    CUDA_TRY(c, cudaSetDevice(c->device));
    GPSS_TRY(flush_pending(c));
    if (c->precision == GPSS_FP32) return energy_impl<float>(c, out, nullptr);
    return energy_impl<double>(c, out, nullptr);
}

// sum |psi|^2 of the device field (no cell volume)
static int raw_mass(gpss_ctx *c, double *out)
{
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "no field uploaded");
    CUDA_TRY(c, cudaSetDevice(c->device));
    GPSS_TRY(flush_pending(c));
    int rc = c->precision == GPSS_FP32 ? diag_passes<float>(c, false, FIN_NONE)
                                       : diag_passes<double>(c, false, FIN_NONE);
    if (rc) return rc;
    double h[4 * RQ_COUNT];
    GPSS_TRY(read_sums(c, h));
    const double m = h[kDiagSlot * RQ_COUNT + RQ_MASS];
    if (!std::isfinite(m)) return fail(c, GPSS_ENONFINITE, "field holds NaN/Inf");
    *out = m;
    return GPSS_OK;
}

int gpss_mass(gpss_ctx *c, double *out)
{
    if (!c || !out) return c ? fail(c, GPSS_EINVAL, "gpss_mass: null out") : GPSS_EINVAL;
    if (c->have_psi && ecache_fresh(c)) {
        *out = c->ecache_mass;
        return GPSS_OK;
    }
    double raw;
    GPSS_TRY(raw_mass(c, &raw));
    *out = times_cell(c, raw);
    return GPSS_OK;
}

int gpss_norm(gpss_ctx *c, double *out)
{
    if (!c || !out) return c ? fail(c, GPSS_EINVAL, "gpss_norm: null out") : GPSS_EINVAL;
    double raw;
    GPSS_TRY(raw_mass(c, &raw));
    // Fields.jl:172-180: sqrt(sum |psi|^2) * sqrt(dx dy [dz])
    *out = std::sqrt(raw) * std::sqrt(cell_volume(c));
    return GPSS_OK;
}

int gpss_normalize(gpss_ctx *c)
{
    NvtxRange nvtx_("gpss_normalize");
    if (!c) return GPSS_EINVAL;
    c->version++;  // the field or the parameters may change
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "no field uploaded");
    CUDA_TRY(c, cudaSetDevice(c->device));
    GPSS_TRY(flush_pending(c));
    return c->precision == GPSS_FP32 ? normalize_impl<float>(c) : normalize_impl<double>(c);
}

int gpss_ground_state(gpss_ctx *c, double dt, double tol, int64_t max_steps, int check_every,
                      double *mu_out, int64_t *steps_out)
{
    NvtxRange nvtx_("gpss_ground_state");
    if (!c) return GPSS_EINVAL;
    c->version++;  // the field or the parameters may change
    if (!(dt > 0) || !(tol > 0) || max_steps < 1 || check_every < 1)
        return fail(c, GPSS_EINVAL, "ground_state: need dt > 0, tol > 0, max_steps >= 1, check_every >= 1");
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "no field uploaded");
    double mu_prev = NAN, e[5] = {0, 0, 0, 0, 0};
    int64_t done = 0;
    GPSS_TRY(gpss_normalize(c));
    while (done < max_steps) {
        int64_t k = check_every;
        if (k > max_steps - done) k = max_steps - done;
        GPSS_TRY(gpss_step(c, (int)k, GPSS_STRANG, 1, dt, nullptr));
        done += k;
        GPSS_TRY(gpss_energy(c, e));
        if (std::isfinite(mu_prev) && std::fabs(e[4] - mu_prev) < tol) break;
        mu_prev = e[4];
    }
    if (mu_out) *mu_out = e[4];
    if (steps_out) *steps_out = done;
    return GPSS_OK;
}

int gpss_select_device(int device)
{
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        g_create_error = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
        return device < 0 ? GPSS_EINVAL : GPSS_ECUDA;
    }
    return GPSS_OK;
}

int gpss_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}


int gpss_sync(gpss_ctx *c)
{
    if (!c) return GPSS_EINVAL;
    CUDA_TRY(c, cudaSetDevice(c->device));
    GPSS_TRY(flush_pending(c));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return GPSS_OK;
}

int gpss_flush(gpss_ctx *c)
{
    if (!c) return GPSS_EINVAL;
    return flush_pending(c);
}

int gpss_event_record(gpss_ctx *c, int slot)
{
    if (!c || slot < 0 || slot >= 8) return c ? fail(c, GPSS_EINVAL, "event slot must be 0..7") : GPSS_EINVAL;
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaEventRecord(c->ev[slot], c->stream));
    return GPSS_OK;
}

int gpss_event_elapsed(gpss_ctx *c, int a, int b, float *ms)
{
    if (!c || !ms || a < 0 || a >= 8 || b < 0 || b >= 8) return c ? fail(c, GPSS_EINVAL, "bad event slots") : GPSS_EINVAL;
    CUDA_TRY(c, cudaEventSynchronize(c->ev[b]));
    CUDA_TRY(c, cudaEventElapsedTime(ms, c->ev[a], c->ev[b]));
    return GPSS_OK;
}

int64_t gpss_launch_count(const gpss_ctx *c) { return c ? c->launches : -1; }

int64_t gpss_device_bytes(const gpss_ctx *c)
{
    if (!c) return -1;
    return c->bytes;
}

int gpss_time_pass(gpss_ctx *c, int axis, int mode, int reps, double dt, double *ms_per_launch)
{
    if (!c || !ms_per_launch) return c ? fail(c, GPSS_EINVAL, "null argument") : GPSS_EINVAL;
    c->version++;  // the field or the parameters may change
    if (axis < 0 || axis >= c->ndim || reps < 1 || (mode != 0 && mode != 1))
        return fail(c, GPSS_EINVAL, "time_pass: bad axis/mode/reps");
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "no field uploaded");
    CUDA_TRY(c, cudaSetDevice(c->device));
    GPSS_TRY(flush_pending(c));
    auto run = [&](auto tag) -> int {
        using T = decltype(tag);
        PassArgs<T> a = axis_args<T>(c, axis, c->psi, c->psi);
        const void *ph;
        GPSS_TRY(get_phase(c, axis, dt, 0, 1, &ph, &a.prow));
        a.phase = (const vec2<T> *)ph;
        a.comp = sizeof(T) == 4 && (c->flags & GPSS_FLAG_COMPENSATED) != 0;
        if (a.comp) {  // the mass bound of the real-time passes (the mass-lock target slot)
            GPSS_TRY(diag_passes<T>(c, false, FIN_NONE));
            a.grid_mass = c->sums + kDiagSlot * RQ_COUNT + RQ_MASS;
        } else if (c->tmap_dev && axis >= 1) {  // the tensor-copy tiles of the real-time y/z passes
            a.tmap = (const char *)c->tmap_dev + (axis - 1) * sizeof(CUtensorMap);
            a.taxis = axis;
            a.tnx = (int)c->n[0];
            a.fin_status = c->status;
            CUDA_TRY(c, cudaMemsetAsync(c->status, 0, sizeof(int), c->stream));
        }
        if (mode == 1) {
            a.nl_mode = NL_REAL;
            a.V = c->have_V ? (const T *)c->V : nullptr;
            a.nl_beta = c->beta;
            a.nl_dt = dt;
            a.nl_split = nl_split(c->beta, dt);
        }
        GPSS_TRY(launch<T>(c, axis, MODE_FUSED, a));  // warm-up
        CUDA_TRY(c, cudaEventRecord(c->ev[6], c->stream));
        for (int i = 0; i < reps; i++) GPSS_TRY(launch<T>(c, axis, MODE_FUSED, a));
        CUDA_TRY(c, cudaEventRecord(c->ev[7], c->stream));
        CUDA_TRY(c, cudaEventSynchronize(c->ev[7]));
        float ms = 0.f;
        CUDA_TRY(c, cudaEventElapsedTime(&ms, c->ev[6], c->ev[7]));
        *ms_per_launch = (double)ms / reps;
        return GPSS_OK;
    };
    return c->precision == GPSS_FP32 ? run(0.0f) : run(0.0);
}

int gpss_host_alloc(void **ptr, int64_t bytes)
{
    if (!ptr || bytes <= 0) return GPSS_EINVAL;
    cudaError_t e = cudaHostAlloc(ptr, (size_t)bytes, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        g_create_error = std::string("cudaHostAlloc: ") + cudaGetErrorString(e);
        return GPSS_ENOMEM;
    }
    return GPSS_OK;
}

int gpss_host_free(void *ptr)
{
    if (!ptr) return GPSS_OK;
    cudaError_t e = cudaFreeHost(ptr);
    return e == cudaSuccess ? GPSS_OK : GPSS_ECUDA;
}

}  // extern "C"
