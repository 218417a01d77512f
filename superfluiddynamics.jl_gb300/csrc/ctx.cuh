// ctx.cuh -- the context of libgpss.so and the host helpers shared by its
// translation units (gpss_api.cu: setup, split steps, energies and the C ABI;
// adjoint_host.cu: the discrete adjoint; solvers.cu: explicit Runge-Kutta and
// the implicit schemes).  Internal: not part of the installed interface.
#pragma once
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <new>
#include <string>
#include <nvtx3/nvToolsExt.h>
#include <cuda.h>
#include "../../include/gpss.h"
#include "gpss_internal.h"

using namespace gpss;


#define GPSS_VERSION_STRING "gpss 0.1.0 (sm_103a)"

static const double kTwoPi = 6.283185307179586;  // Float64(2pi)

struct PhaseEntry {
    int axis, imag, fused;
    double dtl, cD, om;
    void *dev;
    int64_t prow;
};

struct gpss_ctx {
    int ndim = 0;
    int64_t n[3] = {1, 1, 1};
    double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1}, L[3] = {1, 1, 1}, d[3] = {1, 1, 1};
    int64_t total = 0;
    int precision = GPSS_FP64;
    int flags = 0;
    double cD = -0.5, beta = 1.0, omega = 0.0;
    bool have_psi = false;
    bool have_V = false;
    // energies of the field as of `version` (GPSS_FLAG_ENERGY_CACHE); every
    // entry point that may change the field or the parameters bumps version
    uint64_t version = 0, ecache_version = ~uint64_t(0);
    // a merged real-time Strang call leaves its trailing half kinetic flow
    // L(pending_h) unapplied (see flush_pending); pending_scale: the mass
    // lock's factor in `scale` is still to be applied by that flow's first pass
    double pending_h = 0.0;
    bool pending_scale = false;
    double ecache[5] = {0, 0, 0, 0, 0}, ecache_mass = 0;
    int ecache_mass_slot = 0;  // sums slot holding the raw mass the cached energies came with
    // pinned host copy of the sums (4 slots) and the status word, so that the
    // end of a step call reads both with one synchronisation
    double *host_stage = nullptr;
    int device = 0;
    cudaStream_t stream = nullptr;
    void *psi = nullptr;      // device field (float2 or double2)
    void *scratch = nullptr;  // spectrum (plain form) and FP64 staging, total*16 bytes
    void *V = nullptr;        // device potential (float or double)
    void *tw[3] = {nullptr, nullptr, nullptr};  // per axis: register-kernel twiddles, or the generic pass's roots
    // axes whose lines the generic pass runs (not a power of two in [2, 256])
    bool gen[3] = {false, false, false};
    GenPlan gplan[3] = {};
    double *coord_dev[3] = {nullptr, nullptr, nullptr};
    std::vector<double> coord[3];
    double *partials = nullptr;
    int max_blocks = 0;
    // FP32 3D fields: tensor maps of psi for the y and z passes' tile copies
    // (two CUtensorMap, 64-byte aligned, in device memory); null if unused
    void *tmap_dev = nullptr;
    double *sums = nullptr;   // [4][RQ_COUNT]: slots 0..2 per axis, slot 3 diagnostics
    double *scale = nullptr;  // ScaleCell: the factor in FP64 and as a float
    int *status = nullptr;    // [1]
    unsigned int *counter = nullptr;  // arrival counter of the in-kernel reduction finish
    std::vector<PhaseEntry> phases;
    void *rk_buf[4] = {nullptr, nullptr, nullptr, nullptr};  // RK: stage state, lapRot, NL term, sum
    int *rk_lim = nullptr;    // RK: 2/3-rule limits per inner position (the FEAT_MASK pass)
    void *im_buf = nullptr;   // implicit schemes: work fields (implicit_impl)
    size_t im_bytes = 0;
    // discrete adjoint: buffers kept between calls (sized for adj_nck checkpoints, adj_K states)
    void *adj_buf = nullptr;
    size_t adj_bytes = 0;
    // the adjoint's second stream (segment recomputes beside the backward
    // sweep) and its fork/join events, made on first use
    cudaStream_t side = nullptr;
    cudaEvent_t side_ev[3] = {nullptr, nullptr, nullptr};
    // CUDA graphs of repeated launch sequences (graph_run), keyed by what they bake in
    struct GraphEntry {
        std::string key;
        cudaGraphExec_t exec = nullptr;  // null: seen once, captured on the next call
        int64_t launches = 0;
    };
    std::vector<GraphEntry> graphs;
    cudaEvent_t ev[8] = {};
    int64_t launches = 0;
    int64_t bytes = 0;
    std::string err;
};

namespace gpss {
// the message of the last error of a context (or of gpss_create), set by fail()
int fail(gpss_ctx *c, int code, const char *fmt, ...);
// cudaMalloc on behalf of a context (counted in its bytes; honours GPSS_FAULT_ALLOC)
int dev_alloc(gpss_ctx *c, void **p, size_t bytes);
}  // namespace gpss

#define CUDA_TRY(c, call)                                                                   \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail((c), GPSS_ECUDA, "%s failed: %s", #call, cudaGetErrorString(e_));    \
    } while (0)

#define GPSS_TRY(call)            \
    do {                          \
        int rc_ = (call);         \
        if (rc_ != GPSS_OK)       \
            return rc_;           \
    } while (0)

// NVTX range around an entry point (profilers show the C ABI calls as ranges)
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

typedef long double ldouble;

// Grids.jl:78-84: x = LinRange(lo, hi, n+1)[1:end-1] (lerps of Base.LinRange)
static double lerpi(int64_t j, int64_t dd, double a, double b)
{
    double t = (double)j / (double)dd;
    return (1.0 - t) * a + t * b;
}

static void grid_coords(int64_t n, double lo, double hi, std::vector<double> &x)
{
    x.resize((size_t)n);
    if (n <= 1) { x[0] = lo; return; }
    double first = lerpi(0, n, lo, hi), last = lerpi(n - 1, n, lo, hi);
    for (int64_t i = 0; i < n; i++) x[(size_t)i] = lerpi(i, n - 1, first, last);
}

// Plans.jl:829-830: xi_k = kk * ((2pi/dx)/n), kk the signed index of fftfreq
static double xi_mult(const gpss_ctx *c, int axis) { return (kTwoPi / c->d[axis]) / (double)c->n[axis]; }
static double xi_of(const gpss_ctx *c, int axis, int64_t k)
{
    int64_t n = c->n[axis];
    int64_t kk = k < (n + 1) / 2 ? k : k - n;
    return (double)kk * xi_mult(c, axis);
}

static size_t cplx_bytes(const gpss_ctx *c) { return c->precision == GPSS_FP32 ? 8 : 16; }
static size_t real_bytes(const gpss_ctx *c) { return c->precision == GPSS_FP32 ? 4 : 8; }

// Upload complex values v[0..cnt) (cnt = rows * n, row-major) as double-word
// pairs in the field precision: per row hi[n] then lo[n], hi + lo = v.
static int upload_dw(gpss_ctx *c, void **dev, const std::vector<ldouble> &re, const std::vector<ldouble> &im,
                     int64_t rows, int64_t n)
{
    (void)rows;
    if (c->precision == GPSS_FP32) {
        const std::vector<float2> f = dw_split<float>(re, im, n);
        GPSS_TRY(dev_alloc(c, dev, f.size() * sizeof(float2)));
        CUDA_TRY(c, cudaMemcpy(*dev, f.data(), f.size() * sizeof(float2), cudaMemcpyHostToDevice));
        return GPSS_OK;
    }
    const std::vector<double2> h = dw_split<double>(re, im, n);
    GPSS_TRY(dev_alloc(c, dev, h.size() * sizeof(double2)));
    CUDA_TRY(c, cudaMemcpy(*dev, h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice));
    return GPSS_OK;
}

static void clear_graphs(gpss_ctx *c);

// Kinetic factor table for `axis` (splitting.jl:167/172/190/195/200):
// real time  exp(i (cD xi^2 -/+ Om c xi) dtl), imaginary time exp((...) dtl),
// imag == 2: the multiplier cD xi^2 -/+ Om c xi itself (the axis term of
// lapRot, GrossPitaevskii.jl:12-45; dtl unused); fused tables also carry the
// 1/n of the inverse transform.  With Omega != 0 the x (y) table has one row
// per y (x) node.
static int get_phase(gpss_ctx *c, int axis, double dtl, int imag, int fused, const void **dev,
                     int64_t *prow)
{
    for (auto &e : c->phases) {
        if (e.axis == axis && e.dtl == dtl && e.imag == imag && e.fused == fused && e.cD == c->cD &&
            e.om == c->omega) {
            *dev = e.dev;
            *prow = e.prow;
            return GPSS_OK;
        }
    }
    const int64_t n = c->n[axis];
    const bool rot = c->omega != 0.0 && axis < 2 && c->ndim >= 2;
    const int64_t rows = rot ? (axis == 0 ? c->n[1] : c->n[0]) : 1;
    std::vector<ldouble> re((size_t)(n * rows)), im((size_t)(n * rows));
    const ldouble inv_n = fused ? 1.0L / (ldouble)n : 1.0L;
    for (int64_t r = 0; r < rows; r++) {
        const double cr = rot ? (axis == 0 ? c->coord[1][(size_t)r] : c->coord[0][(size_t)r]) : 0.0;
        for (int64_t k = 0; k < n; k++) {
            // the phase argument is the reference's Float64 expression; its
            // exponential is evaluated in long double and kept as hi + lo
            const double xk = xi_of(c, axis, k);
            double ph;
            if (axis == 0) ph = c->cD * (xk * xk) - c->omega * cr * xk;
            else if (axis == 1) ph = c->cD * (xk * xk) + c->omega * cr * xk;
            else ph = c->cD * (xk * xk);
            ldouble fr, fi;
            if (imag == 2) { fr = (ldouble)ph; fi = 0.0L; }  // the multiplier itself (lapRot)
            else if (!imag) { const ldouble t = (ldouble)(ph * dtl); fr = cosl(t); fi = sinl(t); }
            else { fr = expl((ldouble)(ph * dtl)); fi = 0.0L; }
            re[(size_t)(r * n + k)] = fr * inv_n;
            im[(size_t)(r * n + k)] = fi * inv_n;
        }
    }
    PhaseEntry e{axis, imag, fused, dtl, c->cD, c->omega, nullptr, rot ? 2 * n : 0};
    GPSS_TRY(upload_dw(c, &e.dev, re, im, rows, n));
    if (c->phases.size() > 64) {  // bounded cache: drop the oldest
        clear_graphs(c);
        cudaStreamSynchronize(c->stream);
        cudaFree(c->phases.front().dev);
        c->phases.erase(c->phases.begin());
    }
    c->phases.push_back(e);
    *dev = e.dev;
    *prow = e.prow;
    return GPSS_OK;
}

// Graphs hold kernel arguments (table and buffer pointers, beta, V): any change
// of those drops them.
static void clear_graphs(gpss_ctx *c)
{
    if (c->graphs.empty()) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto &e : c->graphs)
        if (e.exec) cudaGraphExecDestroy(e.exec);
    c->graphs.clear();
}

static void clear_phases(gpss_ctx *c)
{
    clear_graphs(c);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto &e : c->phases) cudaFree(e.dev);
    c->phases.clear();
}

// Run a launch sequence that is issued repeatedly with the same arguments: the
// first time eagerly (which also creates its tables and kernel attributes),
// the second time captured into a CUDA graph, afterwards by launching the
// graph.  Small fields spend most of a step in launch overhead; a graph
// replays the sequence with back-to-back kernels.
template <typename F> static int graph_run(gpss_ctx *c, const std::string &key, F issue)
{
    for (auto &e : c->graphs) {
        if (e.key != key) continue;
        if (e.exec) {
            CUDA_TRY(c, cudaGraphLaunch(e.exec, c->stream));
            c->launches += e.launches;
            return GPSS_OK;
        }
        const int64_t l0 = c->launches;
        CUDA_TRY(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = issue();
        cudaGraph_t g = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(c->stream, &g);
        if (rc != GPSS_OK) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (ee != cudaSuccess) return fail(c, GPSS_ECUDA, "graph capture: %s", cudaGetErrorString(ee));
        const cudaError_t ie = cudaGraphInstantiate(&e.exec, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            e.exec = nullptr;
            return fail(c, GPSS_ECUDA, "graph instantiate: %s", cudaGetErrorString(ie));
        }
        e.launches = c->launches - l0;
        CUDA_TRY(c, cudaGraphLaunch(e.exec, c->stream));
        return GPSS_OK;
    }
    if (c->graphs.size() >= 16) {
        cudaStreamSynchronize(c->stream);
        if (c->graphs.front().exec) cudaGraphExecDestroy(c->graphs.front().exec);
        c->graphs.erase(c->graphs.begin());
    }
    c->graphs.push_back(gpss_ctx::GraphEntry{key, nullptr, 0});
    return issue();
}

static std::string graph_key(const char *what, std::initializer_list<double> v)
{
    std::string k(what);
    char buf[40];
    for (double x : v) {
        snprintf(buf, sizeof(buf), ":%a", x);
        k += buf;
    }
    return k;
}

// fields up to this many cells replay their repeated step sequences from CUDA graphs
static const int64_t kGraphCells = int64_t(1) << 21;
static const int kGraphChunk = 32;  // time steps per captured chunk

template <typename T> static PassArgs<T> axis_args(gpss_ctx *c, int axis, const void *in, void *out)
{
    PassArgs<T> a;
    memset(&a, 0, sizeof(a));
    const int64_t nx = c->n[0], ny = c->n[1];
    const int64_t n = c->n[axis];
    a.in = (const vec2<T> *)in;
    a.out = (vec2<T> *)out;
    a.tw = (const vec2<T> *)c->tw[axis];
    a.nlines = (int)(c->total / n);
    if (axis == 0) { a.m0 = a.nlines; a.s0 = nx; a.s1 = 0; a.stride = 1; a.rowmod = (int)ny; }
    else if (axis == 1) { a.m0 = (int)nx; a.s0 = 1; a.s1 = nx * ny; a.stride = nx; a.rowmod = (int)nx; }
    else { a.m0 = a.nlines; a.s0 = 1; a.s1 = 0; a.stride = nx * ny; a.rowmod = 1; }
    a.inv_n = (T)(1.0 / (double)n);
    a.kmult = xi_mult(c, axis);
    a.nl_mode = NL_NONE;
    return a;
}

static bool any_generic(const gpss_ctx *c) { return c->gen[0] || c->gen[1] || c->gen[2]; }

template <typename T> static int blocks_for(gpss_ctx *c, int axis)
{
    if (c->gen[axis]) return (int)((c->total / c->n[axis] + c->gplan[axis].W - 1) / c->gplan[axis].W);
    const int W = PassLauncher<T>::lines((int)c->n[axis], axis == 0);
    const int64_t nl = c->total / c->n[axis];
    return (int)((nl + W - 1) / W);
}

// Does this fused pass go through the pipelined kernel?  Only on request
// (GPSS_FLAG_PIPE) and only for x: an x tile is one contiguous bulk copy,
// while a y/z tile takes n row copies of 128 bytes, which the copy engine
// moves about 3x slower than coalesced loads; at 256^3 the direct kernel's x
// pass is also 6% faster than the pipelined one (issue-bound, more warps).
static bool pipe_ok(const gpss_ctx *c, int axis)
{
    if (!(c->flags & GPSS_FLAG_PIPE)) return false;
    if (axis != 0) return false;
    const int64_t n = c->n[axis];
    if (n != 64 && n != 128 && n != 256) return false;
    const int64_t W = 4096 / n;
    const int64_t nlines = c->total / n;
    if (nlines % W) return false;
    if (axis == 1 && c->n[0] % W) return false;
    return true;
}

// Host-side fault injection for tests: GPSS_FAULT_PIPE_POLLS=v in the
// environment makes the pipelined pass poll a tile's barrier only v times
// before it gives up (0: at once), so the bounded-wait path -- status 2,
// GPSS_ETIMEOUT, the CTA draining its own copies -- runs without any GPU fault.
static unsigned injected_pipe_polls()
{
    const char *v = std::getenv("GPSS_FAULT_PIPE_POLLS");
    if (!v || !*v) return 0u;
    return (unsigned)std::strtoul(v, nullptr, 10) + 1u;
}

template <typename T> static int launch(gpss_ctx *c, int axis, int mode, const PassArgs<T> &a)
{
    if (mode == MODE_FUSED && !a.acc && !a.nl_pre && !a.dot_with && !a.comp && pipe_ok(c, axis)) {
        const int ntiles = (int)(c->total / c->n[axis] / (4096 / c->n[axis]));
        PassArgs<T> ap = a;
        ap.wait_polls = injected_pipe_polls();
        // a wait that gives up is recorded in the status word even when the
        // pass has no reduction of its own (the x pass of a step)
        if (!ap.fin_status) ap.fin_status = c->status;
        cudaError_t e = PassLauncher<T>::pipe(axis == 0, (int)c->n[axis], ap, ntiles, c->stream);
        if (e != cudaSuccess)
            return fail(c, GPSS_ECUDA, "pipelined pass launch (axis %d): %s", axis, cudaGetErrorString(e));
        c->launches++;
        return GPSS_OK;
    }
    if (c->gen[axis]) {
        cudaError_t e = PassLauncher<T>::gen(mode, a, c->gplan[axis], c->stream);
        if (e != cudaSuccess)
            return fail(c, GPSS_ECUDA, "generic pass launch (axis %d, n = %lld, mode %d): %s", axis,
                        (long long)c->n[axis], mode, cudaGetErrorString(e));
        c->launches++;
        return GPSS_OK;
    }
    const int blocks = blocks_for<T>(c, axis);
    cudaError_t e = PassLauncher<T>::launch(mode, axis == 0, (int)c->n[axis], a, blocks, c->stream);
    if (e != cudaSuccess) return fail(c, GPSS_ECUDA, "pass launch (axis %d, mode %d): %s", axis, mode,
                                      cudaGetErrorString(e));
    c->launches++;
    return GPSS_OK;
}

static const int kDiagSlot = 3;  // sums slot of read-only diagnostics (and the mass-lock target)

// arm the in-kernel finish of a pass's reductions into sums slot `slot`
template <typename T> static void set_finish(gpss_ctx *c, PassArgs<T> &a, int slot, int mode)
{
    double dV = 1.0;
    for (int ax = 0; ax < c->ndim; ax++) dV *= c->d[ax];
    a.partials = c->partials;
    a.counter = c->counter;
    a.fin_out = c->sums + slot * RQ_COUNT;
    a.fin_mode = mode;
    a.fin_target = c->sums + kDiagSlot * RQ_COUNT + RQ_MASS;
    a.fin_scale = c->scale;
    a.fin_status = c->status;
    a.dV = dV;
}

// One kinetic flow L(dtl) as fused passes x, y[, z].  The last axis may carry
// the nonlinear flow N(dtnl) as an epilogue and/or the pointwise reductions
// (red_last, finished with fin_last: FIN_NONE, FIN_UNITMASS for the
// imaginary-time renormalisation, FIN_MASSLOCK for restoring the mass of the
// start of the call); diag_kin adds the Parseval kinetic sums on every axis;
// prescale multiplies the first pass by the device scalar c->scale.
template <typename T>
static int kinetic_fused(gpss_ctx *c, double dtl, int imag, bool nl, double dtnl, int red_last,
                         bool diag_kin, bool prescale, int fin_last = FIN_NONE, void *buf = nullptr,
                         bool reverse = false)
{
    void *field = buf ? buf : c->psi;
    for (int step = 0; step < c->ndim; step++) {
        const int axis = reverse ? c->ndim - 1 - step : step;
        PassArgs<T> a = axis_args<T>(c, axis, field, field);
        const void *ph;
        GPSS_TRY(get_phase(c, axis, dtl, imag, 1, &ph, &a.prow));
        a.phase = (const vec2<T> *)ph;
        a.comp = sizeof(T) == 4 && (c->flags & GPSS_FLAG_COMPENSATED) != 0;
        // the FP32 mass lock holds the field at the target mass M0 (its
        // diagnostics slot) through the call: the compensated passes grid on
        // a bound from it
        if (a.comp && fin_last == FIN_MASSLOCK) a.grid_mass = c->sums + kDiagSlot * RQ_COUNT + RQ_MASS;
        // plain FP32 y/z passes of psi under the mass lock (the call checks
        // the status word, where a tile copy that timed out is reported):
        // tiles arrive by tensor copies
        if (c->tmap_dev && !a.comp && axis >= 1 && field == c->psi && fin_last == FIN_MASSLOCK && !diag_kin &&
            a.prow == 0) {
            a.tmap = (const char *)c->tmap_dev + (axis - 1) * sizeof(CUtensorMap);
            a.taxis = axis;
            a.tnx = (int)c->n[0];
            a.fin_status = c->status;
        }
        if (prescale && step == 0) a.scale = c->scale;
        const bool last = step == c->ndim - 1;
        if (last && nl) {
            a.nl_mode = imag ? NL_IMAG : NL_REAL;
            a.V = c->have_V ? (const T *)c->V : nullptr;
            a.nl_beta = c->beta;
            a.nl_dt = dtnl;
            a.nl_split = nl_split(c->beta, dtnl);
        }
        if (last) a.red |= red_last;
        if (a.red & RED_POINT) a.V = c->have_V ? (const T *)c->V : nullptr;
        if (diag_kin) {
            a.red |= RED_KIN;
            a.coord = axis == 0 ? c->coord_dev[1] : (axis == 1 ? c->coord_dev[0] : nullptr);
        }
        if (a.red) set_finish<T>(c, a, axis, last ? fin_last : FIN_NONE);
        GPSS_TRY(launch<T>(c, axis, MODE_FUSED, a));
    }
    return GPSS_OK;
}

// A merged real-time Strang call (Omega = 0, fused) ends with
// L(dt/2) N, leaving its trailing half kinetic flow L(dt/2) unapplied: the
// device holds phi with psi = L(pending_h) phi.  The next such call folds it
// into its first flow (L(a) L(b) = L(a + b) when the flows commute), so a
// loop of one-step calls runs the merged sequence; every other entry point
// that reads or changes the field applies it first (flush_pending), or drops
// it when it replaces the field.  The flow is the same table and launch
// sequence as the trailing half step would have been, so results are
// bitwise those of the eager sequence.
template <typename T> static int flush_pending_t(gpss_ctx *c)
{
    if (c->pending_h == 0.0) return GPSS_OK;
    const double h = c->pending_h;
    const bool ps = c->pending_scale;
    c->pending_h = 0.0;
    c->pending_scale = false;
    return kinetic_fused<T>(c, h, 0, false, 0.0, 0, false, ps);
}
static int flush_pending(gpss_ctx *c)
{
    if (c->pending_h == 0.0) return GPSS_OK;
    CUDA_TRY(c, cudaSetDevice(c->device));
    return c->precision == GPSS_FP32 ? flush_pending_t<float>(c) : flush_pending_t<double>(c);
}
static void drop_pending(gpss_ctx *c)
{
    c->pending_h = 0.0;
    c->pending_scale = false;
}

// Plain form: per axis FFT -> multiply -> iFFT as three launches
// (mul_x!, broadcast, ldiv_x!; Plans.jl:1132-1250, splitting.jl:164-201).
template <typename T> static int kinetic_plain(gpss_ctx *c, double dtl, int imag)
{
    for (int axis = 0; axis < c->ndim; axis++) {
        PassArgs<T> f = axis_args<T>(c, axis, c->psi, c->scratch);
        GPSS_TRY(launch<T>(c, axis, MODE_FWD, f));
        const void *ph;
        int64_t prow;
        GPSS_TRY(get_phase(c, axis, dtl, imag, 0, &ph, &prow));
        cudaError_t e = launch_mul_phase<T>((vec2<T> *)c->scratch, (const vec2<T> *)ph, prow, axis, c->n,
                                            c->total, c->stream);
        if (e != cudaSuccess) return fail(c, GPSS_ECUDA, "mul_phase: %s", cudaGetErrorString(e));
        c->launches++;
        PassArgs<T> b = axis_args<T>(c, axis, c->scratch, c->psi);
        GPSS_TRY(launch<T>(c, axis, MODE_INV, b));
    }
    return GPSS_OK;
}

template <typename T> static int nl_plain(gpss_ctx *c, double dt, int imag)
{
    cudaError_t e = launch_nl<T>((vec2<T> *)c->psi, c->have_V ? (const T *)c->V : nullptr, c->beta, dt, imag,
                                 c->total, c->stream);
    if (e != cudaSuccess) return fail(c, GPSS_ECUDA, "nl: %s", cudaGetErrorString(e));
    c->launches++;
    return GPSS_OK;
}

// sum |psi|^2 (and V|psi|^2, |psi|^4; with kin also the Parseval sums) of the
// current field by read-only passes, into c->sums slot `axis` (kin) or the
// diagnostics slot (mass only)
template <typename T> static int diag_passes(gpss_ctx *c, bool kin, int mode)
{
    const int naxes = kin ? c->ndim : 1;
    for (int axis = 0; axis < naxes; axis++) {
        PassArgs<T> a = axis_args<T>(c, axis, c->psi, c->psi);
        a.red = (axis == 0 ? RED_POINT : 0) | (kin ? RED_KIN : 0);
        a.V = c->have_V ? (const T *)c->V : nullptr;
        a.coord = axis == 0 ? c->coord_dev[1] : (axis == 1 ? c->coord_dev[0] : nullptr);
        set_finish<T>(c, a, kin ? axis : kDiagSlot, axis == 0 ? mode : FIN_NONE);
        GPSS_TRY(launch<T>(c, axis, MODE_DIAG, a));
    }
    return GPSS_OK;
}

// Parseval kinetic sums of one axis of the current field (read-only pass) into
// sums slot `axis`
template <typename T> static int diag_kin_axis(gpss_ctx *c, int axis)
{
    PassArgs<T> a = axis_args<T>(c, axis, c->psi, c->psi);
    a.red = RED_KIN;
    a.coord = axis == 0 ? c->coord_dev[1] : (axis == 1 ? c->coord_dev[0] : nullptr);
    set_finish<T>(c, a, axis, FIN_NONE);
    return launch<T>(c, axis, MODE_DIAG, a);
}

template <typename T> static int apply_scale(gpss_ctx *c)
{
    cudaError_t e = launch_scale<T>((vec2<T> *)c->psi, c->scale, c->total, c->stream);
    if (e != cudaSuccess) return fail(c, GPSS_ECUDA, "scale: %s", cudaGetErrorString(e));
    c->launches++;
    return GPSS_OK;
}

static double cell_volume(const gpss_ctx *c)
{
    double v = 1.0;
    for (int a = 0; a < c->ndim; a++) v *= c->d[a];
    return v;
}

// x * dx * dy [* dz] left to right, as the reference evaluates it
static double times_cell(const gpss_ctx *c, double x)
{
    for (int a = 0; a < c->ndim; a++) x *= c->d[a];
    return x;
}

// normalize! (Fields.jl:196-200) on the device: unit mass from the FP64 sum
template <typename T> static int normalize_impl(gpss_ctx *c)
{
    CUDA_TRY(c, cudaMemsetAsync(c->status, 0, sizeof(int), c->stream));
    GPSS_TRY(diag_passes<T>(c, false, FIN_UNITMASS));
    GPSS_TRY(apply_scale<T>(c));
    int st = 0;
    CUDA_TRY(c, cudaMemcpyAsync(&st, c->status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (st) return fail(c, GPSS_ENONFINITE, "normalize: non-finite or zero norm");
    return GPSS_OK;
}
