// gpss_api.cu -- the C ABI of libgpss.so (include/gpss.h): context setup,
// host-built FP64 tables, and the orchestration of the directional passes
// that make up NumModelSplit1 / NumModelSplit2 time steps.
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
    int device = 0;
    cudaStream_t stream = nullptr;
    void *psi = nullptr;      // device field (float2 or double2)
    void *scratch = nullptr;  // spectrum (plain form) and FP64 staging, total*16 bytes
    void *V = nullptr;        // device potential (float or double)
    void *tw[3] = {nullptr, nullptr, nullptr};
    double *coord_dev[3] = {nullptr, nullptr, nullptr};
    std::vector<double> coord[3];
    double *partials = nullptr;
    int max_blocks = 0;
    double *sums = nullptr;   // [4][RQ_COUNT]: slots 0..2 per axis, slot 3 diagnostics
    double *scale = nullptr;  // ScaleCell: the factor in FP64 and as a float
    int *status = nullptr;    // [1]
    unsigned int *counter = nullptr;  // arrival counter of the in-kernel reduction finish
    std::vector<PhaseEntry> phases;
    void *rk_buf[4] = {nullptr, nullptr, nullptr, nullptr};  // RK: stage state, lapRot, NL term, sum
    int *rk_lim = nullptr;    // RK: 2/3-rule limits per inner position (launch_mask_spectrum)
    void *im_buf = nullptr;   // implicit schemes: work fields (implicit_impl)
    size_t im_bytes = 0;
    // discrete adjoint: buffers kept between calls (sized for adj_nck checkpoints, adj_K states)
    void *adj_buf = nullptr;
    size_t adj_bytes = 0;
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

static thread_local std::string g_create_error;

static int fail(gpss_ctx *c, int code, const char *fmt, ...)
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

static int dev_alloc(gpss_ctx *c, void **p, size_t bytes)
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

typedef long double ldouble;
static const ldouble kHalfPiL = 1.570796326794896619231321691639751442L;

// (cos, sin) of 2 pi k / n in long double, reduced to the first octant so
// that the symmetric values are exact.
static void unit_root(int64_t k, int64_t n, ldouble *cs, ldouble *sn)
{
    k %= n;
    if (k < 0) k += n;
    int64_t q = (4 * k) / n;
    int64_t r4 = 4 * k - q * n;
    ldouble cc, ss;
    if (2 * r4 <= n) {
        ldouble a = kHalfPiL * (ldouble)r4 / (ldouble)n;
        cc = cosl(a); ss = sinl(a);
    } else {
        ldouble a = kHalfPiL * (ldouble)(n - r4) / (ldouble)n;
        cc = sinl(a); ss = cosl(a);
    }
    switch (q) {
    case 0: *cs = cc; *sn = ss; break;
    case 1: *cs = -ss; *sn = cc; break;
    case 2: *cs = -cc; *sn = -ss; break;
    default: *cs = ss; *sn = -cc; break;
    }
}

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
    std::vector<double> h((size_t)(4 * n * rows));  // re/im pairs of hi and lo as doubles
    std::vector<ldouble> lo_re(re.size()), lo_im(im.size());
    if (c->precision == GPSS_FP32) {
        std::vector<float> f((size_t)(4 * n * rows));
        for (int64_t r = 0; r < rows; r++)
            for (int64_t k = 0; k < n; k++) {
                const size_t i = (size_t)(r * n + k);
                const float hr = (float)re[i], hi = (float)im[i];
                const float lr = (float)(re[i] - (ldouble)hr), li = (float)(im[i] - (ldouble)hi);
                f[(size_t)(2 * (r * 2 * n + k))] = hr;
                f[(size_t)(2 * (r * 2 * n + k) + 1)] = hi;
                f[(size_t)(2 * (r * 2 * n + n + k))] = lr;
                f[(size_t)(2 * (r * 2 * n + n + k) + 1)] = li;
            }
        GPSS_TRY(dev_alloc(c, dev, f.size() * 4));
        CUDA_TRY(c, cudaMemcpy(*dev, f.data(), f.size() * 4, cudaMemcpyHostToDevice));
        return GPSS_OK;
    }
    for (int64_t r = 0; r < rows; r++)
        for (int64_t k = 0; k < n; k++) {
            const size_t i = (size_t)(r * n + k);
            const double hr = (double)re[i], hi = (double)im[i];
            h[(size_t)(2 * (r * 2 * n + k))] = hr;
            h[(size_t)(2 * (r * 2 * n + k) + 1)] = hi;
            h[(size_t)(2 * (r * 2 * n + n + k))] = (double)(re[i] - (ldouble)hr);
            h[(size_t)(2 * (r * 2 * n + n + k) + 1)] = (double)(im[i] - (ldouble)hi);
        }
    GPSS_TRY(dev_alloc(c, dev, h.size() * 8));
    CUDA_TRY(c, cudaMemcpy(*dev, h.data(), h.size() * 8, cudaMemcpyHostToDevice));
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

template <typename T> static int blocks_for(gpss_ctx *c, int axis)
{
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

template <typename T> static int launch(gpss_ctx *c, int axis, int mode, const PassArgs<T> &a)
{
    if (mode == MODE_FUSED && !a.acc && pipe_ok(c, axis)) {
        const int ntiles = (int)(c->total / c->n[axis] / (4096 / c->n[axis]));
        cudaError_t e = PassLauncher<T>::pipe(axis == 0, (int)c->n[axis], a, ntiles, c->stream);
        if (e != cudaSuccess)
            return fail(c, GPSS_ECUDA, "pipelined pass launch (axis %d): %s", axis, cudaGetErrorString(e));
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

template <typename T>
static int step_impl(gpss_ctx *c, int nsteps, int scheme, int imag, double dt, gpss_diag *diag)
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
    if (nsteps == 0) {
        if (diag) {
            diag->steps = 0;
            GPSS_TRY(energy_impl<T>(c, diag->energy, &diag->mass));
        }
        return GPSS_OK;
    }
    if (imag || lock) {
        int zero = 0;
        CUDA_TRY(c, cudaMemcpyAsync(c->status, &zero, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    }
    if (lock) GPSS_TRY(diag_passes<T>(c, false, FIN_NONE));  // target mass -> diagnostics slot
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
        // consecutive steps commute (Omega = 0) and compose exactly.
        GPSS_TRY(kinetic_fused<T>(c, dt * 0.5, 0, true, dt, red_nl, false, false, fin_nl));
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
        // with the other axes' derivatives when Omega = 0)
        GPSS_TRY(kinetic_fused<T>(c, dt * 0.5, 0, false, 0.0, diag ? RED_POINT : 0, diag != nullptr, lock));
        diag_done = diag != nullptr;
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
                GPSS_TRY(kinetic_fused<T>(c, dt * 0.5, 0, false, 0.0, 0, false, lock));
            } else {
                GPSS_TRY(kinetic_fused<T>(c, dt, 0, true, dt, red_nl, false, lock && s > 0, fin_nl));
            }
        }
    }
    if (imag || lock) {
        int st = 0;
        CUDA_TRY(c, cudaMemcpyAsync(&st, c->status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
        if (st & 2) return fail(c, GPSS_ETIMEOUT, "a pipelined pass gave up waiting for a tile copy");
        if (st) return fail(c, GPSS_ENONFINITE, "a renormalisation saw a non-finite or zero mass");
    }
    if (diag) {
        diag->steps = nsteps;
        if (diag_done) {
            double h[4 * RQ_COUNT];
            GPSS_TRY(read_sums(c, h));
            const int last = c->ndim - 1;
            if (!std::isfinite(h[last * RQ_COUNT + RQ_MASS]))
                return fail(c, GPSS_ENONFINITE, "field holds NaN/Inf");
            energies_from_sums(c, h, last, diag->energy);
            diag->mass = times_cell(c, h[last * RQ_COUNT + RQ_MASS]);
        } else {
            GPSS_TRY(energy_impl<T>(c, diag->energy, &diag->mass));
        }
    }
    return GPSS_OK;
}

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
// kernels as the forward, so the states are bitwise the forward's).
template <typename T>
static int adjoint_merged(gpss_ctx *c, const double *psi_target, int nsteps, int K, double dt, double *loss,
                          double *dLdV, double *dLdpsi0)
{
    using V = vec2<T>;
    const size_t fb = (size_t)c->total * sizeof(V);
    const int nck = (nsteps + K - 1) / K;
    // psi0, g, tgt, work, states[K], ckpt[nck]; dv (doubles); reduction scratch
    const size_t red_bytes = sizeof(double) * (2 * 152 * 8 + 2);
    const size_t need = fb * (size_t)(4 + K + nck) + (size_t)c->total * sizeof(double) + red_bytes;
    if (c->adj_bytes < need) {
        clear_graphs(c);
        if (c->adj_buf) { cudaStreamSynchronize(c->stream); cudaFree(c->adj_buf); c->adj_buf = nullptr; c->adj_bytes = 0; }
        GPSS_TRY(dev_alloc(c, &c->adj_buf, need));
        c->adj_bytes = need;
    }
    char *base = static_cast<char *>(c->adj_buf);
    void *psi0 = base, *g = base + fb, *tgt = base + 2 * fb, *work = base + 3 * fb;
    auto state = [&](int j) { return static_cast<void *>(base + fb * (size_t)(4 + j)); };
    auto ckpt = [&](int i) { return static_cast<void *>(base + fb * (size_t)(4 + K + i)); };
    double *dv = reinterpret_cast<double *>(base + fb * (size_t)(4 + K + nck));
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
        // backward, segment by segment from the last
        for (int seg = nck - 1; seg >= 0; seg--) {
            const int start = seg * K, end = std::min(start + K, nsteps);
            if (end - start > 1) {
                // work = N(pre_start), then pre_{start+j} = L(dt) N(pre_{start+j-1}) into state(j)
                CUDA_TRY(c, cudaMemcpyAsync(work, ckpt(seg), fb, cudaMemcpyDeviceToDevice, c->stream));
                cudaError_t e = launch_nl<T>((V *)work, c->have_V ? (const T *)c->V : nullptr, c->beta, dt, 0,
                                             c->total, c->stream);
                if (e != cudaSuccess) return fail(c, GPSS_ECUDA, "nl: %s", cudaGetErrorString(e));
                c->launches++;
                for (int j = 1; j < end - start; j++)
                    GPSS_TRY(adj_group<T>(c, work, dt, false, true, dt, state(j), nullptr, nullptr));
            }
            for (int n = end - 1; n >= start; n--) {
                const void *pre = n == start ? ckpt(seg) : state(n - start);
                GPSS_TRY(adj_group<T>(c, g, n == nsteps - 1 ? -h : -dt, true, false, dt, nullptr, pre, dv));
            }
        }
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
template <typename T> static int transform_all(gpss_ctx *c, void *f, bool inverse)
{
    for (int s = 0; s < c->ndim; s++) {
        const int axis = inverse ? c->ndim - 1 - s : s;
        PassArgs<T> a = axis_args<T>(c, axis, f, f);
        GPSS_TRY(launch<T>(c, axis, inverse ? MODE_INV : MODE_FWD, a));
    }
    return GPSS_OK;
}

template <typename T> static int dealias_field(gpss_ctx *c, void *f)
{
    GPSS_TRY(rk_mask_table(c));
    GPSS_TRY(transform_all<T>(c, f, false));
    const int last = c->ndim - 1;
    cudaError_t e = launch_mask_spectrum<T>((vec2<T> *)f, c->rk_lim, c->n[last], c->total / c->n[last], c->total,
                                            c->stream);
    if (e != cudaSuccess) return fail(c, GPSS_ECUDA, "mask: %s", cudaGetErrorString(e));
    c->launches++;
    return transform_all<T>(c, f, true);
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
};

template <typename T> static int im_bufs(gpss_ctx *c, ImBufs &B)
{
    const size_t fb = (size_t)c->total * sizeof(vec2<T>);
    const size_t rb = (size_t)c->total * sizeof(T);
    const size_t pb = sizeof(double) * (2 * 152 * 8 + 2);
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

// krylov! (precond = 0) / krylovPreCond! (precond = 1), krylov.jl:1-67
template <typename T>
static int im_krylov(gpss_ctx *c, ImBufs &B, int scheme, double dt, void *phi, int nkrylov, double tol, int precond,
                     int *niter_out)
{
    using V = vec2<T>;
    const size_t fb = (size_t)c->total * sizeof(V);
    double d[2];
    if (precond) {
        IM_TRY(im_mfield<T>((V *)B.s, (const V *)B.M, (const V *)B.b, c->total, c->stream));
        GPSS_TRY(im_dots<T>(c, B, B.s, B.s, nullptr, nullptr, d));
    } else {
        GPSS_TRY(im_dots<T>(c, B, B.b, B.b, nullptr, nullptr, d));
    }
    const double normb = std::sqrt(d[0]);
    GPSS_TRY(im_apply<T>(c, B, scheme, dt, phi, true, precond, B.r));
    CUDA_TRY(c, cudaMemcpyAsync(B.r2, B.r, fb, cudaMemcpyDeviceToDevice, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(B.p, B.r, fb, cudaMemcpyDeviceToDevice, c->stream));
    int niter = 0;
    for (int it = 1; it <= nkrylov; it++) {
        GPSS_TRY(im_apply<T>(c, B, scheme, dt, B.p, false, precond, B.Ap));
        GPSS_TRY(im_dots<T>(c, B, B.r, B.r2, B.Ap, B.r2, d));
        const double rr2 = d[0], alpha = d[0] / d[1];
        IM_TRY(im_axmy<T>((V *)B.s, (const V *)B.r, alpha, (const V *)B.Ap, c->total, c->stream));
        GPSS_TRY(im_apply<T>(c, B, scheme, dt, B.s, false, precond, B.As));
        GPSS_TRY(im_dots<T>(c, B, B.As, B.s, B.As, B.As, d));
        const double omega = d[0] / d[1];
        IM_TRY(im_update<T>((V *)phi, (const V *)B.p, (const V *)B.s, (const V *)B.As, (V *)B.r, alpha, omega,
                            c->total, c->stream));
        GPSS_TRY(im_dots<T>(c, B, B.r, B.r, B.r, B.r2, d));
        if (!std::isfinite(d[0])) return fail(c, GPSS_ENONFINITE, "Krylov solver: non-finite residual");
        if (std::sqrt(d[0]) / normb < tol) break;
        niter = it;
        const double beta = d[1] / rr2 * alpha / omega;
        IM_TRY(im_pdir<T>((V *)B.p, (const V *)B.r, (const V *)B.Ap, beta, omega, c->total, c->stream));
    }
    *niter_out = niter;
    return GPSS_OK;
}

template <typename T> static int normalize_impl(gpss_ctx *c);

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

// normalize! (Fields.jl:196-200) on the device: unit mass from the FP64 sum
template <typename T> static int normalize_impl(gpss_ctx *c)
{
    int zero = 0;
    CUDA_TRY(c, cudaMemcpyAsync(c->status, &zero, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    GPSS_TRY(diag_passes<T>(c, false, FIN_UNITMASS));
    GPSS_TRY(apply_scale<T>(c));
    int st = 0;
    CUDA_TRY(c, cudaMemcpyAsync(&st, c->status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (st) return fail(c, GPSS_ENONFINITE, "normalize: non-finite or zero norm");
    return GPSS_OK;
}

static bool is_pow2(int64_t v) { return v > 0 && (v & (v - 1)) == 0; }

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
                    c->adj_buf, c->im_buf};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
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
    if (flags & ~(GPSS_FLAG_PLAIN | GPSS_FLAG_NOMERGE | GPSS_FLAG_NOMASSLOCK | GPSS_FLAG_PIPE))
        return fail(nullptr, GPSS_EINVAL, "unknown flags 0x%x", flags);
    for (int a = 0; a < ndim; a++) {
        if (!is_pow2(n[a]) || n[a] < 2 || n[a] > 256)
            return fail(nullptr, GPSS_EINVAL, "n[%d] = %lld: each axis must be a power of two in [2, 256]", a,
                        (long long)n[a]);
        if (!(hi[a] > lo[a]) || !std::isfinite(lo[a]) || !std::isfinite(hi[a]))
            return fail(nullptr, GPSS_EINVAL, "axis %d: need finite lo < hi", a);
    }
    gpss_ctx *c = new (std::nothrow) gpss_ctx();
    if (!c) return fail(nullptr, GPSS_ENOMEM, "host allocation failed");
    c->ndim = ndim;
    c->precision = precision;
    c->flags = flags;
    c->total = 1;
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
        const int64_t N1 = na <= 16 ? na : 16, N2 = na / N1;
        // two rows: stage-A order (k1*N2 + r) and stage-B order (r*N1 + k1)
        std::vector<ldouble> re((size_t)(2 * na)), im((size_t)(2 * na));
        for (int64_t k1 = 0; k1 < N1; k1++)
            for (int64_t r = 0; r < N2; r++) {
                ldouble cs, sn;
                unit_root(r * k1, na, &cs, &sn);
                re[(size_t)(k1 * N2 + r)] = cs;
                im[(size_t)(k1 * N2 + r)] = -sn;
                re[(size_t)(na + r * N1 + k1)] = cs;
                im[(size_t)(na + r * N1 + k1)] = -sn;
            }
        if ((rc = upload_dw(c, &c->tw[a], re, im, 2, na))) return bail(rc);
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
    if (!std::isfinite(coeffD) || !std::isfinite(beta) || !std::isfinite(omega))
        return fail(c, GPSS_EINVAL, "parameters must be finite");
    CUDA_TRY(c, cudaSetDevice(c->device));
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
    CUDA_TRY(c, cudaSetDevice(c->device));
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
    if (!psi) return fail(c, GPSS_EINVAL, "gpss_upload: null psi");
    CUDA_TRY(c, cudaSetDevice(c->device));
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
    if (nsteps < 0) return fail(c, GPSS_EINVAL, "nsteps must be >= 0");
    if (scheme != GPSS_LIE && scheme != GPSS_STRANG) return fail(c, GPSS_EINVAL, "scheme must be 1 (Lie) or 2 (Strang)");
    if (!std::isfinite(dt)) return fail(c, GPSS_EINVAL, "dt must be finite");
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "no field uploaded");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (nsteps == 0 && !diag) return GPSS_OK;
    if (c->precision == GPSS_FP32) return step_impl<float>(c, nsteps, scheme, imag, dt, diag);
    return step_impl<double>(c, nsteps, scheme, imag, dt, diag);
}

int gpss_rk_step(gpss_ctx *c, int nsteps, int stepper, int filter, double dt)
{
    NvtxRange nvtx_("gpss_rk_step");
    if (!c) return GPSS_EINVAL;
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "gpss_rk_step: no field uploaded");
    if (nsteps < 0) return fail(c, GPSS_EINVAL, "gpss_rk_step: nsteps < 0");
    if (stepper != 1 && stepper != 2 && stepper != 4)
        return fail(c, GPSS_EINVAL, "gpss_rk_step: stepper must be 1, 2 or 4 (got %d)", stepper);
    if (filter < 0 || filter > 2) return fail(c, GPSS_EINVAL, "gpss_rk_step: filter must be 0, 1 or 2");
    if (!std::isfinite(dt)) return fail(c, GPSS_EINVAL, "gpss_rk_step: dt must be finite");
    cudaSetDevice(c->device);
    return c->precision == GPSS_FP32 ? rk_step_impl<float>(c, nsteps, stepper, filter, dt)
                                     : rk_step_impl<double>(c, nsteps, stepper, filter, dt);
}

int gpss_implicit_step(gpss_ctx *c, int nsteps, int scheme, double dt, int nkrylov, double tolkrylov, int nnewton,
                       double tolnewton, int64_t *krylov_iters)
{
    NvtxRange nvtx_("gpss_implicit_step");
    if (!c) return GPSS_EINVAL;
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "gpss_implicit_step: no field uploaded");
    if (nsteps < 0 || nkrylov < 1 || nnewton < 1)
        return fail(c, GPSS_EINVAL, "gpss_implicit_step: need nsteps >= 0, nkrylov >= 1, nnewton >= 1");
    if (scheme < GPSS_IMPLICIT_BE || scheme > GPSS_IMPLICIT_CN_QN_T)
        return fail(c, GPSS_EINVAL, "gpss_implicit_step: unknown scheme %d", scheme);
    if (!(dt > 0.0) || !std::isfinite(dt) || !(tolkrylov > 0.0) || !(tolnewton > 0.0))
        return fail(c, GPSS_EINVAL, "gpss_implicit_step: dt and the tolerances must be positive");
    CUDA_TRY(c, cudaSetDevice(c->device));
    return c->precision == GPSS_FP32
               ? implicit_impl<float>(c, nsteps, scheme, dt, nkrylov, tolkrylov, nnewton, tolnewton, krylov_iters)
               : implicit_impl<double>(c, nsteps, scheme, dt, nkrylov, tolkrylov, nnewton, tolnewton, krylov_iters);
}

int gpss_energy(gpss_ctx *c, double *out)
{
    NvtxRange nvtx_("gpss_energy");
    if (!c || !out) return c ? fail(c, GPSS_EINVAL, "gpss_energy: null out") : GPSS_EINVAL;
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "no field uploaded");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (c->precision == GPSS_FP32) return energy_impl<float>(c, out, nullptr);
    return energy_impl<double>(c, out, nullptr);
}

// sum |psi|^2 of the device field (no cell volume)
static int raw_mass(gpss_ctx *c, double *out)
{
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "no field uploaded");
    CUDA_TRY(c, cudaSetDevice(c->device));
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
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "no field uploaded");
    CUDA_TRY(c, cudaSetDevice(c->device));
    return c->precision == GPSS_FP32 ? normalize_impl<float>(c) : normalize_impl<double>(c);
}

int gpss_ground_state(gpss_ctx *c, double dt, double tol, int64_t max_steps, int check_every,
                      double *mu_out, int64_t *steps_out)
{
    NvtxRange nvtx_("gpss_ground_state");
    if (!c) return GPSS_EINVAL;
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

int gpss_adjoint(gpss_ctx *c, const double *psi_target, int nsteps, int K, double dt, double *loss,
                 double *dLdV, double *dLdpsi0)
{
    NvtxRange nvtx_("gpss_adjoint");
    if (!c) return GPSS_EINVAL;
    if (!psi_target || !loss) return fail(c, GPSS_EINVAL, "gpss_adjoint: null psi_target or loss");
    if (nsteps < 1 || K < 1) return fail(c, GPSS_EINVAL, "gpss_adjoint: need nsteps >= 1 and K >= 1");
    if (!std::isfinite(dt)) return fail(c, GPSS_EINVAL, "dt must be finite");
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "no field uploaded");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (c->precision == GPSS_FP32) return adjoint_impl<float>(c, psi_target, nsteps, K, dt, loss, dLdV, dLdpsi0);
    return adjoint_impl<double>(c, psi_target, nsteps, K, dt, loss, dLdV, dLdpsi0);
}

int gpss_sync(gpss_ctx *c)
{
    if (!c) return GPSS_EINVAL;
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return GPSS_OK;
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
    if (axis < 0 || axis >= c->ndim || reps < 1 || (mode != 0 && mode != 1))
        return fail(c, GPSS_EINVAL, "time_pass: bad axis/mode/reps");
    if (!c->have_psi) return fail(c, GPSS_ESTATE, "no field uploaded");
    CUDA_TRY(c, cudaSetDevice(c->device));
    auto run = [&](auto tag) -> int {
        using T = decltype(tag);
        PassArgs<T> a = axis_args<T>(c, axis, c->psi, c->psi);
        const void *ph;
        GPSS_TRY(get_phase(c, axis, dt, 0, 1, &ph, &a.prow));
        a.phase = (const vec2<T> *)ph;
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
