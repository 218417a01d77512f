// noalloc.cu -- gpss_energy_noalloc: the energies of a field that already
// lives in the caller's device memory, computed without allocating anything.
//
// Who needs it: callers whose device memory belongs to another allocator --
// a Julia session whose CuArrays come from CUDA.jl's memory pool, a host
// program that runs under a fixed device-memory budget, or code that must not
// let a library grow its footprint in the middle of a long run.  Such a caller
// cannot let the library cudaMalloc a context (gpss_create does); it passes
// device pointers to psi and V and gets the five energies back.
//
// The kernel is the read-only diagnostic pass of the context path
// (pass_kernel<MODE_DIAG>): per-axis FFTs with Parseval sums and pointwise
// sums, finished on the device by the last CTA.  Its scratch -- the per-CTA
// partial sums, the arrival counter, the sums, the twiddle tables and the
// node coordinates -- lives in one file-scope device array of
// GPSS_NOALLOC_SCRATCH_BYTES (1 MiB), which every GPU that loads the library
// holds until the process exits.
//
// The array's name in host code is only a host-side stand-in, not a device
// address: the first call on each device looks the address up with
// cudaGetSymbolAddress (with that device current) and every launch passes the
// looked-up pointer.  That first call should therefore come before any stream
// capture.  The looked-up address is kept for the life of the process, so a
// cudaDeviceReset between calls (which unloads the library's device code and
// with it the array) is not supported.  Every call shares the array and leaves
// its contents behind; the
// arrival counter is cleared by each call before its kernels run.  Calls whose
// work overlaps on the GPU (other streams, other host threads) race on the
// array: serialise them.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>
#include "../../include/gpss.h"
#include "gpss_internal.h"

using namespace gpss;

#define GPSS_NOALLOC_SCRATCH_BYTES (1u << 20)

static __device__ __align__(256) unsigned char g_noalloc_scratch[GPSS_NOALLOC_SCRATCH_BYTES];

namespace {

// byte offsets of the regions carved from the scratch array
constexpr size_t kOffCounter = 0;                                  // unsigned int
constexpr size_t kOffSums = 256;                                   // 4 slots x RQ_COUNT doubles
constexpr size_t kOffCoord = 512;                                  // 3 x 256 doubles
constexpr size_t kOffTw = kOffCoord + 3 * 256 * sizeof(double);    // 3 x 4 x 256 double2
constexpr size_t kOffPartials = kOffTw + 3 * 4 * 256 * 16;         // RQ_COUNT x CTAs doubles
constexpr size_t kPartialBytes = GPSS_NOALLOC_SCRATCH_BYTES - kOffPartials;

// The largest field the entry point takes (256^3) has at most 256^2 / W
// tiles in one pass, W the lines of a CTA (fewest for the FP64 passes: 4), so
// its partial sums need 16384 x 5 doubles = 640 KiB of the 969.5 KiB region
// (1.5x margin).  The run-time check below therefore never rejects a field of
// lines up to 256; it guards the limit should the CTA shapes change.
static_assert((uint64_t)(256 * 256 / PassShape<double, 256, true>::W) * RQ_COUNT * sizeof(double) <=
                  kPartialBytes, "the partial sums of a 256^3 FP64 field must fit the scratch array");
static_assert((uint64_t)(256 * 256 / PassShape<double, 256, false>::W) * RQ_COUNT * sizeof(double) <=
                  kPartialBytes, "the partial sums of a 256^3 FP64 field must fit the scratch array");

std::mutex g_setup_mutex;
unsigned char *g_scratch_dev[64] = {nullptr};  // looked-up device address, per device

}  // namespace

namespace gpss {
int fail(gpss_ctx *c, int code, const char *fmt, ...);  // gpss_api.cu: the message of gpss_last_error
}

namespace {

// No context holds the message of this entry point: it goes where
// gpss_last_error(NULL) reads it, as for a failed gpss_create.
int noalloc_fail(int code, const char *msg, cudaError_t e = cudaSuccess)
{
    if (e != cudaSuccess) return gpss::fail(nullptr, code, "gpss_energy_noalloc: %s: %s", msg, cudaGetErrorString(e));
    return gpss::fail(nullptr, code, "gpss_energy_noalloc: %s", msg);
}

// twiddle tables of one axis in the pass kernel's layout (stage A hi, lo;
// stage B hi, lo)
template <typename T> std::vector<vec2<T>> twiddle_table(int64_t n)
{
    std::vector<long double> re, im;
    twiddle_rows(n, re, im);
    return dw_split<T>(re, im, n);
}

double lerp_node(int64_t j, int64_t d, double a, double b)
{
    const double t = (double)j / (double)d;
    return (1.0 - t) * a + t * b;
}

template <typename T>
int energy_noalloc_t(int ndim, const int64_t *n3, const double *lo, const double *hi, double cD, double beta,
                     double omega, const void *psi, const void *V, cudaStream_t stream, unsigned char *scratch,
                     double *out)
{
    const int64_t total = n3[0] * n3[1] * n3[2];
    double d[3];
    for (int a = 0; a < 3; a++) d[a] = (a < ndim) ? (hi[a] - lo[a]) / (double)n3[a] : 1.0;
    unsigned int *counter = reinterpret_cast<unsigned int *>(scratch + kOffCounter);
    double *sums = reinterpret_cast<double *>(scratch + kOffSums);
    double *coord = reinterpret_cast<double *>(scratch + kOffCoord);
    unsigned char *tw = scratch + kOffTw;
    double *partials = reinterpret_cast<double *>(scratch + kOffPartials);

    // the counter must start at zero; tables and coordinates of this call
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned int), stream);
    if (e != cudaSuccess) return noalloc_fail(GPSS_ECUDA, "cudaMemsetAsync", e);
    for (int a = 0; a < ndim; a++) {
        std::vector<double> x((size_t)n3[a]);
        const double first = lerp_node(0, n3[a], lo[a], hi[a]), last = lerp_node(n3[a] - 1, n3[a], lo[a], hi[a]);
        for (int64_t i = 0; i < n3[a]; i++) x[(size_t)i] = lerp_node(i, n3[a] - 1, first, last);
        e = cudaMemcpyAsync(coord + 256 * a, x.data(), sizeof(double) * (size_t)n3[a], cudaMemcpyHostToDevice,
                            stream);
        if (e != cudaSuccess) return noalloc_fail(GPSS_ECUDA, "cudaMemcpyAsync (coordinates)", e);
        const std::vector<vec2<T>> t = twiddle_table<T>(n3[a]);
        e = cudaMemcpyAsync(tw + (size_t)a * 4 * 256 * sizeof(vec2<T>), t.data(), sizeof(vec2<T>) * t.size(),
                            cudaMemcpyHostToDevice, stream);
        if (e != cudaSuccess) return noalloc_fail(GPSS_ECUDA, "cudaMemcpyAsync (twiddles)", e);
    }
    const int64_t nx = n3[0], ny = n3[1];
    for (int axis = 0; axis < ndim; axis++) {
        const int64_t na = n3[axis];
        PassArgs<T> a;
        memset(&a, 0, sizeof(a));
        a.in = (const vec2<T> *)psi;
        a.out = nullptr;
        a.tw = reinterpret_cast<const vec2<T> *>(tw + (size_t)axis * 4 * 256 * sizeof(vec2<T>));
        a.nlines = (int)(total / na);
        if (axis == 0) { a.m0 = a.nlines; a.s0 = nx; a.s1 = 0; a.stride = 1; a.rowmod = (int)ny; }
        else if (axis == 1) { a.m0 = (int)nx; a.s0 = 1; a.s1 = nx * ny; a.stride = nx; a.rowmod = (int)nx; }
        else { a.m0 = a.nlines; a.s0 = 1; a.s1 = 0; a.stride = nx * ny; a.rowmod = 1; }
        a.inv_n = (T)(1.0 / (double)na);
        a.kmult = (6.283185307179586 / d[axis]) / (double)na;
        a.nl_mode = NL_NONE;
        a.V = (const T *)V;
        a.red = (axis == 0 ? RED_POINT : 0) | RED_KIN;
        a.coord = axis == 0 ? coord + 256 : (axis == 1 ? coord : nullptr);
        a.partials = partials;
        a.counter = counter;
        a.fin_out = sums + axis * RQ_COUNT;
        a.fin_mode = FIN_NONE;
        const int W = PassLauncher<T>::lines((int)na, axis == 0);
        const int blocks = (int)((a.nlines + W - 1) / W);
        e = PassLauncher<T>::launch(MODE_DIAG, axis == 0, (int)na, a, blocks, stream);
        if (e != cudaSuccess) return noalloc_fail(GPSS_ECUDA, "diagnostic pass launch", e);
    }
    double h[4 * RQ_COUNT];
    e = cudaMemcpyAsync(h, sums, sizeof(double) * 3 * RQ_COUNT, cudaMemcpyDeviceToHost, stream);
    if (e != cudaSuccess) return noalloc_fail(GPSS_ECUDA, "cudaMemcpyAsync (sums)", e);
    e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return noalloc_fail(GPSS_ECUDA, "cudaStreamSynchronize", e);
    if (!std::isfinite(h[RQ_MASS])) return noalloc_fail(GPSS_ENONFINITE, "field holds NaN/Inf");
    // the energies of energy(n), GrossPitaevskii.jl:61-136, from the sums
    auto cell = [&](double x) {
        for (int a = 0; a < ndim; a++) x *= d[a];
        return x;
    };
    double grad = 0.0;
    for (int a = 0; a < ndim; a++) grad += h[a * RQ_COUNT + RQ_KIN];
    const double eom = cell(-omega * (h[RQ_ROT] - h[RQ_COUNT + RQ_ROT]));
    const double edel = cell(-cD * grad + h[RQ_POT]);
    const double ebeta = cell(0.5 * beta * h[RQ_INT]);
    out[0] = eom;
    out[1] = edel;
    out[2] = ebeta;
    out[3] = -eom + edel + ebeta;
    out[4] = -eom + edel + ebeta * 2.0;
    return GPSS_OK;
}

}  // namespace

extern "C" int gpss_energy_noalloc(int ndim, const int64_t *n, const double *lo, const double *hi, int precision,
                                   double coeffD, double beta, double omega, const void *psi_dev,
                                   const void *V_dev, void *stream, double *out)
{
    if (!n || !lo || !hi || !psi_dev || !out) return noalloc_fail(GPSS_EINVAL, "null argument");
    if (ndim != 2 && ndim != 3) return noalloc_fail(GPSS_EINVAL, "ndim must be 2 or 3");
    if (precision != GPSS_FP64 && precision != GPSS_FP32)
        return noalloc_fail(GPSS_EINVAL, "precision must be GPSS_FP64 or GPSS_FP32");
    int64_t n3[3] = {1, 1, 1};
    for (int a = 0; a < ndim; a++) {
        if (n[a] < 2 || n[a] > 256 || (n[a] & (n[a] - 1)))
            return noalloc_fail(GPSS_EINVAL, "each axis must be a power of two in [2, 256]");
        if (!(hi[a] > lo[a])) return noalloc_fail(GPSS_EINVAL, "need lo < hi on every axis");
        n3[a] = n[a];
    }
    // the partial sums of the largest pass must fit the fixed scratch, counted
    // from the tile count (an upper bound on the grid, which may be capped at
    // one wave).  The largest accepted field, 256^3 in FP64 (64-thread CTAs,
    // 4 lines each: 16384 tiles x 5 sums x 8 B = 640 KiB), fits with a 1.6x
    // margin, so today this refusal is a guard for changed launch shapes.
    const int64_t total = n3[0] * n3[1] * n3[2];
    for (int a = 0; a < ndim; a++) {
        const int W = precision == GPSS_FP32 ? pass_lines_per_cta_f32((int)n3[a], a == 0)
                                             : pass_lines_per_cta_f64((int)n3[a], a == 0);
        const int64_t blocks = (total / n3[a] + W - 1) / W;
        if ((uint64_t)blocks * RQ_COUNT * sizeof(double) > kPartialBytes)
            return noalloc_fail(GPSS_EINVAL, "field too large for the fixed 1 MiB scratch of gpss_energy_noalloc");
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(GPSS_ECUDA, "cudaGetDevice", e);
    if (dev < 0 || dev >= 64) return noalloc_fail(GPSS_EINVAL, "device ordinal out of range");
    unsigned char *scratch;
    {
        // set-up, once per device, with that device current
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_dev[dev]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return noalloc_fail(GPSS_ECUDA, "cudaGetSymbolAddress", e);
            g_scratch_dev[dev] = static_cast<unsigned char *>(p);
        }
        scratch = g_scratch_dev[dev];
    }
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (precision == GPSS_FP32)
        return energy_noalloc_t<float>(ndim, n3, lo, hi, coeffD, beta, omega, psi_dev, V_dev, s, scratch, out);
    return energy_noalloc_t<double>(ndim, n3, lo, hi, coeffD, beta, omega, psi_dev, V_dev, s, scratch, out);
}
