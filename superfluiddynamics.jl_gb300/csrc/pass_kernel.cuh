// pass_kernel.cuh -- one directional split-step pass over every line of a
// periodic 2D/3D field.
//
// A "line" is the set of cells that differ only in the coordinate of one
// axis.  The reference moves each axis to the contiguous position with a
// pencil transpose and calls a batched 1D FFT (mul_x!/mul_y!/mul_z!,
// src/Discretization/Plans.jl:1132-1167), multiplies by the kinetic phase
// (src/NumModels/GrossPitaevskii/splitting.jl:167, 172, 190, 195, 200) and
// transforms back (ldiv_x!/..., Plans.jl:1207-1250).  Here one kernel reads
// the lines in place (no transpose), so the whole FFT -> phase -> iFFT costs
// one HBM read and one HBM write of the field.
//
// Line length n = N1 * N2 (N1 = min(n, 16)).  A line is processed by P = N2
// threads, each holding N1 = 16 complex values in registers:
//   stage A  load x[r + N2 j] (j < N1), forward DFT_N1, twiddle w_n^{r k1}
//            -> shared memory slot (k1, r)
//   stage B  thread k1 reads (k1, r) for r < N2, forward DFT_N2 gives
//            X[k1 + N1 k2]; multiply by the phase; backward DFT_N2; twiddle
//            conj(w_n^{r k1}) -> shared slot (k1, r)
//   stage C  thread r reads (k1, r) for k1 < N1, backward DFT_N1 gives
//            x[r + N2 j]; epilogue; store
// The spectrum is never reordered: the forward transform ends and the
// backward one starts in the same registers.  Lines of n <= 16 run entirely in
// one thread.
//
// Two thread layouts:
//   XL  (x axis, stride 1)    the P threads of a line are adjacent lanes, so
//                             global accesses walk along the line;
//   COL (y/z axes, strided)   W adjacent lanes hold W adjacent lines (adjacent
//                             x columns), so each global access is a run of
//                             W * sizeof(complex) >= 128 contiguous bytes.
// Shared-memory layouts are chosen so every stage is bank-conflict free
// (XL: one pad slot per N2-row plus N2 per line; COL: position-major).
//
// Constants (twiddles w_n^{r k1} and the kinetic phase factors) are held as
// double-word pairs hi + lo and applied with cmul2: a rounded constant alone
// would repeat the same relative error on the same mode at every pass.
//
// Modes:
//   MODE_FUSED  FFT -> phase -> iFFT (+ optional NL epilogue, reductions)
//   MODE_FWD    FFT only, writes the natural-order spectrum (plain form)
//   MODE_INV    iFFT (with 1/n) from a natural-order spectrum (plain form)
//   MODE_DIAG   FFT only, writes nothing, accumulates Parseval sums (energy)
#pragma once
#include <cstdint>
#include "fft_core.cuh"
#include "fft_comp.cuh"
#include "nl_phase.cuh"
#include "bulk_async.cuh"

namespace gpss {

enum { MODE_FUSED = 0, MODE_FWD = 1, MODE_INV = 2, MODE_DIAG = 3 };

// reduction slots written by a pass (per-CTA partials, summed on the device)
enum {
    RQ_MASS = 0,   // sum |psi|^2
    RQ_POT = 1,    // sum V |psi|^2
    RQ_INT = 2,    // sum |psi|^4
    RQ_KIN = 3,    // sum over lines of (1/n) sum_k xi_k^2 |X_k|^2
    RQ_ROT = 4,    // sum over lines of c_line (1/n) sum_k xi_k |X_k|^2
    RQ_COUNT = 5
};
enum { RED_POINT = 1, RED_KIN = 2, RED_MASS = 4 };
// how the last CTA finishes a reduction: plain sums, plus the factor of the
// imaginary-time renormalisation (1/sqrt(M dV), normalize!) or of the mass
// lock (sqrt(M0/M)) written to *fin_scale for the next pass
enum { FIN_NONE = 0, FIN_UNITMASS = 1, FIN_MASSLOCK = 2 };
enum { NL_NONE = 0, NL_REAL = 1, NL_IMAG = 2 };
// Optional work a FUSED pass instantiation can do (chosen per launch from the
// arguments; a leaner instantiation keeps fewer values live, which kept the
// hot passes free of register spills under the 80-register bound):
//   FEAT_NL    nonlinear epilogue and the mass sum
//   FEAT_DIAG  energy sums (RED_POINT, RED_KIN), rotation (per-row phases),
//              accumulation into a second field
//   FEAT_PLANE a stack of independent 2D runs of one shape (planes): the
//              nonlinear constants and the deferred renormalisation factor
//              are per plane (plane_nl, plane_scale)
//   FEAT_IMAGM the merged imaginary-time step: the nonlinear flow as a
//              prologue of the first pass (nl_pre, after the deferred
//              factor, its result also stored to nl_pre_out) and the mass sum
//              of the last pass replaced by Re sum conj(dot_with) psi
//   FEAT_ADJ   the discrete adjoint's epilogues (pre_out, adj_pre) without
//              the energy sums (FEAT_DIAG includes them as well)
//   FEAT_SMALL (launch shape, FP32 y/z lines) CTAs of 128 threads, for fields
//              whose pass would otherwise have fewer tiles than SMs
//   FEAT_MASK  the 2/3 dealiasing filter in place of the phase: on the last
//              axis of a spectrum already transformed along the others, keep
//              the modes with |kk| <= mask_lim[line] (scaled by 1/n), zero the rest
//   FEAT_ACC   the `acc` epilogue alone (add the result to a second field:
//              the y/z passes of lapRot in the RK and implicit schemes)
//   FEAT_COMP  (FP32) compensated arithmetic: the transforms, twiddles and
//              phase run on grid-exact two-float values (fft_comp.cuh), so
//              the only FP32 rounding of the pass is the store; combined with
//              FEAT_NONE, FEAT_NL or FEAT_ALL
//   FEAT_GRIDM (with FEAT_COMP, without FEAT_DIAG) one grid for the whole
//              pass from the mass bound `grid_mass` instead of a grid per
//              thread and stage (no re-gridding between stages)
//   FEAT_TMA   (FP32 y/z columns of a 3D field, with FEAT_NONE or FEAT_NL)
//              each tile arrives in shared memory by one tensor copy (TMA,
//              `tmap`), issued while the previous tile is transformed
enum { FEAT_NONE = 0, FEAT_NL = 1, FEAT_DIAG = 2, FEAT_ALL = 3, FEAT_PLANE = 4, FEAT_IMAGM = 8, FEAT_ADJ = 16,
       FEAT_SMALL = 32, FEAT_MASK = 64, FEAT_ACC = 128, FEAT_COMP = 256, FEAT_GRIDM = 512, FEAT_TMA = 1024 };

// Polls of a tile copy's mbarrier before a FEAT_TMA pass gives up (each
// try_wait may suspend the thread for a while; a copy takes microseconds)
constexpr uint32_t kTmaWaitPolls = 1u << 22;

// A renormalisation factor as written by the last CTA of a pass: FP64 for the
// FP64 kernels and a float copy for the FP32 ones (which then need no FP64
// conversion per thread).  Device buffers holding one are 16 bytes.
struct ScaleCell {
    double d;
    float f;
};
template <typename T> __device__ __forceinline__ T load_scale(const double *p);
template <> __device__ __forceinline__ float load_scale<float>(const double *p)
{
    return reinterpret_cast<const ScaleCell *>(p)->f;
}
template <> __device__ __forceinline__ double load_scale<double>(const double *p) { return *p; }
__device__ __forceinline__ void store_scale(double *p, double v)
{
    ScaleCell *c = reinterpret_cast<ScaleCell *>(p);
    c->d = v;
    c->f = (float)v;
}

template <typename T> struct PassArgs {
    const vec2<T> *in;
    vec2<T> *out;
    const vec2<T> *tw;       // 4n entries: stage-A table hi[n], lo[n] at m = k1*N2 + r, then
                             // the stage-B table hi[n], lo[n] at m = r*N1 + k1; both hold
                             // hi[m] + lo[m] = w_n^{r k1} (two index orders so that adjacent
                             // lanes read adjacent entries in either stage)
    const vec2<T> *phase;    // per row: hi[n] then lo[n]; row `row` starts at row*prow
                             // (fused tables already include the 1/n of the inverse)
    int64_t prow;            // 0: one table row for every line (held in shared memory)
    int rowmod;              // row of line g is g % rowmod
    int nlines;
    int m0;                  // base(g) = (g % m0) * s0 + (g / m0) * s1
    int64_t s0, s1, stride;  // stride between positions along the line
    T inv_n;                 // MODE_INV scale (1/n)
    // nonlinear epilogue (MODE_FUSED): psi <- exp(-i (V + beta|psi|^2) dt) psi
    int nl_mode;
    const T *V;              // nullable (zero potential)
    double nl_beta, nl_dt;
    NLSplit nl_split;        // FP32 kernels: beta, dt, beta*dt as float pairs
    // deferred renormalisation: multiply the input by the factor in a
    // ScaleCell (nullable; `scale` points at its FP64 member)
    const double *scale;
    // reductions: per-CTA FP64 partials, finished by the last CTA to arrive
    int red;                 // RED_POINT | RED_KIN | RED_MASS
    double *partials;        // [RQ_COUNT][gridDim.x]
    unsigned int *counter;   // arrival counter (0 between launches)
    double *fin_out;         // RQ_COUNT sums of this pass
    int fin_mode;            // FIN_*
    const double *fin_target;  // M0 of the mass lock
    double *fin_scale;       // factor for the next pass (a ScaleCell)
    int *fin_status;         // set to 1 on a non-finite or non-positive mass
    double dV;
    T kmult;                 // xi_k = kk * kmult, kk the signed wavenumber index
    const double *coord;     // coordinate of each row (rotation energy), nullable
    // FUSED: add the result to this field (same layout as out; may alias it) --
    // the per-axis terms of a sum of directional operators (lapRot of the RK
    // right-hand side); nullable
    const vec2<T> *acc;
    // FUSED with the NL epilogue: also store the value entering the NL stage
    // here (the states the discrete adjoint needs); nullable
    vec2<T> *pre_out;
    // FUSED: replace the NL epilogue by its adjoint at the state adj_pre (the
    // input of the forward NL stage; constants nl_beta/nl_dt/nl_split, V):
    //   g <- conj(f) g + 2 beta dt Im(conj(g) f pre) pre,
    //   adj_dLdV += dt Im(conj(g) f pre),   f = exp(-i (V + beta|pre|^2) dt)
    const vec2<T> *adj_pre;
    double *adj_dLdV;
    // FEAT_PLANE: line g belongs to plane g / plane_lines; per plane the NL
    // constants (FP32 split) and the prescale factor (nullable: no prescale)
    const NLSplit *plane_nl;
    const ScaleCell *plane_scale;
    int plane_lines;
    // FEAT_IMAGM: psi_in <- N(scale * psi_in) before the transform (imaginary
    // time; constants nl_beta/nl_dt/nl_split, V), stored to nl_pre_out
    // (nullable); and RED_MASS sums Re(conj(dot_with) psi_out) (nullable)
    int nl_pre;
    vec2<T> *nl_pre_out;
    const vec2<T> *dot_with;
    // FEAT_MASK: the largest kept |kk| of each line (-1: none)
    const int *mask_lim;
    // FP32 FUSED passes: nonzero selects the compensated instantiation (FEAT_COMP)
    int comp;
    // compensated passes: nullable device pointer to a mass M >= sum |psi|^2
    // of the pass input (after its deferred factor).  Every intermediate of a
    // length-n transform is a sum of at most n unit-weighted values, so its
    // modulus is at most sqrt(n M) <= 16 sqrt(M); with 2 M that bounds all
    // stages of all lines, and one quantum for the whole pass replaces the
    // per-thread, per-stage ones (no re-gridding between stages)
    const double *grid_mass;
    // FEAT_TMA: a CUtensorMap (global memory, 64-byte aligned) of the 3D
    // field `in` with boxes of W x-adjacent columns by the whole line; the
    // line axis (1: y, 2: z) and nx, which W divides
    const void *tmap;
    int taxis, tnx;
    // pipelined pass: 0 waits up to the default number of polls for a tile;
    // v > 0 waits v - 1 polls (host-side fault injection of a timeout)
    unsigned wait_polls;
};

// a double-word constant in shared memory: hi and lo adjacent, so one
// 16-byte load (two for FP64) fetches both
template <typename V> struct __align__(2 * sizeof(V)) DWord {
    V hi, lo;
};

// Threads per CTA and resident CTAs per SM that the kernels are compiled for.
// FP32: 768 threads per SM (at most 80 registers) measured best at 256^3;
// 1024 (64 registers) spills and runs 15-25% slower, no bound lets the fused
// kernels grow past 85 registers and run 1.7x slower.  x lines run in CTAs
// of 128 threads (with their warp barriers 256 runs the same and 64 is 13%
// slower), y/z columns in CTAs of 256 (their global accesses are W = 256/16 =
// 16 adjacent cells, 128 B; with 128 threads they would be 64 B and run 5%
// slower).
#ifndef GPSS_PASS_THREADS_XL_F32
#define GPSS_PASS_THREADS_XL_F32 128
#endif
#ifndef GPSS_PASS_THREADS_COL_F32
#define GPSS_PASS_THREADS_COL_F32 256
#endif
#ifndef GPSS_PASS_SM_THREADS_F32
#define GPSS_PASS_SM_THREADS_F32 768
#endif
// the lean FUSED y/z instantiation (FEAT_NONE: kinetic pass only) fits 64
// registers without spills, so it is compiled for 1024 threads per SM (y pass
// 69.5 -> 67.2 us at 256^3); the x one spills at 64 (6% slower).  With warp
// barriers and dependent launch the lean x pass runs at 768 threads per SM
// (80 registers): alone it is 0.6 us slower than at 896, but the 256^3 step
// is 197.2 -> 195.6 us (the next pass's CTAs find room sooner).  The NL
// instantiation spills at 64 (1% slower).
#ifndef GPSS_PASS_SM_THREADS_LEAN_F32
#define GPSS_PASS_SM_THREADS_LEAN_F32 1024
#endif
#ifndef GPSS_PASS_SM_THREADS_LEAN_XL_F32
#define GPSS_PASS_SM_THREADS_LEAN_XL_F32 768  // 6 CTAs of 128
#endif
// FP64: CTAs of 64 threads.  The FP64 kernels are bound by GB300's FP64 rate
// per SM, so small fields must spread over many SMs (2D 128^2 step 176 -> 88
// us against 256-thread CTAs); 3D fields lose nothing (256^3 plain step 14.75
// -> 14.38 ms, 128^3 fused 1015 -> 946 us).
#ifndef GPSS_PASS_THREADS_F64
#define GPSS_PASS_THREADS_F64 64
#endif
// Small fields (a 2D y pass of 256 columns is 16 tiles of 16): y/z CTAs of 128
// threads (FEAT_SMALL) give twice the tiles (2D 128^2 step 11.4 -> 10.6 us,
// 256^2 13.1 -> 12.5 us); at 256^3 they would cost the y pass 34 %.  The lean
// y/z pass in CTAs of 512 threads (32 columns = 256 B runs, 2 per SM) was
// slower too: y 63.0 -> 67.8 us at 256^3.
#ifndef GPSS_PASS_THREADS_COL_LEAN_F32
#define GPSS_PASS_THREADS_COL_LEAN_F32 256
#endif
// compensated y/z passes: CTAs of 128 threads (8 columns, 64 B runs), four
// per SM: fewer threads wait at each of the two stage barriers (256^3: y
// 152.3 -> 146.6 us, z+NL 159.4 -> 157.2 us against 256-thread CTAs).  Their
// tile count, cells / 2048, is that of the 128-thread x pass, which the
// context's partial-sum buffer already holds.
#ifndef GPSS_PASS_THREADS_COL_COMP_F32
#define GPSS_PASS_THREADS_COL_COMP_F32 128
#endif
template <typename T, bool XL, int FEAT = 0> struct PassGeom {
    static constexpr int THREADS =
        sizeof(T) == 4 ? (XL ? GPSS_PASS_THREADS_XL_F32
                             : ((FEAT & FEAT_SMALL) ? 128
                                : (FEAT & FEAT_COMP) ? GPSS_PASS_THREADS_COL_COMP_F32
                                : (FEAT == FEAT_NONE ? GPSS_PASS_THREADS_COL_LEAN_F32 : GPSS_PASS_THREADS_COL_F32)))
                       : GPSS_PASS_THREADS_F64;
};
// The merged imaginary-time passes (FEAT_IMAGM) fit 72 (x) and 64 (y/z)
// registers without spills; with one more CTA per SM a 128^3 field's x pass
// (1024 tiles) fits one wave of resident CTAs (1064) instead of 1.12 waves
// of 912: the 128^3 imaginary-time trap step 38.8 -> 34.6 us.
#ifndef GPSS_PASS_SM_THREADS_IMAGM_XL_F32
#define GPSS_PASS_SM_THREADS_IMAGM_XL_F32 896
#endif
#ifndef GPSS_PASS_SM_THREADS_IMAGM_F32
#define GPSS_PASS_SM_THREADS_IMAGM_F32 1024
#endif
// Compensated passes (FEAT_COMP) hold every transform value as hi + lo: 512
// threads per SM (128 registers).
#ifndef GPSS_PASS_SM_THREADS_COMP_F32
#define GPSS_PASS_SM_THREADS_COMP_F32 512
#endif
#ifndef GPSS_PASS_SM_THREADS_PLANE_XL_F32
// stacked 2D planes: 7 CTAs per SM give 64 x 256^2 planes' 2048 x tiles 1.9
// waves instead of 2.25 (the 512-run batch 44.1 -> 43.5 ms per 500 steps)
#define GPSS_PASS_SM_THREADS_PLANE_XL_F32 896
#endif
template <typename T, bool XL, int MODE, int FEAT> struct PassOcc {
    static constexpr int SM_THREADS =
        (FEAT & FEAT_COMP) ? GPSS_PASS_SM_THREADS_COMP_F32
        : (MODE == MODE_FUSED && (FEAT & ~FEAT_SMALL) == FEAT_NONE)
            ? (XL ? GPSS_PASS_SM_THREADS_LEAN_XL_F32 : GPSS_PASS_SM_THREADS_LEAN_F32)
        : (MODE == MODE_FUSED && FEAT == FEAT_IMAGM)
            ? (XL ? GPSS_PASS_SM_THREADS_IMAGM_XL_F32 : GPSS_PASS_SM_THREADS_IMAGM_F32)
        : (MODE == MODE_FUSED && XL && (FEAT & FEAT_PLANE))
            ? GPSS_PASS_SM_THREADS_PLANE_XL_F32
            : GPSS_PASS_SM_THREADS_F32;
    static constexpr int MIN_BLOCKS = sizeof(T) == 4 ? SM_THREADS / PassGeom<T, XL, FEAT>::THREADS : 1;
};

template <int N> struct Split {
    static constexpr int N1 = N <= 16 ? N : 16;
    static constexpr int N2 = N / N1;
};

template <typename T, int N, bool XL, int FEAT = 0> struct PassShape {
    static constexpr int N1 = Split<N>::N1;
    static constexpr int N2 = Split<N>::N2;
    static constexpr int P = N2;                       // threads per line
    static constexpr int THREADS = PassGeom<T, XL, FEAT>::THREADS;
    static constexpr int W = THREADS / P;              // lines per CTA
    static constexpr int LS = N + N1 + N2;             // XL padded line stride (slots)
    static constexpr int DATA1 = (N2 == 1) ? 0 : (XL ? W * LS : W * N);
    // compensated passes hold (hi, lo) of a value in one 16-byte slot: DATA1
    // such slots, the size of two value arrays (one 128-bit shared-memory
    // access per value and exchange instead of two 64-bit ones: 256^3 y pass
    // 128.4 -> 123.3 us, z 139.4 -> 136.1 us)
    static constexpr int DATA = DATA1 * ((FEAT & FEAT_COMP) ? 2 : 1);
    // FEAT_TMA: the tile's staging buffer (first, 128-byte aligned) and the
    // copy's mbarrier (after the tables)
    static constexpr bool TMA = (FEAT & FEAT_TMA) != 0 && !XL;
    static constexpr int STAGE = TMA ? W * N : 0;
    // w_n^{r k1} at k1*N2 + r (stage A) and at r*N1 + k1 (stage B) are the same
    // table when N1 == N2: then only one is held
    static constexpr bool TWB = N1 != N2;
    static constexpr int SMEM_SLOTS = STAGE + DATA + (TWB ? 6 : 4) * N + (TMA ? 2 : 0);  // + tables hi and lo
    static constexpr size_t SMEM_BYTES = sizeof(vec2<T>) * SMEM_SLOTS;
};

// sum of `v` over the CTA, written by thread 0 into partials[q * gridDim.x + blockIdx.x]
template <typename T, int THREADS>
__device__ __forceinline__ void block_sum_store(T v, double *partials, int q, T *red_smem)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red_smem[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
#pragma unroll
        for (int i = 0; i < THREADS / 32; i++) s += (double)red_smem[i];
        partials[(size_t)q * gridDim.x + blockIdx.x] = s;
    }
}

// The last CTA of the grid to finish sums every CTA's partials (same fixed
// order whichever CTA is last, so results are deterministic), writes the
// sums and the next-pass factor, and re-arms the counter for the next launch.
// CTA sums of the quantities in qmask (vals[q], q < RQ_COUNT, each thread's
// FP64 total) with one barrier, in FP64 from the thread totals on; thread 0
// writes partials[q * gridDim.x + blockIdx.x]
template <int THREADS>
__device__ __forceinline__ void block_sums_store(const double (&vals)[RQ_COUNT], unsigned qmask, double *partials)
{
    __shared__ double red_smem[RQ_COUNT][THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < RQ_COUNT; q++) {
        if (!(qmask & (1u << q))) continue;
        double v = vals[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red_smem[q][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 0; q < RQ_COUNT; q++) {
            if (!(qmask & (1u << q))) continue;
            double s = 0.0;
#pragma unroll
            for (int i = 0; i < THREADS / 32; i++) s += red_smem[q][i];
            partials[(size_t)q * gridDim.x + blockIdx.x] = s;
        }
    }
}

template <typename T, int THREADS>
__device__ __forceinline__ void finish_reduction(const PassArgs<T> &a, unsigned qmask)
{
    __shared__ bool last;
    __shared__ double red[THREADS];
    if (threadIdx.x == 0) {
        __threadfence();  // this CTA's partials before its arrival
        const unsigned ticket = atomicAdd(a.counter, 1u);
        last = ticket == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int G = gridDim.x;
    for (int q = 0; q < RQ_COUNT; q++) {
        if (!(qmask & (1u << q))) continue;
        double s = 0.0;
        for (int b = threadIdx.x; b < G; b += THREADS) s += __ldcg(a.partials + (size_t)q * G + b);
        red[threadIdx.x] = s;
        __syncthreads();
#pragma unroll
        for (int o = THREADS / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) a.fin_out[q] = red[0];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (a.fin_mode != FIN_NONE) {
            const double m = a.fin_out[RQ_MASS];
            if (!(m > 0.0) || !isfinite(m)) {
                *a.fin_status = 1;
                store_scale(a.fin_scale, 1.0);
            } else if (a.fin_mode == FIN_MASSLOCK) {
                store_scale(a.fin_scale, sqrt(*a.fin_target / m));
            } else {
                store_scale(a.fin_scale, 1.0 / (sqrt(m) * sqrt(a.dV)));
            }
        }
        *a.counter = 0u;
    }
}

template <typename T, int N, bool XL, int MODE, int FEAT = FEAT_ALL>
__global__ void __launch_bounds__(PassGeom<T, XL, FEAT>::THREADS, PassOcc<T, XL, MODE, FEAT>::MIN_BLOCKS)
pass_kernel(const PassArgs<T> a)
{
    constexpr bool kNL = (FEAT & FEAT_NL) != 0, kDiag = (FEAT & FEAT_DIAG) != 0;
    constexpr bool kPlane = (FEAT & FEAT_PLANE) != 0 && sizeof(T) == 4;
    constexpr bool kImagM = (FEAT & FEAT_IMAGM) != 0;
    constexpr bool kAdj = kDiag || (FEAT & FEAT_ADJ) != 0;
    constexpr bool kMask = (FEAT & FEAT_MASK) != 0;
    constexpr bool kAcc = kDiag || (FEAT & FEAT_ACC) != 0;
    constexpr bool kComp = (FEAT & FEAT_COMP) != 0 && sizeof(T) == 4;
    static_assert(!kComp || (MODE == MODE_FUSED && !kMask && !kPlane && !kImagM), "compensated: fused kinetic passes");
    constexpr bool kTma = PassShape<T, N, XL, FEAT>::TMA;
    static_assert(!kTma || (MODE == MODE_FUSED && !kComp && !kDiag && !kPlane && !kImagM && !kMask && !kAdj),
                  "tensor-copy tiles: plain kinetic (+NL) passes");
    const int red = a.red & ((kDiag ? (RED_POINT | RED_KIN) : 0) | (kNL || kDiag || kImagM ? RED_MASS : 0));
    const int64_t prow = kDiag ? a.prow : 0;
    using V = vec2<T>;
    using S = PassShape<T, N, XL, FEAT>;
    constexpr int N1 = S::N1, N2 = S::N2, P = S::P, W = S::W, LS = S::LS;
    constexpr int THREADS = S::THREADS;

    extern __shared__ __align__(128) unsigned char smem_raw[];
    V *stage = reinterpret_cast<V *>(smem_raw);  // FEAT_TMA staging tile (position-major, W per row)
    (void)stage;
    V *sdata = stage + S::STAGE;
    // compensated passes: (hi, lo) of a value as one 16-byte slot, in the
    // layout of sdata with DATA1 such slots
    float4 *sd4 = reinterpret_cast<float4 *>(sdata);
    (void)sd4;
    DWord<V> *stw = reinterpret_cast<DWord<V> *>(sdata + S::DATA);  // stage A [N], stage B [N]
    DWord<V> *stwB = S::TWB ? stw + N : stw;
    DWord<V> *sph = stw + (S::TWB ? 2 : 1) * N;                      // phase [N]
    uint64_t *tbar = reinterpret_cast<uint64_t *>(sph + N);           // FEAT_TMA copy barrier
    (void)tbar;

    const int tid = threadIdx.x;
    if constexpr (kTma) {
        if (tid == 0) {
            mbar_init(tbar, 1u);
            fence_mbar_init();
        }
    }
    // tables into shared memory, hi/lo halves packed per entry
    for (int i = tid; i < N; i += THREADS) {
        stw[i] = DWord<V>{a.tw[i], a.tw[N + i]};
        if (S::TWB) stwB[i] = DWord<V>{a.tw[2 * N + i], a.tw[3 * N + i]};
        if (MODE == MODE_FUSED && !kMask && prow == 0) sph[i] = DWord<V>{a.phase[i], a.phase[N + i]};
    }

    const int w = XL ? tid / P : tid % W;
    const int r = XL ? tid % P : tid / W;
    const uint32_t st = XL ? 1u : (uint32_t)a.stride;

    auto sidx = [&](int q) -> int {
        if constexpr (XL) return w * LS + q + q / N2;
        else return q * W + w;
    };

    // Programmatic dependent launch: a pass may start while the previous
    // kernel of the stream finishes; only the constant tables above are read
    // before the previous grid has completed and its writes are visible.
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const bool scaled = a.scale != nullptr;
    const T scale = scaled ? load_scale<T>(a.scale) : (T)1;
    const T kmult = a.kmult;
    // compensated passes with a mass bound: one grid for every stage (C of
    // the quantum 2^-22 of 32 sqrt(M/2) = 16 sqrt(2 M), rounded up)
    constexpr bool gridm = kComp && (FEAT & FEAT_GRIDM) != 0;
    float2 Cm = make_float2(0.f, 0.f);
    if constexpr (gridm) Cm = grid_for((float)sqrt(0.5 * *a.grid_mass));
    (void)Cm;

    // accumulators: the field precision within a tile (its own cells), FP64
    // across the tiles of the CTA (one FP64 add per tile and quantity, so no
    // FP64 arithmetic per cell), FP64 for the warp and CTA sums
    T acc_mass = 0, acc_pot = 0, acc_int = 0, acc_kin = 0, acc_rot = 0;
    double tot[RQ_COUNT] = {0.0, 0.0, 0.0, 0.0, 0.0};

    // tiles of W lines; a grid smaller than the tile count loops (the tables
    // and the reduction tail are then paid once per CTA, not once per tile)
    const int ntiles = (a.nlines + W - 1) / W;
    // Stage A of a tile writes, and stage C reads, the same slots per thread
    // (k1 * N2 + r for k1 < N1), and stage B's reads and writes of the tile are
    // fenced by the barrier that precedes stage C, and the barrier after
    // stage A keeps the next tile's stage B writes behind every thread's
    // stage C.  So FUSED needs no barrier before a tile's stage A: one barrier
    // for the tables is enough.  FWD and DIAG have no stage C (a fast thread's
    // next stage A would overwrite slots another thread's stage B still
    // reads), INV no stage A (its stage B writes slots other threads' stage C
    // reads): they keep the barrier.
    constexpr bool kTopBarrier = MODE != MODE_FUSED;
    // In the XL layout the P threads of a line are adjacent lanes of one warp
    // (P divides 32) and only they touch the line's shared-memory slots, so
    // the exchanges between stages need only a warp barrier.  COL lines span
    // the CTA (lane stride W).
    static_assert(!XL || 32 % P == 0, "an XL line must not straddle warps");
    auto line_sync = [] {
        if constexpr (XL) __syncwarp();
        else __syncthreads();
    };
    __syncthreads();  // tables ready
    // FEAT_TMA: tile t is the box of W x-adjacent columns at (x0, rest); the
    // first tile's copy starts now, each next one after the stage-A barrier
    // of the current tile (when every thread has read the staging buffer)
    uint32_t tphase = 0;
    bool tdead = false;
    auto tma_issue = [&](int t) {
        const int g0 = t * W, x0 = g0 % a.tnx, rest = g0 / a.tnx;
        mbar_arrive_expect_tx(tbar, (uint32_t)(S::STAGE * sizeof(V)));
        if (a.taxis == 1) tma_load_3d(stage, a.tmap, x0, 0, rest, tbar);
        else tma_load_3d(stage, a.tmap, x0, rest, 0, tbar);
    };
    (void)tma_issue;
    if constexpr (kTma) {
        if (tid == 0 && (int)blockIdx.x < ntiles) {
            asm volatile("fence.proxy.async.global;" ::: "memory");  // the previous grid's field writes
            tma_issue(blockIdx.x);
        }
    }
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int g = tile * W + w;
    const bool valid = g < a.nlines;
    const int gg = valid ? g : 0;
    // a tile never straddles two planes (plane_lines is a multiple of W)
    const int plane = kPlane ? gg / a.plane_lines : 0;
    // (the imaginary-time prologue applies the factor itself, before N)
    const bool tscaled = (scaled && !(kImagM && a.nl_pre)) || (kPlane && a.plane_scale);
    T tscale = scale;
    if constexpr (kPlane) {
        if (a.plane_scale) tscale = a.plane_scale[plane].f;
    }
    // element indices fit 32 bits (at most 256^3 cells); x lines have unit stride
    const uint32_t base = (uint32_t)((gg % a.m0) * a.s0 + (gg / a.m0) * a.s1);
    const int row = gg % a.rowmod;

    V v[N1];
    if constexpr (MODE != MODE_INV) {
        if constexpr (kTma) {
            // the tile's copy: a bounded wait (a copy that never lands is
            // reported, not waited on forever), then the thread's values
            tdead = tdead || !mbar_wait_bounded(tbar, tphase, kTmaWaitPolls);
            tphase ^= 1u;
#pragma unroll
            for (int j = 0; j < N1; j++) v[j] = stage[(r + N2 * j) * W + w];
        } else {
#pragma unroll
            for (int j = 0; j < N1; j++) {
                v[j] = a.in[base + (uint32_t)(r + N2 * j) * st];  // invalid threads read line 0 ...
            }
        }
        if constexpr (MODE == MODE_FUSED || MODE == MODE_DIAG) {
            if (!valid) {  // ... and sum nothing
#pragma unroll
                for (int j = 0; j < N1; j++) v[j] = mk<V>((T)0, (T)0);
            }
        }
        if constexpr (MODE == MODE_FUSED && kImagM) {
            if (a.nl_pre) {  // chi = N(scale * psi), kept for the inner product of the last pass
                const NLConst<T> nlc = nl_const<T>(a.nl_split, a.nl_beta, a.nl_dt);
#pragma unroll
                for (int j = 0; j < N1; j++) {
                    const uint32_t e = base + (uint32_t)(r + N2 * j) * st;
                    const V u = scaled ? cscale(v[j], scale) : v[j];
                    v[j] = nl_apply(u, a.V ? a.V[e] : (T)0, nlc, true);
                    if (valid && a.nl_pre_out) a.nl_pre_out[e] = v[j];
                }
            }
        }
        if constexpr (MODE == MODE_DIAG) {
            if (red & RED_POINT) {
#pragma unroll
                for (int j = 0; j < N1; j++) {
                    T rho = v[j].x * v[j].x + v[j].y * v[j].y;
                    acc_mass += rho;
                    acc_int += rho * rho;
                    if (a.V) acc_pot += a.V[base + (uint32_t)(r + N2 * j) * st] * rho;
                }
            }
        }
        if constexpr (!kComp) dft<N1, -1>(v);
    }
    if constexpr (kTopBarrier) line_sync();  // the previous tile's stage B is done with sdata

    if constexpr (kComp) {
        // compensated kinetic pass: the same stages on gridded two-float
        // values (fft_comp.cuh); each thread grids each stage's values on its
        // own quantum.  The deferred factor enters with the first gridding
        // (an exact product and residual), which is the same linear map as
        // scaling the spectrum.
        cdf c[N1];
        {
            const float sc = tscaled ? (float)tscale : 1.f;
            const float2 C = gridm ? Cm : grid_for(absmax<N1>(v) * fabsf(sc));
            if (tscaled) {
                const float2 S = make_float2(sc, sc);
#pragma unroll
                for (int j = 0; j < N1; j++) c[j] = g_from_scaled(v[j], S, C);
            } else {
#pragma unroll
                for (int j = 0; j < N1; j++) c[j] = g_from(v[j], C);
            }
            g_dft<N1, -1>(c, C);
            if constexpr (N2 == 1) {
                if (red & RED_KIN) {
                    T s2 = 0, s1 = 0;
#pragma unroll
                    for (int k = 0; k < N1; k++) {
                        const int kk = k < N / 2 ? k : k - N;
                        const T xi = (T)kk * kmult;
                        const float2 X = c_round(c[k]);
                        const T m2 = X.x * X.x + X.y * X.y;
                        s2 += xi * xi * m2;
                        s1 += xi * m2;
                    }
                    acc_kin += s2 * (T)(1.0 / N);
                    if (a.coord) acc_rot += s1 * (T)(1.0 / N) * (T)a.coord[row];
                }
#pragma unroll
                for (int k = 0; k < N1; k++) {
                    const DWord<V> p = prow ? DWord<V>{a.phase[row * prow + k], a.phase[row * prow + N + k]}
                                              : sph[k];
                    c[k] = g_cmul2(c[k], p.hi, p.lo, C);
                }
                g_dft<N1, +1>(c, C);
            } else {
                // stage A store: (k1, r) <- c[k1] * w_n^{r k1}, h and l
#pragma unroll
                for (int k1 = 0; k1 < N1; k1++) {
                    const int m = k1 * N2 + r;
                    cdf t = c[k1];
                    if (k1 != 0 && r != 0) {
                        const DWord<V> w2 = stw[m];
                        t = g_cmul2(t, w2.hi, w2.lo, C);
                    }
                    sd4[sidx(m)] = make_float4(t.h.x, t.h.y, t.l.x, t.l.y);
                }
            }
        }
        if constexpr (N2 > 1) {
            line_sync();
            constexpr int NI = N1 / N2;
#pragma unroll
            for (int i = 0; i < NI; i++) {
                const int k1 = r + P * i;
                cdf u[N2];
#pragma unroll
                for (int rr = 0; rr < N2; rr++) {
                    const float4 q4 = sd4[sidx(k1 * N2 + rr)];
                    u[rr].h = make_float2(q4.x, q4.y);
                    u[rr].l = make_float2(q4.z, q4.w);
                }
                float2 C = Cm;
                if constexpr (!gridm) {
                    C = grid_for(absmax<N2>(u));
#pragma unroll
                    for (int rr = 0; rr < N2; rr++) u[rr] = g_regrid(u[rr], C);
                }
                g_dft<N2, -1>(u, C);  // u[k2] = X[k1 + N1 k2]
                if (red & RED_KIN) {
                    T s2 = 0, s1 = 0;
#pragma unroll
                    for (int k2 = 0; k2 < N2; k2++) {
                        const int k = k1 + N1 * k2;
                        const int kk = k < N / 2 ? k : k - N;
                        const T xi = (T)kk * kmult;
                        const float2 X = c_round(u[k2]);
                        const T m2 = X.x * X.x + X.y * X.y;
                        s2 += xi * xi * m2;
                        s1 += xi * m2;
                    }
                    acc_kin += s2 * (T)(1.0 / N);
                    if (a.coord) acc_rot += s1 * (T)(1.0 / N) * (T)a.coord[row];
                }
#pragma unroll
                for (int k2 = 0; k2 < N2; k2++) {
                    const int k = k1 + N1 * k2;
                    const DWord<V> p = prow ? DWord<V>{a.phase[row * prow + k], a.phase[row * prow + N + k]}
                                              : sph[k];
                    u[k2] = g_cmul2(u[k2], p.hi, p.lo, C);
                }
                g_dft<N2, +1>(u, C);
#pragma unroll
                for (int rr = 0; rr < N2; rr++) {
                    cdf t = u[rr];
                    if (k1 != 0 && rr != 0) {
                        const DWord<V> w2 = stwB[rr * N1 + k1];
                        t = g_cmulc2(t, w2.hi, w2.lo, C);
                    }
                    sd4[sidx(k1 * N2 + rr)] = make_float4(t.h.x, t.h.y, t.l.x, t.l.y);
                }
            }
            line_sync();
#pragma unroll
            for (int k1 = 0; k1 < N1; k1++) {
                const float4 q4 = sd4[sidx(k1 * N2 + r)];
                c[k1].h = make_float2(q4.x, q4.y);
                c[k1].l = make_float2(q4.z, q4.w);
            }
            float2 C = Cm;
            if constexpr (!gridm) {
                C = grid_for(absmax<N1>(c));
#pragma unroll
                for (int k1 = 0; k1 < N1; k1++) c[k1] = g_regrid(c[k1], C);
            }
            g_dft<N1, +1>(c, C);
        }
#pragma unroll
        for (int j = 0; j < N1; j++) v[j] = c_round(c[j]);
    } else if constexpr (N2 == 1) {
        // the whole line lives in this thread: v[k] = X[k]
        if constexpr (MODE == MODE_FUSED) {
            if (red & RED_KIN) {
                T s2 = 0, s1 = 0;
#pragma unroll
                for (int k = 0; k < N1; k++) {
                    const int kk = k < N / 2 ? k : k - N;
                    const T xi = (T)kk * kmult;
                    const T m2 = v[k].x * v[k].x + v[k].y * v[k].y;
                    s2 += xi * xi * m2;
                    s1 += xi * m2;
                }
                acc_kin += s2 * (T)(1.0 / N);
                if (a.coord) acc_rot += s1 * (T)(1.0 / N) * (T)a.coord[row];
            }
            if constexpr (kMask) {
                const int lim = a.mask_lim[gg];
#pragma unroll
                for (int k = 0; k < N1; k++) {
                    const int kk = k < (N + 1) / 2 ? k : N - k;
                    v[k] = kk <= lim ? cscale(v[k], a.inv_n) : mk<V>((T)0, (T)0);
                }
            } else {
#pragma unroll
                for (int k = 0; k < N1; k++) {
                    const DWord<V> p = prow ? DWord<V>{a.phase[row * prow + k], a.phase[row * prow + N + k]}
                                              : sph[k];
                    v[k] = cmul2(v[k], p.hi, p.lo);
                    if (tscaled) v[k] = cscale(v[k], tscale);
                }
            }
            dft<N1, +1>(v);
        } else if constexpr (MODE == MODE_DIAG) {
            if (red & RED_KIN) {
                T s2 = 0, s1 = 0;
#pragma unroll
                for (int k = 0; k < N1; k++) {
                    const int kk = k < N / 2 ? k : k - N;
                    const T xi = (T)kk * kmult;
                    const T m2 = v[k].x * v[k].x + v[k].y * v[k].y;
                    s2 += xi * xi * m2;
                    s1 += xi * m2;
                }
                acc_kin += s2 * (T)(1.0 / N);
                if (a.coord) acc_rot += s1 * (T)(1.0 / N) * (T)a.coord[row];
            }
        } else if constexpr (MODE == MODE_FWD) {
            // spectrum out in natural order
        } else {  // MODE_INV
#pragma unroll
            for (int j = 0; j < N1; j++) v[j] = a.in[base + (uint32_t)j * st];
            dft<N1, +1>(v);
#pragma unroll
            for (int j = 0; j < N1; j++) v[j] = cscale(v[j], a.inv_n);
        }
    } else {
        // ---- stage A store: (k1, r) <- v[k1] * w_n^{r k1}
        if constexpr (MODE != MODE_INV) {
#pragma unroll
            for (int k1 = 0; k1 < N1; k1++) {
                const int m = k1 * N2 + r;
                V t = v[k1];
                if (k1 != 0 && r != 0) {
                    const DWord<V> w2 = stw[m];
                    t = cmul2(t, w2.hi, w2.lo);
                }
                sdata[sidx(m)] = t;
            }
            if constexpr (kTma) {
                // every thread has read the staging buffer: the next tile's
                // copy may land in it.  A copy that timed out stops the CTA
                // here (the status word reports it; the CTA still joins the
                // reduction below so the grid's arrival count stays whole).
                if (__syncthreads_or(tdead)) {
                    if (tid == 0) {
                        mbar_wait_bounded(tbar, tphase ^ 1u, kTmaWaitPolls);  // its own copy, if it lands late
                        if (a.fin_status) atomicOr(a.fin_status, 2);
                    }
                    break;
                }
                if (tid == 0 && tile + (int)gridDim.x < ntiles) tma_issue(tile + (int)gridDim.x);
            } else {
                line_sync();
            }
        }
        // ---- stage B: items k1 = r + P*i
        constexpr int NI = N1 / N2;
#pragma unroll
        for (int i = 0; i < NI; i++) {
            const int k1 = r + P * i;
            V u[N2];
            if constexpr (MODE == MODE_INV) {
#pragma unroll
                for (int k2 = 0; k2 < N2; k2++) u[k2] = a.in[base + (uint32_t)(k1 + N1 * k2) * st];
            } else {
#pragma unroll
                for (int rr = 0; rr < N2; rr++) u[rr] = sdata[sidx(k1 * N2 + rr)];
                dft<N2, -1>(u);  // u[k2] = X[k1 + N1 k2]
            }
            if constexpr (MODE == MODE_FWD) {
                if (valid) {
#pragma unroll
                    for (int k2 = 0; k2 < N2; k2++) a.out[base + (uint32_t)(k1 + N1 * k2) * st] = u[k2];
                }
                continue;
            }
            if constexpr (MODE == MODE_FUSED || MODE == MODE_DIAG) {
                if (red & RED_KIN) {
                    T s2 = 0, s1 = 0;
#pragma unroll
                    for (int k2 = 0; k2 < N2; k2++) {
                        const int k = k1 + N1 * k2;
                        const int kk = k < N / 2 ? k : k - N;
                        const T xi = (T)kk * kmult;
                        const T m2 = u[k2].x * u[k2].x + u[k2].y * u[k2].y;
                        s2 += xi * xi * m2;
                        s1 += xi * m2;
                    }
                    acc_kin += s2 * (T)(1.0 / N);
                    if (a.coord) acc_rot += s1 * (T)(1.0 / N) * (T)a.coord[row];
                }
            }
            if constexpr (MODE == MODE_DIAG) continue;
            if constexpr (MODE == MODE_FUSED && kMask) {
                const int lim = a.mask_lim[gg];
#pragma unroll
                for (int k2 = 0; k2 < N2; k2++) {
                    const int k = k1 + N1 * k2;
                    const int kk = k < (N + 1) / 2 ? k : N - k;
                    u[k2] = kk <= lim ? cscale(u[k2], a.inv_n) : mk<V>((T)0, (T)0);
                }
            } else if constexpr (MODE == MODE_FUSED) {
#pragma unroll
                for (int k2 = 0; k2 < N2; k2++) {
                    const int k = k1 + N1 * k2;
                    const DWord<V> p = prow ? DWord<V>{a.phase[row * prow + k], a.phase[row * prow + N + k]}
                                              : sph[k];
                    u[k2] = cmul2(u[k2], p.hi, p.lo);
                    if (tscaled) u[k2] = cscale(u[k2], tscale);
                }
            }
            dft<N2, +1>(u);  // u[rr] = Z[k1][rr]
#pragma unroll
            for (int rr = 0; rr < N2; rr++) {
                V t = u[rr];
                if (k1 != 0 && rr != 0) {
                    const DWord<V> w2 = stwB[rr * N1 + k1];
                    t = cmulc2(t, w2.hi, w2.lo);
                }
                sdata[sidx(k1 * N2 + rr)] = t;
            }
        }
        if constexpr (MODE != MODE_FWD && MODE != MODE_DIAG) {
            line_sync();
            // ---- stage C
#pragma unroll
            for (int k1 = 0; k1 < N1; k1++) v[k1] = sdata[sidx(k1 * N2 + r)];
            dft<N1, +1>(v);  // v[j] = x[r + N2 j] (times n unless folded)
            if constexpr (MODE == MODE_INV) {
#pragma unroll
                for (int j = 0; j < N1; j++) v[j] = cscale(v[j], a.inv_n);
            }
        }
    }

    // ---- epilogue: positions r + N2 j
    if constexpr (MODE == MODE_FUSED || MODE == MODE_INV) {
        if constexpr (MODE == MODE_FUSED && kAdj) {
            if (a.pre_out && valid) {
#pragma unroll
                for (int j = 0; j < N1; j++) a.pre_out[base + (uint32_t)(r + N2 * j) * st] = v[j];
            }
            if (a.adj_pre) {
                const NLConst<T> nlc = nl_const<T>(a.nl_split, a.nl_beta, a.nl_dt);
                const T two_beta_dt = (T)(2.0 * a.nl_beta * a.nl_dt);
#pragma unroll
                for (int j = 0; j < N1; j++) {
                    const uint32_t e = base + (uint32_t)(r + N2 * j) * st;
                    const V pre = a.adj_pre[e];
                    const T vv = a.V ? a.V[e] : (T)0;
                    const V f = nl_factor(pre, vv, nlc, false);
                    const V pout = nl_rotate(f, pre);
                    const T im = v[j].x * pout.y - v[j].y * pout.x;  // Im(conj(g) psi_out)
                    if (valid) a.adj_dLdV[e] += a.nl_dt * (double)im;
                    const V rot = cmulc(v[j], f);                     // conj(f) g
                    v[j] = mk<V>(rot.x + two_beta_dt * im * pre.x, rot.y + two_beta_dt * im * pre.y);
                }
            }
        }
        if constexpr (MODE == MODE_FUSED) {
            if (kNL && a.nl_mode != NL_NONE) {
                const NLConst<T> nlc =
                    nl_const<T>(kPlane ? a.plane_nl[plane] : a.nl_split, a.nl_beta, a.nl_dt);
                const bool imag = a.nl_mode == NL_IMAG;
                bool done = false;
                if constexpr (sizeof(T) == 4) {
                    if (!imag) {
                        // one vote per warp: if every cell of the warp takes the
                        // micro series (the micro or tiny series, a short path),
                        // skip the per-cell choice (measured at 256^3: the z pass
                        // 76.0 -> 73.9 us against the tiny tier alone, with no
                        // loss on the 2D trap)
                        T rmax = 0, vmax = 0;
#pragma unroll
                        for (int j = 0; j < N1; j++) rmax = fmaxf(rmax, fmaf(v[j].x, v[j].x, v[j].y * v[j].y));
                        if (a.V) {
#pragma unroll
                            for (int j = 0; j < N1; j++)
                                vmax = fmaxf(vmax, fabsf(a.V[base + (uint32_t)(r + N2 * j) * st]));
                        }
                        const T tb = nl_theta_bound(rmax, vmax, nlc);
                        if (__all_sync(0xffffffffu, tb <= NL_MICRO_MAX)) {
                            if (a.V) {
#pragma unroll
                                for (int j = 0; j < N1; j++) {
                                    const T vv = a.V[base + (uint32_t)(r + N2 * j) * st];
                                    v[j] = nl_rotate(nl_factor_micro(nl_theta_short(v[j], vv, nlc)), v[j]);
                                }
                            } else {
#pragma unroll
                                for (int j = 0; j < N1; j++)
                                    v[j] = nl_rotate(nl_factor_micro(nl_theta_short(v[j], (T)0, nlc)), v[j]);
                            }
                            done = true;
                        } else if (__all_sync(0xffffffffu, tb <= NL_TINY_MAX)) {
                            if (a.V) {
#pragma unroll
                                for (int j = 0; j < N1; j++) {
                                    const T vv = a.V[base + (uint32_t)(r + N2 * j) * st];
                                    v[j] = nl_rotate(nl_factor_tiny_cell(nl_theta_short(v[j], vv, nlc)), v[j]);
                                }
                            } else {
#pragma unroll
                                for (int j = 0; j < N1; j++)
                                    v[j] = nl_rotate(nl_factor_tiny_cell(nl_theta_short(v[j], (T)0, nlc)), v[j]);
                            }
                            done = true;
                        } else if (__all_sync(0xffffffffu, tb <= NL_SHORT_MAX)) {
#pragma unroll
                            for (int j = 0; j < N1; j++) {
                                const T vv = a.V ? a.V[base + (uint32_t)(r + N2 * j) * st] : (T)0;
                                v[j] = nl_rotate(nl_factor_short(nl_theta_short(v[j], vv, nlc)), v[j]);
                            }
                            done = true;
                        }
                    }
                }
                if (!done) {
#pragma unroll
                    for (int j = 0; j < N1; j++) {
                        const T vv = a.V ? a.V[base + (uint32_t)(r + N2 * j) * st] : (T)0;
                        if constexpr (sizeof(T) == 4) {
                            v[j] = imag ? nl_apply(v[j], vv, nlc, true) : nl_apply_real_cell(v[j], vv, nlc);
                        } else {
                            v[j] = nl_apply(v[j], vv, nlc, imag);
                        }
                    }
                }
            }
            if (red & RED_POINT) {
#pragma unroll
                for (int j = 0; j < N1; j++) {
                    const T rho = v[j].x * v[j].x + v[j].y * v[j].y;
                    acc_mass += rho;
                    acc_int += rho * rho;
                    if (a.V) acc_pot += a.V[base + (uint32_t)(r + N2 * j) * st] * rho;
                }
            } else if (red & RED_MASS) {
                if (kImagM && a.dot_with) {
#pragma unroll
                    for (int j = 0; j < N1; j++) {
                        const V w = a.dot_with[base + (uint32_t)(r + N2 * j) * st];
                        acc_mass += w.x * v[j].x + w.y * v[j].y;
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < N1; j++) acc_mass += v[j].x * v[j].x + v[j].y * v[j].y;
                }
            }
        }
        if (valid) {
            if (MODE == MODE_FUSED && kAcc && a.acc) {
#pragma unroll
                for (int j = 0; j < N1; j++) {
                    const uint32_t e = base + (uint32_t)(r + N2 * j) * st;
                    a.out[e] = cadd(a.acc[e], v[j]);
                }
            } else {
#pragma unroll
                for (int j = 0; j < N1; j++) a.out[base + (uint32_t)(r + N2 * j) * st] = v[j];
            }
        }
    } else if constexpr (MODE == MODE_FWD && N2 == 1) {
        if (valid) {
#pragma unroll
            for (int k = 0; k < N1; k++) a.out[base + (uint32_t)k * st] = v[k];
        }
    }
    if constexpr (MODE == MODE_FUSED || MODE == MODE_DIAG) {
        if (red) {  // this tile's sums into the FP64 totals
            tot[RQ_MASS] += (double)acc_mass;
            tot[RQ_POT] += (double)acc_pot;
            tot[RQ_INT] += (double)acc_int;
            tot[RQ_KIN] += (double)acc_kin;
            tot[RQ_ROT] += (double)acc_rot;
            acc_mass = acc_pot = acc_int = acc_kin = acc_rot = (T)0;
        }
    }

    }  // tiles

    // This CTA's tiles are done: the next kernel of the stream may be
    // scheduled once every CTA has got here (so all of this grid's CTAs have
    // been resident: the dependent grid cannot hold SM slots this one needs),
    // overlapping its launch and table loads with this grid's tail.
    // (Triggering at the top instead was slower at 256^3: 201 vs 197 us per
    // step, the early grid's waiting CTAs sharing SMs with this one's last
    // tiles.)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");

    if constexpr (MODE == MODE_FUSED || MODE == MODE_DIAG) {
        if (red) {
            unsigned qmask = 0;
            if (red & (RED_POINT | RED_MASS)) qmask |= 1u << RQ_MASS;
            if (red & RED_POINT) qmask |= (1u << RQ_POT) | (1u << RQ_INT);
            if (red & RED_KIN) qmask |= (1u << RQ_KIN) | (1u << RQ_ROT);
            block_sums_store<THREADS>(tot, qmask, a.partials);
            finish_reduction<T, THREADS>(a, qmask);
        }
    }
}

}  // namespace gpss
