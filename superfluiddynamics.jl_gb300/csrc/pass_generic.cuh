// pass_generic.cuh -- the directional pass for line lengths that the register
// kernel (pass_kernel.cuh, powers of two up to 256) does not take: any n up to
// GEN_MAX_N whose prime factors are at most 31.  The reference plans every
// length with FFTW (plan_fft, src/Discretization/Plans.jl:846-847); its own
// tests run grids such as 48^3, 48x36 and 64x48x56.
//
// A CTA holds a tile of W lines in shared memory (two buffers, position-major
// so that adjacent threads touch adjacent lines) and runs a mixed-radix
// Stockham transform on it: stage s of radix R with Ns = the product of the
// earlier radices maps
//     v[q] = src[j + q n/R] * w_{Ns R}^{(j mod Ns) q},  DFT_R(v),
//     dst[(j / Ns) Ns R + (j mod Ns) + q Ns] = v[q]
// for j < n/R, which ends in natural order without a reordering pass.  Radices
// 2, 4, 8, 16 use the register DFTs of fft_core.cuh, 3 a closed form, other
// primes a direct DFT; every root of unity is a double-word entry of one table
// w_n^k = exp(-2 pi i k / n), k < n (the same constants the register kernel
// uses, so FP64 results stay within 1e-12 of the oracle).
//
// Modes and features are those of pass_kernel<MODE_FUSED/FWD/INV/DIAG> that the
// split steps, energies, explicit RK and implicit schemes use: phase (one row
// or per-row), deferred scale, nonlinear epilogue, reductions with the
// in-kernel finish, the 2/3 mask, accumulation into a second field.  The
// merged imaginary-time step, the adjoint, stacked planes, the pipelined and
// the compensated passes take power-of-two lines only.
#pragma once
#include "pass_kernel.cuh"

namespace gpss {

constexpr int GEN_MAX_N = 1024;
constexpr int GEN_MAX_STAGES = 12;
constexpr int GEN_THREADS = 256;

struct GenPlan {
    int n;
    int W;                       // lines per tile
    int nst;                     // stages
    int radix[GEN_MAX_STAGES];   // radices in stage order
};

// Stage radices of n (largest power-of-two radices first, then the odd primes
// in increasing order); false if n has a prime factor above 31 or is too long.
inline bool gen_plan_radices(int n, GenPlan &p)
{
    p.n = n;
    p.nst = 0;
    if (n < 2 || n > GEN_MAX_N) return false;
    int m = n;
    for (int r : {16, 8, 4, 2}) {
        while (m % r == 0 && p.nst < GEN_MAX_STAGES) {
            p.radix[p.nst++] = r;
            m /= r;
        }
    }
    for (int r : {3, 5, 7, 11, 13, 17, 19, 23, 29, 31}) {
        while (m % r == 0 && p.nst < GEN_MAX_STAGES) {
            p.radix[p.nst++] = r;
            m /= r;
        }
    }
    return m == 1;
}

// w_n^(m) as a double-word constant from the table (hi[n], lo[n]); DIR = +1
// conjugates (exp(+2 pi i m / n))
template <int DIR, typename V>
__device__ __forceinline__ void gen_root(const V *roots, int n, int m, V &hi, V &lo)
{
    hi = roots[m];
    lo = roots[n + m];
    if (DIR > 0) {
        hi.y = -hi.y;
        lo.y = -lo.y;
    }
}

// radix-3 butterfly: X1,2 = x0 - s/2 +- DIR i (sqrt3/2) d, s = x1 + x2,
// d = x1 - x2; sqrt3/2 = sin(2 pi / 3) is the double-word table entry of
// w_n^(n/3) (its imaginary part is -sin)
template <int DIR, typename V> __device__ __forceinline__ void gen_dft3(V *v, const V *roots, int n)
{
    using T = decltype(V::x);
    const T h = -roots[n / 3].y, l = -roots[n + n / 3].y;
    const V s = cadd(v[1], v[2]), d = csub(v[1], v[2]);
    const V x0 = v[0];
    v[0] = cadd(x0, s);
    const V m = mk<V>(fma((T)-0.5, s.x, x0.x), fma((T)-0.5, s.y, x0.y));
    // t = DIR i (sqrt3/2) d
    const V e = mk<V>(rmul2(d.x, h, l), rmul2(d.y, h, l));
    const V t = DIR < 0 ? mk<V>(e.y, -e.x) : mk<V>(-e.y, e.x);
    v[1] = cadd(m, t);
    v[2] = csub(m, t);
}

// direct DFT of odd prime size R (5, 7) with the table's roots w_R^{jk} = w_n^{jk n/R}
template <int R, int DIR, typename V>
__device__ __forceinline__ void gen_dft_direct(V *v, const V *roots, int n)
{
    V out[R];
    const int step = n / R;
#pragma unroll
    for (int k = 0; k < R; k++) {
        V acc = v[0];
#pragma unroll
        for (int j = 1; j < R; j++) {
            V hi, lo;
            gen_root<DIR>(roots, n, ((j * k) % R) * step, hi, lo);
            acc = cadd(acc, cmul2(v[j], hi, lo));
        }
        out[k] = acc;
    }
#pragma unroll
    for (int k = 0; k < R; k++) v[k] = out[k];
}

template <int R, int DIR, typename V> __device__ __forceinline__ void gen_butterfly(V *v, const V *roots, int n)
{
    if constexpr (R == 2 || R == 4 || R == 8 || R == 16) dft<R, DIR>(v);
    else if constexpr (R == 3) gen_dft3<DIR>(v, roots, n);
    else gen_dft_direct<R, DIR>(v, roots, n);
}

// one Stockham stage of radix R over the W lines of the tile (src -> dst)
template <int R, int DIR, typename V>
__device__ __forceinline__ void gen_stage(const V *src, V *dst, int W, int n, int Ns, const V *roots)
{
    const int L = n / R;
    const int items = W * L;
    for (int t = threadIdx.x; t < items; t += GEN_THREADS) {
        const int w = t % W, j = t / W;
        const int k = j % Ns;
        V v[R];
#pragma unroll
        for (int q = 0; q < R; q++) v[q] = src[(j + q * L) * W + w];
        if (Ns > 1) {
            const int scale = n / (Ns * R);
#pragma unroll
            for (int q = 1; q < R; q++) {
                V hi, lo;
                gen_root<DIR>(roots, n, (k * q * scale) % n, hi, lo);
                v[q] = cmul2(v[q], hi, lo);
            }
        }
        gen_butterfly<R, DIR>(v, roots, n);
        const int base = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int q = 0; q < R; q++) dst[(base + q * Ns) * W + w] = v[q];
    }
}

// one stage of a prime radix R in (7, 31] (rare lengths): the same mapping
// with a run-time radix, not unrolled
template <int DIR, typename V>
__device__ __noinline__ void gen_stage_prime(const V *src, V *dst, int W, int n, int Ns, int R, const V *roots)
{
    const int L = n / R;
    const int items = W * L;
    const int step = n / R;
    for (int t = threadIdx.x; t < items; t += GEN_THREADS) {
        const int w = t % W, j = t / W;
        const int k = j % Ns;
        V v[31];
#pragma unroll 1
        for (int q = 0; q < R; q++) {
            v[q] = src[(j + q * L) * W + w];
            if (Ns > 1 && q > 0) {
                V hi, lo;
                gen_root<DIR>(roots, n, (k * q * (n / (Ns * R))) % n, hi, lo);
                v[q] = cmul2(v[q], hi, lo);
            }
        }
        const int base = (j / Ns) * Ns * R + k;
#pragma unroll 1
        for (int kk = 0; kk < R; kk++) {
            V acc = v[0];
#pragma unroll 1
            for (int q = 1; q < R; q++) {
                V hi, lo;
                gen_root<DIR>(roots, n, ((q * kk) % R) * step, hi, lo);
                acc = cadd(acc, cmul2(v[q], hi, lo));
            }
            dst[(base + kk * Ns) * W + w] = acc;
        }
    }
}

// the whole transform; returns the buffer holding the result
template <int DIR, typename V>
__device__ V *gen_fft(V *b0, V *b1, const GenPlan &p, const V *roots)
{
    V *src = b0, *dst = b1;
    int Ns = 1;
    for (int s = 0; s < p.nst; s++) {
        const int R = p.radix[s];
        switch (R) {
        case 2: gen_stage<2, DIR>(src, dst, p.W, p.n, Ns, roots); break;
        case 3: gen_stage<3, DIR>(src, dst, p.W, p.n, Ns, roots); break;
        case 4: gen_stage<4, DIR>(src, dst, p.W, p.n, Ns, roots); break;
        case 5: gen_stage<5, DIR>(src, dst, p.W, p.n, Ns, roots); break;
        case 7: gen_stage<7, DIR>(src, dst, p.W, p.n, Ns, roots); break;
        case 8: gen_stage<8, DIR>(src, dst, p.W, p.n, Ns, roots); break;
        case 16: gen_stage<16, DIR>(src, dst, p.W, p.n, Ns, roots); break;
        default: gen_stage_prime<DIR>(src, dst, p.W, p.n, Ns, R, roots); break;
        }
        __syncthreads();
        Ns *= R;
        V *t = src;
        src = dst;
        dst = t;
    }
    return src;
}

template <typename T, int MODE>
__global__ void __launch_bounds__(GEN_THREADS)
gen_pass_kernel(const PassArgs<T> a, const GenPlan p)
{
    using V = vec2<T>;
    const int n = p.n, W = p.W;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    V *buf0 = reinterpret_cast<V *>(smem_raw);
    V *buf1 = buf0 + (size_t)W * n;
    const V *roots = a.tw;  // hi[n], lo[n]
    const int red = a.red;
    const T kmult = a.kmult;

    asm volatile("griddepcontrol.wait;" ::: "memory");
    const bool scaled = a.scale != nullptr;
    const T scale = scaled ? load_scale<T>(a.scale) : (T)1;
    T acc_mass = 0, acc_pot = 0, acc_int = 0, acc_kin = 0, acc_rot = 0;
    double tot[RQ_COUNT] = {0.0, 0.0, 0.0, 0.0, 0.0};

    const int ntiles = (a.nlines + W - 1) / W;
    const int cells = W * n;
    auto gbase = [&](int g) -> int64_t { return (int64_t)(g % a.m0) * a.s0 + (int64_t)(g / a.m0) * a.s1; };
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        // ---- load the tile: element (w, pos) at pos * W + w
        for (int t = threadIdx.x; t < cells; t += GEN_THREADS) {
            int w, pos;
            if (a.stride == 1) { w = t / n; pos = t % n; }  // x lines: walk along the line
            else { w = t % W; pos = t / W; }                 // y/z: adjacent columns
            const int g = tile * W + w;
            V x = mk<V>((T)0, (T)0);
            if (g < a.nlines) {
                const int64_t e = gbase(g) + (int64_t)pos * a.stride;
                x = a.in[e];
                if constexpr (MODE == MODE_DIAG) {
                    if (red & RED_POINT) {
                        const T rho = x.x * x.x + x.y * x.y;
                        acc_mass += rho;
                        acc_int += rho * rho;
                        if (a.V) acc_pot += a.V[e] * rho;
                    }
                }
            }
            buf0[pos * W + w] = x;
        }
        __syncthreads();
        V *spec = buf0;
        if constexpr (MODE != MODE_INV) spec = gen_fft<-1>(buf0, buf1, p, roots);  // X[k] at k * W + w
        // ---- spectral work: sums, phase / mask, scale
        if constexpr (MODE == MODE_FWD) {
            for (int t = threadIdx.x; t < cells; t += GEN_THREADS) {
                const int w = t % W, k = t / W, g = tile * W + w;
                if (g < a.nlines) a.out[gbase(g) + (int64_t)k * a.stride] = spec[k * W + w];
            }
            __syncthreads();
        }
        if constexpr (MODE == MODE_FUSED || MODE == MODE_DIAG) {
            for (int t = threadIdx.x; t < cells; t += GEN_THREADS) {
                const int w = t % W, k = t / W, g = tile * W + w;
                if (g >= a.nlines) continue;
                const int row = g % a.rowmod;
                V X = spec[k * W + w];
                if (red & RED_KIN) {
                    const int kk = k < (n + 1) / 2 ? k : k - n;
                    const T xi = (T)kk * kmult;
                    const T m2 = X.x * X.x + X.y * X.y;
                    acc_kin += xi * xi * m2 * (T)(1.0 / n);
                    if (a.coord) acc_rot += xi * m2 * (T)(1.0 / n) * (T)a.coord[row];
                }
                if constexpr (MODE == MODE_FUSED) {
                    if (a.mask_lim) {
                        const int kk = k < (n + 1) / 2 ? k : n - k;
                        X = kk <= a.mask_lim[g] ? cscale(X, a.inv_n) : mk<V>((T)0, (T)0);
                    } else {
                        const V *ph = a.phase + (a.prow ? (int64_t)row * a.prow : 0);
                        X = cmul2(X, ph[k], ph[n + k]);
                        if (scaled) X = cscale(X, scale);
                    }
                    spec[k * W + w] = X;
                }
            }
            __syncthreads();
        }
        if constexpr (MODE == MODE_FUSED || MODE == MODE_INV) {
            V *other = spec == buf0 ? buf1 : buf0;
            V *res = gen_fft<+1>(spec, other, p, roots);
            // ---- epilogue: positions in natural order
            for (int t = threadIdx.x; t < cells; t += GEN_THREADS) {
                int w, pos;
                if (a.stride == 1) { w = t / n; pos = t % n; }
                else { w = t % W; pos = t / W; }
                const int g = tile * W + w;
                if (g >= a.nlines) continue;
                const int64_t e = gbase(g) + (int64_t)pos * a.stride;
                V v = res[pos * W + w];
                if constexpr (MODE == MODE_INV) {
                    v = cscale(v, a.inv_n);
                } else {
                    if (a.nl_mode != NL_NONE) {
                        const NLConst<T> nlc = nl_const<T>(a.nl_split, a.nl_beta, a.nl_dt);
                        const T vv = a.V ? a.V[e] : (T)0;
                        if constexpr (sizeof(T) == 4) {
                            v = a.nl_mode == NL_IMAG ? nl_apply(v, vv, nlc, true) : nl_apply_real_cell(v, vv, nlc);
                        } else {
                            v = nl_apply(v, vv, nlc, a.nl_mode == NL_IMAG);
                        }
                    }
                    if (red & RED_POINT) {
                        const T rho = v.x * v.x + v.y * v.y;
                        acc_mass += rho;
                        acc_int += rho * rho;
                        if (a.V) acc_pot += a.V[e] * rho;
                    } else if (red & RED_MASS) {
                        acc_mass += v.x * v.x + v.y * v.y;
                    }
                    if (a.acc) v = cadd(a.acc[e], v);
                }
                a.out[e] = v;
            }
            __syncthreads();  // the next tile's load reuses the buffers
        }
        if (red) {
            tot[RQ_MASS] += (double)acc_mass;
            tot[RQ_POT] += (double)acc_pot;
            tot[RQ_INT] += (double)acc_int;
            tot[RQ_KIN] += (double)acc_kin;
            tot[RQ_ROT] += (double)acc_rot;
            acc_mass = acc_pot = acc_int = acc_kin = acc_rot = (T)0;
        }
    }
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if constexpr (MODE == MODE_FUSED || MODE == MODE_DIAG) {
        if (red) {
            unsigned qmask = 0;
            if (red & (RED_POINT | RED_MASS)) qmask |= 1u << RQ_MASS;
            if (red & RED_POINT) qmask |= (1u << RQ_POT) | (1u << RQ_INT);
            if (red & RED_KIN) qmask |= (1u << RQ_KIN) | (1u << RQ_ROT);
            block_sums_store<GEN_THREADS>(tot, qmask, a.partials);
            finish_reduction<T, GEN_THREADS>(a, qmask);
        }
    }
}

}  // namespace gpss
