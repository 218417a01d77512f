/*
 * gp_oracle.c -- CPU restatement of SuperfluidDynamics.jl's split-step
 * Gross-Pitaevskii path: the oracle the CUDA library is tested against.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py load this file's library.  The
 * product path (libgpss.so) never links, loads or calls it.
 *
 * What it restates (file:line in the reference project):
 *   grid nodes      src/Discretization/Grids.jl:78-84   x = LinRange(lo,hi,n+1)[1:end-1]
 *   wavenumbers     src/Discretization/Plans.jl:829-830, 967-969   fftfreq(n, 2pi/dx)
 *   Strang step     src/NumModels/GrossPitaevskii/splitting.jl:149-154
 *   Lie step        src/NumModels/GrossPitaevskii/splitting.jl:78-82
 *   kinetic flow    src/NumModels/GrossPitaevskii/splitting.jl:156-203
 *   nonlinear flow  src/NumModels/GrossPitaevskii/splitting.jl:205-209
 *   FFT / iFFT      src/Discretization/Plans.jl:1132-1250 (forward unnormalised,
 *                   inverse = backward transform then *1/n, as AbstractFFTs' ldiv!)
 *   norm            src/Discretization/Fields.jl:172-180
 *   energy          src/NumModels/GrossPitaevskii/GrossPitaevskii.jl:61-136 with
 *                   computeDerivatives!(GradientRotField) src/NumModels/derivatives.jl:27-56, 90-126
 *   explicit RK     src/NumModels/GrossPitaevskii/explicit-rk.jl:96-166 (NumModelGPRK:
 *                   RK1/RK2/RK4, 2/3-rule filter on the nonlinear term or the state),
 *                   lapRot GrossPitaevskii.jl:12-45, xi_max Plans.jl:529-532,
 *                   _dealias_scalar! NavierStokes/NSGP.jl:354-361
 *   implicit        src/NumModels/GrossPitaevskii/backward-euler.jl, crank-nicolson.jl
 *                   (six schemes) with BiCGStab src/NumModels/krylov.jl:1-67
 *   imaginary time  extension (no split-step counterpart in the reference): the
 *                   same stages with t -> -i tau and a unit-mass renormalisation
 *                   (normalize!, Fields.jl:196-200) after every step.
 *
 * The FFT here is this file's own iterative radix-2 transform (FFTW, which the
 * reference calls, is not available); results therefore agree with the
 * reference at the round-off level, and parity is pinned by the reference's
 * analytic known-answer tests (test/runtests.jl:29-90, 644-671, 718-725).
 *
 * Precision: the default build computes in FP64 (the reference's Float64).
 * Built with -DOR_EXTENDED the same code computes in long double (80-bit on
 * x86, 128-bit on Arm) and exports the entry points with an `_ext` suffix:
 * a near-exact reference for measuring the round-off of FP64 implementations.
 * Inputs, grid values and outputs stay doubles at the API either way.
 *
 * Layout: column-major, x fastest (Julia Array order), complex interleaved
 * (re, im) doubles, exactly the memory of a Julia Array{ComplexF64}.
 *
 * Compiled with -ffp-contract=off so x86 and Arm hosts round identically.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_TWO_PI 6.283185307179586 /* Float64(2pi), as Julia's 2pi literal */

#ifdef OR_EXTENDED
typedef long double real;
#define RCOS cosl
#define RSIN sinl
#define REXP expl
#define RSQRT sqrtl
#define RHALFPI 1.570796326794896619231321691639751442L
#define OR_SYM(name) name##_ext
#else
typedef double real;
#define RCOS cos
#define RSIN sin
#define REXP exp
#define RSQRT sqrt
#define RHALFPI 1.5707963267948966
#define OR_SYM(name) name
#endif

typedef struct { real re, im; } ocplx;

/* ---------------------------------------------------------------- grid --- */

/* Julia Base.lerpi: t = j/d; (1-t)*a + t*b  (base/range.jl), in Float64 */
static double lerpi(int64_t j, int64_t d, double a, double b)
{
    double t = (double)j / (double)d;
    return (1.0 - t) * a + t * b;
}

/* Grids.jl:78-84: x = LinRange(lo, hi, n+1)[1:end-1].  Indexing a LinRange
 * with a range builds LinRange(x[1], x[n], n), whose entries are lerps between
 * those two end points. */
static void grid_coords(int64_t n, double lo, double hi, double *x)
{
    if (n <= 1) { x[0] = lo; return; }
    double first = lerpi(0, n, lo, hi);
    double last = lerpi(n - 1, n, lo, hi);
    for (int64_t i = 0; i < n; i++) x[i] = lerpi(i, n - 1, first, last);
}

/* Plans.jl:829-830: xi = fftfreq(n, 2pi/dx) (AbstractFFTs.Frequencies:
 * entry i is (i-1 - (i <= (n+1)>>1 ? 0 : n)) * (fs/n)), in Float64. */
static void fftfreq(int64_t n, double dx, double *xi)
{
    double fs = OR_TWO_PI / dx;
    double mult = fs / (double)n;
    int64_t nneg = (n + 1) >> 1;
    for (int64_t i = 0; i < n; i++) {
        int64_t k = (i < nneg) ? i : i - n;
        xi[i] = (double)k * mult;
    }
}

void OR_SYM(or_grid_coords)(int64_t n, double lo, double hi, double *x) { grid_coords(n, lo, hi, x); }
void OR_SYM(or_fftfreq)(int64_t n, double dx, double *xi) { fftfreq(n, dx, xi); }

/* ----------------------------------------------------------------- FFT --- */

/* (cos, sin) of 2 pi k / n, reduced to the first octant for accuracy and
 * exact symmetries. */
static void unit_root(int64_t k, int64_t n, real *c, real *s)
{
    k %= n; if (k < 0) k += n;
    int64_t q = (4 * k) / n;          /* quadrant 0..3 */
    int64_t r4 = 4 * k - q * n;       /* remainder, [0, n) in units of a quarter turn / n */
    real cc, ss;
    if (2 * r4 <= n) {
        real a = RHALFPI * (real)r4 / (real)n;
        cc = RCOS(a); ss = RSIN(a);
    } else {
        real a = RHALFPI * (real)(n - r4) / (real)n;
        cc = RSIN(a); ss = RCOS(a);
    }
    switch (q) {
    case 0: *c = cc;  *s = ss;  break;
    case 1: *c = -ss; *s = cc;  break;
    case 2: *c = -cc; *s = -ss; break;
    default:*c = ss;  *s = -cc; break;
    }
}

typedef struct {
    int64_t n;
    int pow2;
    ocplx *tw;       /* exp(-2 pi i k / n), k < n */
} fftplan;

static int is_pow2(int64_t n) { return n > 0 && (n & (n - 1)) == 0; }

static int plan_make(fftplan *p, int64_t n)
{
    p->n = n;
    p->pow2 = is_pow2(n);
    p->tw = (ocplx *)malloc(sizeof(ocplx) * (size_t)(n > 0 ? n : 1));
    if (!p->tw) return -1;
    for (int64_t k = 0; k < n; k++) {
        real c, s;
        unit_root(k, n, &c, &s);
        p->tw[k].re = c;
        p->tw[k].im = -s;
    }
    return 0;
}

static void plan_free(fftplan *p) { free(p->tw); p->tw = NULL; }

/* Unnormalised DFT of one contiguous line.  sign = -1 forward (FFTW_FORWARD,
 * exp(-2 pi i jk/n)), +1 backward.  tmp holds n entries of scratch. */
static void fft_line(const fftplan *p, ocplx *a, ocplx *tmp, int sign)
{
    int64_t n = p->n;
    if (n == 1) return;
    if (!p->pow2) { /* direct O(n^2) DFT for sizes that are not powers of two */
        for (int64_t k = 0; k < n; k++) {
            real sr = 0, si = 0;
            for (int64_t j = 0; j < n; j++) {
                int64_t m = (j * k) % n;
                real wr = p->tw[m].re, wi = sign < 0 ? p->tw[m].im : -p->tw[m].im;
                sr += a[j].re * wr - a[j].im * wi;
                si += a[j].re * wi + a[j].im * wr;
            }
            tmp[k].re = sr; tmp[k].im = si;
        }
        memcpy(a, tmp, sizeof(ocplx) * (size_t)n);
        return;
    }
    /* bit reversal permutation */
    int64_t j = 0;
    for (int64_t i = 0; i < n - 1; i++) {
        if (i < j) { ocplx t = a[i]; a[i] = a[j]; a[j] = t; }
        int64_t m = n >> 1;
        while (m >= 1 && j >= m) { j -= m; m >>= 1; }
        j += m;
    }
    /* iterative radix-2 decimation in time */
    for (int64_t len = 2; len <= n; len <<= 1) {
        int64_t half = len >> 1, step = n / len;
        for (int64_t i = 0; i < n; i += len) {
            for (int64_t k = 0; k < half; k++) {
                real wr = p->tw[k * step].re;
                real wi = sign < 0 ? p->tw[k * step].im : -p->tw[k * step].im;
                ocplx u = a[i + k], v = a[i + k + half];
                real tr = v.re * wr - v.im * wi;
                real ti = v.re * wi + v.im * wr;
                a[i + k].re = u.re + tr; a[i + k].im = u.im + ti;
                a[i + k + half].re = u.re - tr; a[i + k + half].im = u.im - ti;
            }
        }
    }
    (void)tmp;
}

/* ---------------------------------------------------------- geometry ----- */

typedef struct {
    int ndim;
    int64_t n[3];
    double lo[3], hi[3], L[3], d[3];   /* Float64 grid description */
    int64_t total;
    double *coord[3];                  /* node positions (Float64) */
    double *xi[3];                     /* wavenumbers (Float64) */
    fftplan plan[3];
} ogrid;

static void grid_free(ogrid *g)
{
    for (int a = 0; a < 3; a++) {
        free(g->coord[a]); free(g->xi[a]);
        if (a < g->ndim) plan_free(&g->plan[a]);
        g->coord[a] = g->xi[a] = NULL;
    }
}

static int grid_make(ogrid *g, int ndim, const int64_t *n, const double *lo, const double *hi)
{
    memset(g, 0, sizeof(*g));
    if (ndim < 1 || ndim > 3) return -1;
    g->ndim = ndim;
    g->total = 1;
    for (int a = 0; a < 3; a++) {
        g->n[a] = a < ndim ? n[a] : 1;
        if (g->n[a] <= 0) return -1;
        g->lo[a] = a < ndim ? lo[a] : 0.0;
        g->hi[a] = a < ndim ? hi[a] : 1.0;
        g->L[a] = g->hi[a] - g->lo[a];
        g->d[a] = g->L[a] / (double)g->n[a];          /* Grids.jl:80 */
        g->total *= g->n[a];
        g->coord[a] = (double *)malloc(sizeof(double) * (size_t)g->n[a]);
        g->xi[a] = (double *)malloc(sizeof(double) * (size_t)g->n[a]);
        if (!g->coord[a] || !g->xi[a]) { grid_free(g); return -1; }
        grid_coords(g->n[a], g->lo[a], g->hi[a], g->coord[a]);
        fftfreq(g->n[a], g->d[a], g->xi[a]);
        if (a < ndim && plan_make(&g->plan[a], g->n[a])) { grid_free(g); return -1; }
    }
    return 0;
}

static real cell_volume(const ogrid *g)
{
    real v = 1;
    for (int a = 0; a < g->ndim; a++) v *= (real)g->d[a];
    return v;
}

/* x * dx * dy [* dz], left to right as Julia evaluates `s * Δx * Δy * Δz` */
static real times_cell(const ogrid *g, real x)
{
    for (int a = 0; a < g->ndim; a++) x *= (real)g->d[a];
    return x;
}

/* Julia's sum is pairwise; so is this one (block of 1024 leaves). */
static real pairwise_sum(const real *v, int64_t n)
{
    if (n <= 1024) {
        real s = 0;
        for (int64_t i = 0; i < n; i++) s += v[i];
        return s;
    }
    int64_t h = n / 2;
    return pairwise_sum(v, h) + pairwise_sum(v + h, n - h);
}

/* double (re, im) pairs <-> internal complex */
static ocplx *load_field(const double *psi, int64_t N)
{
    ocplx *p = (ocplx *)malloc(sizeof(ocplx) * (size_t)N);
    if (!p) return NULL;
    for (int64_t i = 0; i < N; i++) { p[i].re = (real)psi[2 * i]; p[i].im = (real)psi[2 * i + 1]; }
    return p;
}

static void store_field(const ocplx *p, double *psi, int64_t N)
{
    for (int64_t i = 0; i < N; i++) { psi[2 * i] = (double)p[i].re; psi[2 * i + 1] = (double)p[i].im; }
}

static real *load_real(const double *v, int64_t N)
{
    if (!v) return NULL;
    real *r = (real *)malloc(sizeof(real) * (size_t)N);
    if (!r) return NULL;
    for (int64_t i = 0; i < N; i++) r[i] = (real)v[i];
    return r;
}

/* --------------------------------------------------- directional passes -- */

static int64_t line_base(const ogrid *g, int axis, int64_t l)
{
    int64_t nx = g->n[0], ny = g->n[1];
    if (axis == 0) return l * nx;
    if (axis == 1) return (l % nx) + (l / nx) * nx * ny;
    return l;
}

static int64_t line_stride(const ogrid *g, int axis)
{
    return axis == 0 ? 1 : (axis == 1 ? g->n[0] : g->n[0] * g->n[1]);
}

/* coordinate of line l that enters the rotation term of `axis`:
 * the y node for x lines, the x node for y lines */
static real line_coord(const ogrid *g, int axis, int64_t l)
{
    if (axis == 0 && g->ndim >= 2) return (real)g->coord[1][l % g->n[1]];
    if (axis == 1) return (real)g->coord[0][l % g->n[0]];
    return 0;
}

/* For each line along `axis`: FFT, multiply, iFFT (splitting.jl:164-201):
 *   real time   exp(i (cD xi^2 - Om y xi) dtl)   (x)
 *               exp(i (cD xi^2 + Om x xi) dtl)   (y)
 *               exp(i  cD xi^2 dtl)              (z)
 *   imag time   the same with t -> -i tau: exp((cD xi^2 -/+ Om c xi) dtl).
 */
static void kinetic_axis(const ogrid *g, ocplx *psi, int axis, real cD, real Om, real dtl, int imag)
{
    int64_t n = g->n[axis];
    int64_t stride = line_stride(g, axis);
    int64_t nlines = g->total / n;
    const double *xi = g->xi[axis];
    real inv_n = (real)1 / (real)n;
#pragma omp parallel
    {
        ocplx *line = (ocplx *)malloc(sizeof(ocplx) * (size_t)n);
        ocplx *tmp = (ocplx *)malloc(sizeof(ocplx) * (size_t)n);
#pragma omp for schedule(static)
        for (int64_t l = 0; l < nlines; l++) {
            int64_t base = line_base(g, axis, l);
            real c = line_coord(g, axis, l);
            for (int64_t p = 0; p < n; p++) line[p] = psi[base + p * stride];
            fft_line(&g->plan[axis], line, tmp, -1);
            for (int64_t k = 0; k < n; k++) {
                real xk = (real)xi[k], ph;
                /* Julia: coeffD * xi^2 -/+ Om * c * xi  (xi^2 == xi*xi) */
                if (axis == 0) ph = cD * (xk * xk) - Om * c * xk;
                else if (axis == 1) ph = cD * (xk * xk) + Om * c * xk;
                else ph = cD * (xk * xk);
                real fr, fi;
                if (!imag) { real t = ph * dtl; fr = RCOS(t); fi = RSIN(t); }
                else { fr = REXP(ph * dtl); fi = 0; }
                real ar = line[k].re, ai = line[k].im;
                line[k].re = fr * ar - fi * ai;
                line[k].im = fr * ai + fi * ar;
            }
            fft_line(&g->plan[axis], line, tmp, +1);
            for (int64_t p = 0; p < n; p++) {
                psi[base + p * stride].re = line[p].re * inv_n;
                psi[base + p * stride].im = line[p].im * inv_n;
            }
        }
        free(line); free(tmp);
    }
}

/* splitting.jl:156-203 solveLapRot!: x, then y, then z. */
static void solve_lap_rot(const ogrid *g, ocplx *psi, real cD, real Om, real dtl, int imag)
{
    for (int a = 0; a < g->ndim; a++) kinetic_axis(g, psi, a, cD, Om, dtl, imag);
}

/* splitting.jl:205-209 solveNL!: psi <- exp(-i (V + beta |psi|^2) dtl) psi;
 * imaginary time: psi <- exp(-(V + beta |psi|^2) dtl) psi. */
static void solve_nl(const ogrid *g, ocplx *psi, const real *V, real beta, real dtl, int imag)
{
    int64_t N = g->total;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) {
        real ar = psi[i].re, ai = psi[i].im;
        real rho = ar * ar + ai * ai;                   /* abs2 */
        real r = (V ? V[i] : 0) + beta * rho;
        real fr, fi;
        if (!imag) { real t = -r * dtl; fr = RCOS(t); fi = RSIN(t); }
        else { fr = REXP(-r * dtl); fi = 0; }
        psi[i].re = fr * ar - fi * ai;
        psi[i].im = fr * ai + fi * ar;
    }
}

static real sum_abs2(const ogrid *g, const ocplx *psi)
{
    int64_t N = g->total;
    real *tmp = (real *)malloc(sizeof(real) * (size_t)N);
    if (!tmp) return NAN;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) tmp[i] = psi[i].re * psi[i].re + psi[i].im * psi[i].im;
    real s = pairwise_sum(tmp, N);
    free(tmp);
    return s;
}

/* Fields.jl:172-180 */
static real field_norm(const ogrid *g, const ocplx *psi)
{
    return RSQRT(sum_abs2(g, psi)) * RSQRT(cell_volume(g));
}

/* ------------------------------------------------------------ public API -- */

double OR_SYM(or_norm)(int ndim, const int64_t *n, const double *lo, const double *hi, const double *psi)
{
    ogrid g;
    if (grid_make(&g, ndim, n, lo, hi)) return NAN;
    ocplx *p = load_field(psi, g.total);
    double r = p ? (double)field_norm(&g, p) : NAN;
    free(p);
    grid_free(&g);
    return r;
}

/* Batched 1D FFT along one axis (unnormalised forward, or backward*1/n when
 * inverse != 0) -- Plans.jl mul_x!/ldiv_x! etc. without the pencil moves. */
int OR_SYM(or_fft_axis)(int ndim, const int64_t *n, double *psi, int axis, int inverse)
{
    ogrid g;
    const double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    if (grid_make(&g, ndim, n, lo, hi)) return -1;
    if (axis < 0 || axis >= ndim) { grid_free(&g); return -1; }
    int64_t len = g.n[axis], stride = line_stride(&g, axis), nlines = g.total / len;
    ocplx *p = load_field(psi, g.total);
    ocplx *line = (ocplx *)malloc(sizeof(ocplx) * (size_t)len);
    ocplx *tmp = (ocplx *)malloc(sizeof(ocplx) * (size_t)len);
    int rc = (p && line && tmp) ? 0 : -1;
    for (int64_t l = 0; rc == 0 && l < nlines; l++) {
        int64_t base = line_base(&g, axis, l);
        for (int64_t q = 0; q < len; q++) line[q] = p[base + q * stride];
        fft_line(&g.plan[axis], line, tmp, inverse ? +1 : -1);
        real s = inverse ? (real)1 / (real)len : (real)1;
        for (int64_t q = 0; q < len; q++) {
            p[base + q * stride].re = line[q].re * s;
            p[base + q * stride].im = line[q].im * s;
        }
    }
    if (rc == 0) store_field(p, psi, g.total);
    free(p); free(line); free(tmp);
    grid_free(&g);
    return rc;
}

/*
 * nsteps split steps.  scheme 2 = Strang (NumModelSplit2.timeStep!,
 * splitting.jl:149-154), scheme 1 = Lie (NumModelSplit1.timeStep!, :78-82).
 * imag != 0: imaginary time with unit-mass renormalisation after each step.
 * V may be NULL (PotentialZero).  nthreads <= 0 keeps the OpenMP default.
 */
static int step_impl(int ndim, const int64_t *n, const double *lo, const double *hi,
                     double cD, double beta, double Om, const double *V, double *psi,
                     int nsteps, int scheme, int imag, double dt, int nthreads, double *loop_seconds)
{
    ogrid g;
    if (scheme != 1 && scheme != 2) return -1;
    if (grid_make(&g, ndim, n, lo, hi)) return -1;
    ocplx *p = load_field(psi, g.total);
    real *Vr = load_real(V, g.total);
    if (!p || (V && !Vr)) { free(p); free(Vr); grid_free(&g); return -1; }
#ifdef _OPENMP
    int saved = omp_get_max_threads();
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    /* Julia: n.Δt * 0.5 is a Float64 product, then used as the step */
    const real rdt = (real)dt, half = (real)(dt * 0.5);
#ifdef _OPENMP
    const double t0 = omp_get_wtime();
#endif
    for (int s = 0; s < nsteps; s++) {
        if (scheme == 2) {
            solve_lap_rot(&g, p, (real)cD, (real)Om, half, imag);
            solve_nl(&g, p, Vr, (real)beta, rdt, imag);
            solve_lap_rot(&g, p, (real)cD, (real)Om, half, imag);
        } else {
            solve_lap_rot(&g, p, (real)cD, (real)Om, rdt, imag);
            solve_nl(&g, p, Vr, (real)beta, rdt, imag);
        }
        if (imag) {                       /* normalize!, Fields.jl:196-200 */
            real nrm = field_norm(&g, p);
            int64_t N = g.total;
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < N; i++) { p[i].re /= nrm; p[i].im /= nrm; }
        }
    }
#ifdef _OPENMP
    if (loop_seconds) *loop_seconds = omp_get_wtime() - t0;
    omp_set_num_threads(saved);
#else
    if (loop_seconds) *loop_seconds = -1.0;
#endif
    store_field(p, psi, g.total);
    free(p); free(Vr);
    grid_free(&g);
    return 0;
}

int OR_SYM(or_step)(int ndim, const int64_t *n, const double *lo, const double *hi,
                    double cD, double beta, double Om, const double *V, double *psi,
                    int nsteps, int scheme, int imag, double dt, int nthreads)
{
    return step_impl(ndim, n, lo, hi, cD, beta, Om, V, psi, nsteps, scheme, imag, dt, nthreads, NULL);
}

/* or_step that also reports the wall time of the time-step loop alone (grid,
 * plans and field conversion excluded), the part the reference's own
 * benchmark times (benchmarks/scalability_gp.jl:40-51 times timeStep! only). */
int OR_SYM(or_step_timed)(int ndim, const int64_t *n, const double *lo, const double *hi,
                          double cD, double beta, double Om, const double *V, double *psi,
                          int nsteps, int scheme, int imag, double dt, int nthreads, double *loop_seconds)
{
    return step_impl(ndim, n, lo, hi, cD, beta, Om, V, psi, nsteps, scheme, imag, dt, nthreads, loop_seconds);
}

/*
 * Spectral derivatives of GradientRotField (derivatives.jl:27-56 for 2D,
 * 90-126 for 3D): d[axis] = iFFT(i xi FFT psi), dd = iFFT(-xi^2 FFT psi),
 * rx = iFFT_x(i y xi_x FFT_x psi), ry = iFFT_y(-i x xi_y FFT_y psi).
 * Inputs/outputs are internal-precision fields; NULL outputs are skipped.
 */
static void derivatives(const ogrid *g, const ocplx *p, ocplx **d1, ocplx **d2, ocplx **rr)
{
    for (int a = 0; a < g->ndim; a++) {
        int64_t len = g->n[a], stride = line_stride(g, a), nlines = g->total / len;
        real inv_n = (real)1 / (real)len;
#pragma omp parallel
        {
            ocplx *hat = (ocplx *)malloc(sizeof(ocplx) * (size_t)len);
            ocplx *line = (ocplx *)malloc(sizeof(ocplx) * (size_t)len);
            ocplx *tmp = (ocplx *)malloc(sizeof(ocplx) * (size_t)len);
#pragma omp for schedule(static)
            for (int64_t l = 0; l < nlines; l++) {
                int64_t base = line_base(g, a, l);
                real c = line_coord(g, a, l);
                for (int64_t q = 0; q < len; q++) hat[q] = p[base + q * stride];
                fft_line(&g->plan[a], hat, tmp, -1);
                for (int kind = 0; kind < 3; kind++) {
                    ocplx *o = kind == 0 ? d1[a] : (kind == 1 ? d2[a] : rr[a]);
                    if (!o) continue;
                    for (int64_t k = 0; k < len; k++) {
                        real xi = (real)g->xi[a][k], hr = hat[k].re, hi_ = hat[k].im;
                        if (kind == 0) {        /* i xi hat */
                            line[k].re = -xi * hi_; line[k].im = xi * hr;
                        } else if (kind == 1) { /* -xi^2 hat */
                            line[k].re = -(xi * xi) * hr; line[k].im = -(xi * xi) * hi_;
                        } else if (a == 0) {    /* i y xi hat */
                            line[k].re = -(c * xi) * hi_; line[k].im = (c * xi) * hr;
                        } else {                /* -i x xi hat */
                            line[k].re = (c * xi) * hi_; line[k].im = -(c * xi) * hr;
                        }
                    }
                    fft_line(&g->plan[a], line, tmp, +1);
                    for (int64_t q = 0; q < len; q++) {
                        o[base + q * stride].re = line[q].re * inv_n;
                        o[base + q * stride].im = line[q].im * inv_n;
                    }
                }
            }
            free(hat); free(line); free(tmp);
        }
    }
}

int OR_SYM(or_derivatives)(int ndim, const int64_t *n, const double *lo, const double *hi,
                           const double *psi, double *dx, double *dy, double *dz,
                           double *ddx, double *ddy, double *ddz, double *rx, double *ry)
{
    ogrid g;
    if (grid_make(&g, ndim, n, lo, hi)) return -1;
    double *outs[8] = {dx, dy, dz, ddx, ddy, ddz, rx, ry};
    ocplx *in[8] = {0};
    ocplx *p = load_field(psi, g.total);
    int rc = p ? 0 : -1;
    for (int i = 0; i < 8 && rc == 0; i++) {
        if (!outs[i]) continue;
        in[i] = (ocplx *)calloc((size_t)g.total, sizeof(ocplx));
        if (!in[i]) rc = -1;
    }
    if (rc == 0) {
        ocplx *d1[3] = {in[0], in[1], in[2]}, *d2[3] = {in[3], in[4], in[5]}, *rr[3] = {in[6], in[7], NULL};
        derivatives(&g, p, d1, d2, rr);
        for (int i = 0; i < 8; i++)
            if (outs[i]) store_field(in[i], outs[i], g.total);
    }
    for (int i = 0; i < 8; i++) free(in[i]);
    free(p);
    grid_free(&g);
    return rc;
}

/*
 * energy(n) of GrossPitaevskii.jl:61-92 (2D) / 106-136 (3D):
 *   out[0] = E_Omega = sum Re(i conj(psi) Om (rx + ry)) dV
 *   out[1] = E_Delta = (-cD (sum|dx|^2 + sum|dy|^2 [+ sum|dz|^2]) + sum V|psi|^2) dV
 *   out[2] = E_beta  = sum 0.5 beta |psi|^4 dV
 *   out[3] = E       = -E_Omega + E_Delta + E_beta
 *   out[4] = mu      = -E_Omega + E_Delta + 2 E_beta  (GrossPitaevskii.jl:79;
 *                      the 3D method computes no mu, the same formula is used)
 */
int OR_SYM(or_energy)(int ndim, const int64_t *n, const double *lo, const double *hi,
                      double cD, double beta, double Om, const double *V, const double *psi,
                      double *out)
{
    ogrid g;
    if (grid_make(&g, ndim, n, lo, hi)) return -1;
    int64_t N = g.total;
    ocplx *d[3] = {NULL, NULL, NULL}, *rx = NULL, *ry = NULL;
    real *tmp = NULL, *Vr = NULL;
    ocplx *p = load_field(psi, N);
    int rc = -1;
    if (!p) goto done;
    for (int a = 0; a < ndim; a++) {
        d[a] = (ocplx *)calloc((size_t)N, sizeof(ocplx));
        if (!d[a]) goto done;
    }
    rx = (ocplx *)calloc((size_t)N, sizeof(ocplx));
    ry = (ocplx *)calloc((size_t)N, sizeof(ocplx));
    tmp = (real *)malloc(sizeof(real) * (size_t)N);
    Vr = load_real(V, N);
    if (!rx || !ry || !tmp || (V && !Vr)) goto done;
    {
        ocplx *d2[3] = {NULL, NULL, NULL}, *rr[3] = {rx, ndim > 1 ? ry : NULL, NULL};
        derivatives(&g, p, d, d2, rr);
    }
    real grad = 0;
    for (int a = 0; a < ndim; a++) {
        for (int64_t i = 0; i < N; i++) tmp[i] = d[a][i].re * d[a][i].re + d[a][i].im * d[a][i].im;
        grad += pairwise_sum(tmp, N);
    }
    for (int64_t i = 0; i < N; i++) {
        /* real(im * conj(psi) * (Om * (rx + ry))) */
        real sr = (real)Om * (rx[i].re + ry[i].re), si = (real)Om * (rx[i].im + ry[i].im);
        real cr = p[i].re, ci = -p[i].im;                  /* conj(psi) */
        real pi_ = cr * si + ci * sr;
        tmp[i] = -pi_;                                       /* real(i * z) = -imag(z) */
    }
    real eom = times_cell(&g, pairwise_sum(tmp, N));
    for (int64_t i = 0; i < N; i++) {
        real r = p[i].re * p[i].re + p[i].im * p[i].im;
        tmp[i] = (Vr ? Vr[i] : 0) * r;
    }
    real epot = pairwise_sum(tmp, N);
    real edel = times_cell(&g, -(real)cD * grad + epot);
    for (int64_t i = 0; i < N; i++) {
        real r = p[i].re * p[i].re + p[i].im * p[i].im;
        tmp[i] = ((real)0.5 * (real)beta) * (r * r);
    }
    real ebeta = times_cell(&g, pairwise_sum(tmp, N));
    out[0] = (double)eom;
    out[1] = (double)edel;
    out[2] = (double)ebeta;
    out[3] = (double)(-eom + edel + ebeta);
    out[4] = (double)(-eom + edel + ebeta * 2);
    rc = 0;
done:
    for (int a = 0; a < 3; a++) free(d[a]);
    free(rx); free(ry); free(tmp); free(Vr); free(p);
    grid_free(&g);
    return rc;
}

/* ------------------------------------------------ explicit Runge-Kutta -- */

/* Full ND transform, mul_all!/ldiv_all! (Plans.jl:1177-1280): every axis of
 * every line in turn; the inverse scales once by 1/N at the end, as the
 * normalised plan_ifft (AbstractFFTs.ScaledPlan) does. */
static void fft_all(const ogrid *g, ocplx *p, int inverse)
{
    for (int a = 0; a < g->ndim; a++) {
        int64_t len = g->n[a], stride = line_stride(g, a), nlines = g->total / len;
#pragma omp parallel
        {
            ocplx *line = (ocplx *)malloc(sizeof(ocplx) * (size_t)len);
            ocplx *tmp = (ocplx *)malloc(sizeof(ocplx) * (size_t)len);
#pragma omp for schedule(static)
            for (int64_t l = 0; l < nlines; l++) {
                int64_t base = line_base(g, a, l);
                for (int64_t q = 0; q < len; q++) line[q] = p[base + q * stride];
                fft_line(&g->plan[a], line, tmp, inverse ? +1 : -1);
                for (int64_t q = 0; q < len; q++) p[base + q * stride] = line[q];
            }
            free(line); free(tmp);
        }
    }
    if (inverse) {
        real s = (real)1 / (real)g->total;
        int64_t N = g->total;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; i++) { p[i].re *= s; p[i].im *= s; }
    }
}

/* 2/3-rule bound (4/9) min_d max|xi_d|^2, Plans.jl:529-532 (Float64) */
static double xi_max_global(const ogrid *g)
{
    double m = 0;
    for (int a = 0; a < g->ndim; a++) {
        double ma = 0;
        for (int64_t k = 0; k < g->n[a]; k++) {
            double v = g->xi[a][k] * g->xi[a][k];
            if (v > ma) ma = v;
        }
        if (a == 0 || ma < m) m = ma;
    }
    return (4.0 / 9.0) * m;
}

/* _dealias_scalar! (NavierStokes/NSGP.jl:354-361): zero every mode with
 * xi_x^2 + xi_y^2 [+ xi_z^2] >= xi_max (the sum in Float64, left to right) */
static void dealias(const ogrid *g, ocplx *p, double xmax)
{
    int64_t nx = g->n[0], ny = g->n[1], N = g->total;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) {
        int64_t ix = i % nx, iy = (i / nx) % ny, iz = i / (nx * ny);
        double k2 = g->xi[0][ix] * g->xi[0][ix];
        if (g->ndim >= 2) k2 = k2 + g->xi[1][iy] * g->xi[1][iy];
        if (g->ndim >= 3) k2 = k2 + g->xi[2][iz] * g->xi[2][iz];
        if (!(k2 < xmax)) { p[i].re = 0; p[i].im = 0; }
    }
}

typedef struct {
    const ogrid *g;
    const real *V;
    real beta, cD, Om;
    int filter;          /* 0 none, 1 product, 2 solution */
    double xmax;
    ocplx *dd[3], *rr[2], *nl;   /* scratch */
} rk_ctx;

/* gp_rhs! (explicit-rk.jl:96-107):
 *   out = i (lapRot(psi) - N(psi)),  N = (V + beta|psi|^2) psi, 2/3-filtered
 *   when filter = product (_gp_nl!, :117-124);
 * lapRot (GrossPitaevskii.jl:12-45) = -cD (ddx + ddy [+ ddz]) + (Om i)(rx + ry). */
static void gp_rhs(rk_ctx *c, const ocplx *psi, ocplx *out)
{
    const ogrid *g = c->g;
    ocplx *d2[3] = {c->dd[0], g->ndim > 1 ? c->dd[1] : NULL, g->ndim > 2 ? c->dd[2] : NULL};
    ocplx *rr[3] = {c->rr[0], g->ndim > 1 ? c->rr[1] : NULL, NULL};
    ocplx *d1[3] = {NULL, NULL, NULL};
    derivatives(g, psi, d1, d2, rr);
    int64_t N = g->total;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) {
        real r2 = psi[i].re * psi[i].re + psi[i].im * psi[i].im;
        real f = (c->V ? c->V[i] : 0) + c->beta * r2;
        c->nl[i].re = f * psi[i].re;
        c->nl[i].im = f * psi[i].im;
    }
    if (c->filter == 1) {
        fft_all(g, c->nl, 0);
        dealias(g, c->nl, c->xmax);
        fft_all(g, c->nl, 1);
    }
    const real mcD = -c->cD;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) {
        ocplx lap = c->dd[0][i];
        if (g->ndim > 1) { lap.re = lap.re + c->dd[1][i].re; lap.im = lap.im + c->dd[1][i].im; }
        if (g->ndim > 2) { lap.re = lap.re + c->dd[2][i].re; lap.im = lap.im + c->dd[2][i].im; }
        ocplx rot = c->rr[0][i];
        if (g->ndim > 1) { rot.re = rot.re + c->rr[1][i].re; rot.im = rot.im + c->rr[1][i].im; }
        /* -cD * lap + (0 + Om i) * rot */
        real lr = mcD * lap.re - c->Om * rot.im;
        real li = mcD * lap.im + c->Om * rot.re;
        real dr = lr - c->nl[i].re, di = li - c->nl[i].im;
        out[i].re = -di;   /* i * (lin - nl) */
        out[i].im = dr;
    }
}

/*
 * nsteps explicit RK steps, timeStep!(::NumModelGPRK), explicit-rk.jl:135-166:
 * stepper 1 forward Euler, 2 explicit midpoint, 4 classical RK4; filter 0 none,
 * 1 the 2/3 rule on the nonlinear term of every stage, 2 on the state after
 * every step.  The scalar factors are formed as Julia evaluates them
 * (0.5 * dt first, dt / 6 first; k1 + 2k2 + 2k3 + k4 left to right).
 */
int OR_SYM(or_rk_step)(int ndim, const int64_t *n, const double *lo, const double *hi,
                       double cD, double beta, double Om, const double *V, double *psi,
                       int nsteps, int stepper, int filter, double dt, int nthreads)
{
    if (stepper != 1 && stepper != 2 && stepper != 4) return -1;
    if (filter < 0 || filter > 2) return -1;
    ogrid g;
    if (grid_make(&g, ndim, n, lo, hi)) return -1;
    int64_t N = g.total;
    rk_ctx c;
    memset(&c, 0, sizeof(c));
    c.g = &g; c.beta = (real)beta; c.cD = (real)cD; c.Om = (real)Om; c.filter = filter;
    c.xmax = xi_max_global(&g);
    ocplx *p = load_field(psi, N);
    real *Vr = load_real(V, N);
    c.V = Vr;
    ocplx *k[4] = {NULL, NULL, NULL, NULL}, *st = NULL;
    int rc = (p && (!V || Vr)) ? 0 : -1;
    for (int a = 0; a < 3 && rc == 0; a++)
        if (!(c.dd[a] = (ocplx *)calloc((size_t)N, sizeof(ocplx)))) rc = -1;
    for (int a = 0; a < 2 && rc == 0; a++)
        if (!(c.rr[a] = (ocplx *)calloc((size_t)N, sizeof(ocplx)))) rc = -1;
    if (rc == 0 && !(c.nl = (ocplx *)calloc((size_t)N, sizeof(ocplx)))) rc = -1;
    for (int a = 0; a < 4 && rc == 0; a++)
        if (!(k[a] = (ocplx *)calloc((size_t)N, sizeof(ocplx)))) rc = -1;
    if (rc == 0 && !(st = (ocplx *)calloc((size_t)N, sizeof(ocplx)))) rc = -1;
#ifdef _OPENMP
    int saved = omp_get_max_threads();
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    const real Dt = (real)dt, half = (real)(0.5 * dt), sixth = (real)(dt / 6);
    for (int s = 0; rc == 0 && s < nsteps; s++) {
        if (stepper == 1) {
            gp_rhs(&c, p, k[0]);
            for (int64_t i = 0; i < N; i++) { p[i].re = p[i].re + Dt * k[0][i].re; p[i].im = p[i].im + Dt * k[0][i].im; }
        } else if (stepper == 2) {
            gp_rhs(&c, p, k[0]);
            for (int64_t i = 0; i < N; i++) { st[i].re = p[i].re + half * k[0][i].re; st[i].im = p[i].im + half * k[0][i].im; }
            gp_rhs(&c, st, k[1]);
            for (int64_t i = 0; i < N; i++) { p[i].re = p[i].re + Dt * k[1][i].re; p[i].im = p[i].im + Dt * k[1][i].im; }
        } else {
            gp_rhs(&c, p, k[0]);
            for (int64_t i = 0; i < N; i++) { st[i].re = p[i].re + half * k[0][i].re; st[i].im = p[i].im + half * k[0][i].im; }
            gp_rhs(&c, st, k[1]);
            for (int64_t i = 0; i < N; i++) { st[i].re = p[i].re + half * k[1][i].re; st[i].im = p[i].im + half * k[1][i].im; }
            gp_rhs(&c, st, k[2]);
            for (int64_t i = 0; i < N; i++) { st[i].re = p[i].re + Dt * k[2][i].re; st[i].im = p[i].im + Dt * k[2][i].im; }
            gp_rhs(&c, st, k[3]);
            for (int64_t i = 0; i < N; i++) {
                real sr = k[0][i].re + 2 * k[1][i].re, si = k[0][i].im + 2 * k[1][i].im;
                sr = sr + 2 * k[2][i].re; si = si + 2 * k[2][i].im;
                sr = sr + k[3][i].re; si = si + k[3][i].im;
                p[i].re = p[i].re + sixth * sr;
                p[i].im = p[i].im + sixth * si;
            }
        }
        if (filter == 2) {
            fft_all(&g, p, 0);
            dealias(&g, p, c.xmax);
            fft_all(&g, p, 1);
        }
    }
#ifdef _OPENMP
    omp_set_num_threads(saved);
#endif
    if (rc == 0) store_field(p, psi, N);
    for (int a = 0; a < 3; a++) free(c.dd[a]);
    for (int a = 0; a < 2; a++) free(c.rr[a]);
    for (int a = 0; a < 4; a++) free(k[a]);
    free(c.nl); free(st); free(p); free(Vr);
    grid_free(&g);
    return rc;
}

/* -------------------------------------- implicit imaginary-time schemes -- */

/* lapRot(x) = -cD (ddx + ddy [+ ddz]) + (Om i)(rx + ry), GrossPitaevskii.jl:12-45 */
static void lap_rot(const ogrid *g, const ocplx *x, real cD, real Om, ocplx **dd, ocplx **rr, ocplx *out)
{
    ocplx *d2[3] = {dd[0], g->ndim > 1 ? dd[1] : NULL, g->ndim > 2 ? dd[2] : NULL};
    ocplx *r2[3] = {rr[0], g->ndim > 1 ? rr[1] : NULL, NULL};
    ocplx *d1[3] = {NULL, NULL, NULL};
    derivatives(g, x, d1, d2, r2);
    int64_t N = g->total;
    const real mcD = -cD;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) {
        ocplx lap = dd[0][i];
        if (g->ndim > 1) { lap.re = lap.re + dd[1][i].re; lap.im = lap.im + dd[1][i].im; }
        if (g->ndim > 2) { lap.re = lap.re + dd[2][i].re; lap.im = lap.im + dd[2][i].im; }
        ocplx rot = rr[0][i];
        if (g->ndim > 1) { rot.re = rot.re + rr[1][i].re; rot.im = rot.im + rr[1][i].im; }
        out[i].re = mcD * lap.re - Om * rot.im;
        out[i].im = mcD * lap.im + Om * rot.re;
    }
}

/* the six implicit schemes (backward-euler.jl, crank-nicolson.jl) */
enum { IM_BE = 0, IM_BE_NOPRE = 1, IM_CN = 2, IM_CN_QN = 3, IM_CN_T = 4, IM_CN_QN_T = 5 };

typedef struct {
    const ogrid *g;
    int scheme;
    real cD, Om, idt;      /* idt = 1 / dt (Float64, as 1 / n.dt) */
    ocplx *M;              /* real for BE / CN / CN_QN (im = 0), complex for the T schemes */
    real *Anl;
    ocplx *Anl2;
    ocplx *b;
    ocplx *dd[3], *rr[2], *lap;
} im_ctx;

/* prodA of each scheme (backward-euler.jl:87-90, 179-189; crank-nicolson.jl:112-114,
 * 234-236, 356-359, 478-481) */
static void prodA(im_ctx *c, const ocplx *x, ocplx *out)
{
    const ogrid *g = c->g;
    lap_rot(g, x, c->cD, c->Om, c->dd, c->rr, c->lap);
    int64_t N = g->total;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) {
        const ocplx v = x[i], L = c->lap[i];
        ocplx o;
        switch (c->scheme) {
        case IM_BE:       /* x - M lapRot(x) */
            o.re = v.re - c->M[i].re * L.re; o.im = v.im - c->M[i].re * L.im; break;
        case IM_BE_NOPRE: { /* (1/dt + Anl) x - lapRot(x) */
            real a = c->idt + c->Anl[i];
            o.re = a * v.re - L.re; o.im = a * v.im - L.im; break; }
        case IM_CN: {     /* (1/dt + Anl) x + 0.5 Anl2 conj(x) - 0.5 lapRot(x) */
            real a = c->idt + c->Anl[i];
            ocplx h = {(real)0.5 * c->Anl2[i].re, (real)0.5 * c->Anl2[i].im};
            /* h * conj(v) */
            real hr = h.re * v.re + h.im * v.im, hi = h.im * v.re - h.re * v.im;
            o.re = a * v.re + hr - (real)0.5 * L.re; o.im = a * v.im + hi - (real)0.5 * L.im; break; }
        case IM_CN_QN: {  /* (1/dt + 0.5 Anl) x - 0.5 lapRot(x) */
            real a = c->idt + c->Anl[i] * (real)0.5;
            o.re = a * v.re - (real)0.5 * L.re; o.im = a * v.im - (real)0.5 * L.im; break; }
        case IM_CN_T: {   /* (i/dt - 0.5 Anl) x - 0.5 Anl2 conj(x) + 0.5 lapRot(x) */
            real ar = -(real)0.5 * c->Anl[i], ai = c->idt;
            ocplx h = {(real)0.5 * c->Anl2[i].re, (real)0.5 * c->Anl2[i].im};
            real hr = h.re * v.re + h.im * v.im, hi = h.im * v.re - h.re * v.im;
            o.re = (ar * v.re - ai * v.im) - hr + (real)0.5 * L.re;
            o.im = (ar * v.im + ai * v.re) - hi + (real)0.5 * L.im; break; }
        default: {        /* IM_CN_QN_T: (i/dt - 0.5 Anl) x + 0.5 lapRot(x) */
            real ar = -(c->Anl[i] * (real)0.5), ai = c->idt;
            o.re = (ar * v.re - ai * v.im) + (real)0.5 * L.re;
            o.im = (ar * v.im + ai * v.re) + (real)0.5 * L.im; break; }
        }
        out[i] = o;
    }
}

static real re_dot(const ogrid *g, const ocplx *a, const ocplx *b, real *tmp)
{
    int64_t N = g->total;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) tmp[i] = a[i].re * b[i].re + a[i].im * b[i].im;
    return pairwise_sum(tmp, N);
}

static void cmul_field(const ogrid *g, const ocplx *M, ocplx *x)
{
    int64_t N = g->total;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) {
        real xr = M[i].re * x[i].re - M[i].im * x[i].im, xi = M[i].re * x[i].im + M[i].im * x[i].re;
        x[i].re = xr; x[i].im = xi;
    }
}

/* BiCGStab, krylov! (precond = 0) and krylovPreCond! (precond = 1), krylov.jl:1-67;
 * returns the iteration count of the reference (the last completed iteration
 * before the convergence test passes) */
static int krylov_solve(im_ctx *c, ocplx *phi, int nkrylov, real tol, int precond, ocplx **w, real *tmp)
{
    const ogrid *g = c->g;
    int64_t N = g->total;
    ocplx *r = w[0], *r2 = w[1], *p = w[2], *Ap = w[3], *s = w[4], *As = w[5];
    if (precond) {
        for (int64_t i = 0; i < N; i++) s[i] = c->b[i];
        cmul_field(g, c->M, s);
    }
    const real normb = RSQRT(re_dot(g, precond ? s : c->b, precond ? s : c->b, tmp));
    prodA(c, phi, r);
    for (int64_t i = 0; i < N; i++) { r[i].re = c->b[i].re - r[i].re; r[i].im = c->b[i].im - r[i].im; }
    if (precond) cmul_field(g, c->M, r);
    for (int64_t i = 0; i < N; i++) { r2[i] = r[i]; p[i] = r[i]; }
    int niter = 0;
    for (int it = 1; it <= nkrylov; it++) {
        prodA(c, p, Ap);
        if (precond) cmul_field(g, c->M, Ap);
        real rr2 = re_dot(g, r, r2, tmp), Apr2 = re_dot(g, Ap, r2, tmp);
        real alpha = rr2 / Apr2;
        for (int64_t i = 0; i < N; i++) { s[i].re = r[i].re - alpha * Ap[i].re; s[i].im = r[i].im - alpha * Ap[i].im; }
        prodA(c, s, As);
        if (precond) cmul_field(g, c->M, As);
        real Ass = re_dot(g, As, s, tmp), AsAs = re_dot(g, As, As, tmp);
        real omega = Ass / AsAs;
        for (int64_t i = 0; i < N; i++) {
            phi[i].re = (phi[i].re + alpha * p[i].re) + omega * s[i].re;
            phi[i].im = (phi[i].im + alpha * p[i].im) + omega * s[i].im;
        }
        real rr2old = re_dot(g, r, r2, tmp);
        for (int64_t i = 0; i < N; i++) { r[i].re = s[i].re - omega * As[i].re; r[i].im = s[i].im - omega * As[i].im; }
        real rr = re_dot(g, r, r, tmp);
        if (RSQRT(rr) / normb < tol) break;
        niter = it;
        rr2 = re_dot(g, r, r2, tmp);
        real beta = rr2 / rr2old * alpha / omega;
        for (int64_t i = 0; i < N; i++) {
            real qr = p[i].re - omega * Ap[i].re, qi = p[i].im - omega * Ap[i].im;
            p[i].re = r[i].re + beta * qr; p[i].im = r[i].im + beta * qi;
        }
    }
    return niter;
}

/*
 * nsteps of one implicit scheme: scheme IM_BE (NumModelBackwardEuler,
 * backward-euler.jl:62-83), IM_BE_NOPRE (NumModelBackwardEulerNoPrecond,
 * :155-172), IM_CN / IM_CN_QN / IM_CN_T / IM_CN_QN_T (NumModelCrankNicolson*,
 * crank-nicolson.jl:62-103, 186-225, 308-347, 432-468: Newton loop of
 * nnewton iterations to tolnewton around a preconditioned BiCGStab; the
 * stationary schemes renormalise with normalize!, the T schemes do not).
 * kry_total receives the sum of the returned Krylov counts.
 */
int OR_SYM(or_implicit_step)(int ndim, const int64_t *n, const double *lo, const double *hi,
                             double cD, double beta, double Om, const double *V, double *psi,
                             int nsteps, int scheme, double dt, int nkrylov, double tolkrylov,
                             int nnewton, double tolnewton, int64_t *kry_total)
{
    if (scheme < 0 || scheme > 5) return -1;
    ogrid g;
    if (grid_make(&g, ndim, n, lo, hi)) return -1;
    int64_t N = g.total;
    im_ctx c;
    memset(&c, 0, sizeof(c));
    c.g = &g; c.scheme = scheme; c.cD = (real)cD; c.Om = (real)Om; c.idt = (real)(1.0 / dt);
    ocplx *p = load_field(psi, N);
    real *Vr = load_real(V, N);
    ocplx *w[6] = {0}, *psim = NULL, *phi1 = NULL, *phiw = NULL;
    real *tmp = (real *)malloc(sizeof(real) * (size_t)N);
    int rc = (p && (!V || Vr) && tmp) ? 0 : -1;
    ocplx **allc[] = {&c.M, &c.Anl2, &c.b, &c.dd[0], &c.dd[1], &c.dd[2], &c.rr[0], &c.rr[1], &c.lap,
                      &w[0], &w[1], &w[2], &w[3], &w[4], &w[5], &psim, &phi1, &phiw};
    for (size_t i = 0; rc == 0 && i < sizeof(allc) / sizeof(allc[0]); i++)
        if (!(*allc[i] = (ocplx *)calloc((size_t)N, sizeof(ocplx)))) rc = -1;
    if (rc == 0 && !(c.Anl = (real *)calloc((size_t)N, sizeof(real)))) rc = -1;
    const real rbeta = (real)beta, rdt = (real)dt;
    int64_t ktot = 0;
    for (int st = 0; rc == 0 && st < nsteps; st++) {
        if (scheme == IM_BE || scheme == IM_BE_NOPRE) {
            for (int64_t i = 0; i < N; i++) {
                real vv = Vr ? Vr[i] : 0, a2 = p[i].re * p[i].re + p[i].im * p[i].im;
                if (scheme == IM_BE) {
                    real m = (real)1.0 / ((real)1 / rdt + vv + rbeta * a2);
                    c.M[i].re = m; c.M[i].im = 0;
                    c.b[i].re = m * p[i].re / rdt; c.b[i].im = m * p[i].im / rdt;
                } else {
                    c.Anl[i] = vv + rbeta * a2;
                    c.b[i].re = p[i].re / rdt; c.b[i].im = p[i].im / rdt;
                }
            }
            ktot += krylov_solve(&c, p, nkrylov, (real)tolkrylov, 0, w, tmp);
            real nrm = field_norm(&g, p);
            for (int64_t i = 0; i < N; i++) { p[i].re /= nrm; p[i].im /= nrm; }
            continue;
        }
        const int tsch = scheme == IM_CN_T || scheme == IM_CN_QN_T;
        const int newton = scheme == IM_CN || scheme == IM_CN_T;
        for (int64_t i = 0; i < N; i++) { phi1[i] = p[i]; phiw[i].re = 0; phiw[i].im = 0; }
        for (int itn = 1; itn <= nnewton; itn++) {
            for (int64_t i = 0; i < N; i++) {
                psim[i].re = (real)0.5 * (phi1[i].re + p[i].re);
                psim[i].im = (real)0.5 * (phi1[i].im + p[i].im);
                real vv = Vr ? Vr[i] : 0, a2 = psim[i].re * psim[i].re + psim[i].im * psim[i].im;
                c.Anl[i] = newton ? vv + 2 * rbeta * a2 : vv + 3 * rbeta * a2;
                /* beta * psi * psi */
                real qr = rbeta * psim[i].re, qi = rbeta * psim[i].im;
                c.Anl2[i].re = qr * psim[i].re - qi * psim[i].im;
                c.Anl2[i].im = qr * psim[i].im + qi * psim[i].re;
                real d = (vv + 3 * rbeta * a2) * (real)0.5;
                if (!tsch) { c.M[i].re = (real)1.0 / ((real)1.0 / rdt + d); c.M[i].im = 0; }
                else {       /* 1 / (i/dt - d) */
                    real zr = -d, zi = (real)1.0 / rdt, den = zr * zr + zi * zi;
                    c.M[i].re = zr / den; c.M[i].im = -zi / den;
                }
            }
            lap_rot(&g, psim, c.cD, c.Om, c.dd, c.rr, c.lap);
            for (int64_t i = 0; i < N; i++) {
                real vv = Vr ? Vr[i] : 0, a2 = psim[i].re * psim[i].re + psim[i].im * psim[i].im;
                real f = vv + rbeta * a2;
                real dr = phi1[i].re - p[i].re, di = phi1[i].im - p[i].im;
                if (!tsch) {
                    c.b[i].re = (c.idt * dr + f * psim[i].re) - c.lap[i].re;
                    c.b[i].im = (c.idt * di + f * psim[i].im) - c.lap[i].im;
                } else {   /* (i/dt)(phi1 - phi) - f psi + lapRot(psi) */
                    c.b[i].re = (-(c.idt * di) - f * psim[i].re) + c.lap[i].re;
                    c.b[i].im = ((c.idt * dr) - f * psim[i].im) + c.lap[i].im;
                }
            }
            ktot += krylov_solve(&c, phiw, nkrylov, (real)tolkrylov, 1, w, tmp);
            for (int64_t i = 0; i < N; i++) { phi1[i].re -= phiw[i].re; phi1[i].im -= phiw[i].im; }
            for (int64_t i = 0; i < N; i++) tmp[i] = phiw[i].re * phiw[i].re + phiw[i].im * phiw[i].im;
            if (RSQRT(pairwise_sum(tmp, N)) < (real)tolnewton) break;
        }
        for (int64_t i = 0; i < N; i++) p[i] = phi1[i];
        if (!tsch) {
            real nrm = field_norm(&g, p);
            for (int64_t i = 0; i < N; i++) { p[i].re /= nrm; p[i].im /= nrm; }
        }
    }
    if (rc == 0) store_field(p, psi, N);
    if (kry_total) *kry_total = ktot;
    for (size_t i = 0; i < sizeof(allc) / sizeof(allc[0]); i++) free(*allc[i]);
    free(c.Anl); free(tmp); free(p); free(Vr);
    grid_free(&g);
    return rc;
}

int OR_SYM(or_max_threads)(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
