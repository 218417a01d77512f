/*
 * gpss.h -- C ABI of libgpss.so, the GB300 split-step Gross-Pitaevskii
 * library.  It replaces the time-stepping hot path of SuperfluidDynamics.jl
 * (NumModelSplit1 / NumModelSplit2 on a periodic Grid) behind plain C types so
 * that Julia can bind it with ccall.
 *
 * Conventions
 *   - Fields are column-major with x fastest and complex values interleaved
 *     (re, im) as doubles: the memory of a Julia Array{ComplexF64} (the parent
 *     of Field.ϕ, src/Discretization/Fields.jl:94-157).  Potentials are real
 *     doubles of the same shape (param.pot.V, src/Potentials/quadratic.jl:61-67).
 *   - Every entry returns 0 (GPSS_OK) or a negative GPSS_E* code; the message
 *     is available from gpss_last_error().  No entry traps or aborts.
 *   - A context owns all of its device memory and one CUDA stream; it is not
 *     thread-safe.  Distinct contexts may be used from distinct threads.
 *   - Host pointers are only read or written during the call; none is kept.
 */
#ifndef GPSS_H
#define GPSS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPSS_OK 0
#define GPSS_EINVAL (-1)      /* bad argument: sizes, null pointers, ... */
#define GPSS_ENOMEM (-2)      /* device or host allocation failed */
#define GPSS_ECUDA (-3)       /* a CUDA runtime call failed */
#define GPSS_ENONFINITE (-4)  /* a reduction saw NaN/Inf in the field */
#define GPSS_ETIMEOUT (-5)    /* a bounded device-side wait gave up */
#define GPSS_ESTATE (-6)      /* call out of order (e.g. no field uploaded) */
#define GPSS_EIO (-7)         /* a file could not be read or written, or holds an unread form */

/* precision of the device field and of the FFT/phase arithmetic */
#define GPSS_FP64 64
#define GPSS_FP32 32

/* gpss_create flags */
#define GPSS_FLAG_PLAIN 1     /* reference stage order: FFT, multiply, iFFT, NL as
                                 separate launches (no fusion, no merging) */
#define GPSS_FLAG_NOMERGE 2   /* fused passes, but never merge the trailing and
                                 leading half kinetic steps of consecutive steps */
#define GPSS_FLAG_NOMASSLOCK 4 /* FP32 real time: do not restore the mass of the
                                 start of the call after each nonlinear stage */
#define GPSS_FLAG_PIPE 8      /* x passes through the persistent asynchronous-copy
                                 pipeline (same arithmetic; the direct kernel is
                                 faster on GB300 and is the default) */
#define GPSS_FLAG_ENERGY_CACHE 16 /* real-time Strang (fused forms): every
                                 gpss_step also measures the energies of its
                                 final field in its last passes (with Omega != 0
                                 plus one read-only x pass), and gpss_energy /
                                 gpss_mass return them while the field and the
                                 parameters are unchanged -- so solve!'s energy
                                 then timeStep! (NumModels.jl:33-35) costs no
                                 read-only passes, or one with rotation */
#define GPSS_FLAG_COMPENSATED 32 /* FP32 fields: the fused kinetic passes of the
                                 split steps run their transforms, twiddles and
                                 phase on double-float (hi + lo) FP32 values, so
                                 the only FP32 rounding of a pass is the store
                                 of the field (about 3x the instructions of a
                                 plain FP32 pass); the merged imaginary-time
                                 step keeps its plain FP32 passes */

/* split schemes of gpss_step */
#define GPSS_LIE 1            /* NumModelSplit1: L(dt) N(dt) */
#define GPSS_STRANG 2         /* NumModelSplit2: L(dt/2) N(dt) L(dt/2) */

typedef struct gpss_ctx gpss_ctx;

/* Diagnostics of the field at the end of a gpss_step call (FP64). */
typedef struct gpss_diag {
    double mass;        /* sum |psi|^2 dV  (= norm(f)^2, Fields.jl:172-180) */
    double energy[5];   /* E_Omega, E_Delta, E_beta, E, mu (GrossPitaevskii.jl:61-136) */
    int64_t steps;      /* steps performed by the call */
} gpss_diag;

/* Library version string. */
const char *gpss_version(void);

/*
 * Create a context for an ndim-dimensional periodic grid of n[0] x n[1]
 * [x n[2]] nodes on [lo[a], hi[a]).  Replaces Grid(size, bounds)
 * (src/Discretization/Grids.jl:64-129) + Field(grid, ComplexField())
 * (src/Discretization/Fields.jl:94-157) + Plan(f) (src/Discretization/Plans.jl:821-854,
 * 958-999).  ndim is 2 or 3; each n[a] is in [2, 1024] with no prime factor
 * above 31 (the reference plans any length with FFTW, Plans.jl:846-847).
 * Powers of two up to 256 run the register-resident pass kernels; other
 * lengths run the mixed-radix shared-memory pass, which takes every split,
 * energy, explicit RK and implicit entry point but not GPSS_FLAG_COMPENSATED
 * or gpss_adjoint (those return GPSS_EINVAL); the merged imaginary-time step
 * then runs as the unmerged sequence.
 * precision is GPSS_FP64 or GPSS_FP32; flags is a GPSS_FLAG_* mask.
 */
int gpss_create(gpss_ctx **out, int ndim, const int64_t *n, const double *lo, const double *hi,
                int precision, int flags);

/* Release every device resource of the context (NULL is accepted). */
void gpss_destroy(gpss_ctx *ctx);

/* Last error message of ctx (or of the last failed gpss_create when ctx is NULL). */
const char *gpss_last_error(const gpss_ctx *ctx);

/*
 * Equation parameters: i dpsi/dt = coeffD Lap psi + beta |psi|^2 psi + V psi - i Omega Lz psi.
 * Replaces GrossPitaevskiiParameters(coeffΔ, β, pot, Ω) (src/Parameters/Parameters.jl:17-55).
 */
int gpss_set_params(gpss_ctx *ctx, double coeffD, double beta, double omega);

/* Potential V (real, field shape).  NULL selects PotentialZero
 * (src/Potentials/Potentials.jl:12-25); otherwise param.pot.V. */
int gpss_set_potential(gpss_ctx *ctx, const double *V);

/* Copy psi (interleaved complex doubles) to / from the device field. */
int gpss_upload(gpss_ctx *ctx, const double *psi);
int gpss_download(gpss_ctx *ctx, double *psi);

/*
 * nsteps split steps of size dt.  scheme: GPSS_STRANG replaces
 * timeStep!(::NumModelSplit2) (src/NumModels/GrossPitaevskii/splitting.jl:149-154),
 * GPSS_LIE replaces timeStep!(::NumModelSplit1) (splitting.jl:78-82).
 * imag != 0 integrates in imaginary time and renormalises the field to unit
 * mass after every step (an extension; the reference has no imaginary-time
 * split step).  diag may be NULL; when given, it receives the mass and
 * energies of the final field.
 * A real-time Strang call with Omega = 0 (fused forms) runs the merged
 * sequence L(dt/2) N [L(dt) N]^(nsteps-1) and, unless diag is given, leaves
 * its last half kinetic flow L(dt/2) pending: the next such call folds it into
 * its first flow (so a loop of one-step calls costs one kinetic flow per
 * step), and every entry point that reads or changes the field -- download,
 * energy, mass, norm, normalize, set_params, set_potential, the other
 * integrators, sync, flush -- applies it first.  Results are bitwise those of
 * the eager sequence.
 */
int gpss_step(gpss_ctx *ctx, int nsteps, int scheme, int imag, double dt, gpss_diag *diag);

/*
 * nsteps explicit Runge-Kutta steps of size dt of the time-dependent GP
 * equation, dpsi/dt = i [lapRot(psi) - (V + beta|psi|^2) psi]: replaces
 * timeStep!(::NumModelGPRK) (src/NumModels/GrossPitaevskii/explicit-rk.jl:135-166,
 * right-hand side gp_rhs! :96-107, lapRot GrossPitaevskii.jl:12-45).
 * stepper: 1 forward Euler ("RK1"), 2 explicit midpoint ("RK2"), 4 classical
 * RK4 ("RK4").  filter: GPSS_RK_FILTER_* -- where the 2/3 rule (modes with
 * |xi|^2 >= (4/9) min_d max xi_d^2 zeroed, Plans.jl:529-532) is applied.
 */
#define GPSS_RK_FILTER_NONE 0
#define GPSS_RK_FILTER_PRODUCT 1   /* on the nonlinear term of every stage */
#define GPSS_RK_FILTER_SOLUTION 2  /* on the state after every step */
int gpss_rk_step(gpss_ctx *ctx, int nsteps, int stepper, int filter, double dt);

/*
 * nsteps of an implicit scheme of size dt, solving its linear systems with
 * the reference's BiCGStab (krylov!/krylovPreCond!, src/NumModels/krylov.jl:1-67;
 * nkrylov iterations at most, relative residual tolkrylov).  Replaces timeStep! of
 *   GPSS_IMPLICIT_BE          NumModelBackwardEuler            backward-euler.jl:62-83
 *   GPSS_IMPLICIT_BE_NOPRE    NumModelBackwardEulerNoPrecond   backward-euler.jl:155-172
 *   GPSS_IMPLICIT_CN          NumModelCrankNicolson            crank-nicolson.jl:62-103
 *   GPSS_IMPLICIT_CN_QN       NumModelCrankNicolsonQuasiNewton crank-nicolson.jl:186-225
 *   GPSS_IMPLICIT_CN_T        NumModelCrankNicolsonT           crank-nicolson.jl:308-347
 *   GPSS_IMPLICIT_CN_QN_T     NumModelCrankNicolsonQuasiNewtonT crank-nicolson.jl:432-468
 * (the CN schemes iterate Newton at most nnewton times to tolnewton; all but
 * the T schemes renormalise to unit mass).  krylov_iters (nullable) receives
 * the sum of the Krylov counts timeStep! returns.
 */
#define GPSS_IMPLICIT_BE 0
#define GPSS_IMPLICIT_BE_NOPRE 1
#define GPSS_IMPLICIT_CN 2
#define GPSS_IMPLICIT_CN_QN 3
#define GPSS_IMPLICIT_CN_T 4
#define GPSS_IMPLICIT_CN_QN_T 5
int gpss_implicit_step(gpss_ctx *ctx, int nsteps, int scheme, double dt, int nkrylov, double tolkrylov,
                       int nnewton, double tolnewton, int64_t *krylov_iters);

/*
 * Energies of the current field: out = {E_Omega, E_Delta, E_beta, E, mu}.
 * Replaces energy(n) (src/NumModels/GrossPitaevskii/GrossPitaevskii.jl:61-92 2D,
 * 106-136 3D; the 3D method prints no mu, the 2D formula is used for it).
 */
int gpss_energy(gpss_ctx *ctx, double *out);

/* sum |psi|^2 dV of the current field (norm(f)^2, src/Discretization/Fields.jl:172-180). */
int gpss_mass(gpss_ctx *ctx, double *out);

/* norm(f) (Fields.jl:172-180) and normalize! (Fields.jl:196-200) on the device field. */
int gpss_norm(gpss_ctx *ctx, double *out);
int gpss_normalize(gpss_ctx *ctx);

/*
 * Imaginary-time ground state: Strang steps of dt with unit-mass
 * renormalisation until |mu_k - mu_{k-1}| < tol, mu being evaluated every
 * check_every steps, or max_steps steps.  An extension (the reference reaches
 * ground states with Backward-Euler / Crank-Nicolson,
 * src/NumModels/GrossPitaevskii/backward-euler.jl:72-85).
 */
int gpss_ground_state(gpss_ctx *ctx, double dt, double tol, int64_t max_steps, int check_every,
                      double *mu_out, int64_t *steps_out);

/*
 * Discrete adjoint of nsteps real-time Strang steps from the current field
 * (an extension: the reference has no gradient path).  Loss
 *     L = 1 - |<psi_target, psi(T)>|^2,   <a, b> = sum conj(a) b dV.
 * Returns L, dLdV[cell] = dL/dV(cell) (FP64, field shape, nullable) and
 * dLdpsi0 = 2 dL/d conj(psi0) (interleaved complex doubles, nullable; so that
 * dL = Re sum conj(dLdpsi0) dpsi0).  The forward states are checkpointed every
 * K steps and recomputed segment by segment.  FP32 contexts run the forward and
 * the adjoint field in FP32 and accumulate dL/dV in FP64.  The context's
 * field is left at psi0.
 */
int gpss_adjoint(gpss_ctx *ctx, const double *psi_target, int nsteps, int K, double dt, double *loss,
                 double *dLdV, double *dLdpsi0);

/* ---- HDF5 checkpoints ----
 *
 * The file WriterSave writes and reads (src/IO/Writers.jl:41-92 write!,
 * :115-137 read!), "<prefix>-<istep>.h5": float64 datasets "re" and "im" in
 * the root group, the dataspace listing Julia's (nx, ny[, nz]) in reverse
 * (HDF5 is row-major), bytes in the field's own order (x fastest).  Written
 * without an HDF5 library (classic format structures: superblock 0, v1 object
 * headers, a symbol-table group, contiguous storage); read back from files
 * of that classic form as the HDF5 library writes them (user block,
 * continuation blocks, multi-level group B-trees, contiguous or compact
 * float32/float64 storage).  Other forms return GPSS_EIO with a message.
 */

/* Download the device field and write it (write!(WriterSave(f); prefix, istep)). */
int gpss_write_h5(gpss_ctx *ctx, const char *path);
/* Read "re"/"im" of the field's shape and upload them (read!(WriterSave(f); ...)). */
int gpss_read_h5(gpss_ctx *ctx, const char *path);
/* The same for a host field (interleaved complex doubles, n[0..ndim-1] = nx, ny[, nz]);
 * messages go to gpss_last_error(NULL). */
int gpss_h5_write_field(const char *path, int ndim, const int64_t *n, const double *psi);
int gpss_h5_read_field(const char *path, int ndim, const int64_t *n, double *psi);
/* Any float dataset of the root group: rank and dims (slowest first, up to 8)
 * always; values as doubles into out[0..cap) when out is not NULL. */
int gpss_h5_read_dataset(const char *path, const char *name, int *rank, int64_t *dims, double *out,
                         int64_t cap);

/* ---- batched runs (an extension: the reference integrates one field at a time) ---- */

typedef struct gpss_batch gpss_batch;

/*
 * A batch of nruns independent 2D real-time runs (NumModelSplit2 each), run
 * r on an n[r] x n[r] grid (n[r] in {64, 128, 256}) over
 * [lo[2r], hi[2r]) x [lo[2r+1], hi[2r+1]); coeffD shared.  FP32 fields,
 * FP64 masses.  All runs advance together in one persistent kernel launch
 * (captured in a CUDA graph) with a work queue; the first gpss_batch_step
 * autotunes the launch policy on the batch itself.
 */
int gpss_batch_create(gpss_batch **out, int nruns, const int64_t *n, const double *lo, const double *hi,
                      double coeffD);
void gpss_batch_destroy(gpss_batch *b);
const char *gpss_batch_last_error(const gpss_batch *b);
/* beta, potential (real, n x n, x fastest; NULL = zero) and psi (interleaved complex) of one run */
int gpss_batch_set_run(gpss_batch *b, int run, double beta, const double *V, const double *psi);
/* nsteps Strang steps of dt for every run; mass_out[r] = sum |psi_r|^2 (no cell volume), nullable */
int gpss_batch_step(gpss_batch *b, int nsteps, double dt, double *mass_out);
int gpss_batch_download(gpss_batch *b, int run, double *psi);
/* the autotuner's choice (policy 0: runs up to 128^2 in shared memory; 1: up to 64^2),
 * queue order (0: largest first, 1: as given), stacking (the runs of one size and box,
 * two or more, go through the directional pass kernels as one stack of planes: stack 1
 * the 256^2 runs, 2 also the 128^2 ones, 3 every size) and the trial times in ms (16
 * entries: index = 4 stack + 2 policy + order; 1e30 for candidates not tried) */
int gpss_batch_tuning(const gpss_batch *b, int *policy, int *order, int *stack, float *trial_ms);
/* fix the launch choice instead of autotuning it (stack 0 to 3; sizes without a stack
 * stay in the persistent launch) */
int gpss_batch_set_tuning(gpss_batch *b, int policy, int order, int stack);

/* ---- timing and integration helpers (no reference counterpart) ---- */

/* Make `device` the CUDA device that later gpss_create calls on this host
 * thread use (the library links its own CUDA runtime, whose current device
 * is separate from any other runtime loaded in the process). */
int gpss_select_device(int device);

/* Number of CUDA devices visible to the library (0 when there is none). */
int gpss_device_count(void);

/* Block the host until the context's stream is idle (after applying a
 * pending half kinetic flow, see gpss_step). */
int gpss_sync(gpss_ctx *ctx);

/* Record CUDA event `slot` (0..7) on the context's stream. */
int gpss_event_record(gpss_ctx *ctx, int slot);

/*
 * Apply now the half kinetic flow that a merged real-time Strang call of
 * gpss_step leaves pending (see gpss_step).  Every entry point that reads or
 * changes the field does this itself; call it to end a timed region with the
 * field complete.  No counterpart in the reference (its timeStep! is eager).
 */
int gpss_flush(gpss_ctx *ctx);

/* Milliseconds between two recorded events (synchronises on `b`). */
int gpss_event_elapsed(gpss_ctx *ctx, int a, int b, float *ms);

/* Number of kernel launches issued by the context since creation. */
int64_t gpss_launch_count(const gpss_ctx *ctx);

/*
 * Time each directional pass kernel of one fused kinetic step in isolation:
 * runs `reps` launches of the pass along `axis` (0 = x, 1 = y, 2 = z; mode 0 =
 * fused kinetic pass, 1 = fused kinetic pass with the nonlinear epilogue) on
 * the current field, bracketed by CUDA events, and returns the mean
 * milliseconds per launch.  The field is advanced by those launches.
 */
int gpss_time_pass(gpss_ctx *ctx, int axis, int mode, int reps, double dt, double *ms_per_launch);

/*
 * FMA throughput of the current device in TFLOP/s (2 flops per fused
 * multiply-add; precision GPSS_FP32 or GPSS_FP64), measured with CUDA events
 * on a kernel of independent FMA chains.  A diagnostic: it is the compute roof
 * for the roofline reports of the FP64 kernels and of the compensated FP32
 * passes, which their FMA pipe bounds.  No counterpart in the reference.
 */
int gpss_measure_fma_rate(int precision, double *tflops);

/* Page-locked host buffer helpers for fast uploads/downloads. */
int gpss_host_alloc(void **ptr, int64_t bytes);
int gpss_host_free(void *ptr);

/* Device memory held by the context, in bytes. */
int64_t gpss_device_bytes(const gpss_ctx *ctx);

/*
 * Energies of a field that already lives in the caller's device memory,
 * computed without any allocation by the library.  No counterpart in the
 * reference: it exists for callers that cannot let the library cudaMalloc --
 * for example a Julia session whose CuArrays come from CUDA.jl's memory pool,
 * or a program held to a fixed device-memory budget.
 *   psi_dev  device pointer, n[0]*n[1][*n[2]] complex values, x fastest
 *            (double2 for GPSS_FP64, float2 for GPSS_FP32)
 *   V_dev    device pointer to the real potential in the same precision, or NULL
 *   stream   cudaStream_t to run on (NULL: the default stream); the call
 *            returns after the stream has finished its work
 *   out      host array of 5 doubles: E_Omega, E_Delta, E_beta, E, mu (as gpss_energy)
 * Scratch lives in a 1 MiB device array inside the library, held by every GPU
 * that loads it until the process exits.  Fields whose largest reduction
 * needs more partial sums than fit are rejected with GPSS_EINVAL (256^3 fits).
 * The first call on a device looks that array up; make it before any stream
 * capture.  Every call copies its small coordinate and twiddle tables from
 * host memory into the array and waits for `stream` before it returns.  The
 * address is kept for the life of the process: a
 * cudaDeviceReset between calls is not supported.  Calls share the array:
 * calls that overlap on the GPU race, so serialise them.  Returns 0 or a
 * negative GPSS_E* code; the message is available from gpss_last_error(NULL).
 */
int gpss_energy_noalloc(int ndim, const int64_t *n, const double *lo, const double *hi, int precision,
                        double coeffD, double beta, double omega, const void *psi_dev, const void *V_dev,
                        void *stream, double *out);

#ifdef __cplusplus
}
#endif

#endif /* GPSS_H */
