#!/usr/bin/env python3
"""Benchmark of the split-step Gross-Pitaevskii hot path on GB300.

Workload (cfg1): 3D real-time GP, Strang splitting (NumModelSplit2), 256^3
periodic box [0, 2pi]^3, V = 0, coeffD = -xi/sqrt(2), beta = 1/(sqrt(2) xi),
xi = 0.05, psi0 = e^{i theta} with 64 seeded Fourier modes; dt = 2.5e-3.
One bench step = one cfg1 run of 200 time steps through gpss_step from the
cfg1 initial field, which is restored in HBM (outside the timed events)
before every bench step.  The timed form is the FP32 one that meets the
metric's accuracy bar (rel-L2 <= 1e-5 against the FP64 oracle after 200
steps): FP32 storage with compensated (double-float) arithmetic in the fused
passes (GPSS_FLAG_COMPENSATED), FP64 reductions.  The plain FP32 passes are
timed beside it (`fp32_plain`): they are 4x faster but reach 2.5e-5 at step
200, because the Strang step is resonant on the |k| ~ 188 shell of this grid
(|coeffD| |k|^2 dt = pi) and amplifies their rounding.

Metric: Mcell-steps/s = cells x time steps / seconds.  The field (134 MB FP32)
is larger than L2 and every pass streams 268 MB, so no L2 flush is needed.

JSON line keys beyond the base contract:
  e2e            same metric through the public API with host buffers: every
                 step uploads psi (FP64, pinned), runs the 200 steps and
                 downloads psi.
  roofline       the dominant kernel (fused directional pass) against the
                 measured HBM copy bandwidth; algorithmic bytes = 16 B/cell/pass.
  cpu_baseline   the CPU oracle (FP64 C restatement, OpenMP) on a bounded
                 sample of the same workload.
  fp64_plain     the FP64 plain kernels (reference stage order) on the same
                 workload, the comparison the headline metric names.
  batched        cfg3: 512 mixed-size 2D runs in one persistent launch.
  fp32_plain     the plain FP32 fused passes on the same workload (value,
                 per-pass times, roofline).
  accuracy       rel-L2 of the FP32 fields (compensated and plain) and of the
                 FP64 fused field against the FP64 oracle after 50..200 steps.
  imag_time      cfg2: 128^3 imaginary-time steps, FP32 and FP64.
  adjoint        cfg4: one 2000-step gradient through gpss_adjoint.
  rk4            the explicit RK4 integrator (NumModelGPRK) on the cfg1 field.
  solve          solve! iterations (energy + one step) with and without the
                 energy cache; implicit: the BE/CN Krylov schemes (cfg2, 64^3).
  checkpoint     one WriterSave res-<istep>.h5 of the cfg1 field written from
                 and read back into the device field.
  cufft_comparison  the same directional pass through cuFFT (torch.fft).

--impl reference times the CPU restatement of the reference path (the
reference itself is Julia + FFTW, which does not exist on this machine): the
time-step loop of the FP64 C oracle on all host cores, grid and plan setup
excluded (the reference's own benchmark times timeStep! alone), plus a
labelled scipy.fft (pocketfft, threaded) restatement as an FFTW-class leg.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CELLS_N = 256
TIMESTEPS_PER_STEP = 200
BYTES_PER_CELL_PASS = 16  # FP32 complex read + write
PASSES_PER_TIMESTEP = 3   # merged Strang: 3 passes per step (+3 for the final half step)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpss", choices=["gpss", "reference"])
    ap.add_argument("--n", type=int, default=CELLS_N, help="grid points per axis (default 256)")
    ap.add_argument("--timesteps", type=int, default=TIMESTEPS_PER_STEP,
                    help="time steps per bench step (default 200, the cfg1 run length)")
    ap.add_argument("--kernels", default="compensated", choices=["compensated", "plain"],
                    help="FP32 form timed as the headline (default: compensated, the one that meets 1e-5)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the accuracy, cfg2, cfg4 and cuFFT measurements")
    ap.add_argument("--only", choices=["imag", "adjoint", "batch", "rk4", "solve", "implicit", "checkpoint", "passes"],
                    default=None,
                    help="run one secondary measurement alone and print it (profiling runs)")
    ap.add_argument("--only-steps", type=int, default=None,
                    help="with --only imag/solve: time steps (iterations) to time; with --only passes: "
                         "launches per axis")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


class Dist:
    """Barrier and max-over-ranks for torchrun launches (gloo: host-side only)."""

    def __init__(self, world):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, v):
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.out = ""

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            self.out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def measured_hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# FP32 operations (lanes of packed f32x2 instructions; an FMA counts once) that
# a compensated 256-point pass executes per cell, counted from fft_comp.cuh:
# per cell 3 (onto the grid) + 4 x 12.75 (DFT-16: 8 radix-4 butterflies of
# 8 two-word adds, 3 general and 4 sqrt(1/2) products per 16 cells) + 2 x
# 10.55 (twiddle products, 225 of 256 cells) + 12 (phase) + 1 (rounding)
# = 88.1 packed instructions; and ~24 for the nonlinear step and mass sum of
# the last pass of a time step.
COMP_OPS_PER_CELL_PASS = 2 * 88.1
NL_OPS_PER_CELL = 24


def profiled_traffic(kernel_tag):
    """dram bytes per launch of the dominant kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", f"{kernel_tag}.md")
    try:
        for line in open(p):
            if line.strip().startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


# ----------------------------------------------------------------- CPU arm --
def oracle_mod():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import gp_oracle
    gp_oracle.build()
    return gp_oracle


def cpu_sample(c, O, timesteps=1, nthreads=0, psi=None):
    """One bounded sample of the workload on the CPU oracle, timing its
    time-step loop alone; returns (cell-steps/s, cores, seconds, field)."""
    cores = nthreads or os.cpu_count() or 1
    psi = c["psi"] if psi is None else psi
    out, dt = O.c_step_timed(psi, c["bounds"], coeffD=c["coeffD"], beta=c["beta"], V=c["V"],
                             nsteps=timesteps, dt=c["dt"], nthreads=cores)
    cells = float(math.prod(c["shape"]))
    return cells * timesteps / dt, cores, dt, out


METRIC = "GP split-step Mcell-steps/s at 256^3: FP32 fused vs FP64 plain @ relL2<=1e-5"


def workload_name(n):
    return (f"cfg1: 3D real-time GP Strang (NumModelSplit2), {n}^3 on [0,2pi]^3, V=0, xi=0.05, c=1, "
            "dt=2.5e-3")


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    import importlib
    import __graft_entry__ as g
    g.load_package()
    W = importlib.import_module("sfd_gb300.workloads")
    c = W.cfg1(args.n)
    O = oracle_mod()
    cores = os.cpu_count() or 1
    psi = c["psi"]
    for _ in range(args.warmup):
        _, _, _, psi = cpu_sample(c, O, 1, cores, psi)
    secs = 0.0
    for _ in range(args.steps):  # timeStep! after timeStep!, the loop alone timed
        _, _, dt, psi = cpu_sample(c, O, 1, cores, psi)
        secs += dt
    value = (float(math.prod(c["shape"])) * args.steps) / secs / 1e6
    sample = (f"1 Strang time step of cfg1 at {args.n}^3 per bench step, continuing the run (FP64, own "
              "radix-2 FFT, OpenMP); the step loop is timed, grid/plan/field setup is not")
    # FFTW-class leg: the same steps with scipy.fft (pocketfft, threaded)
    sp_steps = 2
    _, sp_s = O.sp_step_timed(c["psi"], c["bounds"], coeffD=c["coeffD"], beta=c["beta"], nsteps=1,
                              dt=c["dt"], workers=cores)
    _, sp_s = O.sp_step_timed(c["psi"], c["bounds"], coeffD=c["coeffD"], beta=c["beta"], nsteps=sp_steps,
                              dt=c["dt"], workers=cores)
    scipy_leg = {"value": float(math.prod(c["shape"])) * sp_steps / sp_s / 1e6, "unit": "Mcell-steps/s",
                 "cores": cores, "kind": "port",
                 "sample": f"{sp_steps} Strang time steps of cfg1 at {args.n}^3: scipy.fft (pocketfft) "
                           f"threaded over {cores} workers, numpy broadcasts single-threaded"}
    line = {
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "Mcell-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded cfg1 phase field, 64 modes |k|<=4)",
        "config": {"workload": workload_name(args.n), "grid": [args.n] * 3,
                   "timesteps_per_step": 1,
                   "note": "a bench step of this CPU arm is one time step (a bounded sample); the metric "
                           "is per cell-step, so it compares directly with the GPU arm"},
        "cpu_baseline": {"value": value, "unit": "Mcell-steps/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "scipy_fft_leg": scipy_leg,
        "note": "CPU restatement of NumModelSplit2 (oracle/gp_oracle.c); the reference's Julia/FFTW "
                "runtime is not installed on this machine",
    }
    print(json.dumps(line), flush=True)
    return 0


def measure_batch(sfd, W, calls=3):
    """cfg3: 512 mixed-size 2D runs, 500 steps per call, one persistent launch
    (CUDA graph) per call; host-timed around the synchronous call."""
    c = W.cfg3()
    runs = c["runs"]
    b = sfd.BatchSplit2([r["n"] for r in runs], [r["bounds"] for r in runs], coeffD=c["coeffD"])
    for i, r in enumerate(runs):
        b.set_run(i, r["beta"], r["V"], r["psi"])
    m0 = b.step(c["nsteps"], c["dt"])  # autotune + capture + one run
    t = []
    for _ in range(calls):
        t0 = time.perf_counter()
        m = b.step(c["nsteps"], c["dt"])
        t.append(time.perf_counter() - t0)
    tune = b.tuning()
    b.close()
    cells = sum(r["n"] * r["n"] for r in runs)
    best = min(t)
    return {"workload": "cfg3: 512 runs (256 x 64^2, 192 x 128^2, 64 x 256^2), 500 steps per call, FP32",
            "value": cells * c["nsteps"] / best / 1e6, "unit": "Mcell-steps/s", "ms_per_call": best * 1e3,
            "calls": calls, "runs": len(runs), "tuning": tune,
            "max_rel_mass_drift": float(np.max(np.abs(m - m0) / m0))}


def _model(sfd, c, precision, form="fused", V=None, steps=1, compensated=False):
    grid = sfd.Grid(c["shape"], c["bounds"])
    f = sfd.Field(grid)
    f.phi = c["psi"]
    pot = sfd.PotentialZero(f) if V is None else sfd.PotentialArray(f, V)
    p = sfd.GrossPitaevskiiParameters(pot, coeffD=c["coeffD"], beta=c["beta"])
    return f, sfd.NumModelSplit2(f, p, c["dt"], steps, steps, precision=precision, form=form,
                                 compensated=compensated)


def measure_accuracy(sfd, c, O, marks=(50, 100, 150, 200)):
    """rel-L2 against the FP64 oracle (oracle/gp_oracle.c run live on the host
    cores, about 40 s for 200 steps at 256^3) after each mark, for the FP32
    compensated form (the headline), the plain FP32 passes and the FP64 fused
    merged form."""
    forms = {"fp32_compensated": dict(precision="fp32", compensated=True),
             "fp32_plain": dict(precision="fp32"),
             "fp64_fused": dict(precision="fp64")}
    models = {k: _model(sfd, c, **kw) for k, kw in forms.items()}
    out = {k: {} for k in forms}
    ref, done = c["psi"], 0
    for k in marks:
        ref = O.c_step(ref, c["bounds"], coeffD=c["coeffD"], beta=c["beta"], nsteps=k - done, dt=c["dt"])
        for name, (f, m) in models.items():
            m.step(k - done)
            out[name][str(k)] = O.rel_l2(f.phi, ref)
        done = k
    for f, m in models.values():
        m.close(download=False)
    return {"rel_l2_vs_fp64_oracle": out, "bar": 1e-5, "bar_met_at_200": {
        k: v[str(marks[-1])] <= 1e-5 for k, v in out.items()}}


def _event_ms(L, h, fn):
    ms = ctypes.c_float()
    L.gpss_event_record(h, 0)
    fn()
    L.gpss_event_record(h, 1)
    L.gpss_event_elapsed(h, 0, 1, ctypes.byref(ms))
    return ms.value


def measure_imag(sfd, W, L, steps=200):
    """cfg2 (128^3 anisotropic trap, imaginary time, per-step FP64 renormalisation):
    fixed-step throughput of the fused FP32 and FP64 kernels."""
    c = W.cfg2(128)
    cells = float(math.prod(c["shape"]))
    out = {"workload": "cfg2: 3D imaginary-time GP, 128^3 on [-10,10]^3, V=(x^2+y^2+4z^2)/2, g=2000, "
                       f"dt=1e-3, {steps} steps per timing"}
    for prec in ("fp32", "fp64"):
        f, m = _model(sfd, c, prec, V=c["V"])
        h = m.handle
        for _ in range(3):
            L.gpss_step(h, 20, 2, 1, c["dt"], None)
        ms = _event_ms(L, h, lambda: L.gpss_step(h, steps, 2, 1, c["dt"], None))
        out[prec] = {"value": cells * steps / (ms / 1e3) / 1e6, "unit": "Mcell-steps/s",
                     "ms_per_timestep": ms / steps}
        m.close(download=False)
    return out


def measure_adjoint(sfd, W):
    """cfg4 (256^2, 2000 steps, checkpoints every 50): one gradient (forward with
    checkpoints, recompute, backward) through gpss_adjoint, host-timed."""
    c = W.cfg4(256)
    out = {"workload": "cfg4: 2D adjoint, 256^2 on [-8,8]^2, trap + learnable V, g=500, dt=1e-3, "
                       "2000 steps, K=50, loss 1-|<psi_t|psi(T)>|^2"}
    grads = {}
    for tag, prec, comp in (("fp32", "fp32", False), ("fp32_compensated", "fp32", True), ("fp64", "fp64", False)):
        f, m = _model(sfd, c, prec, V=c["V"], compensated=comp)
        m.adjoint(c["target"], 100, 50)  # warm-up
        t = []
        for _ in range(3):
            t0 = time.perf_counter()
            loss, dv, g0 = m.adjoint(c["target"], c["nsteps"], c["K"])
            t.append(time.perf_counter() - t0)
        m.close(download=False)
        grads[tag] = dv
        out[tag] = {"s_per_gradient": min(t), "loss": loss,
                    "forward_plus_backward_cell_steps_per_s": 256 * 256 * c["nsteps"] / min(t)}
    for tag in ("fp32", "fp32_compensated"):
        out[tag]["dLdV_rel_l2_vs_fp64"] = float(np.linalg.norm(grads[tag] - grads["fp64"]) /
                                                np.linalg.norm(grads["fp64"]))
    return out


def measure_rk(sfd, c, L, steps=4):
    """The explicit RK4 integrator (NumModelGPRK, 2/3 filter on the product) on
    the cfg1 field at 256^3, FP32 and FP64, CUDA events around gpss_rk_step."""
    cells = float(math.prod(c["shape"]))
    out = {"workload": f"cfg1 field, 256^3, RK4, filter product, dt=1e-3, {steps} steps per timing"}
    for prec in ("fp32", "fp64"):
        grid = sfd.Grid(c["shape"], c["bounds"])
        f = sfd.Field(grid)
        f.phi = c["psi"]
        p = sfd.GrossPitaevskiiParameters(sfd.PotentialZero(f), coeffD=c["coeffD"], beta=c["beta"])
        m = sfd.NumModelGPRK(f, p, 1e-3, steps, steps, stepper="RK4", filter="product", precision=prec)
        h = m.handle
        L.gpss_rk_step(h, 1, 4, 1, 1e-3)
        ms = _event_ms(L, h, lambda: L.gpss_rk_step(h, steps, 4, 1, 1e-3))
        out[prec] = {"value": cells * steps / (ms / 1e3) / 1e6, "unit": "Mcell-steps/s", "ms_per_step": ms / steps}
        m.close(download=False)
    return out


def measure_solve(sfd, c, iters=20):
    """solve! (energy then timeStep! every iteration, NumModels.jl:23-46) on the
    cfg1 field at 256^3, FP32, with and without GPSS_FLAG_ENERGY_CACHE."""
    out = {"workload": f"cfg1 field, 256^3, FP32, solve! with {iters} iterations (energy + one Strang step each)"}
    for cache in (False, True):
        grid = sfd.Grid(c["shape"], c["bounds"])
        f = sfd.Field(grid)
        f.phi = c["psi"]
        p = sfd.GrossPitaevskiiParameters(sfd.PotentialZero(f), coeffD=c["coeffD"], beta=c["beta"])
        m = sfd.NumModelSplit2(f, p, c["dt"], 2, 1000, precision="fp32", energy_cache=cache)
        sfd.solve(m)  # warm-up (3 iterations)
        m.niter = iters - 1
        t0 = time.perf_counter()
        sfd.solve(m)
        t = time.perf_counter() - t0
        m.close(download=False)
        out["cache" if cache else "no_cache"] = {"ms_per_iteration": t / iters * 1e3}
    # a timeStep! loop without energies: one-step calls chain through the
    # pending half kinetic flow (one flow per call), flushed at the end
    grid = sfd.Grid(c["shape"], c["bounds"])
    f = sfd.Field(grid)
    f.phi = c["psi"]
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialZero(f), coeffD=c["coeffD"], beta=c["beta"])
    m = sfd.NumModelSplit2(f, p, c["dt"], iters, iters, precision="fp32")
    from sfd_gb300 import _lib
    L = _lib.lib()
    for _ in range(3):
        sfd.timeStep(m)
    L.gpss_sync(m.handle)
    t0 = time.perf_counter()
    for _ in range(iters):
        sfd.timeStep(m)
    L.gpss_sync(m.handle)
    t = time.perf_counter() - t0
    m.close(download=False)
    out["timestep_loop"] = {"ms_per_call": t / iters * 1e3,
                            "note": "timeStep! called once per step, no energy in between (host-timed, sync at the end)"}
    return out


def measure_checkpoint(sfd, c):
    """WriterSave's res-<istep>.h5 (Writers.jl:41-137) of the cfg1 field at
    256^3 (FP32 on the device), written from the device field and read back
    into it: seconds and GB/s of file per direction (a 268 MB file: "re" and
    "im" as float64)."""
    import shutil
    import tempfile
    grid = sfd.Grid(c["shape"], c["bounds"])
    f = sfd.Field(grid)
    f.phi = c["psi"]
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialZero(f), coeffD=c["coeffD"], beta=c["beta"])
    m = sfd.NumModelSplit2(f, p, c["dt"], 1, 1, precision="fp32")
    d = tempfile.mkdtemp(prefix="gpss_ckpt_")
    try:
        w = sfd.WriterSave(f)
        prefix = os.path.join(d, "res")
        t0 = time.perf_counter()
        w.write(prefix=prefix, istep=0)
        tw = time.perf_counter() - t0
        size = os.path.getsize(prefix + "-0.h5")
        t0 = time.perf_counter()
        w.read(prefix=prefix, istep=0)
        tr = time.perf_counter() - t0
    finally:
        m.close(download=False)
        shutil.rmtree(d, ignore_errors=True)
    return {"workload": "cfg1 field, 256^3 FP32 on the device, one res-<istep>.h5 (float64 re/im) to a temporary directory",
            "file_bytes": size, "write_s": tw, "read_s": tr, "write_GBps": size / tw / 1e9, "read_GBps": size / tr / 1e9}


def measure_implicit(sfd, W, steps=4):
    """The implicit schemes (imaginary-time BE and CN with the reference's
    BiCGStab) on the cfg2 physics at 64^3, FP64: time per step and Krylov
    iterations per step (each iteration reads its FP64 dot products back)."""
    c = W.cfg2(64)
    out = {"workload": f"cfg2 physics at 64^3 (trap, g=2000), FP64, dt=1e-3, {steps} steps per timing"}
    for name, cls in (("backward_euler", sfd.NumModelBackwardEuler), ("crank_nicolson", sfd.NumModelCrankNicolson)):
        grid = sfd.Grid(c["shape"], c["bounds"])
        f = sfd.Field(grid)
        f.phi = c["psi"]
        p = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, c["V"]), coeffD=c["coeffD"], beta=c["beta"])
        m = cls(f, p, c["dt"], steps, steps, precision="fp64")
        m.step(1)
        t0 = time.perf_counter()
        m.step(steps)
        t = time.perf_counter() - t0
        out[name] = {"ms_per_step": t / steps * 1e3, "krylov_iterations_per_step": m.last_krylov / steps}
        m.close(download=False)
    return out


def measure_passes(sfd, c, L, compensated, reps=20):
    """Each fused directional pass of the cfg1 merged step alone (x, y, z with
    the nonlinear epilogue), `reps` launches per axis after one warm-up, CUDA
    events (the command behind the per-pass ncu captures in profiles/)."""
    f, m = _model(sfd, c, "fp32", compensated=compensated)
    out = {"workload": f"cfg1 field, {c['shape'][0]}^3, FP32 {'compensated' if compensated else 'plain'} "
                       f"fused passes, {reps} launches per axis"}
    for axis in range(3):
        ms = ctypes.c_double()
        rc = L.gpss_time_pass(m.handle, axis, 1 if axis == 2 else 0, reps, c["dt"], ctypes.byref(ms))
        if rc != 0:
            raise RuntimeError(L.gpss_last_error(m.handle).decode())
        out["xyz"[axis] + "_ms"] = ms.value
    m.close(download=False)
    return out


def run_only(args):
    """One secondary measurement alone (for profiling it), one JSON line."""
    import importlib
    import __graft_entry__ as g
    sfd = g.load_package()
    from sfd_gb300 import _lib
    W = importlib.import_module("sfd_gb300.workloads")
    L = _lib.lib()
    if args.only == "imag":
        r = measure_imag(sfd, W, L, steps=args.only_steps or 200)
    elif args.only == "adjoint":
        r = measure_adjoint(sfd, W)
    elif args.only == "batch":
        r = measure_batch(sfd, W)
    elif args.only == "rk4":
        r = measure_rk(sfd, W.cfg1(256), L)
    elif args.only == "implicit":
        r = measure_implicit(sfd, W)
    elif args.only == "checkpoint":
        r = measure_checkpoint(sfd, W.cfg1(256))
    elif args.only == "passes":
        r = measure_passes(sfd, W.cfg1(args.n), L, args.kernels == "compensated", reps=args.only_steps or 20)
    else:
        r = measure_solve(sfd, W.cfg1(256), iters=args.only_steps or 20)
    print(json.dumps(r), flush=True)
    return 0


def measure_cufft(c, n, reps=20):
    """The same directional pass (FFT -> phase multiply -> inverse FFT) through
    cuFFT (torch.fft, complex64) on the 256^3 field, per axis, for comparison."""
    try:
        import torch
        if not torch.cuda.is_available():
            return None
    except ImportError:
        return None
    x = torch.from_numpy(np.ascontiguousarray(c["psi"].reshape(-1, order="F")).astype(np.complex64))
    x = x.cuda().reshape(n, n, n)  # [z][y][x]
    k = torch.fft.fftfreq(n, d=1.0 / n, device="cuda")
    ph = torch.exp(1j * (c["coeffD"] * (k * k) * c["dt"]).to(torch.float32)).to(torch.complex64)
    out = {"note": "torch.fft (cuFFT) complex64 at 256^3, per axis: fft -> multiply by exp(i coeffD k^2 dt) "
                   "-> ifft, CUDA events, mean of 20"}
    for dim, name in ((2, "x"), (1, "y"), (0, "z")):
        shape = [1, 1, 1]
        shape[dim] = n
        p = ph.reshape(shape)
        f = lambda: torch.fft.ifft(torch.fft.fft(x, dim=dim) * p, dim=dim)
        for _ in range(3):
            f()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            f()
        e1.record()
        torch.cuda.synchronize()
        out[name + "_pass_ms"] = e0.elapsed_time(e1) / reps
    del x
    torch.cuda.empty_cache()
    return out


# ----------------------------------------------------------------- GPU arm --
def run_gpss(args, rank, world, local):
    import importlib
    import numpy as np
    import __graft_entry__ as g
    sfd = g.load_package()
    from sfd_gb300 import _lib
    W = importlib.import_module("sfd_gb300.workloads")
    L = _lib.lib()
    dist = Dist(world)
    _lib.check(L.gpss_select_device(local))
    c = W.cfg1(args.n)
    cells = float(math.prod(c["shape"]))
    nt = args.timesteps

    grid = sfd.Grid(c["shape"], c["bounds"])
    f = sfd.Field(grid)
    f.phi = c["psi"]
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialZero(f), coeffD=c["coeffD"], beta=c["beta"])
    comp = args.kernels == "compensated"
    model = sfd.NumModelSplit2(f, p, c["dt"], nt, nt, precision="fp32", compensated=comp)
    h = model.handle
    ck = lambda rc: _lib.check(rc, h)

    # ---- device-resident throughput (value).  Every bench step is the cfg1
    # run itself: the initial field is restored (uploaded, outside the timed
    # events) before each one, so the run never drifts into a different state
    # (the nonlinear epilogue's cost depends on the field through |psi|^2).
    psi0 = np.asfortranarray(c["psi"], dtype=np.complex128)
    p0 = psi0.ctypes.data_as(ctypes.POINTER(ctypes.c_double))

    def restore():
        ck(L.gpss_upload(h, p0))
        ck(L.gpss_sync(h))

    for _ in range(args.warmup):
        restore()
        ck(L.gpss_step(h, nt, 2, 0, c["dt"], None))
        ck(L.gpss_flush(h))
    ck(L.gpss_sync(h))
    dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    launches = 0
    t_sum = 0.0
    ms = ctypes.c_float()
    for _ in range(args.steps):
        restore()
        l0 = L.gpss_launch_count(h)
        ck(L.gpss_event_record(h, 0))
        ck(L.gpss_step(h, nt, 2, 0, c["dt"], None))
        ck(L.gpss_flush(h))  # the call's last half kinetic flow, inside the timed region
        ck(L.gpss_event_record(h, 1))
        ck(L.gpss_event_elapsed(h, 0, 1, ctypes.byref(ms)))
        launches += L.gpss_launch_count(h) - l0
        t_sum += ms.value
    clk = clocks.stop()
    dist.barrier()
    t_ms = dist.max(t_sum)
    value = world * cells * nt * args.steps / (t_ms / 1e3) / 1e6
    restore()

    # ---- dominant kernel timing (roofline): each fused pass alone, CUDA events
    alg_bytes = BYTES_PER_CELL_PASS * cells
    peak, peak_kind = measured_hbm_peak()
    passes_per_call = PASSES_PER_TIMESTEP * (nt + 1)  # 3 per merged step + the final half step

    def pass_times(hh):
        per = {}
        for axis in range(3):
            out = ctypes.c_double()
            _lib.check(L.gpss_time_pass(hh, axis, 1 if axis == 2 else 0, 20, c["dt"], ctypes.byref(out)), hh)
            per["xyz"[axis]] = out.value
        return per

    def roofline(per, tagform, ms_step):
        dom = max(per, key=per.get)
        achieved = alg_bytes / (per[dom] / 1e3) / 1e9
        step_gbs = BYTES_PER_CELL_PASS * cells * passes_per_call / (ms_step / 1e3) / 1e9
        return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": profiled_traffic(f"pass_{tagform}_{dom}_cfg1_{args.n}"), "kernel": f"fused {dom} pass",
                "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)" if peak_kind == "measured"
                else "fallback 6800 GB/s",
                "algorithmic_bytes_per_launch": alg_bytes, "ms_per_launch": per,
                "whole_step_gbs": step_gbs, "whole_step_frac": step_gbs / peak,
                "whole_step_bytes_per_cell_step": BYTES_PER_CELL_PASS * PASSES_PER_TIMESTEP,
                "note": "per-pass frac: 16 B/cell per launch (one read and one write of the FP32 field); "
                        "whole step: the 3 merged passes per time step (48 B/cell-step)"}

    per_axis = pass_times(h)
    roof = roofline(per_axis, "fp32c" if comp else "fp32", t_ms / args.steps)
    if comp:
        roof["note"] += ("; the compensated passes are bound by the FMA pipe (grid-exact two-float "
                         "arithmetic), not by HBM: see compute_fp32_pipe and profiles/")

    # ---- end to end through the public API with host buffers
    nbytes = int(cells) * 16
    e2e = None
    e2e_steps = 0
    if not args.no_e2e:
        hbuf = ctypes.c_void_p()
        _lib.check(L.gpss_host_alloc(ctypes.byref(hbuf), nbytes))
        host = np.frombuffer((ctypes.c_char * nbytes).from_address(hbuf.value), dtype=np.complex128)
        host[:] = c["psi"].reshape(-1, order="F")
        hp = ctypes.cast(hbuf, ctypes.POINTER(ctypes.c_double))
        e2e_steps = max(3, min(args.steps, 10))
        ck(L.gpss_upload(h, hp))
        ck(L.gpss_step(h, nt, 2, 0, c["dt"], None))
        ck(L.gpss_download(h, hp))
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            ck(L.gpss_upload(h, hp))
            ck(L.gpss_step(h, nt, 2, 0, c["dt"], None))
            ck(L.gpss_download(h, hp))
        ck(L.gpss_sync(h))
        e2e_s = dist.max(time.perf_counter() - t0)
        e2e = world * cells * nt * e2e_steps / e2e_s / 1e6
        del host
        _lib.check(L.gpss_host_free(hbuf))
    model.close(download=False)

    # ---- the other FP32 form on the same workload (the plain passes when the
    # compensated ones are the headline)
    other = None
    if not args.no_extra:
        f2 = sfd.Field(grid)
        f2.phi = c["psi"]
        p2 = sfd.GrossPitaevskiiParameters(sfd.PotentialZero(f2), coeffD=c["coeffD"], beta=c["beta"])
        m2 = sfd.NumModelSplit2(f2, p2, c["dt"], nt, nt, precision="fp32", compensated=not comp)
        h2 = m2.handle
        k2 = 5
        t2 = 0.0
        for i in range(k2 + 2):
            _lib.check(L.gpss_upload(h2, p0), h2)
            _lib.check(L.gpss_sync(h2), h2)
            _lib.check(L.gpss_event_record(h2, 0), h2)
            _lib.check(L.gpss_step(h2, nt, 2, 0, c["dt"], None), h2)
            _lib.check(L.gpss_flush(h2), h2)
            _lib.check(L.gpss_event_record(h2, 1), h2)
            _lib.check(L.gpss_event_elapsed(h2, 0, 1, ctypes.byref(ms)), h2)
            if i >= 2:
                t2 += ms.value
        per2 = pass_times(h2)
        m2.close(download=False)
        other = {"form": "compensated" if not comp else "plain", "value": cells * nt * k2 / (t2 / 1e3) / 1e6,
                 "unit": "Mcell-steps/s", "ms_per_step": t2 / k2, "steps": k2,
                 "roofline": roofline(per2, "fp32" if comp else "fp32c", t2 / k2)}

    # ---- measured FMA roofs (FP32 for the compensated passes, FP64 for the
    # FP64 kernels): both are bound by their FMA pipe, not by HBM
    peaks = {}
    for prec, key in ((32, "fp32_tflops"), (64, "fp64_tflops")):
        t = ctypes.c_double()
        if L.gpss_measure_fma_rate(prec, ctypes.byref(t)) == 0:
            peaks[key] = t.value
    # algorithmic flops per cell and time step (5 n log2 n per length-n FFT,
    # 6 per complex phase multiply, ~20 for the nonlinear factor): merged
    # step = 3 kinetic flows; the plain form = 2 half-step flows of 3 axes
    lg = math.log2(args.n)
    flops_merged = 3 * (2 * 5 * lg + 6) + 20
    flops_plain = 2 * 3 * (2 * 5 * lg + 6) + 20
    if peaks.get("fp32_tflops"):
        ach = flops_merged * value / world * 1e6 / 1e12
        roof["compute"] = {"unit": "TFLOP/s", "algorithmic_flops_per_cell_step": flops_merged,
                           "achieved": ach, "fp32_fma_peak_measured": peaks["fp32_tflops"],
                           "frac": ach / peaks["fp32_tflops"],
                           "note": "textbook FFT flops of the merged step (5 n log2 n per transform)"}
        if comp and args.n == 256:
            # the compensated passes are bound by the FMA pipe: their executed
            # FP32 operations (each lane of a packed f32x2 instruction counted,
            # an FMA counted once) against the measured FMA rate in the same
            # unit (FMA/s = FLOP/s / 2)
            peak_ops = peaks["fp32_tflops"] / 2
            xo = COMP_OPS_PER_CELL_PASS * cells / (per_axis["x"] * 1e-3) / 1e12
            so = (PASSES_PER_TIMESTEP * COMP_OPS_PER_CELL_PASS + NL_OPS_PER_CELL) * value / world * 1e6 / 1e12
            roof["compute_fp32_pipe"] = {
                "unit": "T FP32 ops/s", "peak": peak_ops,
                "peak_source": "gpss_measure_fma_rate (FP32 FMA chains, CUDA events)",
                "ops_per_cell_per_pass": COMP_OPS_PER_CELL_PASS, "nl_ops_per_cell": NL_OPS_PER_CELL,
                "x_pass_achieved": xo, "x_pass_frac": xo / peak_ops,
                "whole_step_achieved": so, "whole_step_frac": so / peak_ops,
                "note": "FP32 operations the compensated 256-point pass executes per cell (88.1 packed "
                        "f32x2 instructions: entering the grid 3, four DFT-16 51, two twiddles 21.1, "
                        "phase 12, final rounding 1); the x pass carries no nonlinear epilogue"}

    # ---- FP64 plain kernels on the same workload (fewer time steps)
    fp64 = None
    if not args.no_fp64:
        f64 = sfd.Field(grid)
        f64.phi = c["psi"]
        p64 = sfd.GrossPitaevskiiParameters(sfd.PotentialZero(f64), coeffD=c["coeffD"], beta=c["beta"])
        m64 = sfd.NumModelSplit2(f64, p64, c["dt"], 10, 10, precision="fp64", form="plain")
        h64 = m64.handle
        k64 = 10
        _lib.check(L.gpss_step(h64, 2, 2, 0, c["dt"], None), h64)
        _lib.check(L.gpss_event_record(h64, 0), h64)
        _lib.check(L.gpss_step(h64, k64, 2, 0, c["dt"], None), h64)
        _lib.check(L.gpss_event_record(h64, 1), h64)
        ms64 = ctypes.c_float()
        _lib.check(L.gpss_event_elapsed(h64, 0, 1, ctypes.byref(ms64)), h64)
        m64.close(download=False)
        v64 = cells * k64 / (ms64.value / 1e3) / 1e6
        fp64 = {"value": v64, "unit": "Mcell-steps/s", "timesteps": k64,
                "ms_per_timestep": ms64.value / k64, "fp32_over_fp64_plain": value / world / v64}
        if peaks.get("fp64_tflops"):
            ach64 = flops_plain * v64 * 1e6 / 1e12
            fp64["roofline"] = {"bound": "fp64_fma", "unit": "TFLOP/s", "algorithmic_flops_per_cell_step": flops_plain,
                                "achieved": ach64, "peak": peaks["fp64_tflops"], "frac": ach64 / peaks["fp64_tflops"],
                                "peak_source": "gpss_measure_fma_rate (FP64 FMA chains, CUDA events)"}
        if other:
            other["fp32_over_fp64_plain"] = other["value"] / v64

    # ---- batched runs (cfg3)
    batch = None
    if not args.no_batch:
        batch = measure_batch(sfd, W)

    # ---- accuracy, imaginary time (cfg2), adjoint (cfg4), cuFFT comparison
    extra = {}
    if not args.no_extra and rank == 0 and args.n == 256:
        extra["accuracy"] = measure_accuracy(sfd, c, oracle_mod())
        extra["imag_time"] = measure_imag(sfd, W, L)
        extra["adjoint"] = measure_adjoint(sfd, W)
        extra["rk4"] = measure_rk(sfd, c, L)
        extra["solve"] = measure_solve(sfd, c)
        extra["implicit"] = measure_implicit(sfd, W)
        extra["checkpoint"] = measure_checkpoint(sfd, c)
        cu = measure_cufft(c, args.n)
        if cu:
            cu["gpss_pass_ms"] = per_axis
            extra["cufft_comparison"] = cu

    # ---- CPU baseline (rank 0, N=1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        O = oracle_mod()
        v, cores, dt, _ = cpu_sample(c, O, 1, os.cpu_count() or 1)
        steps = max(1, min(128, int(12.0 / max(dt, 1e-3))))  # about 12 s of CPU work
        if steps > 1:
            v, cores, dt, _ = cpu_sample(c, O, steps, os.cpu_count() or 1)
        cpu = {"value": v / 1e6, "unit": "Mcell-steps/s", "cores": cores, "kind": "port",
               "sample": f"{steps} Strang time step(s) of cfg1 at {args.n}^3 on the FP64 C oracle "
                         f"(own radix-2 FFT, OpenMP), step loop {dt:.1f} s (setup not timed)"}

    dist.close()
    if rank != 0:
        return 0
    line = {
        "metric": METRIC,
        "value": value, "unit": "Mcell-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded cfg1 phase field, 64 modes |k|<=4)",
        "config": {"workload": workload_name(args.n),
                   "kernels": ("FP32 fused, compensated (double-float arithmetic, FP32 storage)" if comp
                               else "FP32 fused, plain"),
                   "grid": [args.n] * 3, "timesteps_per_step": nt,
                   "l2": "inputs larger than L2 (134 MB field, 268 MB streamed per pass); no flush",
                   "initial_field": "restored before every bench step (outside the timed events)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "gpu_launches": int(launches),
        "e2e": None if e2e is None else {"value": e2e, "unit": "Mcell-steps/s", "h2d_bytes_per_step": nbytes,
                                         "d2h_bytes_per_step": nbytes, "steps": e2e_steps},
        "roofline": roof,
        "fma_peaks_measured": peaks,
        "cpu_baseline": cpu,
        "fp64_plain": fp64,
        ("fp32_plain" if comp else "fp32_compensated"): other,
        "batched": batch,
    }
    line.update(extra)
    if clk:
        line["clocks"] = clk
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.only:
        return run_only(args)
    return run_gpss(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
