"""CPU oracle for the split-step Gross-Pitaevskii path -- TEST INFRASTRUCTURE ONLY.

Two independent FP64 restatements of SuperfluidDynamics.jl's `NumModelSplit1` /
`NumModelSplit2` path (src/NumModels/GrossPitaevskii/splitting.jl:78-82, 149-209):

* ``C*`` functions wrap ``gp_oracle.c`` (own radix-2 FFT, OpenMP), compiled by
  ``oracle/Makefile`` into ``oracle/_build/libgporacle.so``;
* ``np_*`` functions restate the same stages with ``numpy.fft`` (pocketfft), a
  second FFT implementation, for small cross-checks.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline arm use
this module, and only as the oracle.  Fields are numpy arrays of shape
``(nx, ny[, nz])`` in Fortran order, i.e. x fastest in memory like the
reference's Julia ``Array{ComplexF64}``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libgporacle.so")
_EXT_PATH = os.path.join(_HERE, "_build", "libgporacle_ext.so")
_lib = None
_ext = None

_i64p = ctypes.POINTER(ctypes.c_int64)
_f64p = ctypes.POINTER(ctypes.c_double)


def build(force: bool = False) -> str:
    """Compile gp_oracle.c (FP64 and extended builds) with oracle/Makefile."""
    # make rebuilds only what is out of date
    subprocess.run(["make", "-s", "-C", _HERE] + (["-B"] if force else []), check=True)
    return _LIB_PATH


class _Bound:
    """The or_* entry points of one build (suffix '' or '_ext')."""

    def __init__(self, path, suffix):
        L = ctypes.CDLL(path)
        g = lambda nm: getattr(L, nm + suffix)
        self.or_grid_coords = g("or_grid_coords")
        self.or_grid_coords.argtypes = [ctypes.c_int64, ctypes.c_double, ctypes.c_double, _f64p]
        self.or_fftfreq = g("or_fftfreq")
        self.or_fftfreq.argtypes = [ctypes.c_int64, ctypes.c_double, _f64p]
        self.or_norm = g("or_norm")
        self.or_norm.argtypes = [ctypes.c_int, _i64p, _f64p, _f64p, _f64p]
        self.or_norm.restype = ctypes.c_double
        self.or_fft_axis = g("or_fft_axis")
        self.or_fft_axis.argtypes = [ctypes.c_int, _i64p, _f64p, ctypes.c_int, ctypes.c_int]
        self.or_step = g("or_step")
        self.or_step.argtypes = [ctypes.c_int, _i64p, _f64p, _f64p, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, _f64p, _f64p, ctypes.c_int,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int]
        self.or_step_timed = g("or_step_timed")
        self.or_step_timed.argtypes = self.or_step.argtypes + [_f64p]
        self.or_derivatives = g("or_derivatives")
        self.or_derivatives.argtypes = [ctypes.c_int, _i64p, _f64p, _f64p, _f64p] + [_f64p] * 8
        self.or_energy = g("or_energy")
        self.or_energy.argtypes = [ctypes.c_int, _i64p, _f64p, _f64p, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_double, _f64p, _f64p, _f64p]
        self.or_rk_step = g("or_rk_step")
        self.or_rk_step.argtypes = [ctypes.c_int, _i64p, _f64p, _f64p, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_double, _f64p, _f64p, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int]
        self.or_implicit_step = g("or_implicit_step")
        self.or_implicit_step.argtypes = [ctypes.c_int, _i64p, _f64p, _f64p, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double, _f64p, _f64p, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                          ctypes.c_double, _i64p]
        self.or_max_threads = g("or_max_threads")
        self.or_max_threads.restype = ctypes.c_int


def lib(extended: bool = False):
    """FP64 oracle, or (extended=True) the long-double build of the same code."""
    global _lib, _ext
    if extended:
        if _ext is None:
            build()
            _ext = _Bound(_EXT_PATH, "_ext")
        return _ext
    if _lib is None:
        build()
        _lib = _Bound(_LIB_PATH, "")
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(_f64p)


def _geom(shape, bounds):
    nd = len(shape)
    n = np.array(list(shape) + [1] * (3 - nd), dtype=np.int64)
    lo = np.array([b[0] for b in bounds] + [0.0] * (3 - nd), dtype=np.float64)
    hi = np.array([b[1] for b in bounds] + [1.0] * (3 - nd), dtype=np.float64)
    return nd, n, lo, hi


def _field(psi):
    a = np.asfortranarray(psi, dtype=np.complex128)
    return a


# ------------------------------------------------------------------ grid --
def grid_coords(n: int, lo: float, hi: float) -> np.ndarray:
    """Grids.jl:78-84 node positions (LinRange(lo, hi, n+1)[1:end-1])."""
    out = np.empty(n, dtype=np.float64)
    lib().or_grid_coords(n, float(lo), float(hi), _p(out))
    return out


def fftfreq(n: int, d: float) -> np.ndarray:
    """Plans.jl:829-830 wavenumbers fftfreq(n, 2pi/d)."""
    out = np.empty(n, dtype=np.float64)
    lib().or_fftfreq(n, float(d), _p(out))
    return out


def spacing(shape, bounds):
    return [(b[1] - b[0]) / n for n, b in zip(shape, bounds)]


def quadratic_potential(shape, bounds, gammas=None, alpha=0.0):
    """PotentialQuadratic (src/Potentials/quadratic.jl:61-67):
    V = 0.5 (1 - alpha) (gx x^2 + gy y^2 [+ gz z^2]), evaluated in Julia's order."""
    nd = len(shape)
    gammas = gammas or [1.0] * nd
    xs = [grid_coords(n, b[0], b[1]) for n, b in zip(shape, bounds)]
    grids = np.meshgrid(*xs, indexing="ij")
    acc = gammas[0] * grids[0] ** 2
    for a in range(1, nd):
        acc = acc + gammas[a] * grids[a] ** 2
    return np.asfortranarray(0.5 * (1 - alpha) * acc)


# ---------------------------------------------------------------- C path --
def c_norm(psi, bounds) -> float:
    psi = _field(psi)
    nd, n, lo, hi = _geom(psi.shape, bounds)
    return lib().or_norm(nd, n.ctypes.data_as(_i64p), _p(lo), _p(hi), _p(psi))


def c_fft_axis(psi, axis: int, inverse: bool = False):
    out = _field(psi).copy(order="F")
    nd, n, lo, hi = _geom(out.shape, [(0, 1)] * out.ndim)
    rc = lib().or_fft_axis(nd, n.ctypes.data_as(_i64p), _p(out), axis,
                           1 if inverse else 0)
    assert rc == 0
    return out


def c_step(psi, bounds, *, coeffD=-0.5, beta=1.0, omega=0.0, V=None, nsteps=1, scheme=2,
           imag=False, dt=1e-3, nthreads=0, extended=False, inplace=False):
    """nsteps of NumModelSplit2 (scheme=2) or NumModelSplit1 (scheme=1).  Returns a
    new array (or steps `psi` itself when inplace=True and it is an F-ordered
    complex128 array).  extended=True runs the long-double build."""
    if inplace and isinstance(psi, np.ndarray) and psi.dtype == np.complex128 and psi.flags.f_contiguous:
        out = psi
    else:
        out = _field(psi).copy(order="F")
    nd, n, lo, hi = _geom(out.shape, bounds)
    Vp = None if V is None else np.asfortranarray(V, dtype=np.float64)
    rc = lib(extended).or_step(nd, n.ctypes.data_as(_i64p), _p(lo), _p(hi), coeffD, beta, omega,
                       _p(Vp), _p(out), int(nsteps), int(scheme),
                       1 if imag else 0, float(dt), int(nthreads))
    if rc != 0:
        raise ValueError("or_step failed")
    return out


def c_step_timed(psi, bounds, *, coeffD=-0.5, beta=1.0, omega=0.0, V=None, nsteps=1, scheme=2,
                 imag=False, dt=1e-3, nthreads=0):
    """c_step that also returns the seconds of the time-step loop alone (setup
    of grid, plans and field excluded): (field, seconds)."""
    out = _field(psi).copy(order="F")
    nd, n, lo, hi = _geom(out.shape, bounds)
    Vp = None if V is None else np.asfortranarray(V, dtype=np.float64)
    secs = ctypes.c_double(-1.0)
    L = lib()
    rc = L.or_step_timed(nd, n.ctypes.data_as(_i64p), _p(lo), _p(hi), coeffD, beta, omega, _p(Vp),
                         _p(out), int(nsteps), int(scheme), 1 if imag else 0, float(dt), int(nthreads),
                         ctypes.cast(ctypes.byref(secs), _f64p))
    if rc != 0:
        raise ValueError("or_step_timed failed")
    return out, secs.value


RK_STEPPERS = {"RK1": 1, "RK2": 2, "RK4": 4}
RK_FILTERS = {"none": 0, "product": 1, "solution": 2}


def c_rk_step(psi, bounds, *, coeffD=-0.5, beta=1.0, omega=0.0, V=None, nsteps=1, stepper="RK4",
              filter="product", dt=1e-3, nthreads=0, extended=False):
    """nsteps of NumModelGPRK.timeStep! (explicit-rk.jl:135-166)."""
    out = _field(psi).copy(order="F")
    nd, n, lo, hi = _geom(out.shape, bounds)
    Vp = None if V is None else np.asfortranarray(V, dtype=np.float64)
    rc = lib(extended).or_rk_step(nd, n.ctypes.data_as(_i64p), _p(lo), _p(hi), coeffD, beta, omega,
                                  _p(Vp), _p(out), int(nsteps), RK_STEPPERS[stepper], RK_FILTERS[filter],
                                  float(dt), int(nthreads))
    if rc != 0:
        raise ValueError("or_rk_step failed")
    return out


def np_rk_step(psi, bounds, *, coeffD=-0.5, beta=1.0, omega=0.0, V=None, nsteps=1, stepper="RK4",
               filter="product", dt=1e-3):
    """Same scheme as c_rk_step with numpy.fft (an independent transform): the
    right-hand side i[(sum_d L_d) psi - N(psi)] with L_d the per-axis spectral
    multipliers of lapRot (cD xi_x^2 - Om y xi_x, cD xi_y^2 + Om x xi_y, cD xi_z^2)."""
    p = np.array(psi, dtype=np.complex128, order="F", copy=True)
    nd = p.ndim
    shape = p.shape
    d = spacing(shape, bounds)
    xs = [grid_coords(n, b[0], b[1]) for n, b in zip(shape, bounds)]
    xis = [fftfreq(n, dd) for n, dd in zip(shape, d)]
    Vv = 0.0 if V is None else np.asarray(V, dtype=np.float64)

    def bshape(v, axis):
        s = [1] * nd
        s[axis] = v.size
        return v.reshape(s)

    xmax = (4.0 / 9.0) * min(float(np.max(x * x)) for x in xis)
    k2 = sum(bshape(x, a) ** 2 for a, x in enumerate(xis))
    mask = k2 < xmax

    def filt(f):
        return np.fft.ifftn(mask * np.fft.fftn(f))

    def rhs(q):
        lin = np.zeros_like(q)
        for a in range(nd):
            xi = bshape(xis[a], a)
            if a == 0 and nd >= 2:
                m = coeffD * (xi * xi) - omega * bshape(xs[1], 1) * xi
            elif a == 1:
                m = coeffD * (xi * xi) + omega * bshape(xs[0], 0) * xi
            else:
                m = coeffD * (xi * xi)
            lin += np.fft.ifft(m * np.fft.fft(q, axis=a), axis=a)
        nlt = (Vv + beta * (q.real ** 2 + q.imag ** 2)) * q
        if filter == "product":
            nlt = filt(nlt)
        return 1j * (lin - nlt)

    for _ in range(nsteps):
        if stepper == "RK1":
            p = p + dt * rhs(p)
        elif stepper == "RK2":
            k1 = rhs(p)
            p = p + dt * rhs(p + 0.5 * dt * k1)
        else:
            k1 = rhs(p)
            k2 = rhs(p + 0.5 * dt * k1)
            k3 = rhs(p + 0.5 * dt * k2)
            k4 = rhs(p + dt * k3)
            p = p + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
        if filter == "solution":
            p = filt(p)
    return np.asfortranarray(p)


IMPLICIT_SCHEMES = {"BackwardEuler": 0, "BackwardEulerNoPrecond": 1, "CrankNicolson": 2,
                    "CrankNicolsonQuasiNewton": 3, "CrankNicolsonT": 4, "CrankNicolsonQuasiNewtonT": 5}


def c_implicit_step(psi, bounds, *, scheme="BackwardEuler", coeffD=-0.5, beta=1.0, omega=0.0, V=None,
                    nsteps=1, dt=1e-3, nkrylov=70, tolkrylov=1e-8, nnewton=15, tolnewton=1e-6,
                    extended=False):
    """nsteps of one implicit scheme (backward-euler.jl / crank-nicolson.jl with
    the BiCGStab of krylov.jl).  Returns (psi, total Krylov count)."""
    out = _field(psi).copy(order="F")
    nd, n, lo, hi = _geom(out.shape, bounds)
    Vp = None if V is None else np.asfortranarray(V, dtype=np.float64)
    tot = np.zeros(1, dtype=np.int64)
    rc = lib(extended).or_implicit_step(nd, n.ctypes.data_as(_i64p), _p(lo), _p(hi), coeffD, beta, omega,
                                        _p(Vp), _p(out), int(nsteps), IMPLICIT_SCHEMES[scheme], float(dt),
                                        int(nkrylov), float(tolkrylov), int(nnewton), float(tolnewton),
                                        tot.ctypes.data_as(_i64p))
    if rc != 0:
        raise ValueError("or_implicit_step failed")
    return out, int(tot[0])


def np_implicit_step(psi, bounds, *, scheme="BackwardEuler", coeffD=-0.5, beta=1.0, omega=0.0, V=None,
                     nsteps=1, dt=1e-3, nkrylov=70, tolkrylov=1e-8, nnewton=15, tolnewton=1e-6):
    """The same schemes with numpy.fft and numpy reductions (independent of the
    C restatement): lapRot as the sum of the per-axis spectral multipliers."""
    p = np.array(psi, dtype=np.complex128, order="F", copy=True)
    nd = p.ndim
    d = spacing(p.shape, bounds)
    xs = [grid_coords(n, b[0], b[1]) for n, b in zip(p.shape, bounds)]
    xis = [fftfreq(n, dd) for n, dd in zip(p.shape, d)]
    Vv = 0.0 if V is None else np.asarray(V, dtype=np.float64)

    def bshape(v, axis):
        sh = [1] * nd
        sh[axis] = v.size
        return v.reshape(sh)

    def lap_rot(q):
        out = np.zeros_like(q)
        for a in range(nd):
            xi = bshape(xis[a], a)
            if a == 0 and nd >= 2:
                m = coeffD * (xi * xi) - omega * bshape(xs[1], 1) * xi
            elif a == 1:
                m = coeffD * (xi * xi) + omega * bshape(xs[0], 0) * xi
            else:
                m = coeffD * (xi * xi)
            out += np.fft.ifft(m * np.fft.fft(q, axis=a), axis=a)
        return out

    idt = 1.0 / dt
    st = {}

    def prodA(x):
        L = lap_rot(x)
        if scheme == "BackwardEuler":
            return x - st["M"] * L
        if scheme == "BackwardEulerNoPrecond":
            return (idt + st["Anl"]) * x - L
        if scheme == "CrankNicolson":
            return (idt + st["Anl"]) * x + 0.5 * st["Anl2"] * np.conj(x) - 0.5 * L
        if scheme == "CrankNicolsonQuasiNewton":
            return (idt + st["Anl"] * 0.5) * x - 0.5 * L
        if scheme == "CrankNicolsonT":
            return (1j * idt - 0.5 * st["Anl"]) * x - 0.5 * st["Anl2"] * np.conj(x) + 0.5 * L
        return (1j * idt - st["Anl"] * 0.5) * x + 0.5 * L

    def rdot(a, b):
        return float(np.sum((a * np.conj(b)).real))

    def krylov(phi, precond):
        M = st["M"] if precond else 1.0
        b = st["b"]
        normb = np.sqrt(rdot(M * b, M * b))
        r = M * (b - prodA(phi))
        r2 = r.copy()
        pp = r.copy()
        niter = 0
        for it in range(1, nkrylov + 1):
            Ap = M * prodA(pp)
            rr2 = rdot(r, r2)
            alpha = rr2 / rdot(Ap, r2)
            s_ = r - alpha * Ap
            As = M * prodA(s_)
            omega_ = rdot(As, s_) / rdot(As, As)
            phi += alpha * pp + omega_ * s_
            rr2old = rdot(r, r2)
            r = s_ - omega_ * As
            if np.sqrt(rdot(r, r)) / normb < tolkrylov:
                break
            niter = it
            beta_ = rdot(r, r2) / rr2old * alpha / omega_
            pp = r + beta_ * (pp - omega_ * Ap)
        return niter

    def normalize(q):
        return q / (np.sqrt(np.sum(np.abs(q) ** 2)) * np.sqrt(np.prod(d)))

    tot = 0
    for _ in range(nsteps):
        if scheme in ("BackwardEuler", "BackwardEulerNoPrecond"):
            a2 = np.abs(p) ** 2
            st["M"] = 1.0 / (idt + Vv + beta * a2)
            st["Anl"] = Vv + beta * a2
            st["b"] = st["M"] * p / dt if scheme == "BackwardEuler" else p / dt
            tot += krylov(p, False)
            p = normalize(p)
            continue
        tsch = scheme.endswith("T")
        newton = scheme in ("CrankNicolson", "CrankNicolsonT")
        phi1 = p.copy()
        phiw = np.zeros_like(p)
        for _ in range(nnewton):
            q = 0.5 * (phi1 + p)
            a2 = np.abs(q) ** 2
            st["Anl"] = Vv + (2 if newton else 3) * beta * a2
            st["Anl2"] = beta * q * q
            dd = (Vv + 3 * beta * a2) * 0.5
            st["M"] = 1.0 / ((1j * idt - dd) if tsch else (idt + dd))
            f = Vv + beta * a2
            if tsch:
                st["b"] = 1j * idt * (phi1 - p) - f * q + lap_rot(q)
            else:
                st["b"] = idt * (phi1 - p) + f * q - lap_rot(q)
            tot += krylov(phiw, True)
            phi1 = phi1 - phiw
            if np.sqrt(np.sum(np.abs(phiw) ** 2)) < tolnewton:
                break
        p = phi1 if tsch else normalize(phi1)
    return np.asfortranarray(p), tot


def c_derivatives(psi, bounds):
    """computeDerivatives!(GradientRotField) -> dict of dx, dy, [dz], ddx, ..., rx, ry."""
    psi = _field(psi)
    nd, n, lo, hi = _geom(psi.shape, bounds)
    names = ["dx", "dy", "dz", "ddx", "ddy", "ddz", "rx", "ry"]
    outs = {}
    ptrs = []
    for nm in names:
        axis = {"x": 0, "y": 1, "z": 2}[nm[-1]]
        if axis < nd and not (nm.startswith("r") and nd < 2):
            outs[nm] = np.zeros(psi.shape, dtype=np.complex128, order="F")
            ptrs.append(_p(outs[nm]))
        else:
            ptrs.append(None)
    rc = lib().or_derivatives(nd, n.ctypes.data_as(_i64p), _p(lo), _p(hi),
                              _p(psi), *ptrs)
    assert rc == 0
    return outs


def c_energy(psi, bounds, *, coeffD=-0.5, beta=1.0, omega=0.0, V=None, extended=False):
    """energy(n) of GrossPitaevskii.jl:61-136 -> (E_Omega, E_Delta, E_beta, E, mu)."""
    psi = _field(psi)
    nd, n, lo, hi = _geom(psi.shape, bounds)
    out = np.zeros(5, dtype=np.float64)
    Vp = None if V is None else np.asfortranarray(V, dtype=np.float64)
    rc = lib(extended).or_energy(nd, n.ctypes.data_as(_i64p), _p(lo), _p(hi), coeffD, beta, omega,
                         _p(Vp), _p(psi), _p(out))
    assert rc == 0
    return tuple(float(v) for v in out)


def max_threads() -> int:
    return int(lib().or_max_threads())


# ------------------------------------------------------------ numpy path --
def np_step(psi, bounds, *, coeffD=-0.5, beta=1.0, omega=0.0, V=None, nsteps=1, scheme=2,
            imag=False, dt=1e-3):
    """Same stages as c_step, with numpy.fft as the (independent) transform."""
    p = np.array(psi, dtype=np.complex128, order="F", copy=True)
    nd = p.ndim
    shape = p.shape
    d = spacing(shape, bounds)
    xs = [grid_coords(n, b[0], b[1]) for n, b in zip(shape, bounds)]
    xis = [fftfreq(n, dd) for n, dd in zip(shape, d)]
    Vv = None if V is None else np.asarray(V, dtype=np.float64)

    def bshape(v, axis):
        s = [1] * nd
        s[axis] = v.size
        return v.reshape(s)

    def lap(dtl):
        for a in range(nd):
            xi = bshape(xis[a], a)
            if a == 0 and nd >= 2:
                ph = coeffD * (xi * xi) - omega * bshape(xs[1], 1) * xi
            elif a == 1:
                ph = coeffD * (xi * xi) + omega * bshape(xs[0], 0) * xi
            else:
                ph = coeffD * (xi * xi)
            fac = np.exp(ph * dtl) if imag else np.exp(1j * (ph * dtl))
            p[...] = np.fft.ifft(fac * np.fft.fft(p, axis=a), axis=a)

    def nl(dtl):
        r = (0.0 if Vv is None else Vv) + beta * (p.real ** 2 + p.imag ** 2)
        fac = np.exp(-r * dtl) if imag else np.exp(1j * (-r * dtl))
        p[...] = fac * p

    for _ in range(nsteps):
        if scheme == 2:
            lap(dt * 0.5); nl(dt); lap(dt * 0.5)
        else:
            lap(dt); nl(dt)
        if imag:
            nrm = np.sqrt(np.sum(np.abs(p) ** 2)) * np.sqrt(np.prod(d))
            p /= nrm
    return p


def sp_step_timed(psi, bounds, *, coeffD=-0.5, beta=1.0, V=None, nsteps=1, dt=1e-3, workers=0):
    """Strang steps (scheme 2, real time, Omega = 0) with scipy.fft (pocketfft,
    threaded over `workers`) as the transform and numpy broadcasts (single
    threaded, like the reference's Julia broadcasts) for the phase and
    nonlinear stages: an FFTW-class CPU restatement for timing.  Returns
    (field, seconds of the step loop)."""
    import time
    import scipy.fft as sfft
    workers = workers or os.cpu_count() or 1
    p = np.array(psi, dtype=np.complex128, order="F", copy=True)
    nd = p.ndim
    d = spacing(p.shape, bounds)
    facs = []
    for a in range(nd):
        xi = fftfreq(p.shape[a], d[a])
        s = [1] * nd
        s[a] = xi.size
        facs.append(np.exp(1j * ((coeffD * (xi * xi)) * (dt * 0.5))).reshape(s))
    Vv = None if V is None else np.asarray(V, dtype=np.float64)
    t0 = time.perf_counter()
    for _ in range(nsteps):
        for half in range(2):
            for a in range(nd):
                p = sfft.ifft(facs[a] * sfft.fft(p, axis=a, workers=workers), axis=a, workers=workers)
            if half == 0:
                r = (0.0 if Vv is None else Vv) + beta * (p.real ** 2 + p.imag ** 2)
                p = np.exp(1j * (-r * dt)) * p
    return p, time.perf_counter() - t0


def rel_l2(a, b) -> float:
    """Relative L2 distance ||a-b|| / ||b|| (the reference's GPU test metric,
    test/runtests.jl:1416-1417)."""
    a = np.asarray(a); b = np.asarray(b)
    return float(np.sqrt(np.sum(np.abs(a - b) ** 2)) / np.sqrt(np.sum(np.abs(b) ** 2)))


def relerr_max(a, b) -> float:
    """Max-norm relative error, test/runtests.jl:5."""
    a = np.asarray(a); b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


# ------------------------------------------------- forward-mode (dual numbers) --
def np_tangent_loss(psi0, dpsi0, V, dV, psi_target, bounds, *, coeffD=-0.5, beta=1.0, nsteps=1, dt=1e-3):
    """Loss L = 1 - |<psi_target, psi(T)>|^2 of nsteps real-time Strang steps
    (splitting.jl:149-209, Omega = 0) and its directional derivative along
    (dpsi0, dV), by dual numbers: every value carries a tangent, the FFT stages
    are linear (the tangent goes through the same transform), the nonlinear
    stage psi_out = exp(-i theta) psi with theta = (V + beta|psi|^2) dt gives
    dpsi_out = exp(-i theta) (dpsi - i dtheta psi),
    dtheta = (dV + 2 beta Re(conj(psi) dpsi)) dt.  Returns (L, dL)."""
    p = np.array(psi0, dtype=np.complex128, order="F", copy=True)
    t = np.array(dpsi0, dtype=np.complex128, order="F", copy=True)
    nd = p.ndim
    shape = p.shape
    d = spacing(shape, bounds)
    xis = [fftfreq(n, dd) for n, dd in zip(shape, d)]
    Vv = np.zeros(shape) if V is None else np.asarray(V, dtype=np.float64)
    dVv = np.zeros(shape) if dV is None else np.asarray(dV, dtype=np.float64)

    def lap(dtl):
        for a in range(nd):
            s = [1] * nd
            s[a] = shape[a]
            xi = xis[a].reshape(s)
            fac = np.exp(1j * ((coeffD * (xi * xi)) * dtl))
            p[...] = np.fft.ifft(fac * np.fft.fft(p, axis=a), axis=a)
            t[...] = np.fft.ifft(fac * np.fft.fft(t, axis=a), axis=a)

    for _ in range(nsteps):
        lap(dt * 0.5)
        rho = p.real ** 2 + p.imag ** 2
        theta = (Vv + beta * rho) * dt
        dtheta = (dVv + 2.0 * beta * (p.real * t.real + p.imag * t.imag)) * dt
        f = np.exp(-1j * theta)
        t[...] = f * (t - 1j * dtheta * p)
        p[...] = f * p
        lap(dt * 0.5)
    cell = float(np.prod(d))
    z = np.sum(np.conj(psi_target) * p) * cell
    dz = np.sum(np.conj(psi_target) * t) * cell
    L = 1.0 - abs(z) ** 2
    dL = -2.0 * float(np.real(np.conj(z) * dz))
    return float(L), dL
