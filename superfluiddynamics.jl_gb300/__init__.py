"""GB300 split-step Gross-Pitaevskii integrator with SuperfluidDynamics.jl's API.

Host-side mirror of the reference's split-step path, written over the C ABI
of ``libgpss.so`` (include/gpss.h).  The names follow the reference:

=====================================  =============================================
reference (Julia)                      here
=====================================  =============================================
``Grid(size, bounds)``                 ``Grid(size, bounds)``   (Grids.jl:64-129)
``Field(grid, ComplexField())``        ``Field(grid)``          (Fields.jl:94-157)
``norm(f)`` / ``normalize!(f)``        ``norm(f)`` / ``normalize(f)`` (Fields.jl:172-200)
``GrossPitaevskiiParameters(...)``     ``GrossPitaevskiiParameters(...)`` (Parameters.jl:49-55)
``PotentialZero(f)``                   ``PotentialZero(f)``     (Potentials.jl:12-25)
``PotentialQuadratic(f; α, γx, ...)``  ``PotentialQuadratic(f, alpha, gx, gy, gz)`` (quadratic.jl)
``NumModelSplit1(f, p, Δt, n, fb)``    ``NumModelSplit1(f, p, dt, niter, freqbckp)`` (splitting.jl:58)
``NumModelSplit2(f, p, Δt, n, fb)``    ``NumModelSplit2(f, p, dt, niter, freqbckp)`` (splitting.jl:129)
``timeStep!(n)``                       ``timeStep(n[, nsteps])`` (splitting.jl:78, 149)
``energy(n[, show])``                  ``energy(n[, show])``    (GrossPitaevskii.jl:61, 106)
``solve!(n; istart)``                  ``solve(n, istart=1)``   (NumModels.jl:23-46)
``write!/read!(WriterSave(f); ...)``   ``WriterSave(f).write/read(prefix, istep)`` (Writers.jl:41-137)
=====================================  =============================================

Fields are numpy arrays of shape ``(nx, ny[, nz])`` in Fortran order: x is
fastest in memory, exactly like the reference's Julia arrays.  The model keeps
the field resident on the GPU; ``field.phi`` downloads it on access after the
model has stepped it.  The time stepping always runs in libgpss (CUDA); there
is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from ._lib import (GPSSError, GPSS_FP32, GPSS_FP64, GPSS_FLAG_COMPENSATED, GPSS_FLAG_ENERGY_CACHE,
                   GPSS_FLAG_NOMASSLOCK, GPSS_FLAG_NOMERGE, GPSS_FLAG_PIPE, GPSS_FLAG_PLAIN)

__all__ = ["Grid", "Field", "norm", "normalize", "GrossPitaevskiiParameters", "PotentialZero",
           "PotentialQuadratic", "NumModelSplit1", "NumModelSplit2", "timeStep", "energy",
           "solve", "BatchSplit2", "GPSSError", "version", "NumModelGPRK", "NumModelBackwardEuler", "NumModelBackwardEulerNoPrecond",
           "NumModelCrankNicolson", "NumModelCrankNicolsonQuasiNewton", "NumModelCrankNicolsonT",
           "NumModelCrankNicolsonQuasiNewtonT", "WriterSave", "read_h5_dataset"]

_f64p = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)


def version() -> str:
    return _lib.lib().gpss_version().decode()


# --------------------------------------------------------------------- Grid --
def _lerpi(j, d, a, b):
    t = j / d
    return (1 - t) * a + t * b


def grid_coords(n: int, lo: float, hi: float) -> np.ndarray:
    """Node positions of Grids.jl:78-84, ``LinRange(lo, hi, n+1)[1:end-1]``
    (Base.LinRange lerps, reproduced value by value)."""
    lo = float(lo); hi = float(hi)
    if n <= 1:
        return np.array([lo])
    first, last = _lerpi(0, n, lo, hi), _lerpi(n - 1, n, lo, hi)
    j = np.arange(n, dtype=np.float64)
    t = j / float(n - 1)
    return (1 - t) * first + t * last


class Grid:
    """Periodic grid of ``size`` nodes on ``bounds`` (Grids.jl:24-129)."""

    def __init__(self, size, bounds):
        size = tuple(int(v) for v in size)
        bounds = tuple((float(b[0]), float(b[1])) for b in bounds)
        if len(size) not in (2, 3) or len(bounds) != len(size):
            raise ValueError("Grid: size and bounds must both be 2D or 3D")
        for n, (lo, hi) in zip(size, bounds):
            if n <= 0 or not hi > lo:
                raise ValueError("Grid: need n > 0 and lo < hi on every axis")
        self.n = size
        self.min = tuple(b[0] for b in bounds)
        self.max = tuple(b[1] for b in bounds)
        self.L = tuple(hi - lo for lo, hi in bounds)
        self.delta = tuple(L / n for L, n in zip(self.L, size))
        self.data = tuple(grid_coords(n, lo, hi) for n, (lo, hi) in zip(size, bounds))

    ndim = property(lambda s: len(s.n))
    bounds = property(lambda s: tuple(zip(s.min, s.max)))
    x = property(lambda s: s.data[0])
    y = property(lambda s: s.data[1])
    z = property(lambda s: s.data[2] if len(s.n) > 2 else None)

    def __repr__(self):
        return f"Grid{self.ndim}D({'x'.join(map(str, self.n))} on {self.bounds})"


# -------------------------------------------------------------------- Field --
class Field:
    """Complex field on a Grid (Fields.jl:35-157); ``phi`` is its array."""

    def __init__(self, grid: Grid):
        self.g = grid
        self._phi = np.zeros(grid.n, dtype=np.complex128, order="F")
        self._owner = None  # model holding a newer copy on the device

    @property
    def phi(self) -> np.ndarray:
        if self._owner is not None and self._owner._device_newer:
            self._owner.download()
        return self._phi

    @phi.setter
    def phi(self, value):
        arr = np.asarray(value, dtype=np.complex128)
        if arr.shape != self.g.n:
            raise ValueError(f"phi must have shape {self.g.n}, got {arr.shape}")
        self._phi = np.asfortranarray(arr).copy(order="F")
        if self._owner is not None:
            self._owner.upload()

    def mesh(self):
        """Broadcastable coordinate arrays (x, y[, z]), the reference's ``f.x``, ``f.y``."""
        nd = self.g.ndim
        out = []
        for a in range(nd):
            shape = [1] * nd
            shape[a] = self.g.n[a]
            out.append(self.g.data[a].reshape(shape))
        return tuple(out)

    x = property(lambda s: s.mesh()[0])
    y = property(lambda s: s.mesh()[1])
    z = property(lambda s: s.mesh()[2] if s.g.ndim > 2 else None)


def norm(f: Field) -> float:
    """Fields.jl:172-180, ``sqrt(sum |phi|^2) * sqrt(dx dy [dz])``.  Uses the
    device copy when a model owns the field."""
    if f._owner is not None:
        return f._owner.norm()
    a = f._phi
    s = float(np.sum(a.real * a.real + a.imag * a.imag))
    return math.sqrt(s) * math.sqrt(float(np.prod(f.g.delta)))


def normalize(f: Field) -> None:
    """Fields.jl:196-200, ``phi ./= norm(f)`` (on the device when a model owns it)."""
    if f._owner is not None:
        f._owner.normalize()
        return
    f._phi /= norm(f)


# --------------------------------------------------------- parameters/pots --
class PotentialZero:
    """V = 0 (Potentials.jl:12-25)."""

    def __init__(self, f: Field):
        self.f = f
        self.V = np.zeros(f.g.n, dtype=np.float64, order="F")
        self.is_zero = True


class PotentialQuadratic:
    """V = 0.5 (1 - alpha) (gx x^2 + gy y^2 [+ gz z^2])  (quadratic.jl:29-67)."""

    def __init__(self, f: Field, alpha=0.0, gx=1.0, gy=1.0, gz=1.0):
        self.f = f
        self.alpha, self.gx, self.gy, self.gz = float(alpha), float(gx), float(gy), float(gz)
        X = f.mesh()
        acc = self.gx * X[0] ** 2 + self.gy * X[1] ** 2
        if f.g.ndim > 2:
            acc = acc + self.gz * X[2] ** 2
        self.V = np.asfortranarray(0.5 * (1 - self.alpha) * acc)
        self.is_zero = False


class PotentialArray:
    """Any real array as the potential (what the C ABI's gpss_set_potential takes)."""

    def __init__(self, f: Field, V):
        self.f = f
        self.V = np.asfortranarray(np.asarray(V, dtype=np.float64))
        if self.V.shape != f.g.n:
            raise ValueError("potential shape must match the grid")
        self.is_zero = False


class GrossPitaevskiiParameters:
    """i dphi/dt = coeffD Lap phi + beta |phi|^2 phi + V phi - i Omega Lz phi (Parameters.jl:17-55)."""

    def __init__(self, pot, coeffD=-0.5, beta=1.0, Omega=0.0):
        self.coeffD = float(coeffD)
        self.beta = float(beta)
        self.pot = pot
        self.Omega = float(Omega)


# ------------------------------------------------------------------- models --
_PRECISION = {"fp64": GPSS_FP64, "fp32": GPSS_FP32, 64: GPSS_FP64, 32: GPSS_FP32}


class _SplitModel:
    scheme = 2

    def __init__(self, f: Field, param: GrossPitaevskiiParameters, dt, niter, freqbckp, *,
                 precision="fp64", form="fused", merge=True, masslock=True, pipeline=False,
                 energy_cache=False, compensated=False, writers=()):
        if f._owner is not None:
            raise ValueError("this field already belongs to a model")
        if form not in ("fused", "plain"):
            raise ValueError("form must be 'fused' or 'plain'")
        self.f = f
        self.param = param
        self.dt = float(dt)
        self.niter = int(niter)
        self.freqbckp = int(freqbckp)
        self.precision = precision
        self.form = form
        self.writers = list(writers)
        self._device_newer = False
        L = _lib.lib()
        g = f.g
        nd = g.ndim
        n = (ctypes.c_int64 * 3)(*(list(g.n) + [1] * (3 - nd)))
        lo = (ctypes.c_double * 3)(*(list(g.min) + [0.0] * (3 - nd)))
        hi = (ctypes.c_double * 3)(*(list(g.max) + [1.0] * (3 - nd)))
        flags = ((GPSS_FLAG_PLAIN if form == "plain" else 0) | (0 if merge else GPSS_FLAG_NOMERGE)
                 | (0 if masslock else GPSS_FLAG_NOMASSLOCK) | (GPSS_FLAG_PIPE if pipeline else 0)
                 | (GPSS_FLAG_ENERGY_CACHE if energy_cache else 0)
                 | (GPSS_FLAG_COMPENSATED if compensated else 0))
        h = ctypes.c_void_p()
        _lib.check(L.gpss_create(ctypes.byref(h), nd, n, lo, hi, _PRECISION[precision], flags))
        self._h = h
        try:
            self.set_params(param)
            f._owner = self
            self.upload()
        except Exception:
            L.gpss_destroy(h)
            self._h = None
            raise

    # -- plumbing
    def _ck(self, rc):
        return _lib.check(rc, self._h)

    def set_params(self, param: GrossPitaevskiiParameters):
        L = _lib.lib()
        self.param = param
        self._ck(L.gpss_set_params(self._h, param.coeffD, param.beta, param.Omega))
        pot = param.pot
        if pot is None or getattr(pot, "is_zero", False):
            self._ck(L.gpss_set_potential(self._h, None))
        else:
            V = np.asfortranarray(np.asarray(pot.V, dtype=np.float64))
            if V.shape != self.f.g.n:
                raise ValueError("potential shape must match the grid")
            self._ck(L.gpss_set_potential(self._h, V.ctypes.data_as(_f64p)))

    def upload(self):
        a = np.asfortranarray(self.f._phi, dtype=np.complex128)
        self._ck(_lib.lib().gpss_upload(self._h, a.ctypes.data_as(_f64p)))
        self._device_newer = False

    def download(self):
        a = self.f._phi
        if not (a.flags.f_contiguous and a.dtype == np.complex128):
            a = np.zeros(self.f.g.n, dtype=np.complex128, order="F")
        self._ck(_lib.lib().gpss_download(self._h, a.ctypes.data_as(_f64p)))
        self.f._phi = a
        self._device_newer = False

    def close(self, download=True):
        """Release the device context (downloading the field first by default)."""
        if getattr(self, "_h", None):
            if download and self._device_newer:
                self.download()
            _lib.lib().gpss_destroy(self._h)
            self._h = None
            self.f._owner = None

    def __del__(self):
        try:
            self.close(download=False)
        except Exception:
            pass

    # -- physics
    def step(self, nsteps=1, imag=False, diag=False):
        d = _lib.Diag() if diag else None
        self._ck(_lib.lib().gpss_step(self._h, int(nsteps), self.scheme, 1 if imag else 0, self.dt,
                                      ctypes.byref(d) if d is not None else None))
        self._device_newer = True
        if d is not None:
            return {"mass": d.mass, "energy": tuple(d.energy), "steps": d.steps}
        return None

    def energies(self):
        out = (ctypes.c_double * 5)()
        self._ck(_lib.lib().gpss_energy(self._h, out))
        return tuple(out)

    def mass(self):
        out = ctypes.c_double()
        self._ck(_lib.lib().gpss_mass(self._h, ctypes.byref(out)))
        return out.value

    def norm(self):
        out = ctypes.c_double()
        self._ck(_lib.lib().gpss_norm(self._h, ctypes.byref(out)))
        return out.value

    def normalize(self):
        self._ck(_lib.lib().gpss_normalize(self._h))
        self._device_newer = True

    def ground_state(self, tol=1e-10, max_steps=100000, check_every=10):
        mu = ctypes.c_double()
        steps = ctypes.c_int64()
        self._ck(_lib.lib().gpss_ground_state(self._h, self.dt, float(tol), int(max_steps),
                                              int(check_every), ctypes.byref(mu),
                                              ctypes.byref(steps)))
        self._device_newer = True
        return mu.value, steps.value

    def adjoint(self, psi_target, nsteps, K=50):
        """Loss L = 1 - |<psi_target, psi(T)>|^2 after nsteps Strang steps from
        the current field, with dL/dV (real, field shape) and the Wirtinger
        gradient 2 dL/d conj(psi0).  The field is left unchanged."""
        tgt = np.asfortranarray(np.asarray(psi_target, dtype=np.complex128))
        if tgt.shape != self.f.g.n:
            raise ValueError("psi_target must have the field's shape")
        loss = ctypes.c_double()
        dv = np.zeros(self.f.g.n, dtype=np.float64, order="F")
        gp = np.zeros(self.f.g.n, dtype=np.complex128, order="F")
        self._ck(_lib.lib().gpss_adjoint(self._h, tgt.ctypes.data_as(_f64p), int(nsteps), int(K), self.dt,
                                         ctypes.byref(loss), dv.ctypes.data_as(_f64p), gp.ctypes.data_as(_f64p)))
        return loss.value, dv, gp

    def timestep_value(self):
        return self.scheme

    @property
    def handle(self):
        return self._h

    def __repr__(self):
        return (f"Splitting Order {self.scheme}\n  ├───────  time step: {self.dt}\n"
                f"  └──────────── solve: number of iterations {self.niter}, "
                f"backup frequency {self.freqbckp}")


class NumModelSplit1(_SplitModel):
    """First-order Lie splitting, L(dt) N(dt) (splitting.jl:1-82)."""
    scheme = 1


class NumModelSplit2(_SplitModel):
    """Second-order Strang splitting, L(dt/2) N(dt) L(dt/2) (splitting.jl:84-154)."""
    scheme = 2


class NumModelGPRK(_SplitModel):
    """Explicit Runge-Kutta integrator of the time-dependent GP equation,
    NumModelGPRK(f, param, dt, niter, freqbckp; stepper="RK4", filter=:product)
    (explicit-rk.jl:1-167): stepper "RK1" | "RK2" | "RK4", filter "product"
    (2/3 rule on the nonlinear term of every stage) | "solution" (on the state
    after every step) | "none".  timeStep returns 0 as the reference does."""
    scheme = 0
    _STEPPERS = {"RK1": 1, "RK2": 2, "RK4": 4}
    _FILTERS = {"none": 0, "product": 1, "solution": 2}

    def __init__(self, f: Field, param: GrossPitaevskiiParameters, dt, niter, freqbckp, *,
                 stepper="RK4", filter="product", precision="fp64", writers=()):
        filt = filter.lstrip(":") if isinstance(filter, str) else filter
        if filt not in self._FILTERS:
            raise ValueError(f"NumModelGPRK filter {filter} unknown (use :product, :solution or :none).")
        self.stepper = stepper
        self.filter = filt
        super().__init__(f, param, dt, niter, freqbckp, precision=precision, writers=writers)

    def step(self, nsteps=1, imag=False, diag=False):
        if imag:
            raise ValueError("NumModelGPRK integrates in real time only")
        if self.stepper not in self._STEPPERS:
            raise ValueError(f'NumModelGPRK stepper "{self.stepper}" unknown (use "RK1", "RK2" or "RK4").')
        self._ck(_lib.lib().gpss_rk_step(self._h, int(nsteps), self._STEPPERS[self.stepper],
                                         self._FILTERS[self.filter], self.dt))
        self._device_newer = True
        if diag:
            eom, edel, ebeta, e, mu = self.energies()
            return {"mass": self.mass(), "energy": (eom, edel, ebeta, e, mu), "steps": int(nsteps)}
        return None

    def __repr__(self):
        return (f"Gross-Pitaevskii explicit {self.stepper} (2/3 filter: {self.filter})\n"
                f"  ├───────  time step: {self.dt}\n"
                f"  └──────────── solve: number of iterations {self.niter}, backup frequency {self.freqbckp}")


class _ImplicitModel(_SplitModel):
    """Common part of the implicit schemes: a linear system per step (per
    Newton iteration for Crank-Nicolson) solved by the reference's BiCGStab
    (krylov.jl).  timeStep returns the summed Krylov counts, as the reference's
    timeStep! does."""
    scheme = 0
    implicit = 0
    newton = False

    def __init__(self, f: Field, param: GrossPitaevskiiParameters, dt, niter, freqbckp, *, nkrylov=70,
                 tolkrylov=1e-8, nnewton=15, tolnewton=1e-6, precision="fp64", writers=()):
        self.nkrylov = int(nkrylov)
        self.tolkrylov = float(tolkrylov)
        self.nnewton = int(nnewton)
        self.tolnewton = float(tolnewton)
        self.last_krylov = 0
        super().__init__(f, param, dt, niter, freqbckp, precision=precision, writers=writers)

    def step(self, nsteps=1, imag=False, diag=False):
        k = ctypes.c_int64()
        self._ck(_lib.lib().gpss_implicit_step(self._h, int(nsteps), self.implicit, self.dt, self.nkrylov,
                                               self.tolkrylov, self.nnewton, self.tolnewton, ctypes.byref(k)))
        self._device_newer = True
        self.last_krylov = k.value
        if diag:
            eom, edel, ebeta, e, mu = self.energies()
            return {"mass": self.mass(), "energy": (eom, edel, ebeta, e, mu), "steps": int(nsteps)}
        return None

    def timestep_value(self):
        return self.last_krylov

    def __repr__(self):
        lines = [self._title, f"  ├──────────  krylov: n iterations {self.nkrylov}, tolerance {self.tolkrylov}"]
        if self.newton:
            lines.append(f"  ├──────────  newton: n iterations {self.nnewton}, tolerance {self.tolnewton}")
        lines += [f"  ├───────  time step: {self.dt}",
                  f"  └──────────── solve: number of iterations {self.niter}, backup frequency {self.freqbckp}"]
        return "\n".join(lines)


class NumModelBackwardEuler(_ImplicitModel):
    """Preconditioned backward Euler in imaginary time (backward-euler.jl:1-90)."""
    implicit = 0
    _title = "Backward Euler"


class NumModelBackwardEulerNoPrecond(_ImplicitModel):
    """Backward Euler without preconditioning (backward-euler.jl:92-197)."""
    implicit = 1
    _title = "Backward Euler without preconditionning"


class NumModelCrankNicolson(_ImplicitModel):
    """Stationary Crank-Nicolson, Newton-Raphson (crank-nicolson.jl:1-123)."""
    implicit = 2
    newton = True
    _title = "Stationnary Crank-Nicolson Newton-Raphson scheme"


class NumModelCrankNicolsonQuasiNewton(_ImplicitModel):
    """Stationary Crank-Nicolson, quasi-Newton (crank-nicolson.jl:125-245)."""
    implicit = 3
    newton = True
    _title = "Stationnary Crank-Nicolson Quasi-Newton scheme"


class NumModelCrankNicolsonT(_ImplicitModel):
    """Time-dependent Crank-Nicolson, Newton-Raphson (crank-nicolson.jl:247-368)."""
    implicit = 4
    newton = True
    _title = "Time dependant Crank-Nicolson Newton-Raphson scheme"


class NumModelCrankNicolsonQuasiNewtonT(_ImplicitModel):
    """Time-dependent Crank-Nicolson, quasi-Newton (crank-nicolson.jl:370-489)."""
    implicit = 5
    newton = True
    _title = "Time dependant Crank-Nicolson Quasi-Newton scheme"


def timeStep(n: _SplitModel, nsteps: int = 1) -> int:
    """timeStep!(n): one (or nsteps) steps; returns what the reference's
    timeStep! returns (1 for Lie, 2 for Strang, splitting.jl:81, 153; 0 for
    explicit RK; the Krylov iteration count for the implicit schemes)."""
    n.step(nsteps)
    return n.timestep_value()


def energy(n: _SplitModel, show: bool = False):
    """energy(n) (GrossPitaevskii.jl:61-136) -> (E_Omega, E_Delta, E_beta, E)."""
    eom, edel, ebeta, e, mu = n.energies()
    if show:
        if n.f.g.ndim == 2:
            print(f"Chemical potential : {mu}")
        print(f"Angular Momentum Energy : {eom}")
        print(f"Kinetic + Potential Energy : {edel}")
        print(f"Interaction Energy : {ebeta}")
        print(f"Total Energy: {e}")
    return eom, edel, ebeta, e


def chemical_potential(n: _SplitModel) -> float:
    """mu = -E_Omega + E_Delta + 2 E_beta (GrossPitaevskii.jl:79)."""
    return n.energies()[4]


class WriterSave:
    """WriterSave(f) (Writers.jl:17-20; write! :41-92, read! :115-137): the
    field as "<prefix>-<istep>.h5" holding float64 datasets "re" and "im"
    (dataspace (nz, ny, nx) / (ny, nx), x fastest, as Julia writes its
    column-major arrays).  A field owned by a model is written from the
    device buffer and read straight back into it; the library writes the
    HDF5 structures itself (gpss_write_h5 / gpss_h5_write_field).  An
    instance is also a writer hook for ``solve``."""

    def __init__(self, f: Field):
        self.f = f

    @staticmethod
    def path(prefix="res", istep=0):
        return f"{prefix}-{int(istep)}.h5"

    def _shape(self):
        g = self.f.g
        return g.ndim, (ctypes.c_int64 * 3)(*(list(g.n) + [1] * (3 - g.ndim)))

    def write(self, prefix="res", istep=0, dt=1.0):
        path = self.path(prefix, istep).encode()
        owner = self.f._owner
        if owner is not None and owner._h:
            owner._ck(_lib.lib().gpss_write_h5(owner._h, path))
            return
        nd, n = self._shape()
        a = np.asfortranarray(self.f._phi, dtype=np.complex128)
        _lib.check(_lib.lib().gpss_h5_write_field(path, nd, n, a.ctypes.data_as(_f64p)))

    def read(self, prefix="res", istep=0, dt=1.0):
        path = self.path(prefix, istep).encode()
        owner = self.f._owner
        if owner is not None and owner._h:
            owner._ck(_lib.lib().gpss_read_h5(owner._h, path))
            owner._device_newer = True  # the host copy is stale until read
            return
        nd, n = self._shape()
        a = np.zeros(self.f.g.n, dtype=np.complex128, order="F")
        _lib.check(_lib.lib().gpss_h5_read_field(path, nd, n, a.ctypes.data_as(_f64p)))
        self.f._phi = a

    def __call__(self, field, prefix, istep, dt):
        self.write(prefix, istep, dt)


def read_h5_dataset(path, name):
    """Any float dataset of an HDF5 file's root group, as a float64 array of
    the dataset's (row-major) shape."""
    L = _lib.lib()
    rank = ctypes.c_int()
    dims = (ctypes.c_int64 * 8)()
    _lib.check(L.gpss_h5_read_dataset(str(path).encode(), name.encode(), ctypes.byref(rank), dims, None, 0))
    shape = tuple(dims[i] for i in range(rank.value))
    out = np.zeros(shape, dtype=np.float64)
    _lib.check(L.gpss_h5_read_dataset(str(path).encode(), name.encode(), ctypes.byref(rank), dims,
                                      out.ctypes.data_as(_f64p), out.size))
    return out


def solve(n: _SplitModel, istart: int = 1):
    """solve!(n; istart) (NumModels.jl:23-46): energy then timeStep! every
    iteration, writers every freqbckp iterations.  Writers are callables
    ``w(field, prefix, istep, dt)``.  A model made with ``energy_cache=True``
    (real time, Omega = 0, fused) measures the energies inside each step's
    last passes, so the energy call of the next iteration launches nothing."""
    res = []
    nkt = 0
    for w in n.writers:
        w(n.f, "res", istart, n.dt)
    for it in range(istart, istart + n.niter + 1):
        E = energy(n)
        nk = timeStep(n)
        nkt += nk
        res.append((nk, nkt) + tuple(E))
        if it % n.freqbckp == 0:
            for w in n.writers:
                w(n.f, "res", it, n.dt)
    return res


class BatchSplit2:
    """Many independent 2D NumModelSplit2 runs (FP32 fields, FP64 masses)
    advanced together by one persistent kernel launch (gpss_batch_*).

    sizes: grid size n of each run (n x n, n in {64, 128, 256});
    bounds: ((xmin, xmax), (ymin, ymax)) per run."""

    def __init__(self, sizes, bounds, coeffD=-0.5):
        L = _lib.lib()
        self.sizes = [int(n) for n in sizes]
        self.bounds = [tuple(tuple(float(v) for v in ax) for ax in b) for b in bounds]
        nr = len(self.sizes)
        n = (ctypes.c_int64 * nr)(*self.sizes)
        lo = (ctypes.c_double * (2 * nr))(*[b[a][0] for b in self.bounds for a in range(2)])
        hi = (ctypes.c_double * (2 * nr))(*[b[a][1] for b in self.bounds for a in range(2)])
        h = ctypes.c_void_p()
        rc = L.gpss_batch_create(ctypes.byref(h), nr, n, lo, hi, float(coeffD))
        if rc != 0:
            raise GPSSError(rc, "gpss_batch_create failed (sizes must be 64, 128 or 256; a GPU is needed)")
        self._h = h

    def _ck(self, rc):
        if rc != 0:
            msg = _lib.lib().gpss_batch_last_error(self._h)
            raise GPSSError(rc, msg.decode() if msg else "")

    def set_run(self, r, beta, V, psi):
        n = self.sizes[r]
        p = np.asfortranarray(np.asarray(psi, dtype=np.complex128))
        if p.shape != (n, n):
            raise ValueError("psi shape must be (n, n) of that run")
        Vp = None
        if V is not None:
            Vp = np.asfortranarray(np.asarray(V, dtype=np.float64))
            if Vp.shape != (n, n):
                raise ValueError("V shape must be (n, n) of that run")
        self._ck(_lib.lib().gpss_batch_set_run(self._h, int(r), float(beta),
                                               None if Vp is None else Vp.ctypes.data_as(_f64p),
                                               p.ctypes.data_as(_f64p)))

    def step(self, nsteps, dt):
        m = np.zeros(len(self.sizes), dtype=np.float64)
        self._ck(_lib.lib().gpss_batch_step(self._h, int(nsteps), float(dt), m.ctypes.data_as(_f64p)))
        return m

    def download(self, r):
        n = self.sizes[r]
        out = np.zeros((n, n), dtype=np.complex128, order="F")
        self._ck(_lib.lib().gpss_batch_download(self._h, int(r), out.ctypes.data_as(_f64p)))
        return out

    def tuning(self):
        """The launch choice: policy (0: runs up to 128^2 in shared memory, 1: up
        to 64^2), queue order (0: largest first, 1: as given), stack level (runs
        of one size and box as planes through the pass kernels: 1 the 256^2
        runs, 2 also 128^2, 3 every size) and the 16 trial times in ms (index
        4 stack + 2 policy + order; 1e30 for candidates not tried)."""
        pol, order, stack = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ms = (ctypes.c_float * 16)()
        self._ck(_lib.lib().gpss_batch_tuning(self._h, ctypes.byref(pol), ctypes.byref(order), ctypes.byref(stack),
                                              ms))
        return {"policy": pol.value, "order": order.value, "stack": stack.value, "trial_ms": list(ms)}

    def set_tuning(self, policy, order, stack=0):
        """Fix the launch choice (skips the autotuner); stack level 0 to 3."""
        self._ck(_lib.lib().gpss_batch_set_tuning(self._h, int(policy), int(order), int(stack)))

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().gpss_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
