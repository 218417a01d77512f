"""Seeded synthetic inputs of the benchmark configurations.

No public dataset is involved: each configuration is a synthetic initial
state and potential with the shapes and value distributions of the
split-step workloads this library is measured on.  All seeds are fixed here;
tests, the bench and the oracle comparisons read the same arrays.

cfg0  2D 128^2 on [-8,8]^2, V = (x^2+y^2)/2, beta = 500, coeffD = -0.5,
      psi0 = exp(-(x^2+y^2)/4) e^{i theta}, theta = 16 Fourier modes with
      |k| <= 3, amplitudes N(0, 0.05^2); unit mass; dt = 1e-3, 1000 steps.
cfg1  3D 256^3 on [0,2pi]^3, V = 0, rho = 1, xi = 0.05, c = 1:
      coeffD = -c xi / sqrt(2), beta = c / (sqrt(2) xi) (so c = sqrt(2|coeffD| beta),
      xi = sqrt(|coeffD|/beta)); psi0 = e^{i theta}, 64 modes |k| <= 4,
      amplitudes N(0, 0.3^2); dt = 2.5e-3, 200 steps.
cfg2  3D 128^3 on [-10,10]^3, V = (x^2 + y^2 + 4 z^2)/2, beta = 2000, imaginary
      time; psi0 = unit-mass Gaussian + U(-1e-3, 1e-3) noise on re and im,
      renormalised; dt = 1e-3.
cfg3  512 independent 2D runs: 256 x 64^2, 192 x 128^2, 64 x 256^2, all on
      [-8,8]^2 (a box chosen here; the workload gives none), V = (a x^2 + b y^2)/2 with
      a, b ~ U(0.5, 2) plus 8 Gaussian bumps (heights U(0, 2), centres
      U(-6, 6)^2, width 0.5), g ~ U(100, 1000), psi0 = the trap's oscillator
      ground state times a cfg0-style phase imprint, unit mass; dt = 1e-3,
      500 steps; FP32 fields, FP64 masses.
cfg4  2D 256^2 on [-8,8]^2, trap V = (x^2+y^2)/2 plus a learnable V1 = 0,
      g = 500, dt = 1e-3, 2000 steps, checkpoints every 50 steps; psi0 as
      cfg0 (at 256^2); loss 1 - |<psi_target, psi(T)>|^2 with psi_target a
      seeded vortex dipole: the psi0 envelope times tanh(r+/0.5) tanh(r-/0.5)
      exp(i (atan2(y-y0, x-x0) - atan2(y-y0, x+x0))), vortices at (+-x0, y0),
      x0 ~ U(1, 2), y0 ~ U(-0.5, 0.5); unit mass.
"""
from __future__ import annotations

import math

import numpy as np

SQRT2 = math.sqrt(2.0)


def _coords(n, lo, hi):
    from . import grid_coords
    return grid_coords(n, lo, hi)


def _mesh(shape, bounds):
    xs = [_coords(n, b[0], b[1]) for n, b in zip(shape, bounds)]
    return np.meshgrid(*xs, indexing="ij")


def _modes(rng, count, kmax, L):
    """`count` integer wave-vector indices p with 0 < |2 pi p / L| <= kmax."""
    unit = [2 * math.pi / l for l in L]
    pmax = [int(math.floor(kmax / u)) for u in unit]
    cands = []
    for idx in np.ndindex(*[2 * p + 1 for p in pmax]):
        p = [i - pm for i, pm in zip(idx, pmax)]
        k2 = sum((pi * u) ** 2 for pi, u in zip(p, unit))
        if 0 < k2 <= kmax * kmax + 1e-12:
            cands.append(p)
    sel = rng.choice(len(cands), size=count, replace=len(cands) < count)
    return [cands[i] for i in sel], unit


def _phase_field(rng, shape, bounds, count, kmax, sigma):
    """theta = sum_m a_m cos(k_m . x + phi_m) on the grid nodes x_j = lo + j dx,
    evaluated exactly (integer modes) with one inverse FFT."""
    L = [b[1] - b[0] for b in bounds]
    ps, unit = _modes(rng, count, kmax, L)
    amps = rng.normal(0.0, sigma, size=count)
    phis = rng.uniform(0.0, 2 * math.pi, size=count)
    coef = np.zeros(shape, dtype=np.complex128)
    for p, a, ph in zip(ps, amps, phis):
        shift = sum(pi * u * b[0] for pi, u, b in zip(p, unit, bounds))
        idx = tuple(int(pi) % n for pi, n in zip(p, shape))
        coef[idx] += a * np.exp(1j * (ph + shift))
    try:  # multithreaded transform when scipy is present
        import scipy.fft as sfft
        theta = sfft.ifftn(coef, workers=-1).real
    except ImportError:
        theta = np.fft.ifftn(coef).real
    theta *= float(np.prod(shape))
    return theta


def _cis(theta):
    out = np.empty(theta.shape, dtype=np.complex128, order="F")
    out.real = np.cos(theta)
    out.imag = np.sin(theta)
    return out


def _unit_mass(psi, bounds):
    dV = np.prod([(b[1] - b[0]) / n for n, b in zip(psi.shape, bounds)])
    nrm = math.sqrt(float(np.sum(np.abs(psi) ** 2))) * math.sqrt(dV)
    return psi / nrm


def cfg0(n=128, seed=0):
    """2D trapped BEC with a seeded phase imprint (FP64 parity run)."""
    shape = (n, n)
    bounds = ((-8.0, 8.0), (-8.0, 8.0))
    rng = np.random.default_rng(1000 + seed)
    X, Y = _mesh(shape, bounds)
    theta = _phase_field(rng, shape, bounds, 16, 3.0, 0.05)
    psi = np.exp(-(X ** 2 + Y ** 2) / 4.0) * np.exp(1j * theta)
    psi = np.asfortranarray(_unit_mass(psi, bounds))
    V = np.asfortranarray(0.5 * (1 - 0.0) * (1.0 * X ** 2 + 1.0 * Y ** 2))
    return dict(name=f"cfg0-2d-{n}", shape=shape, bounds=bounds, psi=psi, V=V, coeffD=-0.5,
                beta=500.0, omega=0.0, dt=1e-3, nsteps=1000, imag=False)


def cfg1(n=256, seed=0):
    """3D quantum-turbulence-like phase field in a periodic box (headline)."""
    shape = (n, n, n)
    bounds = ((0.0, 2 * math.pi),) * 3
    rng = np.random.default_rng(2000 + seed)
    xi, c = 0.05, 1.0
    theta = _phase_field(rng, shape, bounds, 64, 4.0, 0.3)
    psi = _cis(np.asfortranarray(theta))
    return dict(name=f"cfg1-3d-{n}", shape=shape, bounds=bounds, psi=psi, V=None,
                coeffD=-c * xi / SQRT2, beta=c / (SQRT2 * xi), omega=0.0, dt=2.5e-3, nsteps=200,
                imag=False)


def cfg2(n=128, seed=0):
    """3D anisotropic trap, imaginary-time ground state."""
    shape = (n, n, n)
    bounds = ((-10.0, 10.0),) * 3
    rng = np.random.default_rng(3000 + seed)
    X, Y, Z = _mesh(shape, bounds)
    psi = np.exp(-0.5 * (X ** 2 + Y ** 2 + 2.0 * Z ** 2)).astype(np.complex128)
    psi = _unit_mass(psi, bounds)
    psi = psi + rng.uniform(-1e-3, 1e-3, size=shape) + 1j * rng.uniform(-1e-3, 1e-3, size=shape)
    psi = np.asfortranarray(_unit_mass(psi, bounds))
    V = np.asfortranarray(0.5 * (1 - 0.0) * (1.0 * X ** 2 + 1.0 * Y ** 2 + 4.0 * Z ** 2))
    return dict(name=f"cfg2-3d-{n}", shape=shape, bounds=bounds, psi=psi, V=V, coeffD=-0.5,
                beta=2000.0, omega=0.0, dt=1e-3, nsteps=200, imag=True)


def cfg4(n=256, seed=0):
    """2D gradient workload: trap + learnable potential, vortex-dipole target."""
    c = cfg0(n, seed)
    rng = np.random.default_rng(4000 + seed)
    X, Y = _mesh(c["shape"], c["bounds"])
    x0, y0 = rng.uniform(1.0, 2.0), rng.uniform(-0.5, 0.5)
    rp = np.hypot(X - x0, Y - y0)
    rm = np.hypot(X + x0, Y - y0)
    phase = np.arctan2(Y - y0, X - x0) - np.arctan2(Y - y0, X + x0)
    env = np.exp(-(X ** 2 + Y ** 2) / 4.0)
    tgt = env * np.tanh(rp / 0.5) * np.tanh(rm / 0.5) * np.exp(1j * phase)
    c.update(name=f"cfg4-2d-{n}", target=np.asfortranarray(_unit_mass(tgt, c["bounds"])), nsteps=2000, K=50)
    return c


def cfg3_run(n, seed):
    """One run of the batched workload (see cfg3)."""
    shape = (n, n)
    bounds = ((-8.0, 8.0), (-8.0, 8.0))
    rng = np.random.default_rng(5000 + seed)
    X, Y = _mesh(shape, bounds)
    a, b = rng.uniform(0.5, 2.0, size=2)
    V = 0.5 * (a * X ** 2 + b * Y ** 2)
    for _ in range(8):
        h = rng.uniform(0.0, 2.0)
        cx, cy = rng.uniform(-6.0, 6.0, size=2)
        V = V + h * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * 0.5 ** 2))
    g = rng.uniform(100.0, 1000.0)
    theta = _phase_field(rng, shape, bounds, 16, 3.0, 0.05)
    psi = np.exp(-0.5 * (np.sqrt(a) * X ** 2 + np.sqrt(b) * Y ** 2)) * np.exp(1j * theta)
    return dict(n=n, bounds=bounds, V=np.asfortranarray(V), beta=float(g),
                psi=np.asfortranarray(_unit_mass(psi, bounds)))


def cfg3(counts=(256, 192, 64), sizes=(64, 128, 256), seed=0):
    """The batched workload: a list of runs (sizes mixed, seeded) and dt, steps."""
    runs = []
    k = 0
    for cnt, n in zip(counts, sizes):
        for _ in range(cnt):
            runs.append(cfg3_run(n, seed * 100000 + k))
            k += 1
    return dict(name="cfg3-batch", runs=runs, coeffD=-0.5, dt=1e-3, nsteps=500)
