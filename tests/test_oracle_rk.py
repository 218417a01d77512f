"""The oracle's restatement of NumModelGPRK (explicit-rk.jl:96-166) against
an independent numpy restatement, a closed-form linear case and the schemes'
convergence orders (no GPU)."""
import math

import numpy as np
import pytest


def _field(shape, seed, amp=0.3):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(amp * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)))


@pytest.mark.parametrize("stepper", ["RK1", "RK2", "RK4"])
@pytest.mark.parametrize("filt", ["none", "product", "solution"])
@pytest.mark.parametrize("shape,omega", [((32, 16), 0.7), ((16, 8, 8), 0.0), ((8, 16, 8), 0.4)])
def test_c_rk_matches_numpy(O, stepper, filt, shape, omega):
    b = tuple((-4.0 + a, 3.0 + 2 * a) for a in range(len(shape)))
    p = _field(shape, 3)
    V = O.quadratic_potential(shape, b)
    kw = dict(coeffD=-0.5, beta=3.0, omega=omega, V=V, nsteps=5, stepper=stepper, filter=filt, dt=2e-3)
    assert O.rel_l2(O.c_rk_step(p, b, **kw), O.np_rk_step(p, b, **kw)) < 1e-13


@pytest.mark.parametrize("stepper,order", [("RK1", 1), ("RK2", 2), ("RK4", 4)])
def test_rk_linear_case_is_the_stability_polynomial(O, stepper, order):
    """beta = V = Omega = 0: every Fourier mode is multiplied per step by the
    Taylor polynomial of exp(z), z = i coeffD |xi|^2 dt, of the scheme's order."""
    shape, b = (16, 8, 16), ((-math.pi, math.pi), (-2.0, 2.0), (0.0, 3.0))
    p = _field(shape, 4)
    dt, nsteps = 2e-3, 7
    got = O.c_rk_step(p, b, coeffD=-0.5, beta=0.0, nsteps=nsteps, stepper=stepper, filter="none", dt=dt)
    k2 = 0
    for a, (n, bb) in enumerate(zip(shape, b)):
        xi = np.fft.fftfreq(n, (bb[1] - bb[0]) / n) * 2 * math.pi
        s = [1, 1, 1]
        s[a] = n
        k2 = k2 + xi.reshape(s) ** 2
    z = 1j * -0.5 * k2 * dt
    R = sum(z ** j / math.factorial(j) for j in range(order + 1))
    want = np.fft.ifftn(np.fft.fftn(p) * R ** nsteps)
    assert O.rel_l2(got, want) < 1e-13


@pytest.mark.parametrize("stepper,lo,hi", [("RK1", 0.85, 1.15), ("RK2", 1.85, 2.15), ("RK4", 3.7, 4.3)])
def test_rk_convergence_order(O, stepper, lo, hi):
    """Halving dt divides the error at a fixed time by 2^order (nonlinear,
    rotating, trapped 2D case; filter on the product keeps the order)."""
    shape, b = (32, 32), ((-6.0, 6.0), (-6.0, 6.0))
    X, Y = np.meshgrid(np.linspace(-6, 6, 32, endpoint=False), np.linspace(-6, 6, 32, endpoint=False), indexing="ij")
    p = np.asfortranarray(np.exp(-(X ** 2 + Y ** 2) / 2) * np.exp(0.3j * X) + 0j)
    V = O.quadratic_potential(shape, b)
    kw = dict(coeffD=-0.5, beta=1.0, omega=0.2, V=V, stepper=stepper, filter="product")
    T = 0.08
    ref = O.c_rk_step(p, b, nsteps=1280, dt=T / 1280, **{**kw, "stepper": "RK4"})
    errs = [O.rel_l2(O.c_rk_step(p, b, nsteps=m, dt=T / m, **kw), ref) for m in (40, 80)]
    assert lo < math.log2(errs[0] / errs[1]) < hi


def test_rk_filter_zeroes_high_modes(O):
    """filter = solution leaves no mode at or above the 2/3-rule bound."""
    shape, b = (32, 16), ((0.0, 2 * math.pi), (0.0, math.pi))
    p = _field(shape, 5)
    out = O.c_rk_step(p, b, coeffD=-0.5, beta=1.0, nsteps=1, stepper="RK1", filter="solution", dt=1e-3)
    F = np.fft.fftn(out)
    xis = [np.fft.fftfreq(n, (bb[1] - bb[0]) / n) * 2 * math.pi for n, bb in zip(shape, b)]
    xmax = 4.0 / 9.0 * min(np.max(x * x) for x in xis)
    k2 = xis[0][:, None] ** 2 + xis[1][None, :] ** 2
    assert np.max(np.abs(F[k2 >= xmax])) < 1e-12 * np.max(np.abs(F))
    assert np.min(np.abs(F[k2 < xmax])) > 0
