"""The FP32 nonlinear factor exp(-i theta), theta = (V + beta |psi|^2) dt
(splitting.jl:205-209), through every tier of the FP32 kernels: the micro
and tiny series (|theta| <= 1/16, <= 1/8), the short path without range
reduction (<= 0.78) and the double-float argument with Cody-Waite reduction
(up to 1e4 here), against float64 sin/cos of the float64 argument.

The factor is isolated with a one-step Lie split (L(dt) N(dt)) at coeffD = 0
on the compensated passes: the kinetic flow is then the identity to far
below FP32 rounding of the line's largest value, so the stored field is the
nonlinear epilogue applied to the input, rounded once.  What the identity
flow leaves on a cell is measured by the same run with the factor exactly 1
(beta = V = 0) and allowed on top.  Bound: 4 ulp of |psi| (2^-22 relative)
per cell -- one rounding of each factor component, the complex product and
the store."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ULP = 2.0 ** -24


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def _run(sfd, psi, V, beta, dt, bounds):
    g = sfd.Grid(psi.shape, bounds)
    f = sfd.Field(g)
    f.phi = psi
    pot = sfd.PotentialZero(f) if V is None else sfd.PotentialArray(f, V)
    p = sfd.GrossPitaevskiiParameters(pot, coeffD=0.0, beta=beta)
    n = sfd.NumModelSplit1(f, p, dt, 1, 1, precision="fp32", compensated=True, masslock=False)
    n.step(1)
    out = f.phi.copy()
    n.close()
    return out


@pytest.mark.parametrize("source", ["potential", "density"])
def test_nl_factor_all_tiers(sfd, source):
    nx, ny = 256, 64
    bounds = ((0.0, 1.0), (0.0, 1.0))
    rng = np.random.default_rng(5)
    dt = 1e-3
    ang = rng.uniform(0, 2 * np.pi, (nx, ny))
    if source == "potential":
        # |psi| ~ 1, theta = (V + |psi|^2) dt with V from 1e-6 to 1e7 along x
        amp = 1.0 + 0.25 * rng.uniform(-1, 1, (nx, ny))
        V = np.repeat(np.logspace(-6, 7, nx)[:, None], ny, axis=1).astype(np.float32).astype(np.float64)
        beta = 1.0
    else:
        # V = 0, theta = beta |psi|^2 dt with |psi|^2 from 1e-7 to 10 along x
        amp = np.repeat(np.sqrt(np.logspace(-7, 1, nx))[:, None], ny, axis=1) * (1 + 0.1 * rng.uniform(-1, 1, (nx, ny)))
        V = None
        beta = 1e6
    psi = (amp * np.exp(1j * ang)).astype(np.complex64).astype(np.complex128)
    psi = np.asfortranarray(psi)
    got = _run(sfd, psi, V, beta, dt, bounds)
    # the same passes with the factor exactly 1 (beta = V = 0): what the
    # kinetic identity itself leaves on each cell (a few 2^-24 of the cell
    # where |psi| is 1e-3.5 of its line's largest value, ~2^-40 elsewhere)
    kin = np.abs(_run(sfd, psi, None, 0.0, dt, bounds) - psi) / np.abs(psi)
    theta = ((0.0 if V is None else V) + beta * (psi.real ** 2 + psi.imag ** 2)) * dt
    want = np.exp(-1j * theta) * psi
    rel = np.abs(got - want) / np.abs(psi) - kin
    tiers = {"micro": theta <= 1 / 16, "tiny": (theta > 1 / 16) & (theta <= 0.125),
             "short": (theta > 0.125) & (theta <= 0.78), "reduced": theta > 0.78}
    report = {k: (int(m.sum()), float(rel[m].max()) / ULP if m.any() else 0.0) for k, m in tiers.items()}
    for k, (count, _) in report.items():
        assert count >= 64, f"tier {k} barely covered: {report}"
    assert theta.max() > 1e3
    assert rel.max() <= 4 * ULP, f"max error per tier in ulp: {report}"
