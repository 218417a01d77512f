"""NumModelGPRK on the GPU (gpss_rk_step) against the oracle's restatement of
explicit-rk.jl:96-166.  Bars: FP64 rel-L2 <= 1e-12, FP32 <= 1e-5."""
import numpy as np
import pytest

from helpers import random_field

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def run_rk(sfd, shape, bounds, psi0, *, V=None, precision="fp64", nsteps=1, calls=1, **kw):
    g = sfd.Grid(shape, bounds)
    f = sfd.Field(g)
    f.phi = psi0
    pot = sfd.PotentialZero(f) if V is None else sfd.PotentialArray(f, V)
    p = sfd.GrossPitaevskiiParameters(pot, coeffD=kw.get("coeffD", -0.5), beta=kw.get("beta", 1.0),
                                      Omega=kw.get("omega", 0.0))
    n = sfd.NumModelGPRK(f, p, kw["dt"], nsteps, nsteps, stepper=kw["stepper"], filter=kw["filter"],
                         precision=precision)
    for _ in range(calls):
        n.step(nsteps // calls)
    out = f.phi.copy(order="F")
    n.close()
    return out


CASES = [
    ((64, 32), ((-6.0, 6.0), (-4.0, 5.0)), 0.6, True),
    ((32, 16, 16), ((-4.0, 4.0), (-3.0, 3.0), (-2.0, 2.0)), 0.3, True),
    ((16, 32, 8), ((0.0, 6.0), (0.0, 6.0), (0.0, 3.0)), 0.0, False),
]


@pytest.mark.parametrize("stepper", ["RK1", "RK2", "RK4"])
@pytest.mark.parametrize("filt", ["none", "product", "solution"])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_rk_fp64_matches_oracle(sfd, O, stepper, filt, case):
    shape, b, omega, trap = CASES[case]
    psi0 = 0.5 * random_field(shape, seed=10 + case)
    V = O.quadratic_potential(shape, b) if trap else None
    kw = dict(coeffD=-0.5, beta=2.0, omega=omega, dt=1e-3, stepper=stepper, filter=filt)
    got = run_rk(sfd, shape, b, psi0, V=V, nsteps=12, calls=3, **kw)
    want = O.c_rk_step(psi0, b, V=V, nsteps=12, **kw)
    assert O.rel_l2(got, want) < 1e-12


@pytest.mark.parametrize("stepper", ["RK2", "RK4"])
@pytest.mark.parametrize("filt", ["product", "solution"])
def test_rk_fp32_matches_oracle(sfd, O, stepper, filt):
    shape, b, omega, trap = CASES[1]
    psi0 = 0.5 * random_field(shape, seed=21)
    V = O.quadratic_potential(shape, b)
    kw = dict(coeffD=-0.5, beta=2.0, omega=omega, dt=1e-3, stepper=stepper, filter=filt)
    got = run_rk(sfd, shape, b, psi0, V=V, precision="fp32", nsteps=40, **kw)
    want = O.c_rk_step(psi0, b, V=V, nsteps=40, **kw)
    assert O.rel_l2(got, want) < 1e-5


def test_rk4_cfg1_slab_fp64(sfd, O, W):
    """The cfg1 state (its phase field on a 64^3 copy) through 10 RK4 steps
    with the 2/3 filter on the product, FP64."""
    c = W.cfg1(64)
    kw = dict(coeffD=c["coeffD"], beta=c["beta"], dt=1e-3, stepper="RK4", filter="product")
    got = run_rk(sfd, c["shape"], c["bounds"], c["psi"], nsteps=10, **kw)
    want = O.c_rk_step(c["psi"], c["bounds"], nsteps=10, **kw)
    assert O.rel_l2(got, want) < 1e-12


def test_rk_rejects_bad_arguments(sfd):
    g = sfd.Grid((16, 16), ((0.0, 1.0), (0.0, 1.0)))
    f = sfd.Field(g)
    f.phi = np.ones((16, 16), dtype=np.complex128)
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialZero(f))
    with pytest.raises(ValueError):
        sfd.NumModelGPRK(f, p, 1e-3, 1, 1, filter="bogus")
    n = sfd.NumModelGPRK(f, p, 1e-3, 1, 1, stepper="RK3")
    with pytest.raises(ValueError):
        n.step(1)
    from sfd_gb300 import _lib
    assert _lib.lib().gpss_rk_step(n.handle, 1, 3, 1, 1e-3) == -1
    assert _lib.lib().gpss_rk_step(n.handle, 1, 4, 7, 1e-3) == -1
    n.close()


@pytest.mark.parametrize("name", ["rk4_product_2d_rot", "rk2_solution_3d"])
def test_rk_golden(sfd, name):
    """The committed explicit-RK fixtures (the oracle's field): FP64 within
    1e-12, FP32 within 1e-5."""
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".solver.npz"))
    b = tuple(tuple(r) for r in z["bounds"])
    kw = dict(coeffD=float(z["coeffD"]), beta=float(z["beta"]), omega=float(z["omega"]), dt=float(z["dt"]),
              stepper=str(z["stepper"]), filter=str(z["filter"]))
    want = z["psi"]
    for precision, tol in (("fp64", 1e-12), ("fp32", 1e-5)):
        got = run_rk(sfd, want.shape, b, z["psi0"], V=z["V"], precision=precision, nsteps=int(z["nsteps"]), **kw)
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < tol, precision
