"""The oracle's restatement of the implicit schemes (backward-euler.jl,
crank-nicolson.jl, krylov.jl) against an independent numpy restatement and a
physics cross-check: imaginary-time backward Euler converges to the same
ground state as the imaginary-time split step (no GPU)."""
import numpy as np
import pytest

SCHEMES = ["BackwardEuler", "BackwardEulerNoPrecond", "CrankNicolson", "CrankNicolsonQuasiNewton",
           "CrankNicolsonT", "CrankNicolsonQuasiNewtonT"]


def _gauss(shape, bounds):
    axes = [np.linspace(b[0], b[1], n, endpoint=False) for n, b in zip(shape, bounds)]
    mesh = np.meshgrid(*axes, indexing="ij")
    psi = np.exp(-0.5 * sum(m ** 2 for m in mesh)) * (1 + 0.1 * mesh[0]) + 0j
    dV = np.prod([(b[1] - b[0]) / n for n, b in zip(shape, bounds)])
    return np.asfortranarray(psi / np.sqrt(np.sum(np.abs(psi) ** 2) * dV))


@pytest.mark.parametrize("scheme", SCHEMES)
@pytest.mark.parametrize("shape,omega", [((32, 16), 0.3), ((8, 8, 8), 0.0)])
def test_c_implicit_matches_numpy(O, scheme, shape, omega):
    b = tuple((-5.0 + a, 5.0 - a) for a in range(len(shape)))
    psi = _gauss(shape, b)
    V = O.quadratic_potential(shape, b)
    kw = dict(scheme=scheme, coeffD=-0.5, beta=5.0, omega=omega, V=V, nsteps=2, dt=1e-2)
    a, na = O.c_implicit_step(psi, b, **kw)
    c, nc = O.np_implicit_step(psi, b, **kw)
    assert na == nc
    assert O.rel_l2(a, c) < 1e-12


def test_backward_euler_ground_state_matches_split_step(O):
    """Imaginary-time BE and imaginary-time Strang reach the same ground state
    (their fixed points differ only by the O(dt) splitting error)."""
    shape, b = (32, 32), ((-6.0, 6.0), (-6.0, 6.0))
    psi = _gauss(shape, b)
    V = O.quadratic_potential(shape, b)
    be, _ = O.c_implicit_step(psi, b, scheme="BackwardEuler", beta=10.0, V=V, nsteps=300, dt=5e-2)
    sp = O.c_step(psi, b, beta=10.0, V=V, nsteps=3000, dt=5e-3, imag=True)
    e_be = O.c_energy(be, b, beta=10.0, V=V)
    e_sp = O.c_energy(sp, b, beta=10.0, V=V)
    assert abs(e_be[3] - e_sp[3]) < 1e-3 * abs(e_sp[3])
    assert O.rel_l2(np.abs(be), np.abs(sp)) < 1e-2
