"""Grid sizes that are not powers of two up to 256 (the mixed-radix pass,
csrc/pass_generic.cuh) against the oracle.

The reference plans every length with FFTW (src/Discretization/Plans.jl:846-847);
its own tests run 48^3 (test/runtests.jl:46,78), 48x36 (:1076) and 64x48x56
(:769), and its split-step notes measure 512^2 (splitting.jl:41-46,117).  The
oracle transforms such lengths with a direct O(n^2) DFT in FP64.

Bars as in test_gpu_parity.py: FP64 <= 1e-12 (relative L2), FP32 <= 1e-5.
"""
import ctypes

import numpy as np
import pytest

from helpers import random_field, run_model

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def _bounds(nd):
    return tuple((-4.0 - 0.5 * a, 4.0 + a) for a in range(nd))


# the reference's own grid sizes, then radices 3/5/7 and primes up to 31,
# lengths above 256, and mixes with register-kernel axes
SHAPES = [
    (48, 48, 48), (48, 36), (64, 48, 56), (512, 512),
    (12, 20), (3, 5), (96, 100), (31, 62), (1024, 8), (8, 768), (1000, 6),
    (7, 11, 13), (256, 24, 5), (18, 128, 30), (44, 26, 34), (50, 16, 2),
]


@pytest.mark.parametrize("form", ["fused", "plain"])
@pytest.mark.parametrize("shape", SHAPES)
def test_generic_fp64_strang(sfd, O, shape, form):
    nd = len(shape)
    b = _bounds(nd)
    psi0 = random_field(shape, seed=sum(shape) + 1)
    V = O.quadratic_potential(shape, b, gammas=[1.0, 0.7, 1.3][:nd])
    kw = dict(coeffD=-0.5, beta=3.0, V=V, dt=2e-3)
    got = run_model(sfd, shape, b, psi0, nsteps=4, form=form, **kw)
    ref = O.c_step(psi0, b, nsteps=4, **kw)
    assert O.rel_l2(got, ref) < TOL64
    # unitary flow: mass kept to FP64 round-off
    m0, m1 = np.sum(np.abs(psi0) ** 2), np.sum(np.abs(got) ** 2)
    assert abs(m1 - m0) <= 1e-12 * m0


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("imag", [False, True])
@pytest.mark.parametrize("shape", [(48, 36), (24, 20, 18)])
def test_generic_fp64_rotation_and_imaginary_time(sfd, O, shape, scheme, imag):
    nd = len(shape)
    b = tuple((-5.0, 5.0 + a) for a in range(nd))
    psi0 = random_field(shape, seed=7)
    V = O.quadratic_potential(shape, b)
    kw = dict(coeffD=-0.5, beta=20.0, omega=0.7, V=V, dt=5e-3, scheme=scheme, imag=imag)
    got = run_model(sfd, shape, b, psi0, nsteps=5, **kw)
    ref = O.c_step(psi0, b, nsteps=5, **kw)
    assert O.rel_l2(got, ref) < TOL64


def test_generic_fp64_imaginary_time_merged_request(sfd, O):
    """Omega = 0 imaginary time: the merged step needs power-of-two axes, so a
    48^3 field runs the unmerged sequence and still meets the FP64 bar, with
    unit mass after every call."""
    shape = (48, 48, 48)
    b = ((-6.0, 6.0),) * 3
    psi0 = random_field(shape, seed=9)
    V = O.quadratic_potential(shape, b, gammas=[1.0, 1.0, 2.0])
    kw = dict(coeffD=-0.5, beta=50.0, V=V, dt=1e-2, imag=True)
    got = run_model(sfd, shape, b, psi0, nsteps=6, **kw)
    ref = O.c_step(psi0, b, nsteps=6, **kw)
    assert O.rel_l2(got, ref) < TOL64
    dV = np.prod([(hi - lo) / n for n, (lo, hi) in zip(shape, b)])
    assert abs(np.sum(np.abs(got) ** 2) * dV - 1.0) < 1e-12


@pytest.mark.parametrize("shape", [(48, 48, 48), (512, 512), (64, 48, 56)])
def test_generic_fp32_fused(sfd, O, shape):
    nd = len(shape)
    b = _bounds(nd)
    psi0 = random_field(shape, seed=3)
    V = O.quadratic_potential(shape, b)
    kw = dict(coeffD=-0.5, beta=5.0, V=V, dt=1e-3)
    got = run_model(sfd, shape, b, psi0, nsteps=20, precision="fp32", **kw)
    ref = O.c_step(psi0, b, nsteps=20, **kw)
    assert O.rel_l2(got, ref) < TOL32


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-6)])
@pytest.mark.parametrize("shape", [(48, 36), (30, 24, 20), (512, 64)])
def test_generic_energy(sfd, O, shape, precision, tol):
    nd = len(shape)
    b = tuple((-5.0, 6.0) for _ in range(nd))
    psi0 = random_field(shape, seed=21)
    V = O.quadratic_potential(shape, b)
    g = sfd.Grid(shape, b)
    f = sfd.Field(g)
    f.phi = psi0
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, V), coeffD=-0.4, beta=7.0, Omega=0.6)
    n = sfd.NumModelSplit2(f, p, 1e-3, 1, 1, precision=precision)
    got = n.energies()
    n.close()
    ref = O.c_energy(psi0, b, coeffD=-0.4, beta=7.0, omega=0.6, V=V)
    scale = max(abs(v) for v in ref)
    for x, y in zip(got, ref):
        assert abs(x - y) <= tol * scale


@pytest.mark.parametrize("stepper,filt", [("RK4", "product"), ("RK2", "solution"), ("RK1", "none")])
def test_generic_rk_fp64(sfd, O, stepper, filt):
    shape, b = (48, 36), ((-6.0, 6.0), (-4.0, 5.0))
    psi0 = 0.5 * random_field(shape, seed=10)
    V = O.quadratic_potential(shape, b)
    kw = dict(coeffD=-0.5, beta=2.0, omega=0.6, dt=1e-3, stepper=stepper, filter=filt)
    g = sfd.Grid(shape, b)
    f = sfd.Field(g)
    f.phi = psi0
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, V), coeffD=-0.5, beta=2.0, Omega=0.6)
    n = sfd.NumModelGPRK(f, p, 1e-3, 8, 8, stepper=stepper, filter=filt, precision="fp64")
    n.step(8)
    got = f.phi.copy(order="F")
    n.close()
    want = O.c_rk_step(psi0, b, V=V, nsteps=8, **kw)
    assert O.rel_l2(got, want) < TOL64


def test_generic_backward_euler_fp64(sfd, O):
    shape, b = (24, 20, 18), ((-5.0, 5.0), (-4.0, 4.0), (-3.0, 3.0))
    axes = [np.linspace(lo, hi, n, endpoint=False) for n, (lo, hi) in zip(shape, b)]
    mesh = np.meshgrid(*axes, indexing="ij")
    psi = np.exp(-0.5 * sum(m ** 2 for m in mesh)) * (1 + 0.1 * mesh[0]) + 0j
    dV = np.prod([(hi - lo) / n for n, (lo, hi) in zip(shape, b)])
    psi = np.asfortranarray(psi / np.sqrt(np.sum(np.abs(psi) ** 2) * dV))
    V = O.quadratic_potential(shape, b)
    kw = dict(coeffD=-0.5, beta=5.0, omega=0.0, dt=1e-2)
    g = sfd.Grid(shape, b)
    f = sfd.Field(g)
    f.phi = psi
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, V), coeffD=-0.5, beta=5.0, Omega=0.0)
    n = sfd.NumModelBackwardEuler(f, p, 1e-2, 2, 2, precision="fp64", nkrylov=70, tolkrylov=1e-8)
    counts = [sfd.timeStep(n) for _ in range(2)]
    got = f.phi.copy(order="F")
    n.close()
    want, nw = O.c_implicit_step(psi, b, scheme="BackwardEuler", V=V, nsteps=2, **kw)
    err = O.rel_l2(got, want)
    assert err < (1e-10 if sum(counts) == nw else 1e-7), (counts, nw, err)


def test_generic_rejections(sfd):
    """Compensated passes and the adjoint take power-of-two axes only: a clear
    GPSS_EINVAL, and the context keeps working."""
    L = sfd._lib.lib()
    shape, b = (48, 32), ((-4.0, 4.0), (-4.0, 4.0))
    g = sfd.Grid(shape, b)
    f = sfd.Field(g)
    f.phi = random_field(shape, seed=1)
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialZero(f), coeffD=-0.5, beta=1.0)
    with pytest.raises(Exception):
        sfd.NumModelSplit2(f, p, 1e-3, 1, 1, precision="fp32", compensated=True)
    n = sfd.NumModelSplit2(f, p, 1e-3, 1, 1, precision="fp64")
    tgt = np.asfortranarray(random_field(shape, seed=2))
    loss = ctypes.c_double()
    dV = np.zeros(shape, order="F")
    dpsi = np.zeros(shape, dtype=np.complex128, order="F")
    rc = L.gpss_adjoint(n._h, tgt.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 4, 2, 1e-3,
                        ctypes.byref(loss), dV.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                        dpsi.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert rc == -1
    assert b"power of two" in L.gpss_last_error(n._h)
    n.step(2)
    assert np.isfinite(f.phi).all()
    n.close()
