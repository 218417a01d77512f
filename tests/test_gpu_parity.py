"""Parity of the CUDA split-step path with the CPU oracle (FP64 restatement of
src/NumModels/GrossPitaevskii/splitting.jl), through the library's public API.

Tolerances (relative L2, ||a-b|| / ||b||, the metric of test/runtests.jl:1416):
  FP64 forms  <= 1e-12   vs the FP64 oracle (the reference asserts 1e-10 for
                         CuArray vs Array), and vs the long-double oracle
                         stored in tests/golden (near-exact), where the GPU
                         must be no farther from exact than the FP64 oracle is
  FP32 fused  <= 1e-5    vs the FP64 oracle
"""
import math

import numpy as np
import pytest

from helpers import random_field, run_model

pytestmark = pytest.mark.gpu

# full-size properties of the compensated passes (measured on GB300: linear
# flow 2.0e-7 against 1.0e-6 for the plain passes, time reversal 5.5e-7
# against 2.3e-6)
LINEAR_FLOW_BAR_COMP = 5e-7
REVERSAL_BAR_COMP = 1.5e-6

TOL64 = 1e-12
TOL32 = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


# -------------------------------------------------- the reference's own case --
@pytest.mark.parametrize("form", ["fused", "plain"])
def test_reference_gpu_vs_cpu_split2(sfd, O, form):
    """test/runtests.jl:1438-1454: 32^2 on [-6,6]^2, Gaussian*(1+0.1x),
    normalised, beta=10, harmonic trap, dt=0.01, 20 steps of NumModelSplit2."""
    g = sfd.Grid((32, 32), ((-6, 6), (-6, 6)))
    f = sfd.Field(g)
    X, Y = f.mesh()
    f.phi = np.exp(-0.5 * (X ** 2 + Y ** 2)) * (1 + 0.1 * X)
    sfd.normalize(f)
    psi0 = f.phi.copy(order="F")
    pot = sfd.PotentialQuadratic(f, gx=1.0, gy=1.0)
    p = sfd.GrossPitaevskiiParameters(pot, coeffD=-0.5, beta=10.0, Omega=0.0)
    n = sfd.NumModelSplit2(f, p, 0.01, 20, 20, precision="fp64", form=form)
    for _ in range(20):
        assert sfd.timeStep(n) == 2
    got = f.phi.copy()
    n.close()
    ref = O.c_step(psi0, g.bounds, coeffD=-0.5, beta=10.0, V=pot.V, nsteps=20, dt=0.01)
    assert O.rel_l2(got, ref) < TOL64


# ------------------------------------------------------------ FP64 coverage --
SHAPES = [
    ((2, 4), 2), ((8, 8), 2), ((16, 32), 2), ((64, 16), 2), ((256, 8), 2), ((8, 256), 2),
    ((128, 128), 2), ((256, 256), 2),
    ((4, 8, 2), 3), ((32, 16, 8), 3), ((8, 16, 32), 3), ((64, 32, 16), 3), ((16, 16, 256), 3),
    ((256, 16, 8), 3),
]


@pytest.mark.parametrize("shape,nd", SHAPES)
def test_fp64_fused_shapes(sfd, O, shape, nd):
    bounds = tuple((-3.0 - a, 4.0 + 0.5 * a) for a in range(nd))
    psi0 = random_field(shape, seed=sum(shape))
    V = O.quadratic_potential(shape, bounds, gammas=[1.0, 0.7, 1.3][:nd])
    kw = dict(coeffD=-0.5, beta=3.0, V=V, dt=2e-3, nsteps=5)
    got = run_model(sfd, shape, bounds, psi0, **kw)
    ref = O.c_step(psi0, bounds, coeffD=-0.5, beta=3.0, V=V, nsteps=5, dt=2e-3)
    assert O.rel_l2(got, ref) < TOL64


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("form", ["fused", "plain"])
@pytest.mark.parametrize("shape", [(32, 64), (16, 32, 8)])
def test_fp64_rotation(sfd, O, scheme, form, shape):
    nd = len(shape)
    bounds = tuple((-5.0, 5.0 + a) for a in range(nd))
    psi0 = random_field(shape, seed=7)
    V = O.quadratic_potential(shape, bounds)
    got = run_model(sfd, shape, bounds, psi0, coeffD=-0.5, beta=20.0, omega=0.7, V=V, dt=5e-3,
                    nsteps=6, scheme=scheme, form=form)
    ref = O.c_step(psi0, bounds, coeffD=-0.5, beta=20.0, omega=0.7, V=V, nsteps=6, scheme=scheme,
                   dt=5e-3)
    assert O.rel_l2(got, ref) < TOL64


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("form", ["fused", "plain"])
@pytest.mark.parametrize("shape", [(64, 32), (16, 8, 32)])
def test_fp64_imaginary_time(sfd, O, scheme, form, shape):
    nd = len(shape)
    bounds = tuple((-6.0, 6.0) for _ in range(nd))
    psi0 = random_field(shape, seed=3)
    V = O.quadratic_potential(shape, bounds)
    got = run_model(sfd, shape, bounds, psi0, coeffD=-0.5, beta=50.0, omega=0.3, V=V, dt=1e-2,
                    nsteps=7, scheme=scheme, imag=True, form=form)
    ref = O.c_step(psi0, bounds, coeffD=-0.5, beta=50.0, omega=0.3, V=V, nsteps=7, scheme=scheme,
                   imag=True, dt=1e-2)
    assert O.rel_l2(got, ref) < TOL64
    dV = np.prod([(b[1] - b[0]) / n for n, b in zip(shape, bounds)])
    assert abs(np.sum(np.abs(got) ** 2) * dV - 1.0) < 1e-12


def test_merge_is_exact_reordering(sfd, O):
    """Merging L(dt/2) L(dt/2) of consecutive steps (Omega = 0) only changes round-off."""
    shape, bounds = (64, 32, 16), ((-4, 4), (-4, 4), (-2, 2))
    psi0 = random_field(shape, seed=11)
    V = O.quadratic_potential(shape, bounds)
    a = run_model(sfd, shape, bounds, psi0, beta=30.0, V=V, dt=1e-3, nsteps=20, merge=True)
    b = run_model(sfd, shape, bounds, psi0, beta=30.0, V=V, dt=1e-3, nsteps=20, merge=False)
    c = run_model(sfd, shape, bounds, psi0, beta=30.0, V=V, dt=1e-3, nsteps=20, per_call=1)
    ref = O.c_step(psi0, bounds, beta=30.0, V=V, nsteps=20, dt=1e-3)
    for x in (a, b, c):
        assert O.rel_l2(x, ref) < TOL64


# --------------------------------------------------------- known answers --
def test_linear_flow_is_exact(sfd, O):
    """beta = V = Omega = 0: psi_hat(t) = exp(i coeffD k^2 t) psi_hat(0) exactly
    (the split step is exact for the linear flow)."""
    shape, bounds = (32, 16, 64), ((-np.pi, np.pi), (-2.0, 2.0), (0.0, 3.0))
    psi0 = random_field(shape, seed=5)
    t = 40 * 1e-2
    got = run_model(sfd, shape, bounds, psi0, beta=0.0, dt=1e-2, nsteps=40)
    F = np.fft.fftn(psi0)
    for a, (n, b) in enumerate(zip(shape, bounds)):
        xi = np.fft.fftfreq(n, (b[1] - b[0]) / n) * 2 * np.pi
        s = [1] * 3
        s[a] = n
        F = F * np.exp(1j * (-0.5) * xi.reshape(s) ** 2 * t)
    exact = np.fft.ifftn(F)
    assert O.rel_l2(got, exact) < 1e-13


def test_split_order_and_mass(sfd, O):
    """test/runtests.jl:644-671 on the GPU: temporal order 1 (Lie) / 2 (Strang)
    by step refinement, mass conserved to 1e-12."""
    N, L, beta, T = 32, 2 * np.pi, 20.0, 0.2
    bounds = ((-L, L), (-L, L))
    g = sfd.Grid((N, N), bounds)
    f = sfd.Field(g)
    X, Y = f.mesh()
    psi0 = np.asfortranarray((1 + 0.3 * np.cos(X) + 0.2 * np.sin(2 * Y)) * np.exp(1j * 0.5 * X))
    psi0 = psi0 / O.c_norm(psi0, bounds)
    for order, lo, hi, ns in ((1, 0.85, 1.15, (50, 100, 200)), (2, 1.85, 2.15, (25, 50, 100))):
        runs = [run_model(sfd, (N, N), bounds, psi0, beta=beta, dt=T / k, nsteps=k, scheme=order)
                for k in ns]
        d = [np.sqrt(np.sum(np.abs(runs[i] - runs[i + 1]) ** 2) / np.sum(np.abs(runs[i + 1]) ** 2))
             for i in range(2)]
        assert lo < math.log2(d[0] / d[1]) < hi
        masses = [np.sum(np.abs(r) ** 2) for r in runs]
        assert max(abs(m - masses[0]) for m in masses) < 1e-12


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-6)])
def test_energy_matches_oracle(sfd, O, precision, tol):
    for shape in ((64, 32), (32, 16, 8)):
        nd = len(shape)
        bounds = tuple((-5.0, 6.0) for _ in range(nd))
        psi0 = random_field(shape, seed=21)
        V = O.quadratic_potential(shape, bounds)
        g = sfd.Grid(shape, bounds)
        f = sfd.Field(g)
        f.phi = psi0
        p = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, V), coeffD=-0.4, beta=7.0, Omega=0.6)
        n = sfd.NumModelSplit2(f, p, 1e-3, 1, 1, precision=precision)
        got = n.energies()
        n.close()
        ref = O.c_energy(psi0, bounds, coeffD=-0.4, beta=7.0, omega=0.6, V=V)
        scale = max(abs(v) for v in ref)
        for a, b in zip(got, ref):
            assert abs(a - b) <= tol * scale


def test_step_diagnostics_fused_equal_separate(sfd, O):
    """The diagnostics fused into the final half step equal energy() after it."""
    shape, bounds = (64, 64, 32), ((-5, 5), (-5, 5), (-3, 3))
    psi0 = random_field(shape, seed=2)
    V = O.quadratic_potential(shape, bounds)
    g = sfd.Grid(shape, bounds)
    f = sfd.Field(g)
    f.phi = psi0
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, V), coeffD=-0.5, beta=15.0)
    n = sfd.NumModelSplit2(f, p, 1e-3, 10, 10, precision="fp64")
    d = n.step(10, diag=True)
    e = n.energies()
    m = n.mass()
    n.close()
    assert abs(d["mass"] - m) <= 1e-13 * abs(m)
    for a, b in zip(d["energy"], e):
        assert abs(a - b) <= 1e-12 * max(abs(x) for x in e)


# ------------------------------------------------------ benchmark configs --
def _cfg0_golden():
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "cfg0_2d_128_1000.npz"))
    return z, tuple(tuple(r) for r in z["bounds"])


@pytest.mark.parametrize("form", ["fused", "plain"])
def test_cfg0_fp64_full(sfd, O, form):
    """cfg0 at its full size: 128^2, g=500, trap, dt=1e-3, 1000 steps (FP64).
    Two independent FP64 FFT codes differ by ~1.7e-12 here (round-off growth
    under g = 500); against the near-exact long-double run the GPU must be
    within 1e-13, and within 1e-12 of the FP64 oracle (whose own error is 8.8e-13)."""
    z, b = _cfg0_golden()
    psi0 = z["psi0"]
    kw = dict(coeffD=float(z["coeffD"]), beta=float(z["beta"]), V=z["V"], dt=float(z["dt"]),
              nsteps=int(z["nsteps"]))
    ref = O.c_step(psi0, b, **kw)
    got = run_model(sfd, psi0.shape, b, psi0, form=form, per_call=250, **kw)
    assert O.rel_l2(got, z["psi_ext"]) < 1e-13
    assert O.rel_l2(got, ref) < TOL64
    dV = (16.0 / 128) ** 2
    assert abs(np.sum(np.abs(got) ** 2) * dV - 1.0) < 1e-12


def test_cfg0_fp32(sfd, O):
    """cfg0 in FP32 (double-word constants + mass lock): 1000 steps within 1e-5
    of the near-exact run."""
    z, b = _cfg0_golden()
    got = run_model(sfd, z["psi0"].shape, b, z["psi0"], coeffD=float(z["coeffD"]), beta=float(z["beta"]),
                    V=z["V"], dt=float(z["dt"]), nsteps=int(z["nsteps"]), precision="fp32")
    assert O.rel_l2(got, z["psi_ext"]) < TOL32


def test_cfg1_fp32_128_vs_oracle(sfd, O, W):
    """cfg1 physics at 128^3 (the oracle finishes in about a minute): FP32 fused
    after 200 steps within 1e-5 of the FP64 oracle."""
    c = W.cfg1(128)
    ref = O.c_step(c["psi"], c["bounds"], coeffD=c["coeffD"], beta=c["beta"], nsteps=c["nsteps"],
                   dt=c["dt"])
    got = run_model(sfd, c["shape"], c["bounds"], c["psi"], coeffD=c["coeffD"], beta=c["beta"],
                    dt=c["dt"], nsteps=c["nsteps"], precision="fp32")
    assert O.rel_l2(got, ref) < TOL32


@pytest.fixture(scope="module")
def cfg1_full(O, W):
    """cfg1 at its full size (256^3) run by the FP64 oracle: the fields after
    150 and 200 steps (about 40 s on 16 host cores)."""
    c = W.cfg1(256)
    kw = dict(coeffD=c["coeffD"], beta=c["beta"], dt=c["dt"])
    r150 = O.c_step(c["psi"], c["bounds"], nsteps=150, **kw)
    r200 = O.c_step(r150, c["bounds"], nsteps=50, **kw)
    return c, r150, r200


def _cfg1_run(sfd, c, **kw):
    """150 + 50 steps of cfg1 through the public API: the fields after 150 and
    200 steps, the mass and energies before, and the fused diagnostics after."""
    g = sfd.Grid(c["shape"], c["bounds"])
    f = sfd.Field(g)
    f.phi = c["psi"]
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialZero(f), coeffD=c["coeffD"], beta=c["beta"])
    n = sfd.NumModelSplit2(f, p, c["dt"], c["nsteps"], c["nsteps"], **kw)
    m0, e0 = n.mass(), n.energies()
    n.step(150)
    a150 = f.phi.copy(order="F")
    d = n.step(50, diag=True)
    a200 = f.phi.copy(order="F")
    n.close()
    return a150, a200, m0, e0, d


@pytest.mark.parametrize("form", ["plain", "fused"])
def test_cfg1_fullsize_fp64_vs_oracle(sfd, O, cfg1_full, form):
    """cfg1 at 256^3 in FP64 against the FP64 oracle after 150 and 200 steps
    (splitting.jl:149-209): the plain form (the reference's stage order) and
    the fused merged form within 1e-12, mass conserved to 1e-12."""
    c, r150, r200 = cfg1_full
    a150, a200, m0, _, d = _cfg1_run(sfd, c, precision="fp64", form=form)
    assert O.rel_l2(a150, r150) < TOL64
    assert O.rel_l2(a200, r200) < TOL64
    assert abs(d["mass"] - m0) / m0 < 1e-12


def test_cfg1_fullsize_fp32_compensated_vs_oracle(sfd, O, cfg1_full):
    """The FP32 form of the headline measurement (compensated passes: FP32
    storage, double-float FFT arithmetic) against the FP64 oracle at 256^3:
    within 1e-5 after 200 steps.  Measured on GB300: 9.7e-7 (150 steps),
    5.8e-6 (200 steps)."""
    c, r150, r200 = cfg1_full
    a150, a200, m0, e0, d = _cfg1_run(sfd, c, precision="fp32", compensated=True)
    e150, e200 = O.rel_l2(a150, r150), O.rel_l2(a200, r200)
    print(f"cfg1 256^3 compensated FP32 vs oracle: {e150:.3e} (150 steps), {e200:.3e} (200 steps)")
    assert e150 < TOL32
    assert e200 < TOL32
    assert abs(d["mass"] - m0) / m0 < 1e-6
    assert abs(d["energy"][3] - e0[3]) / abs(e0[3]) < 1e-3


def test_cfg1_fullsize_fp32_plain_vs_oracle(sfd, O, cfg1_full):
    """Plain FP32 passes (no compensation) at 256^3 against the FP64 oracle.
    They meet 1e-5 through 150 steps (5.1e-6 measured) but not at 200
    (2.5e-5): |coeffD| |k|^2 dt reaches pi on the shell |k| ~ 188 of this
    grid, where the Strang step is resonant and amplifies round-off about
    2.7x per 25 steps; 90% of the 200-step error sits in 184 <= |k| < 192.
    This test pins that behaviour (<= 1e-5 at 150, < 4e-5 at 200); the
    compensated passes above are the FP32 form that meets 1e-5 at 200."""
    c, r150, r200 = cfg1_full
    a150, a200, m0, _, d = _cfg1_run(sfd, c, precision="fp32")
    assert O.rel_l2(a150, r150) < TOL32
    assert O.rel_l2(a200, r200) < 4e-5
    assert abs(d["mass"] - m0) / m0 < 1e-5


@pytest.mark.parametrize("nsteps,per_call", [(1, None), (2, None), (3, 1), (40, None), (70, 33)])
@pytest.mark.parametrize("shape", [(64, 32), (16, 8, 32)])
def test_merged_imaginary_time(sfd, O, shape, nsteps, per_call):
    """Imaginary-time Strang with Omega = 0 takes one kinetic flow per step
    (renormalisation from <chi, L(dt) chi>, the nonlinear stage as the next
    pass's prologue): FP64 against the oracle and against the unmerged
    sequence, FP32 against the oracle; calls of one step and chunks that
    cross the graph-captured blocks of 32 steps."""
    nd = len(shape)
    bounds = tuple((-6.0, 6.0 + a) for a in range(nd))
    psi0 = random_field(shape, seed=11)
    V = O.quadratic_potential(shape, bounds)
    kw = dict(coeffD=-0.5, beta=40.0, V=V, dt=1e-2, nsteps=nsteps, imag=True, per_call=per_call)
    ref = O.c_step(psi0, bounds, coeffD=-0.5, beta=40.0, V=V, nsteps=nsteps, imag=True, dt=1e-2)
    got = run_model(sfd, shape, bounds, psi0, **kw)
    unmerged = run_model(sfd, shape, bounds, psi0, merge=False, **kw)
    assert O.rel_l2(got, ref) < TOL64
    assert O.rel_l2(got, unmerged) < TOL64
    dV = np.prod([(b[1] - b[0]) / n for n, b in zip(shape, bounds)])
    assert abs(np.sum(np.abs(got) ** 2) * dV - 1.0) < 1e-12
    got32 = run_model(sfd, shape, bounds, psi0, precision="fp32", **kw)
    assert O.rel_l2(got32, ref) < TOL32


def test_cfg2_ground_state_small(sfd, O, W):
    """Imaginary time (cfg2 physics at 32^3): FP32 stages with FP64 reductions
    track the FP64 oracle; mu agrees."""
    c = W.cfg2(32)
    nsteps = 300
    ref = O.c_step(c["psi"], c["bounds"], coeffD=c["coeffD"], beta=c["beta"], V=c["V"],
                   nsteps=nsteps, dt=c["dt"], imag=True)
    for prec, tol in (("fp64", TOL64), ("fp32", TOL32)):
        got = run_model(sfd, c["shape"], c["bounds"], c["psi"], coeffD=c["coeffD"], beta=c["beta"],
                        V=c["V"], dt=c["dt"], nsteps=nsteps, imag=True, precision=prec)
        assert O.rel_l2(got, ref) < tol
    mu_ref = O.c_energy(ref, c["bounds"], coeffD=c["coeffD"], beta=c["beta"], V=c["V"])[4]
    g = sfd.Grid(c["shape"], c["bounds"])
    f = sfd.Field(g)
    f.phi = c["psi"]
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, c["V"]), coeffD=c["coeffD"], beta=c["beta"])
    n = sfd.NumModelSplit2(f, p, c["dt"], nsteps, nsteps, precision="fp32")
    n.step(nsteps, imag=True)
    mu = n.energies()[4]
    n.close()
    assert abs(mu - mu_ref) / abs(mu_ref) < 1e-5


def test_cfg2_fullsize_ground_state(sfd, O, W):
    """cfg2 at its full size (128^3, g = 2000, anisotropic trap, dt = 1e-3)
    run to the ground state, against the FP64 oracle's run
    (tests/golden/cfg2_3d_128.ground.npz, made by make_cfg2_ground.py: 16410
    steps to |mu_n - mu_{n-10}| < 1e-10).
    * FP64 gpss_ground_state stops at the oracle's step -- or one check later:
      the oracle's last difference is 9.98e-11, within rounding of the
      tolerance -- with mu within 1e-10 of the oracle's;
    * FP64, the oracle's step count: the five energies within 1e-11 and the
      field within 1e-10 (of its largest value) of the oracle's;
    * FP32 stages with FP64 reductions and renormalisation, the same steps:
      mu within 1e-6, the field within 2e-4 of its largest value.  Near the
      ground state each step damps the slowest excitation only by about
      gap * dt ~ 1e-3, so the FP32 rounding of every step accumulates there
      about 1/(gap dt) ~ 1e3 times (measured: 5.3e-5); mu is variational
      (second order in that error)."""
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "cfg2_3d_128.ground.npz"))
    c = W.cfg2(128)
    nref, eref = int(z["nsteps"]), z["energies"]
    mid = [n // 2 for n in c["shape"]]

    def close(got, tol):
        scale = float(z["max_abs"])
        assert np.max(np.abs(got[::8, ::8, ::8] - z["sample"])) <= tol * scale
        assert np.max(np.abs(got[:, mid[1], mid[2]] - z["line_x"])) <= tol * scale
        assert np.max(np.abs(got[mid[0], :, mid[2]] - z["line_y"])) <= tol * scale
        assert np.max(np.abs(got[mid[0], mid[1], :] - z["line_z"])) <= tol * scale

    def model(precision):
        g = sfd.Grid(c["shape"], c["bounds"])
        f = sfd.Field(g)
        f.phi = c["psi"]
        p = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, c["V"]), coeffD=c["coeffD"], beta=c["beta"])
        return f, sfd.NumModelSplit2(f, p, c["dt"], 1, 1, precision=precision)

    f, n = model("fp64")
    mu, steps = n.ground_state(tol=1e-10, max_steps=2 * nref, check_every=10)
    n.close()
    assert steps in (nref, nref + 10), (steps, nref)
    assert abs(mu - eref[4]) <= 1e-10
    out = {}
    for prec in ("fp64", "fp32"):
        f, n = model(prec)
        n.normalize()
        n.step(nref, imag=True)
        out[prec] = (n.energies(), f.phi.copy())
        n.close()
    e64, got64 = out["fp64"]
    for a, b in zip(e64, eref):
        assert abs(a - b) <= 1e-11 * max(abs(x) for x in eref)
    close(got64, 1e-10)
    e32, got32 = out["fp32"]
    assert abs(e32[4] - eref[4]) <= 1e-6 * abs(eref[4])
    close(got32, 2e-4)
    print(f"cfg2 128^3 ground state: {steps} steps (oracle {nref}), mu FP64 {mu:.12f} "
          f"(oracle {eref[4]:.12f}), FP32 {e32[4]:.10f}")


# ----------------------------------------------------------------- errors --
def test_nonfinite_is_reported(sfd):
    g = sfd.Grid((16, 16), ((-1, 1), (-1, 1)))
    f = sfd.Field(g)
    a = np.ones((16, 16), dtype=complex)
    a[3, 4] = np.nan
    f.phi = a
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialZero(f), beta=1.0)
    n = sfd.NumModelSplit2(f, p, 1e-3, 1, 1)
    with pytest.raises(sfd.GPSSError) as ei:
        n.energies()
    assert ei.value.code == -4
    with pytest.raises(sfd.GPSSError):
        n.step(2, imag=True)
    n.close(download=False)


# ------------------------------------------------------------ golden files --
def _golden():
    import os
    here = os.path.join(os.path.dirname(__file__), "golden")
    return sorted(os.path.join(here, f) for f in os.listdir(here)
                  if f.endswith(".npz") and not f.endswith((".grad.npz", ".solver.npz", ".ground.npz")))


@pytest.mark.parametrize("path", _golden(), ids=lambda p: p.split("/")[-1][:-4])
@pytest.mark.parametrize("form", ["fused", "plain"])
def test_golden_fixture(sfd, O, path, form):
    """GPU FP64 vs the FP64 oracle's golden output (<= 1e-12) and vs the
    long-double output: no farther from exact than the FP64 oracle itself."""
    z = np.load(path)
    b = tuple(tuple(r) for r in z["bounds"])
    V = z["V"] if z["has_V"] else None
    got = run_model(sfd, z["psi0"].shape, b, z["psi0"], coeffD=float(z["coeffD"]), beta=float(z["beta"]),
                    omega=float(z["omega"]), V=V, dt=float(z["dt"]), nsteps=int(z["nsteps"]),
                    scheme=int(z["scheme"]), imag=bool(z["imag"]), form=form)
    assert O.rel_l2(got, z["psi"]) < TOL64
    oracle_err = O.rel_l2(z["psi"], z["psi_ext"])
    assert O.rel_l2(got, z["psi_ext"]) <= max(oracle_err, 1e-14)


@pytest.mark.parametrize("path", _golden(), ids=lambda p: p.split("/")[-1][:-4])
@pytest.mark.parametrize("precision,tol_m,tol_e", [("fp64", 1e-12, 1e-11), ("fp32", 3e-6, 2e-5)])
def test_golden_traces(sfd, path, precision, tol_m, tol_e):
    """Mass and energy(n) (E_Omega, E_Delta, E_beta, E, mu) every
    trace_every steps against the oracle's recorded traces; energies relative
    to the largest of the five.  FP32: the mass lock rescales with the mass
    taken before the last half kinetic step, so the FP32 round-off of those
    passes stays in the mass (measured worst 9e-7, cfg1 at 32^3)."""
    z = np.load(path)
    shape = z["psi0"].shape
    if precision == "fp32" and any(n & (n - 1) for n in shape):
        pytest.skip("the FP32 path takes power-of-two sizes")
    b = tuple(tuple(r) for r in z["bounds"])
    g = sfd.Grid(shape, b)
    f = sfd.Field(g)
    f.phi = z["psi0"]
    pot = sfd.PotentialArray(f, z["V"]) if z["has_V"] else sfd.PotentialZero(f)
    p = sfd.GrossPitaevskiiParameters(pot, coeffD=float(z["coeffD"]), beta=float(z["beta"]), Omega=float(z["omega"]))
    cls = sfd.NumModelSplit2 if int(z["scheme"]) == 2 else sfd.NumModelSplit1
    n = cls(f, p, float(z["dt"]), int(z["nsteps"]), int(z["nsteps"]), precision=precision)
    steps = z["trace_steps"]
    worst_m = worst_e = 0.0
    for i, st in enumerate(steps):
        if i:
            n.step(int(st - steps[i - 1]), imag=bool(z["imag"]))
        m, e = n.mass(), np.array(n.energies())
        worst_m = max(worst_m, abs(m - z["trace_mass"][i]) / z["trace_mass"][i])
        worst_e = max(worst_e, np.max(np.abs(e - z["trace_energy"][i])) / np.max(np.abs(z["trace_energy"][i])))
    n.close()
    print(f"{path.split('/')[-1]} {precision}: mass {worst_m:.2e} energies {worst_e:.2e}")
    assert worst_m <= tol_m
    assert worst_e <= tol_e


# ---------------------------------------------------- pipelined pass kernel --
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("shape", [(256, 256, 16), (64, 128, 256), (128, 64, 64), (256, 64), (64, 256)])
def test_pipelined_pass_matches_direct_kernel(sfd, O, precision, shape):
    """The asynchronous-copy pipeline changes how tiles move, not the
    arithmetic: without the mass lock (whose FP64 sums are accumulated in a
    different order) results are bitwise identical."""
    nd = len(shape)
    bounds = tuple((-4.0, 4.0 + a) for a in range(nd))
    psi0 = random_field(shape, seed=17)
    V = O.quadratic_potential(shape, bounds)
    kw = dict(coeffD=-0.5, beta=25.0, V=V, dt=2e-3, nsteps=6, precision=precision, masslock=False)
    a = run_model(sfd, shape, bounds, psi0, pipeline=True, **kw)
    b = run_model(sfd, shape, bounds, psi0, pipeline=False, **kw)
    assert np.array_equal(a, b)
    if precision == "fp32":
        c = run_model(sfd, shape, bounds, psi0, pipeline=True, **dict(kw, masslock=True))
        d = run_model(sfd, shape, bounds, psi0, pipeline=False, **dict(kw, masslock=True))
        assert O.rel_l2(c, d) < 1e-6


# ------------------------------------------------ FP32 coverage, every size --
@pytest.mark.parametrize("shape,nd", SHAPES)
def test_fp32_fused_shapes(sfd, O, shape, nd):
    """Every line length 2..256 and both layouts in FP32 (lean and full
    instantiations: trap potential and rotation), vs the FP64 oracle."""
    bounds = tuple((-3.0 - a, 4.0 + 0.5 * a) for a in range(nd))
    psi0 = random_field(shape, seed=7 + sum(shape))
    V = O.quadratic_potential(shape, bounds, gammas=[1.0, 0.7, 1.3][:nd])
    for omega in (0.0, 0.3):
        kw = dict(coeffD=-0.5, beta=3.0, omega=omega, V=V, dt=2e-3, nsteps=5)
        got = run_model(sfd, shape, bounds, psi0, precision="fp32", **kw)
        ref = O.c_step(psi0, bounds, **kw)
        assert O.rel_l2(got, ref) < TOL32


@pytest.mark.parametrize("shape,nd", SHAPES)
def test_fp32_compensated_shapes(sfd, O, shape, nd):
    """Compensated FP32 passes (GPSS_FLAG_COMPENSATED) at every line length
    2..256 in both layouts, trap potential and rotation, Strang and Lie: within
    1e-6 of the FP64 oracle, and no farther from it than the plain FP32 passes."""
    bounds = tuple((-3.0 - a, 4.0 + 0.5 * a) for a in range(nd))
    psi0 = random_field(shape, seed=7 + sum(shape))
    V = O.quadratic_potential(shape, bounds, gammas=[1.0, 0.7, 1.3][:nd])
    for omega in (0.0, 0.3):
        for scheme in (2, 1):
            kw = dict(coeffD=-0.5, beta=3.0, omega=omega, V=V, dt=2e-3, nsteps=5, scheme=scheme)
            ref = O.c_step(psi0, bounds, **kw)
            comp = run_model(sfd, shape, bounds, psi0, precision="fp32", compensated=True, **kw)
            plain = run_model(sfd, shape, bounds, psi0, precision="fp32", **kw)
            ec, ep = O.rel_l2(comp, ref), O.rel_l2(plain, ref)
            assert ec < 1e-6, (omega, scheme, ec)
            assert ec <= 1.05 * ep + 1e-8, (omega, scheme, ec, ep)


@pytest.mark.parametrize("shape", [(64, 32), (16, 8, 32)])
def test_fp32_compensated_imaginary_unmerged(sfd, O, shape):
    """Imaginary time with the unmerged sequence (GPSS_FLAG_NOMERGE) runs the
    compensated passes too: within 1e-6 of the FP64 oracle after 20 steps."""
    nd = len(shape)
    bounds = tuple((-6.0, 6.0 + a) for a in range(nd))
    psi0 = random_field(shape, seed=13)
    V = O.quadratic_potential(shape, bounds)
    kw = dict(coeffD=-0.5, beta=40.0, V=V, dt=1e-2, nsteps=20, imag=True)
    ref = O.c_step(psi0, bounds, **kw)
    got = run_model(sfd, shape, bounds, psi0, precision="fp32", compensated=True, merge=False, **kw)
    assert O.rel_l2(got, ref) < 1e-6


# ------------------------------------------- full-size (256^3) properties --
@pytest.mark.parametrize("compensated,bar", [(False, 3e-6), (True, LINEAR_FLOW_BAR_COMP)])
def test_fullsize_linear_flow_is_exact_fp32(sfd, O, W, compensated, bar):
    """beta = V = 0 at 256^3: every merged FP32 pass applies the exact kinetic
    factor, so 20 steps equal exp(i coeffD |k|^2 t) on the spectrum (numpy
    FFT in complex128 of the same input) to FP32 round-off.  The compensated
    passes leave only the rounding of each pass's store (63 of them here)."""
    c = W.cfg1(256)
    got = run_model(sfd, c["shape"], c["bounds"], c["psi"], coeffD=c["coeffD"], beta=0.0, dt=c["dt"],
                    nsteps=20, precision="fp32", compensated=compensated)
    F = np.fft.fftn(c["psi"])
    k2 = 0
    for a in range(3):
        xi = np.fft.fftfreq(256, 2 * math.pi / 256) * 2 * math.pi
        s = [1, 1, 1]
        s[a] = 256
        k2 = k2 + xi.reshape(s) ** 2
    want = np.fft.ifftn(F * np.exp(1j * c["coeffD"] * k2 * (20 * c["dt"])))
    err = O.rel_l2(got, want)
    print(f"linear flow, compensated={compensated}: rel-L2 {err:.3e}")
    assert err < bar


@pytest.mark.parametrize("compensated,bar", [(False, 1e-5), (True, REVERSAL_BAR_COMP)])
def test_fullsize_time_reversal_fp32(sfd, O, W, compensated, bar):
    """Strang splitting is time-reversible: N(-dt) undoes N(dt) (it keeps
    |psi|), the kinetic flows are unitary.  40 steps forward then 40 with -dt
    at 256^3 in FP32 return the initial field to round-off, and the FP64
    reductions see the mass and energy come back."""
    c = W.cfg1(256)
    g = sfd.Grid(c["shape"], c["bounds"])
    f = sfd.Field(g)
    f.phi = c["psi"]
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialZero(f), coeffD=c["coeffD"], beta=c["beta"])
    n = sfd.NumModelSplit2(f, p, c["dt"], 1, 1, precision="fp32", compensated=compensated)
    e0 = n.energies()
    n.step(40)
    mid = f.phi.copy()
    n.dt = -c["dt"]
    n.step(40)
    back = f.phi.copy()
    e1 = n.energies()
    n.close()
    err = O.rel_l2(back, c["psi"])
    print(f"time reversal, compensated={compensated}: rel-L2 {err:.3e}, energy {abs(e1[3] - e0[3]) / abs(e0[3]):.2e}")
    assert O.rel_l2(mid, c["psi"]) > 1e-2          # the field did move
    assert err < bar
    assert abs(e1[3] - e0[3]) < 1e-5 * abs(e0[3])


# ----------------------------------------------------------- energy cache --
@pytest.mark.parametrize("omega", [0.0, 0.4])
@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp32c"])
def test_energy_cache_solve(sfd, O, precision, omega):
    """GPSS_FLAG_ENERGY_CACHE: solve!'s energy-then-timeStep! sequence gives
    the same energy records as without the cache, with fewer passes per
    iteration (none beyond the step at Omega = 0, one read-only x pass with
    rotation, against 3); the cache follows every change of the field and of
    the parameters.  fp32c: FP32 with the compensated passes."""
    comp = precision == "fp32c"
    precision = "fp32" if comp else precision
    shape, bounds = (32, 16, 8), ((-5.0, 5.0), (-4.0, 4.0), (-3.0, 3.0))
    psi0 = random_field(shape, seed=5)
    V = O.quadratic_potential(shape, bounds)
    L = sfd._lib.lib()
    res, launches = {}, {}
    for cache in (False, True):
        g = sfd.Grid(shape, bounds)
        f = sfd.Field(g)
        f.phi = psi0
        p = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, V), coeffD=-0.5, beta=30.0, Omega=omega)
        n = sfd.NumModelSplit2(f, p, 2e-3, 20, 100, precision=precision, energy_cache=cache, compensated=comp)
        l0 = L.gpss_launch_count(n.handle)
        res[cache] = np.array(sfd.solve(n))
        launches[cache] = L.gpss_launch_count(n.handle) - l0
        if cache:
            # a new field, then new parameters: the energies follow
            n.f.phi = psi0
            n.upload()
            f2 = sfd.Field(sfd.Grid(shape, bounds))
            f2.phi = psi0
            fresh = sfd.NumModelSplit2(f2, p, 2e-3, 1, 1, precision=precision, compensated=comp)
            assert np.allclose(n.energies(), fresh.energies(), rtol=1e-12, atol=0)
            p2 = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, V), coeffD=-0.5, beta=10.0, Omega=omega)
            n.step(3)
            n.set_params(p2)
            fresh.set_params(p2)
            fresh.step(3)  # the same 3 steps, now under the new parameters
            n.f.phi = psi0
            n.upload()
            n.step(3)
            assert np.allclose(n.energies(), fresh.energies(), rtol=1e-12 if precision == "fp64" else 1e-6, atol=0)
            fresh.close()
        n.close()
    tol = 1e-12 if precision == "fp64" else 1e-6
    scale = np.max(np.abs(res[False][:, 2:]))
    assert np.max(np.abs(res[True] - res[False])) <= tol * scale
    assert launches[True] < launches[False]


# ------------------------------------------- pending trailing half step --
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_pending_half_step_chains_calls(sfd, O, precision):
    """A merged real-time Strang call leaves its last half kinetic flow
    pending and the next call folds it into its first flow: K one-step calls
    are bitwise one K-step call, with one kinetic flow per call instead of
    two; reading the field (download) applies the pending flow.  Calls with
    diagnostics run their trailing half step eagerly (two half flows per
    step instead of one merged flow: equal to round-off)."""
    shape, bounds = (32, 16, 8), ((-4.0, 4.0), (-3.0, 3.0), (-2.0, 2.0))
    psi0 = random_field(shape, seed=31)
    V = O.quadratic_potential(shape, bounds)
    L = sfd._lib.lib()
    K = 10

    def model():
        g = sfd.Grid(shape, bounds)
        f = sfd.Field(g)
        f.phi = psi0
        p = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, V), coeffD=-0.5, beta=3.0)
        return f, sfd.NumModelSplit2(f, p, 1e-3, K, K, precision=precision)

    f1, n1 = model()
    n1.step(K)
    one_call = f1.phi.copy()
    n1.close()
    f2, n2 = model()
    l0 = L.gpss_launch_count(n2.handle)
    for _ in range(K):
        n2.step(1)
    l1 = L.gpss_launch_count(n2.handle)
    chained = f2.phi.copy()  # download applies the pending flow
    n2.close()
    assert np.array_equal(chained, one_call)
    assert l1 - l0 <= 3 * K + 1  # one flow per call (+ the FP32 mass-lock target of the first call)
    # the eager trailing half step (diagnostics requested) gives the same field
    f3, n3 = model()
    for _ in range(K):
        n3.step(1, diag=True)
    eager = f3.phi.copy()
    n3.close()
    assert O.rel_l2(eager, one_call) < (1e-13 if precision == "fp64" else 1e-6)
    ref = O.c_step(psi0, bounds, coeffD=-0.5, beta=3.0, V=V, nsteps=K, dt=1e-3)
    assert O.rel_l2(chained, ref) < (TOL64 if precision == "fp64" else TOL32)


def test_pending_half_step_flushes_before_parameter_change(sfd, O):
    """A pending flow belongs to the parameters it was computed with:
    set_params applies it first, so changing coeffD between one-step calls
    matches the oracle's two runs back to back."""
    shape, bounds = (32, 16, 8), ((-4.0, 4.0), (-3.0, 3.0), (-2.0, 2.0))
    psi0 = random_field(shape, seed=32)
    g = sfd.Grid(shape, bounds)
    f = sfd.Field(g)
    f.phi = psi0
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialZero(f), coeffD=-0.5, beta=3.0)
    n = sfd.NumModelSplit2(f, p, 1e-3, 4, 4, precision="fp64")
    n.step(1)
    n.step(1)
    n.set_params(sfd.GrossPitaevskiiParameters(sfd.PotentialZero(f), coeffD=-0.3, beta=3.0))
    n.step(2)
    got = f.phi.copy()
    n.close()
    mid = O.c_step(psi0, bounds, coeffD=-0.5, beta=3.0, nsteps=2, dt=1e-3)
    ref = O.c_step(mid, bounds, coeffD=-0.3, beta=3.0, nsteps=2, dt=1e-3)
    assert O.rel_l2(got, ref) < TOL64


@pytest.mark.parametrize("shape", [(64, 32), (32, 16, 8)])
def test_energy_cache_rotation_vs_oracle(sfd, O, shape):
    """GPSS_FLAG_ENERGY_CACHE with Omega != 0: the energies solve! records at
    every iteration (from the last passes of each step plus one read-only x
    pass) match the oracle's energy of its own run (GrossPitaevskii.jl:61-81,
    E_Omega from the rotation sums; NumModels.jl:32-35), FP64."""
    nd = len(shape)
    bounds = tuple((-5.0 + a, 5.0) for a in range(nd))
    psi0 = random_field(shape, seed=41)
    V = O.quadratic_potential(shape, bounds)
    kw = dict(coeffD=-0.5, beta=30.0, omega=0.4, V=V)
    g = sfd.Grid(shape, bounds)
    f = sfd.Field(g)
    f.phi = psi0
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, V), coeffD=-0.5, beta=30.0, Omega=0.4)
    n = sfd.NumModelSplit2(f, p, 2e-3, 6, 100, precision="fp64", energy_cache=True)
    rec = np.array(sfd.solve(n))
    n.close()
    ref = psi0
    for row in rec:
        e_ref = O.c_energy(ref, bounds, **kw)
        scale = max(abs(v) for v in e_ref[:4])
        assert np.max(np.abs(row[2:6] - np.array(e_ref[:4]))) <= 1e-11 * scale
        ref = O.c_step(ref, bounds, nsteps=1, dt=2e-3, **kw)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-14), ("fp32", 2e-7)])
def test_device_norm_and_normalize(sfd, O, precision, tol):
    """norm(f) and normalize!(f) (Fields.jl:172-200) on a model-owned field run
    on the device (gpss_norm, gpss_normalize: FP64 sums) and match the oracle's
    c_norm; after a step (whose last half flow may be pending) too."""
    shape, bounds = (64, 32, 16), ((-4.0, 4.0), (-3.0, 5.0), (-2.0, 2.0))
    psi0 = 3.7 * random_field(shape, seed=51)
    g = sfd.Grid(shape, bounds)
    f = sfd.Field(g)
    f.phi = psi0
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialZero(f), coeffD=-0.5, beta=2.0)
    n = sfd.NumModelSplit2(f, p, 1e-3, 1, 1, precision=precision)
    src = psi0.astype(np.complex64).astype(np.complex128) if precision == "fp32" else psi0
    want = O.c_norm(src, bounds)
    assert abs(sfd.norm(f) - want) <= tol * want
    sfd.normalize(f)
    assert abs(sfd.norm(f) - 1.0) <= tol
    assert O.rel_l2(f.phi, src / want) <= tol
    n.step(3)  # leaves its last half kinetic flow pending: norm applies it first
    nrm = sfd.norm(f)
    after = f.phi.copy()
    assert abs(nrm - O.c_norm(after, bounds)) <= 2 * tol
    n.close()
