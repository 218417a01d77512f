"""The CPU oracle pinned against the reference's own known-answer tests
(test/runtests.jl), and against a second, independent restatement that uses
numpy's FFT.  No GPU is needed."""
import math

import numpy as np
import pytest

TOL_FFT = 1e-10  # test/runtests.jl:9


def relerr(a, b):  # test/runtests.jl:5
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(np.asarray(b))))


def plane_wave(O, shape, bounds, modes):
    xs = [O.grid_coords(n, b[0], b[1]) for n, b in zip(shape, bounds)]
    X = np.meshgrid(*xs, indexing="ij")
    ks = [2 * math.pi * m / (b[1] - b[0]) for m, b in zip(modes, bounds)]
    return np.asfortranarray(np.exp(1j * sum(k * x for k, x in zip(ks, X)))), X, ks


def test_grid_nodes_and_wavenumbers(O):
    x = O.grid_coords(128, -8, 8)
    assert x[0] == -8.0 and abs(x[-1] - (8 - 0.125)) < 1e-14
    assert np.allclose(np.diff(x), 0.125, atol=1e-14)
    xi = O.fftfreq(8, 0.5)
    assert np.allclose(xi, np.fft.fftfreq(8, 0.5) * 2 * math.pi, rtol=0, atol=1e-15)
    assert xi[4] < 0  # Nyquist entry is negative, as AbstractFFTs.fftfreq


def test_fft_derivatives_2d_rotation(O):
    """runtests.jl:29-46: 64^2 on [-12,12]^2, mode (2,3)."""
    b = ((-12, 12), (-12, 12))
    psi, (X, Y), (kx, ky) = plane_wave(O, (64, 64), b, (2, 3))
    d = O.c_derivatives(psi, b)
    assert relerr(d["dx"], 1j * kx * psi) < TOL_FFT
    assert relerr(d["dy"], 1j * ky * psi) < TOL_FFT
    assert relerr(d["rx"], Y * d["dx"]) < TOL_FFT
    assert relerr(d["ry"], -X * d["dy"]) < TOL_FFT


def test_fft_derivatives_3d_rotation(O):
    """runtests.jl:48-62: 48^3 on [-12,12]^3 (not a power of two), mode (2,3,4)."""
    b = ((-12, 12),) * 3
    psi, (X, Y, Z), (kx, ky, kz) = plane_wave(O, (48, 48, 48), b, (2, 3, 4))
    d = O.c_derivatives(psi, b)
    assert relerr(d["dx"], 1j * kx * psi) < TOL_FFT
    assert relerr(d["dy"], 1j * ky * psi) < TOL_FFT
    assert relerr(d["dz"], 1j * kz * psi) < TOL_FFT
    assert relerr(d["rx"], Y * d["dx"]) < TOL_FFT
    assert relerr(d["ry"], -X * d["dy"]) < TOL_FFT


def test_fft_round_trip(O):
    """runtests.jl:673-692 (non-cubic 32x24x40 box): transform and back per axis."""
    rng = np.random.default_rng(0)
    a = np.asfortranarray(rng.standard_normal((32, 24, 40)) + 1j * rng.standard_normal((32, 24, 40)))
    for ax in range(3):
        f = O.c_fft_axis(a, ax)
        assert relerr(f, np.fft.fft(a, axis=ax)) < TOL_FFT
        back = O.c_fft_axis(f, ax, inverse=True)
        assert relerr(back, a) < TOL_FFT


def test_norm_and_normalize(O):
    """runtests.jl:718-725: phi = 1 on [-12,12]^2 has norm sqrt(Lx Ly)."""
    b = ((-12, 12), (-12, 12))
    a = np.ones((64, 64), dtype=complex, order="F")
    assert abs(O.c_norm(a, b) - math.sqrt(24 * 24)) < 1e-12
    a2 = a / O.c_norm(a, b)
    assert abs(O.c_norm(a2, b) - 1.0) < 1e-14


def _order_runs(O, step):
    N, L, beta, T = 32, 2 * math.pi, 20.0, 0.2
    b = ((-L, L), (-L, L))
    x = O.grid_coords(N, -L, L)
    X, Y = x[:, None], x[None, :]
    p = np.asfortranarray((1 + 0.3 * np.cos(X) + 0.2 * np.sin(2 * Y)) * np.exp(1j * 0.5 * X))
    p = p / O.c_norm(p, b)
    out = {}
    for order, ns in ((1, (50, 100, 200)), (2, (25, 50, 100))):
        out[order] = [step(p, b, coeffD=-0.5, beta=beta, nsteps=k, scheme=order, dt=T / k) for k in ns]
    return out


@pytest.mark.parametrize("impl", ["c", "numpy"])
def test_split_order_and_mass_conservation(O, impl):
    """runtests.jl:644-671: order bands (0.85,1.15) Lie / (1.85,2.15) Strang,
    mass conserved to 1e-12."""
    step = O.c_step if impl == "c" else O.np_step
    runs = _order_runs(O, step)
    for order, lo, hi in ((1, 0.85, 1.15), (2, 1.85, 2.15)):
        r = runs[order]
        d = [np.sqrt(np.sum(np.abs(r[i] - r[i + 1]) ** 2) / np.sum(np.abs(r[i + 1]) ** 2)) for i in range(2)]
        assert lo < math.log2(d[0] / d[1]) < hi
        m = [np.sum(np.abs(q) ** 2) for q in r]
        assert max(abs(v - m[0]) for v in m) < 1e-12


def test_linear_flow_exact(O):
    """beta = V = Omega = 0: the split step reproduces exp(i coeffD k^2 t) exactly."""
    shape, b = (16, 8, 32), ((-math.pi, math.pi), (-2.0, 2.0), (0.0, 3.0))
    rng = np.random.default_rng(1)
    p = np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    got = O.c_step(p, b, coeffD=-0.5, beta=0.0, nsteps=10, dt=1e-2)
    F = np.fft.fftn(p)
    for a, (n, bb) in enumerate(zip(shape, b)):
        xi = np.fft.fftfreq(n, (bb[1] - bb[0]) / n) * 2 * math.pi
        s = [1, 1, 1]
        s[a] = n
        F = F * np.exp(1j * -0.5 * xi.reshape(s) ** 2 * 0.1)
    assert O.rel_l2(got, np.fft.ifftn(F)) < 1e-13


@pytest.mark.parametrize("imag", [False, True])
@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("shape", [(16, 32), (8, 16, 4)])
def test_c_oracle_matches_numpy_oracle(O, imag, scheme, shape):
    nd = len(shape)
    b = tuple((-4.0 - a, 5.0) for a in range(nd))
    rng = np.random.default_rng(2)
    p = np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    V = O.quadratic_potential(shape, b)
    kw = dict(coeffD=-0.5, beta=3.0, omega=0.4, V=V, nsteps=4, scheme=scheme, imag=imag, dt=1e-2)
    assert O.rel_l2(O.c_step(p, b, **kw), O.np_step(p, b, **kw)) < 1e-13


def test_timed_legs_match_the_oracle(O):
    """The timing legs of the CPU baseline step the same field as c_step: the
    loop-timed C entry point bit for bit, the scipy.fft restatement to FP64
    round-off; both report a positive loop time."""
    shape, bounds = (16, 8, 32), ((0.0, 6.0), (0.0, 5.0), (0.0, 7.0))
    rng = np.random.default_rng(3)
    psi = np.asfortranarray(np.exp(1j * rng.uniform(0, 0.3, shape)))
    kw = dict(coeffD=-0.0353, beta=14.1, nsteps=4, dt=2.5e-3)
    ref = O.c_step(psi, bounds, **kw)
    a, ta = O.c_step_timed(psi, bounds, **kw)
    b, tb = O.sp_step_timed(psi, bounds, workers=2, **kw)
    assert np.array_equal(a, ref) and ta > 0
    assert O.rel_l2(b, ref) < 1e-13 and tb > 0


def test_energy_formulas(O):
    """Derivative route of GrossPitaevskii.jl:61-136 vs a Parseval evaluation."""
    shape, b = (32, 16, 8), ((-5.0, 6.0),) * 3
    rng = np.random.default_rng(3)
    p = np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    V = O.quadratic_potential(shape, b)
    cD, beta, om = -0.4, 7.0, 0.6
    got = O.c_energy(p, b, coeffD=cD, beta=beta, omega=om, V=V)
    dV = np.prod([(bb[1] - bb[0]) / n for n, bb in zip(shape, b)])
    xs = [O.grid_coords(n, bb[0], bb[1]) for n, bb in zip(shape, b)]
    xis = [np.fft.fftfreq(n, (bb[1] - bb[0]) / n) * 2 * math.pi for n, bb in zip(shape, b)]
    grad, rot = 0.0, [0.0, 0.0]
    for a in range(3):
        F = np.fft.fft(p, axis=a)
        s = [1, 1, 1]
        s[a] = shape[a]
        xi = xis[a].reshape(s)
        grad += np.sum(xi ** 2 * np.abs(F) ** 2) / shape[a]
        if a < 2:
            other = 1 - a
            so = [1, 1, 1]
            so[other] = shape[other]
            rot[a] = np.sum(xs[other].reshape(so) * xi * np.abs(F) ** 2) / shape[a]
    rho = np.abs(p) ** 2
    eom = -om * (rot[0] - rot[1]) * dV
    edel = (-cD * grad + np.sum(V * rho)) * dV
    eb = 0.5 * beta * np.sum(rho ** 2) * dV
    ref = (eom, edel, eb, -eom + edel + eb, -eom + edel + 2 * eb)
    for a, r in zip(got, ref):
        assert abs(a - r) <= 1e-12 * max(abs(v) for v in ref)


def test_golden_fixtures_reproduce(O):
    """The committed golden vectors (tests/golden/) are what the oracle computes."""
    import os
    here = os.path.join(os.path.dirname(__file__), "golden")
    names = sorted(f for f in os.listdir(here) if f.endswith(".npz") and not f.endswith((".grad.npz", ".solver.npz", ".ground.npz")))
    assert names, "no golden fixtures"
    for nm in names:
        z = np.load(os.path.join(here, nm))
        b = tuple(tuple(r) for r in z["bounds"])
        V = z["V"] if z["has_V"] else None
        out = O.c_step(z["psi0"], b, coeffD=float(z["coeffD"]), beta=float(z["beta"]),
                       omega=float(z["omega"]), V=V, nsteps=int(z["nsteps"]), scheme=int(z["scheme"]),
                       imag=bool(z["imag"]), dt=float(z["dt"]))
        assert O.rel_l2(out, z["psi"]) < 1e-13, nm
        # the FP64 oracle's own distance to the long-double reference
        assert O.rel_l2(z["psi"], z["psi_ext"]) < 1e-12, nm
        e = O.c_energy(z["psi"], b, coeffD=float(z["coeffD"]), beta=float(z["beta"]),
                       omega=float(z["omega"]), V=V)
        assert np.allclose(e, z["energy"], rtol=1e-12, atol=1e-14), nm
        # the traces: chunked runs give the recorded mass and energy(n) values
        kw = dict(coeffD=float(z["coeffD"]), beta=float(z["beta"]), omega=float(z["omega"]), V=V)
        p = z["psi0"].copy(order="F")
        steps = z["trace_steps"]
        for i, s in enumerate(steps):
            if i:
                p = O.c_step(p, b, nsteps=int(s - steps[i - 1]), scheme=int(z["scheme"]), imag=bool(z["imag"]),
                             dt=float(z["dt"]), **kw)
            assert abs(O.c_norm(p, b) ** 2 - z["trace_mass"][i]) <= 1e-12 * z["trace_mass"][i], (nm, s)
            e = np.array(O.c_energy(p, b, **kw))
            assert np.max(np.abs(e - z["trace_energy"][i])) <= 1e-12 * np.max(np.abs(e)), (nm, s)


def test_golden_cfg_fixtures_present():
    """Seeded workloads 0-4 each have a golden fixture (1-3 at reduced sizes)."""
    import os
    here = os.path.join(os.path.dirname(__file__), "golden")
    names = set(os.listdir(here))
    for nm in ("cfg0_2d_128_1000.npz", "cfg1_3d_32_200.npz", "cfg2_3d_32_200.npz", "cfg3_run_64_s0.npz",
               "cfg3_run_64_s2.npz", "cfg4_grad_32.grad.npz"):
        assert nm in names, nm


def test_golden_gradient_reproduces(O):
    """The cfg4 gradient fixture: the dual-number restatement gives the
    recorded loss and directional derivatives."""
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "cfg4_grad_32.grad.npz"))
    b = tuple(tuple(r) for r in z["bounds"])
    for dv, dpsi, dL in zip(z["dV"], z["dpsi0"], z["dL"]):
        L, d = O.np_tangent_loss(z["psi0"], np.asfortranarray(dpsi), z["V"], np.asfortranarray(dv), z["target"], b,
                                 coeffD=float(z["coeffD"]), beta=float(z["beta"]), nsteps=int(z["nsteps"]),
                                 dt=float(z["dt"]))
        assert abs(L - float(z["L"])) < 1e-13
        assert abs(d - dL) <= 1e-12 * abs(dL)


def _solver_fixtures():
    import os
    here = os.path.join(os.path.dirname(__file__), "golden")
    return sorted(os.path.join(here, f) for f in os.listdir(here) if f.endswith(".solver.npz"))


def test_solver_fixtures_present():
    import os
    names = {os.path.basename(p) for p in _solver_fixtures()}
    assert names == {"rk4_product_2d_rot.solver.npz", "rk2_solution_3d.solver.npz", "backwardeuler_2d.solver.npz",
                     "cranknicolson_2d.solver.npz"}


@pytest.mark.parametrize("path", _solver_fixtures(), ids=lambda p: p.rsplit("/", 1)[-1])
def test_golden_solver_reproduces(O, path):
    """The committed explicit-RK and implicit-scheme fixtures: the oracle
    reproduces the field (and the implicit schemes' Krylov count)."""
    z = np.load(path)
    b = tuple(tuple(r) for r in z["bounds"])
    kw = dict(coeffD=float(z["coeffD"]), beta=float(z["beta"]), omega=float(z["omega"]), V=z["V"],
              nsteps=int(z["nsteps"]), dt=float(z["dt"]))
    if str(z["kind"]) == "rk":
        out = O.c_rk_step(z["psi0"], b, stepper=str(z["stepper"]), filter=str(z["filter"]), **kw)
    else:
        out, iters = O.c_implicit_step(z["psi0"], b, scheme=str(z["scheme"]), **kw)
        assert iters == int(z["krylov"])
    assert O.rel_l2(out, z["psi"]) < 1e-14
