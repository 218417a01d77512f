"""The discrete adjoint of the Strang step (gpss_adjoint) against central
finite differences of the GPU's own FP64 forward map, and against the
dual-number (forward-mode) restatement of the reference path in the oracle.

Bar: the gradient agrees with finite differences to 1e-6 relative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# FP32 adjoints against the FP64 one (relative L2 of the gradients; measured
# on GB300: cfg4 full size 1.7e-5 plain, 5.6e-7 compensated; 64^2 cases
# 0.9-1.3e-6 for dL/dV and 3-4e-6 for dL/dpsi0, compensated)
BAR_CFG4_PLAIN = 1e-4
BAR_CFG4_COMP = 1e-5
BAR_SMALL_COMP = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def _model(sfd, c, V, precision="fp64", compensated=False, Omega=0.0):
    g = sfd.Grid(c["shape"], c["bounds"])
    f = sfd.Field(g)
    f.phi = c["psi"]
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, V), coeffD=c["coeffD"], beta=c["beta"], Omega=Omega)
    return f, sfd.NumModelSplit2(f, p, c["dt"], c["nsteps"], c["nsteps"], precision=precision,
                                 merge=False, masslock=False, compensated=compensated)


def _loss(sfd, O, c, V, nsteps, psi0=None):
    """L of the GPU FP64 forward map (unmerged Strang, as in the adjoint)."""
    cc = dict(c, psi=c["psi"] if psi0 is None else psi0)
    f, n = _model(sfd, cc, V)
    n.step(nsteps)
    psi = f.phi.copy(order="F")
    n.close()
    dV = np.prod([(b[1] - b[0]) / m for m, b in zip(c["shape"], c["bounds"])])
    z = np.sum(np.conj(c["target"]) * psi) * dV
    return 1.0 - abs(z) ** 2


def _directions(shape, count, seed, smooth=4.0):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        a = rng.standard_normal(shape)
        F = np.fft.fft2(a)
        kx = np.fft.fftfreq(shape[0])[:, None] * shape[0]
        ky = np.fft.fftfreq(shape[1])[None, :] * shape[1]
        a = np.fft.ifft2(F * np.exp(-(kx ** 2 + ky ** 2) / smooth ** 2)).real
        out.append(np.asfortranarray(a / np.max(np.abs(a))))
    return out


def test_adjoint_dV_vs_finite_differences(sfd, O, W):
    """32 seeded directions, 32^2 copy of the gradient workload, 60 steps,
    checkpoints every 7 steps (a partial last segment)."""
    c = W.cfg4(32)
    nsteps, K = 60, 7
    f, n = _model(sfd, c, c["V"])
    L, dLdV, _ = n.adjoint(c["target"], nsteps, K)
    n.close()
    eps = 1e-4
    worst = 0.0
    for dv in _directions(c["shape"], 32, seed=5):
        fd = (_loss(sfd, O, c, c["V"] + eps * dv, nsteps) - _loss(sfd, O, c, c["V"] - eps * dv, nsteps)) / (2 * eps)
        adj = float(np.sum(dLdV * dv))
        worst = max(worst, abs(fd - adj) / max(abs(adj), 1e-300))
    assert abs(L - _loss(sfd, O, c, c["V"], nsteps)) < 1e-13
    assert worst < 1e-6


def test_adjoint_dpsi0_vs_finite_differences(sfd, O, W):
    c = W.cfg4(32)
    nsteps, K = 40, 10
    f, n = _model(sfd, c, c["V"])
    L, _, g0 = n.adjoint(c["target"], nsteps, K)
    n.close()
    rng = np.random.default_rng(9)
    eps = 1e-5
    for _ in range(8):
        d = rng.standard_normal(c["shape"]) + 1j * rng.standard_normal(c["shape"])
        d = np.asfortranarray(d / np.max(np.abs(d)))
        fd = (_loss(sfd, O, c, c["V"], nsteps, c["psi"] + eps * d)
              - _loss(sfd, O, c, c["V"], nsteps, c["psi"] - eps * d)) / (2 * eps)
        adj = float(np.real(np.sum(np.conj(g0) * d)))
        assert abs(fd - adj) <= 1e-6 * abs(adj)


def test_adjoint_vs_dual_numbers_of_the_reference_path(sfd, O, W):
    """Directional derivative from the oracle's dual-number restatement of
    the reference's Strang step on a 32^2 copy."""
    c = W.cfg4(32)
    nsteps, K = 50, 8
    f, n = _model(sfd, c, c["V"])
    L, dLdV, g0 = n.adjoint(c["target"], nsteps, K)
    n.close()
    rng = np.random.default_rng(3)
    for dv in _directions(c["shape"], 4, seed=11):
        dpsi = np.asfortranarray(0.1 * (rng.standard_normal(c["shape"]) + 1j * rng.standard_normal(c["shape"])))
        Lo, dLo = O.np_tangent_loss(c["psi"], dpsi, c["V"], dv, c["target"], c["bounds"], coeffD=c["coeffD"],
                                    beta=c["beta"], nsteps=nsteps, dt=c["dt"])
        adj = float(np.sum(dLdV * dv)) + float(np.real(np.sum(np.conj(g0) * dpsi)))
        assert abs(L - Lo) < 1e-12
        assert abs(adj - dLo) <= 1e-8 * abs(dLo)


def test_adjoint_cfg4_full_size(sfd, O, W):
    """cfg4 at full size (256^2, 2000 steps, K = 50): FP64 gradient against
    central differences on 4 of the seeded directions; FP32 forward with FP64
    dL/dV accumulation against the FP64 gradient."""
    c = W.cfg4(256)
    nsteps, K = c["nsteps"], c["K"]
    res = {}
    for prec in ("fp64", "fp32"):
        f, n = _model(sfd, c, c["V"], precision=prec)
        res[prec] = n.adjoint(c["target"], nsteps, K)
        n.close()
    L64, dV64, g64 = res["fp64"]
    L32, dV32, g32 = res["fp32"]
    eps = 1e-4
    for dv in _directions(c["shape"], 4, seed=21, smooth=16.0):
        fd = (_loss(sfd, O, c, c["V"] + eps * dv, nsteps) - _loss(sfd, O, c, c["V"] - eps * dv, nsteps)) / (2 * eps)
        adj = float(np.sum(dV64 * dv))
        assert abs(fd - adj) <= 1e-6 * abs(adj)
    assert abs(L32 - L64) < 1e-6
    assert np.linalg.norm(dV32 - dV64) / np.linalg.norm(dV64) < BAR_CFG4_PLAIN


def test_adjoint_with_rotation_vs_finite_differences(sfd, O, W):
    """Omega != 0 (the x and y flows do not commute, so the unmerged
    sequence is differentiated): dL/dV against central differences."""
    c = W.cfg4(32)
    nsteps, K = 30, 7
    g = sfd.Grid(c["shape"], c["bounds"])

    def model(V):
        f = sfd.Field(g)
        f.phi = c["psi"]
        p = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, V), coeffD=c["coeffD"], beta=c["beta"], Omega=0.4)
        return f, sfd.NumModelSplit2(f, p, c["dt"], nsteps, nsteps, merge=False, masslock=False)

    def loss(V):
        f, n = model(V)
        n.step(nsteps)
        psi = f.phi.copy(order="F")
        n.close()
        dV = np.prod([(b[1] - b[0]) / m for m, b in zip(c["shape"], c["bounds"])])
        return 1.0 - abs(np.sum(np.conj(c["target"]) * psi) * dV) ** 2

    f, n = model(c["V"])
    L, dLdV, _ = n.adjoint(c["target"], nsteps, K)
    n.close()
    assert abs(L - loss(c["V"])) < 1e-13
    eps = 1e-4
    for dv in _directions(c["shape"], 4, seed=13):
        fd = (loss(c["V"] + eps * dv) - loss(c["V"] - eps * dv)) / (2 * eps)
        assert abs(fd - float(np.sum(dLdV * dv))) <= 1e-6 * abs(fd)


def test_adjoint_golden_cfg4_32(sfd, W):
    """The committed cfg4 gradient fixture (32^2, 50 steps): loss and four
    directional derivatives from the oracle's dual-number restatement."""
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "cfg4_grad_32.grad.npz"))
    b = tuple(tuple(r) for r in z["bounds"])
    c = dict(shape=z["psi0"].shape, bounds=b, psi=z["psi0"], coeffD=float(z["coeffD"]), beta=float(z["beta"]),
             dt=float(z["dt"]), nsteps=int(z["nsteps"]))
    f, n = _model(sfd, c, z["V"])
    L, dLdV, g0 = n.adjoint(z["target"], int(z["nsteps"]), 8)
    n.close()
    assert abs(L - float(z["L"])) < 1e-12
    for dv, dpsi, dL in zip(z["dV"], z["dpsi0"], z["dL"]):
        adj = float(np.sum(dLdV * dv)) + float(np.real(np.sum(np.conj(g0) * dpsi)))
        assert abs(adj - dL) <= 1e-8 * abs(dL)


def test_overlap_loss_autograd_function(sfd, W):
    """overlap_loss as a torch.autograd.Function: its loss and gradients are
    those of gpss_adjoint, they chain through other torch operations, and a
    central difference of the function itself agrees with the gradient."""
    import importlib
    torch = pytest.importorskip("torch")
    AD = importlib.import_module("sfd_gb300.autodiff")
    c = W.cfg4(32)
    nsteps, K = 40, 7
    f, n = _model(sfd, c, c["V"])
    L_ref, dV_ref, g_ref = n.adjoint(c["target"], nsteps, K)
    V = torch.tensor(np.ascontiguousarray(c["V"]), dtype=torch.float64, requires_grad=True)
    psi0 = torch.tensor(np.ascontiguousarray(c["psi"]), dtype=torch.complex128, requires_grad=True)
    L = AD.overlap_loss(n, V, psi0, c["target"], nsteps, K)
    (3.0 * L + (V * V).sum()).backward()
    assert abs(L.item() - L_ref) < 1e-14
    assert np.allclose(V.grad.numpy(), 3.0 * dV_ref + 2.0 * c["V"], rtol=0, atol=1e-13 * np.abs(dV_ref).max())
    assert np.allclose(psi0.grad.numpy(), 3.0 * g_ref, rtol=0, atol=1e-13 * np.abs(g_ref).max())
    # central difference through the function along one smooth direction of V
    dv = torch.tensor(np.ascontiguousarray(_directions(c["shape"], 1, seed=17)[0]))
    eps = 1e-4
    with torch.no_grad():
        lp = AD.overlap_loss(n, V + eps * dv, psi0, c["target"], nsteps, K).item()
        lm = AD.overlap_loss(n, V - eps * dv, psi0, c["target"], nsteps, K).item()
    adj = float((torch.from_numpy(np.ascontiguousarray(dV_ref)) * dv).sum())
    assert abs((lp - lm) / (2 * eps) - adj) <= 1e-6 * abs(adj)
    n.close()


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_adjoint_cfg4_full_size_compensated(sfd, O, W):
    """cfg4 at full size (256^2, 2000 steps, K = 50) in FP32 storage with the
    compensated passes (forward, recompute and backward): the gradient against
    the FP64 gradient (itself checked against central differences above).
    The FP32 field of this trap (g = 500) drifts from FP64 by round-off that
    the dynamics amplify; the compensated passes leave only the storage
    rounding, so their gradient is far closer to FP64 than the plain FP32
    passes' one."""
    c = W.cfg4(256)
    nsteps, K = c["nsteps"], c["K"]
    res = {}
    for tag, prec, comp in (("fp64", "fp64", False), ("fp32", "fp32", False), ("fp32c", "fp32", True)):
        f, n = _model(sfd, c, c["V"], precision=prec, compensated=comp)
        res[tag] = n.adjoint(c["target"], nsteps, K)
        n.close()
    L64, dV64, g64 = res["fp64"]
    Lc, dVc, gc = res["fp32c"]
    e_plain = _rel(res["fp32"][1], dV64)
    e_comp = _rel(dVc, dV64)
    print(f"dL/dV rel-L2 vs FP64: plain FP32 {e_plain:.2e}, compensated {e_comp:.2e}; "
          f"dL/dpsi0 {_rel(gc, g64):.2e}; loss {abs(Lc - L64):.1e}")
    assert abs(Lc - L64) < 1e-8
    assert e_comp < BAR_CFG4_COMP
    assert _rel(gc, g64) < BAR_CFG4_COMP
    assert e_comp < 0.2 * e_plain


@pytest.mark.parametrize("omega", [0.0, 0.4])
def test_adjoint_compensated_small(sfd, O, W, omega):
    """64^2 copy of the gradient workload, 300 steps, checkpoints every 20:
    the compensated FP32 adjoint (merged sequence with Omega = 0, the unmerged
    one with rotation) against the FP64 adjoint."""
    c = W.cfg4(64)
    nsteps, K = 300, 20
    res = {}
    for tag, prec, comp in (("fp64", "fp64", False), ("fp32c", "fp32", True)):
        f, n = _model(sfd, c, c["V"], precision=prec, compensated=comp, Omega=omega)
        res[tag] = n.adjoint(c["target"], nsteps, K)
        n.close()
    (L64, dV64, g64), (Lc, dVc, gc) = res["fp64"], res["fp32c"]
    print(f"omega {omega}: dL/dV {_rel(dVc, dV64):.2e}, dL/dpsi0 {_rel(gc, g64):.2e}, loss {abs(Lc - L64):.1e}")
    assert abs(Lc - L64) < 1e-7
    assert _rel(dVc, dV64) < BAR_SMALL_COMP
    assert _rel(gc, g64) < BAR_SMALL_COMP

