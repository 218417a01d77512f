"""Race check without a sanitizer: every GPU path is deterministic (fixed
reduction orders, no atomics in sums), so running the same case twice must
give bitwise-identical results.  A missing barrier or an out-of-order
shared-memory access would show up here as run-to-run differences."""
import numpy as np
import pytest

from helpers import random_field, run_model

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_split_step_is_bitwise_reproducible(sfd, O, precision):
    shape, b = (128, 64, 32), ((-5.0, 5.0), (-4.0, 4.0), (-3.0, 3.0))
    psi0 = random_field(shape, seed=3)
    V = O.quadratic_potential(shape, b)
    kw = dict(coeffD=-0.5, beta=4.0, omega=0.2, V=V, dt=2e-3, nsteps=20, precision=precision)
    a = run_model(sfd, shape, b, psi0, **kw)
    c = run_model(sfd, shape, b, psi0, **kw)
    assert np.array_equal(a, c)


def test_rk_and_adjoint_are_bitwise_reproducible(sfd, W):
    c = W.cfg4(64)
    outs = []
    for _ in range(2):
        g = sfd.Grid(c["shape"], c["bounds"])
        f = sfd.Field(g)
        f.phi = c["psi"]
        p = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, c["V"]), coeffD=c["coeffD"], beta=c["beta"])
        n = sfd.NumModelSplit2(f, p, c["dt"], 1, 1, precision="fp32")
        L, dv, g0 = n.adjoint(c["target"], 60, 8)
        n.close()
        f2 = sfd.Field(g)
        f2.phi = c["psi"]
        p2 = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f2, c["V"]), coeffD=c["coeffD"], beta=c["beta"])
        m = sfd.NumModelGPRK(f2, p2, c["dt"], 1, 1, precision="fp32")
        m.step(20)
        outs.append((L, dv, g0, f2.phi.copy()))
        m.close()
    assert outs[0][0] == outs[1][0]
    for i in (1, 2, 3):
        assert np.array_equal(outs[0][i], outs[1][i])


def test_batch_is_bitwise_reproducible(sfd, W):
    runs = [W.cfg3_run(n, 500 + i) for i, n in enumerate((64, 128, 256, 256))]
    res = []
    for stack in (0, 1):
        for _ in range(2):
            b = sfd.BatchSplit2([r["n"] for r in runs], [r["bounds"] for r in runs])
            for i, r in enumerate(runs):
                b.set_run(i, r["beta"], r["V"], r["psi"])
            b.set_tuning(0, 0, stack)
            m = b.step(30, 1e-3)
            res.append((stack, m, [b.download(i) for i in range(len(runs))]))
            b.close()
    for k in (0, 2):
        assert np.array_equal(res[k][1], res[k + 1][1])
        for x, y in zip(res[k][2], res[k + 1][2]):
            assert np.array_equal(x, y)
