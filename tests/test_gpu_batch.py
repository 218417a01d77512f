"""Batched runs (gpss_batch_*): one persistent launch over runs of mixed
sizes; every run against the single-field FP32 path and the FP64 oracle."""
import numpy as np
import pytest

from helpers import run_model

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


@pytest.mark.parametrize("tuning", [None, (0, 0, 0), (1, 1, 0), (0, 0, 1), (1, 0, 1), (0, 0, 2), (1, 1, 2),
                                    (0, 0, 3)],
                         ids=["autotuned", "p0", "p1", "p0-stacked", "p1-stacked", "p0-stacked128",
                              "p1-stacked128", "all-stacked"])
def test_batch_matches_single_runs_and_oracle(sfd, O, W, tuning):
    """Every launch choice: the persistent kernel's policies, and the 256^2
    runs as a stack of planes through the directional pass kernels."""
    runs = [W.cfg3_run(n, 77 + i) for i, n in enumerate((64, 128, 256, 64, 128, 256, 64, 256))]
    nsteps, dt = 40, 1e-3
    b = sfd.BatchSplit2([r["n"] for r in runs], [r["bounds"] for r in runs])
    for i, r in enumerate(runs):
        b.set_run(i, r["beta"], r["V"], r["psi"])
    if tuning is not None:
        b.set_tuning(*tuning)
    masses = b.step(nsteps, dt)
    tune = b.tuning()
    assert tune["policy"] in (0, 1) and tune["order"] in (0, 1) and tune["stack"] in (0, 1, 2, 3)
    if tuning is not None:
        assert (tune["policy"], tune["order"], tune["stack"]) == tuning
    for i, r in enumerate(runs):
        got = b.download(i)
        single = run_model(sfd, (r["n"], r["n"]), r["bounds"], r["psi"], coeffD=-0.5, beta=r["beta"], V=r["V"],
                           dt=dt, nsteps=nsteps, precision="fp32")
        ref = O.c_step(r["psi"], r["bounds"], coeffD=-0.5, beta=r["beta"], V=r["V"], nsteps=nsteps, dt=dt)
        assert O.rel_l2(got, single) < 5e-6  # two FP32 paths, mass sums ordered differently
        assert O.rel_l2(got, ref) < 1e-5
        m0 = np.sum(np.abs(r["psi"].astype(np.complex64)) ** 2)
        assert abs(masses[i] - m0) / m0 < 1e-6
    b.close()


def test_batch_repeated_calls_are_consistent(sfd, O, W):
    """Two calls of k steps equal one call of 2k steps up to FP32 round-off
    (the graph is re-captured for a new step count)."""
    runs = [W.cfg3_run(n, 300 + i) for i, n in enumerate((64, 128, 256))]
    a = sfd.BatchSplit2([r["n"] for r in runs], [r["bounds"] for r in runs])
    c = sfd.BatchSplit2([r["n"] for r in runs], [r["bounds"] for r in runs])
    for i, r in enumerate(runs):
        a.set_run(i, r["beta"], r["V"], r["psi"])
        c.set_run(i, r["beta"], r["V"], r["psi"])
    a.step(15, 1e-3)
    a.step(15, 1e-3)
    c.step(30, 1e-3)
    for i, r in enumerate(runs):
        ref = O.c_step(r["psi"], r["bounds"], coeffD=-0.5, beta=r["beta"], V=r["V"], nsteps=30, dt=1e-3)
        assert O.rel_l2(a.download(i), ref) < 1e-5
        assert O.rel_l2(c.download(i), ref) < 1e-5
    a.close()
    c.close()


def test_batch_golden_cfg3_runs(sfd, O):
    """The committed cfg3 fixtures (two 64^2 runs, 500 steps) through one
    batch, against the FP64 oracle's golden output and mass trace."""
    import os
    here = os.path.join(os.path.dirname(__file__), "golden")
    zs = [np.load(os.path.join(here, nm)) for nm in ("cfg3_run_64_s0.npz", "cfg3_run_64_s2.npz")]
    b = sfd.BatchSplit2([z["psi0"].shape[0] for z in zs], [tuple(tuple(r) for r in z["bounds"]) for z in zs])
    for i, z in enumerate(zs):
        b.set_run(i, float(z["beta"]), z["V"], z["psi0"])
    masses = b.step(int(zs[0]["nsteps"]), float(zs[0]["dt"]))
    for i, z in enumerate(zs):
        err = O.rel_l2(b.download(i), z["psi"])
        print(f"cfg3 golden run {i}: rel L2 {err:.2e}")
        assert err < 2e-5
        cell = np.prod([(r[1] - r[0]) / m for r, m in zip(z["bounds"], z["psi0"].shape)])
        assert abs(masses[i] * cell - z["trace_mass"][-1]) <= 1e-6 * z["trace_mass"][-1]
    b.close()


def test_batch_full_cfg3_vs_oracle(sfd, O, W):
    """The full cfg3 batch the bench times: 512 runs (256 x 64^2, 192 x 128^2,
    64 x 256^2), 500 steps in one call, autotuned launch.  Every 256^2 run and
    16 runs of each smaller size against the FP64 oracle within 1e-5; every
    run's FP64 mass sum within 1e-6 of its initial mass."""
    c = W.cfg3()
    runs = c["runs"]
    b = sfd.BatchSplit2([r["n"] for r in runs], [r["bounds"] for r in runs], coeffD=c["coeffD"])
    for i, r in enumerate(runs):
        b.set_run(i, r["beta"], r["V"], r["psi"])
    masses = b.step(c["nsteps"], c["dt"])
    picked = [i for i, r in enumerate(runs) if r["n"] == 256]
    for n in (64, 128):
        idx = [i for i, r in enumerate(runs) if r["n"] == n]
        picked += idx[:: len(idx) // 16][:16]
    worst = 0.0
    for i in picked:
        r = runs[i]
        ref = O.c_step(r["psi"], r["bounds"], coeffD=c["coeffD"], beta=r["beta"], V=r["V"], nsteps=c["nsteps"],
                       dt=c["dt"])
        err = O.rel_l2(b.download(i), ref)
        worst = max(worst, err)
        assert err < 1e-5, (i, r["n"], r["beta"], err)
    for i, r in enumerate(runs):
        m0 = np.sum(np.abs(r["psi"].astype(np.complex64)) ** 2)
        assert abs(masses[i] - m0) / m0 < 1e-6
    print(f"cfg3 full batch: {len(picked)} runs vs the oracle, worst rel-L2 {worst:.2e}")
    b.close()
