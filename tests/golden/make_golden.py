"""Generates the golden vectors of tests/golden/*.npz with the CPU oracle
(oracle/gp_oracle.c), cross-checked against the independent numpy restatement
before writing.  Each file holds the input, the FP64 oracle's output `psi`
and the long-double oracle's output `psi_ext` (a near-exact reference: FP64
implementations differ from it only by their own round-off), plus traces of
the mass and of energy(n)'s five values (E_Omega, E_Delta, E_beta, E, mu;
GrossPitaevskii.jl:61-136) every `trace_every` steps.

The cfg1..cfg4 fixtures are the seeded workloads of sfd_gb300.workloads at
reduced sizes (the full-size fields are hundreds of MB): cfg1 at 32^3 (200
steps), cfg2 at 32^3 (200 imaginary-time steps), two cfg3 runs at 64^2 (seeds 0 and 2, 500
steps) and the cfg4 gradient workload at 32^2 (`cfg4_grad_32.grad.npz`: the
loss and its directional derivatives along seeded (dV, dpsi0) directions from
the oracle's dual-number restatement, checked here against central
differences of the FP64 oracle).  The `*.solver.npz` fixtures hold explicit
RK and implicit (Backward-Euler, Crank-Nicolson) runs of the oracle, each
cross-checked against the numpy restatement (and its Krylov count).

Run from the repository root on an x86 host (80-bit long double):
    python tests/golden/make_golden.py
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)
import gp_oracle as O  # noqa: E402


def field(shape, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    F = np.fft.fftn(a)
    for ax, n in enumerate(shape):
        k = np.fft.fftfreq(n) * n
        s = [1] * len(shape)
        s[ax] = n
        F *= np.exp(-(k.reshape(s) / max(2.0, n / 8)) ** 2)
    a = np.fft.ifftn(F)
    return np.asfortranarray(a / np.sqrt(np.mean(np.abs(a) ** 2)))


def cases():
    # the reference's GPU-vs-CPU Split2 case, test/runtests.jl:1438-1454
    b = ((-6.0, 6.0), (-6.0, 6.0))
    x = O.grid_coords(32, -6, 6)
    X, Y = x[:, None], x[None, :]
    p = np.asfortranarray(np.exp(-0.5 * (X ** 2 + Y ** 2)) * (1 + 0.1 * X))
    p = p / O.c_norm(p, b)
    yield "ref_split2_gpu_case", dict(psi0=p, bounds=b, V=O.quadratic_potential((32, 32), b), coeffD=-0.5,
                                      beta=10.0, omega=0.0, nsteps=20, scheme=2, imag=False, dt=0.01)
    b = ((-5.0, 5.0), (-4.0, 4.0))
    yield "split1_rotation_2d", dict(psi0=field((32, 16), 1), bounds=b, V=O.quadratic_potential((32, 16), b),
                                     coeffD=-0.5, beta=20.0, omega=0.7, nsteps=10, scheme=1, imag=False, dt=5e-3)
    b = ((-3.0, 3.0), (-2.0, 2.0), (-4.0, 4.0))
    yield "split2_3d_trap", dict(psi0=field((16, 8, 32), 2), bounds=b,
                                 V=O.quadratic_potential((16, 8, 32), b, gammas=[1.0, 2.0, 0.5]),
                                 coeffD=-0.5, beta=5.0, omega=0.0, nsteps=10, scheme=2, imag=False, dt=4e-3)
    b = ((-6.0, 6.0),) * 3
    yield "split2_3d_imag_rot", dict(psi0=field((16, 16, 8), 3), bounds=b, V=O.quadratic_potential((16, 16, 8), b),
                                     coeffD=-0.5, beta=50.0, omega=0.3, nsteps=20, scheme=2, imag=True, dt=1e-2)
    b = ((0.0, 2 * math.pi),) * 3
    # cfg0 at full size: 2D 128^2 trap, g = 500, 1000 steps (the FP64 parity run)
    sys.path.insert(0, ROOT)
    import __graft_entry__ as g
    g.load_package()
    import importlib
    c0 = importlib.import_module("sfd_gb300.workloads").cfg0()
    yield "cfg0_2d_128_1000", dict(psi0=c0["psi"], bounds=c0["bounds"], V=c0["V"], coeffD=c0["coeffD"],
                                   beta=c0["beta"], omega=0.0, nsteps=c0["nsteps"], scheme=2, imag=False,
                                   dt=c0["dt"], trace_every=100)
    W = importlib.import_module("sfd_gb300.workloads")
    c1 = W.cfg1(32)
    yield "cfg1_3d_32_200", dict(psi0=c1["psi"], bounds=c1["bounds"], V=None, coeffD=c1["coeffD"],
                                 beta=c1["beta"], omega=0.0, nsteps=c1["nsteps"], scheme=2, imag=False,
                                 dt=c1["dt"], trace_every=20)
    c2 = W.cfg2(32)
    yield "cfg2_3d_32_200", dict(psi0=c2["psi"], bounds=c2["bounds"], V=c2["V"], coeffD=c2["coeffD"],
                                 beta=c2["beta"], omega=0.0, nsteps=c2["nsteps"], scheme=2, imag=True,
                                 dt=c2["dt"], trace_every=20)
    # seed 1 (g = 913) is left out: at 64^2 its 500 steps amplify round-off to
    # ~1e-9 (two FP64 restatements differ by that much), no 1e-12 parity case
    for seed in (0, 2):
        r = W.cfg3_run(64, seed)
        yield f"cfg3_run_64_s{seed}", dict(psi0=r["psi"], bounds=r["bounds"], V=r["V"], coeffD=-0.5,
                                           beta=r["beta"], omega=0.0, nsteps=500, scheme=2, imag=False,
                                           dt=1e-3, trace_every=100, cfg3_seed=seed)
    yield "split2_3d_periodic_box", dict(psi0=np.asfortranarray(np.exp(1j * field((16, 16, 16), 4).real)),
                                         bounds=b, V=None, coeffD=-0.05 / math.sqrt(2),
                                         beta=1 / (math.sqrt(2) * 0.05), omega=0.0, nsteps=20, scheme=2,
                                         imag=False, dt=2.5e-3)


def trace(c):
    """(steps, mass, energies) every trace_every steps, by chunked oracle runs."""
    every = c.get("trace_every", c["nsteps"])
    kw = dict(coeffD=c["coeffD"], beta=c["beta"], omega=c["omega"], V=c["V"])
    p = c["psi0"].copy(order="F")
    steps, mass, en = [0], [O.c_norm(p, c["bounds"]) ** 2], [O.c_energy(p, c["bounds"], **kw)]
    done = 0
    while done < c["nsteps"]:
        k = min(every, c["nsteps"] - done)
        p = O.c_step(p, c["bounds"], nsteps=k, scheme=c["scheme"], imag=c["imag"], dt=c["dt"], **kw)
        done += k
        steps.append(done)
        mass.append(O.c_norm(p, c["bounds"]) ** 2)
        en.append(O.c_energy(p, c["bounds"], **kw))
    return np.array(steps), np.array(mass), np.array(en), p


def grad_case():
    """cfg4 at 32^2, 50 steps: L and dL along 4 seeded (dV, dpsi0) directions."""
    import importlib
    import __graft_entry__ as g
    g.load_package()
    W = importlib.import_module("sfd_gb300.workloads")
    c = W.cfg4(32)
    nsteps = 50
    rng = np.random.default_rng(4242)
    dVs, dpsis, dLs = [], [], []
    kx = np.fft.fftfreq(32)[:, None] * 32
    ky = np.fft.fftfreq(32)[None, :] * 32
    L = None
    for _ in range(4):
        a = np.fft.ifft2(np.fft.fft2(rng.standard_normal(c["shape"])) * np.exp(-(kx ** 2 + ky ** 2) / 16.0)).real
        dv = np.asfortranarray(a / np.max(np.abs(a)))
        dpsi = np.asfortranarray(0.1 * (rng.standard_normal(c["shape"]) + 1j * rng.standard_normal(c["shape"])))
        L, dL = O.np_tangent_loss(c["psi"], dpsi, c["V"], dv, c["target"], c["bounds"], coeffD=c["coeffD"],
                                  beta=c["beta"], nsteps=nsteps, dt=c["dt"])
        dVs.append(dv)
        dpsis.append(dpsi)
        dLs.append(dL)

    def loss(V, psi0):
        p = O.c_step(psi0, c["bounds"], coeffD=c["coeffD"], beta=c["beta"], V=V, nsteps=nsteps, dt=c["dt"])
        z = np.sum(np.conj(c["target"]) * p) * np.prod(O.spacing(c["shape"], c["bounds"]))
        return 1.0 - abs(z) ** 2

    assert abs(loss(c["V"], c["psi"]) - L) < 1e-13
    eps = 1e-5
    for dv, dpsi, dL in zip(dVs, dpsis, dLs):
        fd = (loss(c["V"] + eps * dv, c["psi"] + eps * dpsi) - loss(c["V"] - eps * dv, c["psi"] - eps * dpsi)) / (2 * eps)
        assert abs(fd - dL) <= 1e-6 * abs(dL), (fd, dL)
    np.savez_compressed(os.path.join(HERE, "cfg4_grad_32.grad.npz"), psi0=c["psi"], V=c["V"], target=c["target"],
                        bounds=np.array(c["bounds"]), coeffD=c["coeffD"], beta=c["beta"], dt=c["dt"],
                        nsteps=nsteps, L=L, dV=np.array(dVs), dpsi0=np.array(dpsis), dL=np.array(dLs))
    print("cfg4_grad_32", "L", L, "dL", dLs)


def solver_cases():
    """Fixtures of the integrators beside the split step: NumModelGPRK
    (explicit-rk.jl:96-166) and the implicit Krylov schemes
    (backward-euler.jl, crank-nicolson.jl, krylov.jl)."""
    b2 = ((-6.0, 6.0), (-4.0, 5.0))
    V2 = O.quadratic_potential((64, 32), b2)
    yield "rk4_product_2d_rot", dict(kind="rk", psi0=0.5 * field((64, 32), 11), bounds=b2, V=V2, coeffD=-0.5,
                                     beta=2.0, omega=0.6, nsteps=20, dt=1e-3, stepper="RK4", filter="product")
    b3 = ((-4.0, 4.0), (-3.0, 3.0), (-2.0, 2.0))
    yield "rk2_solution_3d", dict(kind="rk", psi0=0.5 * field((32, 16, 16), 12), bounds=b3,
                                  V=O.quadratic_potential((32, 16, 16), b3), coeffD=-0.5, beta=2.0, omega=0.3,
                                  nsteps=12, dt=1e-3, stepper="RK2", filter="solution")
    b = ((-6.0, 6.0), (-6.0, 6.0))
    p0 = field((32, 32), 13)
    p0 = np.asfortranarray(p0 / O.c_norm(p0, b))
    for scheme in ("BackwardEuler", "CrankNicolson"):
        yield f"{scheme.lower()}_2d", dict(kind="implicit", psi0=p0, bounds=b, V=O.quadratic_potential((32, 32), b),
                                          coeffD=-0.5, beta=5.0, omega=0.0, nsteps=3, dt=1e-2, scheme=scheme)


def solver_main():
    for name, c in solver_cases():
        kw = dict(coeffD=c["coeffD"], beta=c["beta"], omega=c["omega"], V=c["V"], nsteps=c["nsteps"], dt=c["dt"])
        extra = {}
        if c["kind"] == "rk":
            kw.update(stepper=c["stepper"], filter=c["filter"])
            out = O.c_rk_step(c["psi0"], c["bounds"], **kw)
            chk = O.np_rk_step(c["psi0"], c["bounds"], **kw)
            extra = dict(stepper=c["stepper"], filter=c["filter"])
        else:
            kw.update(scheme=c["scheme"])
            out, iters = O.c_implicit_step(c["psi0"], c["bounds"], **kw)
            chk, iters_np = O.np_implicit_step(c["psi0"], c["bounds"], **kw)
            assert iters == iters_np, name
            extra = dict(scheme=c["scheme"], krylov=iters)
        assert O.rel_l2(out, chk) < 1e-11, (name, O.rel_l2(out, chk))
        np.savez_compressed(os.path.join(HERE, name + ".solver.npz"), kind=c["kind"], psi0=c["psi0"], psi=out,
                            V=c["V"], bounds=np.array(c["bounds"]), coeffD=c["coeffD"], beta=c["beta"],
                            omega=c["omega"], nsteps=c["nsteps"], dt=c["dt"], **extra)
        print(name, out.shape, "numpy vs C oracle", O.rel_l2(out, chk), extra.get("krylov", ""))


def main():
    solver_main()
    grad_case()
    for name, c in cases():
        kw = dict(coeffD=c["coeffD"], beta=c["beta"], omega=c["omega"], V=c["V"], nsteps=c["nsteps"],
                  scheme=c["scheme"], imag=c["imag"], dt=c["dt"])
        out = O.c_step(c["psi0"], c["bounds"], **kw)
        ext = O.c_step(c["psi0"], c["bounds"], extended=True, **kw)
        chk = O.np_step(c["psi0"], c["bounds"], **kw)
        assert O.rel_l2(out, chk) < 4e-12, name
        e = O.c_energy(out, c["bounds"], coeffD=c["coeffD"], beta=c["beta"], omega=c["omega"], V=c["V"])
        V = c["V"] if c["V"] is not None else np.zeros(c["psi0"].shape)
        steps, mass, en, tp = trace(c)
        assert O.rel_l2(tp, out) < 1e-13, name
        extra = {"cfg3_seed": c["cfg3_seed"]} if "cfg3_seed" in c else {}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), psi0=c["psi0"], psi=out, V=V,
                            trace_steps=steps, trace_mass=mass, trace_energy=en, **extra,
                            has_V=c["V"] is not None, bounds=np.array(c["bounds"]), coeffD=c["coeffD"],
                            beta=c["beta"], omega=c["omega"], nsteps=c["nsteps"], scheme=c["scheme"],
                            imag=c["imag"], dt=c["dt"], energy=np.array(e), psi_ext=ext)
        print(name, out.shape, "numpy vs FP64 oracle", O.rel_l2(out, chk), "FP64 oracle vs extended",
              O.rel_l2(out, ext))


if __name__ == "__main__":
    main()
