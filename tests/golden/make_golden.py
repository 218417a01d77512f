"""Generates the golden vectors of tests/golden/*.npz with the CPU oracle
(oracle/gp_oracle.c), cross-checked against the independent numpy restatement
before writing.  Each file holds the input, the FP64 oracle's output `psi`
and the long-double oracle's output `psi_ext` (a near-exact reference: FP64
implementations differ from it only by their own round-off).

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
                                   dt=c0["dt"])
    yield "split2_3d_periodic_box", dict(psi0=np.asfortranarray(np.exp(1j * field((16, 16, 16), 4).real)),
                                         bounds=b, V=None, coeffD=-0.05 / math.sqrt(2),
                                         beta=1 / (math.sqrt(2) * 0.05), omega=0.0, nsteps=20, scheme=2,
                                         imag=False, dt=2.5e-3)


def main():
    for name, c in cases():
        kw = dict(coeffD=c["coeffD"], beta=c["beta"], omega=c["omega"], V=c["V"], nsteps=c["nsteps"],
                  scheme=c["scheme"], imag=c["imag"], dt=c["dt"])
        out = O.c_step(c["psi0"], c["bounds"], **kw)
        ext = O.c_step(c["psi0"], c["bounds"], extended=True, **kw)
        chk = O.np_step(c["psi0"], c["bounds"], **kw)
        assert O.rel_l2(out, chk) < 4e-12, name
        e = O.c_energy(out, c["bounds"], coeffD=c["coeffD"], beta=c["beta"], omega=c["omega"], V=c["V"])
        V = c["V"] if c["V"] is not None else np.zeros(c["psi0"].shape)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), psi0=c["psi0"], psi=out, V=V,
                            has_V=c["V"] is not None, bounds=np.array(c["bounds"]), coeffD=c["coeffD"],
                            beta=c["beta"], omega=c["omega"], nsteps=c["nsteps"], scheme=c["scheme"],
                            imag=c["imag"], dt=c["dt"], energy=np.array(e), psi_ext=ext)
        print(name, out.shape, "numpy vs FP64 oracle", O.rel_l2(out, chk), "FP64 oracle vs extended",
              O.rel_l2(out, ext))


if __name__ == "__main__":
    main()
