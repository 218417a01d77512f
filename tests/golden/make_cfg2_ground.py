"""Generates tests/golden/cfg2_3d_128.ground.npz: the cfg2 imaginary-time
ground state at its full size (128^3 on [-10, 10]^3, V = (x^2 + y^2 + 4 z^2)/2,
g = 2000, dt = 1e-3) run by the FP64 oracle (oracle/gp_oracle.c) until
|mu_n - mu_{n-10}| < 1e-10 with mu evaluated every 10 steps -- the stopping
rule of the library's gpss_ground_state, so the GPU run stops at the same
step.  The 128^3 field (33 MB) is not stored: the fixture keeps the step
count, the five energies and the mass of the final field, its values on
every 8th node of each axis (16^3), and the full lines through the trap
centre along each axis.

16410 steps; about 6.5 minutes on 16 host cores (the oracle is OpenMP-parallel).  Run
from the repository root (an optional argument names another output file):
    python tests/golden/make_cfg2_ground.py [out.npz]
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)
import gp_oracle as O  # noqa: E402


def main():
    import __graft_entry__ as g
    g.load_package()
    import importlib
    W = importlib.import_module("sfd_gb300.workloads")
    O.build()
    c = W.cfg2(128)
    kw = dict(coeffD=c["coeffD"], beta=c["beta"], V=c["V"], dt=c["dt"], imag=True)
    psi = c["psi"] / O.c_norm(c["psi"], c["bounds"])
    mu_prev, done, t0 = None, 0, time.time()
    while True:
        psi = O.c_step(psi, c["bounds"], nsteps=10, **kw)
        done += 10
        e = O.c_energy(psi, c["bounds"], coeffD=c["coeffD"], beta=c["beta"], V=c["V"])
        if mu_prev is not None and abs(e[4] - mu_prev) < 1e-10:
            break
        mu_prev = e[4]
        if done % 1000 == 0:
            print(done, e[4], time.time() - t0, flush=True)
    mid = [n // 2 for n in c["shape"]]
    out = dict(nsteps=done, energies=np.array(e), mu_prev=mu_prev,
               mass=O.c_norm(psi, c["bounds"]) ** 2,
               sample=np.ascontiguousarray(psi[::8, ::8, ::8]),
               line_x=psi[:, mid[1], mid[2]].copy(), line_y=psi[mid[0], :, mid[2]].copy(),
               line_z=psi[mid[0], mid[1], :].copy(), max_abs=np.max(np.abs(psi)))
    path = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "cfg2_3d_128.ground.npz")
    np.savez_compressed(path, **out)
    print("steps", done, "mu", e[4], "seconds", time.time() - t0)


if __name__ == "__main__":
    main()
