"""Shared helpers of the GPU tests: run a case through the library's public
API and through the oracle."""
import numpy as np


def run_model(sfd, shape, bounds, psi0, *, coeffD=-0.5, beta=1.0, omega=0.0, V=None, dt=1e-3,
              nsteps=1, scheme=2, imag=False, precision="fp64", form="fused", merge=True,
              per_call=None, masslock=True, pipeline=False, compensated=False):
    g = sfd.Grid(shape, bounds)
    f = sfd.Field(g)
    f.phi = psi0
    pot = sfd.PotentialZero(f) if V is None else sfd.PotentialArray(f, V)
    p = sfd.GrossPitaevskiiParameters(pot, coeffD=coeffD, beta=beta, Omega=omega)
    cls = sfd.NumModelSplit2 if scheme == 2 else sfd.NumModelSplit1
    n = cls(f, p, dt, nsteps, nsteps, precision=precision, form=form, merge=merge, masslock=masslock,
            pipeline=pipeline, compensated=compensated)
    done = 0
    k = per_call or nsteps
    while done < nsteps:
        kk = min(k, nsteps - done)
        n.step(kk, imag=imag)
        done += kk
    out = f.phi.copy(order="F")
    n.close()
    return out


def random_field(shape, seed=0, smooth=True):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    if smooth:  # low-pass so the state is resolved
        F = np.fft.fftn(a)
        for ax, n in enumerate(shape):
            k = np.fft.fftfreq(n) * n
            s = [1] * len(shape)
            s[ax] = n
            F *= np.exp(-(k.reshape(s) / max(2.0, n / 8)) ** 2)
        a = np.fft.ifftn(F)
    a = a / np.sqrt(np.mean(np.abs(a) ** 2))
    return np.asfortranarray(a)
