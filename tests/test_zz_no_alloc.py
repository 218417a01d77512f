"""gpss_energy_noalloc: energies of a field held in the caller's device memory,
computed by the library without allocating.

Callers that cannot let a library cudaMalloc (device memory owned by another
allocator, such as CUDA.jl's pool in a Julia session, or a fixed device-memory
budget) pass device pointers and get the energies back; the library's scratch
is a fixed array inside it.  This file is collected last so that a run that
stops at its first failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

from helpers import random_field

pytestmark = pytest.mark.gpu

# (shape, bounds, with a potential, Omega): a 3D trap with rotation, a 2D trap
# with rotation (x coordinates for the y pass), a 3D field with V = NULL
CASES = {
    "3d_trap_rot": ((64, 32, 16), ((-5.0, 6.0),) * 3, True, 0.6),
    "2d_trap_rot": ((128, 64), ((-6.0, 6.0), (-4.0, 5.0)), True, 0.6),
    "3d_free": ((32, 16, 64), ((0.0, 6.0), (0.0, 5.0), (0.0, 7.0)), False, 0.0),
}


def _c_args(shape, bounds):
    nd = len(shape)
    nn = (ctypes.c_int64 * 3)(*(list(shape) + [1] * (3 - nd)))
    lo = (ctypes.c_double * 3)(*([b[0] for b in bounds] + [0.0] * (3 - nd)))
    hi = (ctypes.c_double * 3)(*([b[1] for b in bounds] + [1.0] * (3 - nd)))
    return nd, nn, lo, hi


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-6)])
def test_energy_noalloc_matches_context_path(sfd, O, built_lib, case, precision, tol):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sfd_gb300 import _lib
    L = _lib.lib()
    shape, bounds, with_v, om = CASES[case]
    psi0 = random_field(shape, seed=21)
    V = O.quadratic_potential(shape, bounds) if with_v else None
    cD, beta = -0.4, 7.0
    # the existing entry point (context path) on the same field
    g = sfd.Grid(shape, bounds)
    f = sfd.Field(g)
    f.phi = psi0
    pot = sfd.PotentialArray(f, V) if with_v else sfd.PotentialZero(f)
    p = sfd.GrossPitaevskiiParameters(pot, coeffD=cD, beta=beta, Omega=om)
    n = sfd.NumModelSplit2(f, p, 1e-3, 1, 1, precision=precision)
    ref = n.energies()
    n.close(download=False)
    # device copies owned by the caller (torch's allocator), x fastest in memory
    cdt, rdt = (torch.complex128, torch.float64) if precision == "fp64" else (torch.complex64, torch.float32)
    psi_dev = torch.from_numpy(np.ascontiguousarray(psi0.ravel(order="F"))).to("cuda").to(cdt)
    V_dev = torch.from_numpy(np.ascontiguousarray(V.ravel(order="F"))).to("cuda").to(rdt) if with_v else None
    torch.cuda.synchronize()
    nd, nn, lo, hi = _c_args(shape, bounds)
    prec = 64 if precision == "fp64" else 32
    scale = max(abs(v) for v in ref)
    free_before = None
    for call in range(2):  # two calls in a row share the library's scratch
        out = (ctypes.c_double * 5)()
        rc = L.gpss_energy_noalloc(nd, nn, lo, hi, prec, cD, beta, om, ctypes.c_void_p(psi_dev.data_ptr()),
                                   ctypes.c_void_p(V_dev.data_ptr()) if with_v else None, None, out)
        assert rc == 0, L.gpss_last_error(None)
        for a, b in zip(out, ref):
            assert abs(a - b) <= tol * scale
        if call == 0:
            free_before = torch.cuda.mem_get_info()[0]
    assert torch.cuda.mem_get_info()[0] == free_before  # the second call allocated nothing


def test_energy_noalloc_rejects_bad_arguments(sfd, built_lib):
    """Sizes the fixed scratch does not cover, or a bad box, return GPSS_EINVAL
    with a message in gpss_last_error(NULL); nothing runs on the device."""
    from sfd_gb300 import _lib
    L = _lib.lib()
    out = (ctypes.c_double * 5)()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the arguments are refused first
    for shape, bounds in (((48, 32, 16), ((0.0, 1.0),) * 3),       # not a power of two
                          ((512, 32), ((0.0, 1.0),) * 2),          # longer than 256
                          ((32, 32), ((0.0, 1.0), (2.0, 2.0)))):   # lo >= hi
        nd, nn, lo, hi = _c_args(shape, bounds)
        rc = L.gpss_energy_noalloc(nd, nn, lo, hi, 64, -0.5, 1.0, 0.0, dummy, None, None, out)
        assert rc == _lib.GPSS_EINVAL
        assert b"gpss_energy_noalloc" in L.gpss_last_error(None)
