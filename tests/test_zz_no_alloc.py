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


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-6)])
def test_energy_noalloc_matches_context_path(sfd, O, built_lib, precision, tol):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sfd_gb300 import _lib
    L = _lib.lib()
    shape, bounds = (64, 32, 16), ((-5.0, 6.0),) * 3
    psi0 = random_field(shape, seed=21)
    V = O.quadratic_potential(shape, bounds)
    cD, beta, om = -0.4, 7.0, 0.6
    # the existing entry point (context path) on the same field
    g = sfd.Grid(shape, bounds)
    f = sfd.Field(g)
    f.phi = psi0
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, V), coeffD=cD, beta=beta, Omega=om)
    n = sfd.NumModelSplit2(f, p, 1e-3, 1, 1, precision=precision)
    ref = n.energies()
    n.close(download=False)
    # device copies owned by the caller (torch's allocator), x fastest in memory
    cdt, rdt = (torch.complex128, torch.float64) if precision == "fp64" else (torch.complex64, torch.float32)
    psi_dev = torch.from_numpy(np.ascontiguousarray(psi0.ravel(order="F"))).to("cuda").to(cdt)
    V_dev = torch.from_numpy(np.ascontiguousarray(V.ravel(order="F"))).to("cuda").to(rdt)
    torch.cuda.synchronize()
    nn = (ctypes.c_int64 * 3)(*shape)
    lo = (ctypes.c_double * 3)(*[b[0] for b in bounds])
    hi = (ctypes.c_double * 3)(*[b[1] for b in bounds])
    prec = 64 if precision == "fp64" else 32
    scale = max(abs(v) for v in ref)
    free_before = None
    for call in range(2):  # two calls in a row share the library's scratch
        out = (ctypes.c_double * 5)()
        rc = L.gpss_energy_noalloc(3, nn, lo, hi, prec, cD, beta, om, ctypes.c_void_p(psi_dev.data_ptr()),
                                   ctypes.c_void_p(V_dev.data_ptr()), None, out)
        assert rc == 0
        for a, b in zip(out, ref):
            assert abs(a - b) <= tol * scale
        if call == 0:
            free_before = torch.cuda.mem_get_info()[0]
    assert torch.cuda.mem_get_info()[0] == free_before  # the second call allocated nothing
