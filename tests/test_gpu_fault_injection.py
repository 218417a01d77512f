"""Host-side fault injection (no GPU fault): with GPSS_FAULT_ALLOC=N the
N-th device allocation of a process fails.  Every entry point must then
return GPSS_ENOMEM with a message, leak nothing it can free, and leave the
process usable."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import ctypes, json, sys
import numpy as np
sys.path.insert(0, {root!r})
import __graft_entry__ as g
sfd = g.load_package()
from sfd_gb300 import _lib
L = _lib.lib()
h = ctypes.c_void_p()
n = (ctypes.c_int64 * 3)(32, 32, 16)
lo = (ctypes.c_double * 3)(0, 0, 0)
hi = (ctypes.c_double * 3)(1, 1, 1)
out = {{"create": L.gpss_create(ctypes.byref(h), 3, n, lo, hi, 32, 0)}}
if out["create"] == 0:
    psi = np.ones((32, 32, 16), dtype=np.complex128, order="F")
    out["upload"] = L.gpss_upload(h, psi.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    out["rk"] = L.gpss_rk_step(h, 1, 4, 1, 1e-3)
    out["msg"] = L.gpss_last_error(h).decode()
    out["step"] = L.gpss_step(h, 2, 2, 0, 1e-3, None)  # the context still works
    L.gpss_destroy(h)
else:
    out["msg"] = L.gpss_last_error(None).decode()
print(json.dumps(out))
"""


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def _child(k):
    env = dict(os.environ, GPSS_FAULT_ALLOC=str(k))
    r = subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT)], env=env, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_allocation_failures_are_reported():
    seen_create_fail = seen_rk_fail = False
    for k in range(1, 25):
        out = _child(k)
        if out["create"] != 0:
            assert out["create"] == -2 and "injected" in out["msg"]
            seen_create_fail = True
            continue
        assert out["upload"] == 0
        if out["rk"] != 0:
            assert out["rk"] == -2 and "injected" in out["msg"]
            assert out["step"] == 0
            seen_rk_fail = True
            break
    assert seen_create_fail and seen_rk_fail


def test_pipelined_wait_timeout_is_reported(sfd, O):
    """The pipelined x pass bounds every wait on a tile's barrier.  With
    GPSS_FAULT_PIPE_POLLS=0 every CTA gives up at once (no GPU fault: each CTA
    still waits, bounded, for the copies it issued before it returns): the step
    returns GPSS_ETIMEOUT, and the same context then steps normally, bitwise
    equal to the direct kernel."""
    from helpers import random_field, run_model
    shape, bounds = (64, 32, 16), ((-4.0, 4.0), (-3.0, 3.0), (-2.0, 2.0))
    psi0 = random_field(shape, seed=17)
    kw = dict(coeffD=-0.5, beta=2.0, dt=1e-3, nsteps=4, precision="fp32", masslock=False)
    g = sfd.Grid(shape, bounds)
    f = sfd.Field(g)
    f.phi = psi0
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialZero(f), coeffD=-0.5, beta=2.0)
    n = sfd.NumModelSplit2(f, p, 1e-3, 4, 4, precision="fp32", pipeline=True, masslock=False)
    os.environ["GPSS_FAULT_PIPE_POLLS"] = "0"
    try:
        with pytest.raises(sfd.GPSSError) as ei:
            n.step(4)
    finally:
        del os.environ["GPSS_FAULT_PIPE_POLLS"]
    assert "ETIMEOUT" in str(ei.value) or "gave up" in str(ei.value)
    f.phi = psi0  # the context is still usable
    n.step(4)
    got = f.phi.copy()
    n.close()
    ref = run_model(sfd, shape, bounds, psi0, pipeline=False, **kw)
    assert np.array_equal(got, ref)
