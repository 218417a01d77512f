"""Host-side fault injection (no GPU fault): with GPSS_FAULT_ALLOC=N the
N-th device allocation of a process fails.  Every entry point must then
return GPSS_ENOMEM with a message, leak nothing it can free, and leave the
process usable."""
import json
import os
import subprocess
import sys

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
