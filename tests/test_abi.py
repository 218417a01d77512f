"""The C ABI library loads, exports every function include/gpss.h declares,
and validates arguments on the host; the host mirror matches the reference's
grid/potential conventions.  No kernel is launched (no GPU needed)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest


@pytest.fixture(scope="module")
def L(sfd, built_lib):
    from sfd_gb300 import _lib
    return _lib.lib()


def test_every_header_function_is_exported(L, sfd):
    from sfd_gb300 import _lib
    names = _lib.header_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    for nm in names:
        assert nm in exported, nm
        assert hasattr(L, nm)
    assert set(names) == set(_lib.SIGNATURES), "ctypes signatures must cover the header exactly"


def test_version(L):
    assert b"sm_103a" in L.gpss_version()


def _create(L, ndim, n, lo, hi, prec=64, flags=0):
    from sfd_gb300 import _lib
    h = ctypes.c_void_p()
    arr = lambda t, v: (t * 3)(*(list(v) + [0] * (3 - len(v))))
    rc = L.gpss_create(ctypes.byref(h), ndim, arr(ctypes.c_int64, n), arr(ctypes.c_double, lo),
                       arr(ctypes.c_double, hi), prec, flags)
    return rc, h


@pytest.mark.parametrize("ndim,n,lo,hi,prec,flags", [
    (1, (32,), (0,), (1,), 64, 0),              # 1D is not a split-step field here
    (2, (37, 32), (0, 0), (1, 1), 64, 0),       # prime factor above 31
    (2, (32, 74), (0, 0), (1, 1), 64, 0),       # 2 x 37
    (2, (2048, 32), (0, 0), (1, 1), 64, 0),     # above 1024 per axis
    (2, (48, 32), (0, 0), (1, 1), 32, 32),      # compensated passes need powers of two up to 256
    (2, (1, 32), (0, 0), (1, 1), 64, 0),        # below 2
    (2, (32, 32), (1, 0), (1, 1), 64, 0),       # lo == hi
    (2, (32, 32), (0, 0), (1, 1), 16, 0),       # unknown precision
    (3, (8, 8, 8), (0, 0, 0), (1, 1, 1), 32, 64),  # unknown flag
])
def test_create_rejects_bad_arguments(L, ndim, n, lo, hi, prec, flags):
    rc, h = _create(L, ndim, n, lo, hi, prec, flags)
    assert rc == -1
    assert not h.value
    assert L.gpss_last_error(None)


def test_null_arguments(L):
    assert L.gpss_create(None, 2, None, None, None, 64, 0) == -1
    assert L.gpss_set_params(None, 0, 0, 0) == -1
    assert L.gpss_step(None, 1, 2, 0, 1e-3, None) == -1
    assert L.gpss_rk_step(None, 1, 4, 1, 1e-3) == -1
    assert L.gpss_implicit_step(None, 1, 0, 1e-3, 70, 1e-8, 15, 1e-6, None) == -1
    L.gpss_destroy(None)


def test_create_without_gpu_fails_cleanly(L):
    if L.gpss_device_count() > 0:
        pytest.skip("a GPU is visible")
    rc, h = _create(L, 2, (32, 32), (0, 0), (1, 1))
    assert rc == -3  # GPSS_ECUDA, no crash
    assert b"cuda" in L.gpss_last_error(None).lower()


def test_host_grid_matches_oracle(sfd, O):
    for n, lo, hi in ((128, -8, 8), (256, 0.0, 2 * np.pi), (48, -12, 12), (5, -1.5, 2.25)):
        assert np.array_equal(sfd.grid_coords(n, lo, hi), O.grid_coords(n, lo, hi))


def test_host_potential_matches_oracle(sfd, O):
    g = sfd.Grid((32, 16, 8), ((-3, 4), (-2, 2), (0, 5)))
    f = sfd.Field(g)
    p = sfd.PotentialQuadratic(f, gx=1.0, gy=0.5, gz=2.0)
    ref = O.quadratic_potential((32, 16, 8), g.bounds, gammas=[1.0, 0.5, 2.0])
    assert np.array_equal(p.V, ref)
    assert p.V.flags.f_contiguous


def test_host_norm_normalize(sfd):
    g = sfd.Grid((64, 64), ((-12, 12), (-12, 12)))
    f = sfd.Field(g)
    f.phi = np.ones((64, 64))
    assert abs(sfd.norm(f) - 24.0) < 1e-12
    sfd.normalize(f)
    assert abs(sfd.norm(f) - 1.0) < 1e-14


def test_field_layout_is_julia_order(sfd):
    g = sfd.Grid((8, 4, 2), ((0, 1), (0, 1), (0, 1)))
    f = sfd.Field(g)
    a = np.arange(64).reshape((8, 4, 2), order="F").astype(complex)
    f.phi = a
    flat = np.frombuffer(f.phi.tobytes(order="A"), dtype=np.complex128)
    assert np.array_equal(flat.real, np.arange(64))  # x fastest


def test_workloads_are_seeded(W):
    a, b = W.cfg0(32), W.cfg0(32)
    assert np.array_equal(a["psi"], b["psi"])
    c = W.cfg1(16)
    assert np.allclose(np.abs(c["psi"]), 1.0)
    assert abs(np.sqrt(2 * abs(c["coeffD"]) * c["beta"]) - 1.0) < 1e-14  # sound speed c = 1
    assert abs(np.sqrt(abs(c["coeffD"]) / c["beta"]) - 0.05) < 1e-14   # healing length xi


def test_build_recipe_targets_sm103a(sfd):
    import importlib.util
    import __graft_entry__ as g
    spec = importlib.util.spec_from_file_location("b", os.path.join(g.PKG_DIR, "build.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    assert "arch=compute_103a,code=sm_103a" in m.ARCH


def test_overlap_loss_checks_arguments_on_the_host(sfd):
    """The autograd wrapper of gpss_adjoint rejects mismatched shapes and
    dtypes before any call into the library."""
    import importlib
    import types
    torch = pytest.importorskip("torch")
    AD = importlib.import_module("sfd_gb300.autodiff")
    model = types.SimpleNamespace(f=types.SimpleNamespace(g=types.SimpleNamespace(n=(8, 8))))
    V = torch.zeros(8, 8, dtype=torch.float64)
    psi = torch.zeros(8, 8, dtype=torch.complex128)
    with pytest.raises(ValueError):
        AD.overlap_loss(model, torch.zeros(8, 4, dtype=torch.float64), psi, None, 1)
    with pytest.raises(TypeError):
        AD.overlap_loss(model, psi, psi, None, 1)
    with pytest.raises(TypeError):
        AD.overlap_loss(model, V, V, None, 1)
