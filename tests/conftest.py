import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libgpss kernels)")


@pytest.fixture(scope="session")
def sfd():
    import __graft_entry__ as g
    return g.load_package()


@pytest.fixture(scope="session")
def W(sfd):
    import importlib
    return importlib.import_module("sfd_gb300.workloads")


@pytest.fixture(scope="session")
def O():
    import gp_oracle
    gp_oracle.build()
    return gp_oracle


@pytest.fixture(scope="session")
def built_lib():
    """Builds libgpss.so if it is missing (GPU tests call through it)."""
    import __graft_entry__ as g
    from importlib import util
    spec = util.spec_from_file_location("sfd_gb300_build", os.path.join(g.PKG_DIR, "build.py"))
    mod = util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()
