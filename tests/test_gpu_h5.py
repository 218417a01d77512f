"""HDF5 checkpoints from device buffers: WriterSave on a field a model owns
writes the device field (gpss_write_h5) and reads a file straight into it
(gpss_read_h5); solve()'s writer hook produces the reference's
res-<istep>.h5 files, and a run restarted from one of them (read! then
solve!(n; istart)) ends bitwise where the uninterrupted run ends."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def _model(sfd, c, precision, niter, freqbckp, writers=()):
    g = sfd.Grid(c["shape"], c["bounds"])
    f = sfd.Field(g)
    f.phi = c["psi"]
    p = sfd.GrossPitaevskiiParameters(sfd.PotentialArray(f, c["V"]) if c.get("V") is not None else None,
                                      coeffD=c["coeffD"], beta=c["beta"])
    n = sfd.NumModelSplit2(f, p, c["dt"], niter, freqbckp, precision=precision)
    n.writers = [w(f) for w in writers]
    return f, n


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_device_field_round_trip(sfd, W, tmp_path, precision):
    c = W.cfg0(64)
    f, n = _model(sfd, c, precision, 10, 10)
    n.step(5)
    w = sfd.WriterSave(f)
    w.write(prefix=str(tmp_path / "res"), istep=5)
    dev = f.phi.copy(order="F")  # downloads the stepped field
    on_file = sfd.read_h5_dataset(str(tmp_path / "res-5.h5"), "re") + 1j * sfd.read_h5_dataset(
        str(tmp_path / "res-5.h5"), "im")
    assert np.array_equal(on_file, dev.T)
    # read! into the model: the device field becomes the file's field
    n.step(3)
    w.read(prefix=str(tmp_path / "res"), istep=5)
    assert np.array_equal(f.phi, dev)
    n.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_solve_restart_from_checkpoint(sfd, W, tmp_path, precision):
    c = W.cfg0(64)
    prefix = tmp_path / "res"

    class Writer(sfd.WriterSave):
        def __call__(self, field, _prefix, istep, dt):
            self.write(prefix=str(prefix), istep=istep, dt=dt)

    f, n = _model(sfd, c, precision, 19, 5, writers=[Writer])
    sfd.solve(n, istart=1)  # iterations 1..20, checkpoints 1 (start), 5, 10, 15, 20
    full = f.phi.copy(order="F")
    n.close()
    for k in (1, 5, 10, 15, 20):
        assert (tmp_path / f"res-{k}.h5").exists()
    f2, n2 = _model(sfd, dict(c, psi=np.zeros(c["shape"], dtype=complex)), precision, 9, 5)
    sfd.WriterSave(f2).read(prefix=str(prefix), istep=10)
    sfd.solve(n2, istart=11)  # iterations 11..20
    assert np.array_equal(f2.phi, full)
    n2.close()
