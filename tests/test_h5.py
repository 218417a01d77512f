"""HDF5 checkpoints (WriterSave's "<prefix>-<istep>.h5", src/IO/Writers.jl:41-137)
written and read by libgpss without an HDF5 library.  Host code only.

The reader is pinned on a file the HDF5 library itself wrote (scipy's MATLAB
7.3 test file: a 512-byte user block, superblock 0, layout message 2), whose
variable is also stored in a MATLAB v7 file that scipy reads; the writer's
structures are re-parsed here by a second, independent parser that checks
the invariants the format sets (node sizes, heap free list, key order,
header sizes, end-of-file address)."""
import ctypes
import os
import struct

import numpy as np
import pytest


@pytest.fixture(scope="module")
def L(sfd, built_lib):
    from sfd_gb300 import _lib
    return _lib.lib()


def _scipy_data(name):
    scipy = pytest.importorskip("scipy")
    p = os.path.join(os.path.dirname(scipy.__file__), "io", "matlab", "tests", "data", name)
    if not os.path.exists(p):
        pytest.skip(f"scipy test data {name} not installed")
    return p


def test_reads_a_file_written_by_the_hdf5_library(sfd):
    import scipy.io as sio
    ref = sio.loadmat(_scipy_data("testdouble_7.4_GLNX86.mat"))["testdouble"]
    got = sfd.read_h5_dataset(_scipy_data("testhdf5_7.4_GLNX86.mat"), "testdouble")
    assert got.shape == (9, 1)  # MATLAB's 1 x 9 row, dims listed in reverse
    assert np.array_equal(got.ravel(), ref.ravel())


# ---- an independent parser of the classic structures the writer emits
def _u(b, off, n):
    return int.from_bytes(b[off:off + n], "little")


UNDEF = (1 << 64) - 1


def _parse(path):
    b = open(path, "rb").read()
    assert b[:8] == b"\x89HDF\r\n\x1a\n"
    assert b[8] == 0 and b[13] == 8 and b[14] == 8
    leaf_k, node_k = _u(b, 16, 2), _u(b, 18, 2)
    base, fs, eof, drv = (_u(b, 24 + 8 * i, 8) for i in range(4))
    assert base == 0 and fs == UNDEF and drv == UNDEF
    assert eof == len(b), "end-of-file address must be the file size"
    root_oh, cache = _u(b, 64, 8), _u(b, 72, 4)
    bt, hp = _u(b, 80, 8), _u(b, 88, 8)
    assert cache == 1

    def ohdr(a):
        assert a % 8 == 0 and b[a] == 1
        nmsg, size = _u(b, a + 2, 2), _u(b, a + 8, 4)
        msgs, p = {}, a + 16
        for _ in range(nmsg):
            t, n = _u(b, p, 2), _u(b, p + 2, 2)
            assert n % 8 == 0
            msgs[t] = b[p + 8:p + 8 + n]
            p += 8 + n
        assert p == a + 16 + size, "header size must cover its messages exactly"
        return msgs

    root = ohdr(root_oh)
    assert set(root) == {0x11} and (_u(root[0x11], 0, 8), _u(root[0x11], 8, 8)) == (bt, hp)
    # local heap: free list head inside the segment, one block ending the list
    assert b[hp:hp + 4] == b"HEAP" and b[hp + 4] == 0
    dsize, free, daddr = _u(b, hp + 8, 8), _u(b, hp + 16, 8), _u(b, hp + 24, 8)
    assert free + 16 <= dsize and _u(b, daddr + free, 8) == 1 and free + _u(b, daddr + free + 8, 8) <= dsize
    name = lambda off: b[daddr + off:b.index(b"\0", daddr + off)].decode()
    assert name(0) == ""
    # B-tree: one group leaf at the full node size, keys bracketing the names
    assert b[bt:bt + 4] == b"TREE" and b[bt + 4] == 0 and b[bt + 5] == 0 and _u(b, bt + 6, 2) == 1
    assert _u(b, bt + 8, 8) == UNDEF and _u(b, bt + 16, 8) == UNDEF
    node_size = 24 + 2 * node_k * 8 + (2 * node_k + 1) * 8
    snod = _u(b, bt + 32, 8)
    assert _u(b, bt + 24, 8) == 0 and snod >= bt + node_size
    assert b[snod:snod + 4] == b"SNOD" and b[snod + 4] == 1
    nsym = _u(b, snod + 6, 2)
    assert 1 <= nsym <= 2 * leaf_k
    ents = [(name(_u(b, snod + 8 + 40 * i, 8)), _u(b, snod + 16 + 40 * i, 8)) for i in range(nsym)]
    names = [e[0] for e in ents]
    assert names == sorted(names) and name(_u(b, bt + 40, 8)) == names[-1]
    out = {}
    for nm, a in ents:
        m = ohdr(a)
        assert set(m) == {0x1, 0x3, 0x5, 0x8}
        sp, ty, ly = m[0x1], m[0x3], m[0x8]
        assert sp[0] == 1 and sp[2] == 0
        dims = struct.unpack_from("<%dQ" % sp[1], sp, 8)
        assert ty[:4] == bytes([0x11, 0x20, 63, 0]) and _u(ty, 4, 4) == 8
        assert struct.unpack_from("<HHBBBBI", ty, 8) == (0, 64, 52, 11, 0, 52, 1023)
        assert ly[0] == 3 and ly[1] == 1
        addr, n = _u(ly, 2, 8), _u(ly, 10, 8)
        assert n == 8 * int(np.prod(dims)) and addr + n <= len(b)
        out[nm] = np.frombuffer(b, dtype="<f8", count=n // 8, offset=addr).reshape(dims)
    return out


@pytest.mark.parametrize("shape", [(8, 6, 4), (16, 8), (1, 1, 1), (64, 32, 2)])
def test_write_read_round_trip_and_structure(L, sfd, tmp_path, shape):
    g = sfd.Grid(shape, tuple((-1.0, 1.0) for _ in shape))
    rng = np.random.default_rng(len(shape) * 100 + shape[0])
    psi = np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    psi.flat[0] = np.inf - 1j * 0.0  # any bit pattern goes through unchanged
    psi.flat[-1] = -0.0 + 1j * 5e-324
    f = sfd.Field(g)
    f.phi = psi
    w = sfd.WriterSave(f)
    prefix = str(tmp_path / "res")
    w.write(prefix=prefix, istep=7)
    path = prefix + "-7.h5"
    parsed = _parse(path)
    assert sorted(parsed) == ["im", "re"]
    # Julia's (nx, ny, nz) column-major array is the HDF5 (nz, ny, nx) row-major one
    assert parsed["re"].shape == shape[::-1]
    assert np.array_equal(parsed["re"].view(np.uint64), psi.real.T.view(np.uint64))
    assert np.array_equal(parsed["im"].view(np.uint64), psi.imag.T.view(np.uint64))
    f2 = sfd.Field(g)
    sfd.WriterSave(f2).read(prefix=prefix, istep=7)
    assert np.array_equal(f2.phi.ravel(order="F").view(np.uint64), psi.ravel(order="F").view(np.uint64))


def test_read_errors(L, sfd, tmp_path):
    from sfd_gb300 import _lib
    g = sfd.Grid((8, 4), ((0, 1), (0, 1)))
    f = sfd.Field(g)
    f.phi = np.ones((8, 4))
    sfd.WriterSave(f).write(prefix=str(tmp_path / "a"), istep=0)
    path = str(tmp_path / "a-0.h5")
    with pytest.raises(_lib.GPSSError, match="EIO.*cannot open"):
        sfd.WriterSave(f).read(prefix=str(tmp_path / "missing"), istep=0)
    with pytest.raises(_lib.GPSSError, match="EINVAL.*shape"):
        sfd.WriterSave(sfd.Field(sfd.Grid((4, 8), ((0, 1), (0, 1))))).read(prefix=str(tmp_path / "a"), istep=0)
    with pytest.raises(_lib.GPSSError, match='EIO.*no dataset "U1"'):
        sfd.read_h5_dataset(path, "U1")
    b = bytearray(open(path, "rb").read())
    bad = tmp_path / "v2.h5"
    b2 = bytearray(b)
    b2[8] = 2
    bad.write_bytes(bytes(b2))
    with pytest.raises(_lib.GPSSError, match="superblock version 2"):
        sfd.read_h5_dataset(str(bad), "re")
    bad.write_bytes(b"not an hdf5 file" * 8)
    with pytest.raises(_lib.GPSSError, match="no HDF5 signature"):
        sfd.read_h5_dataset(str(bad), "re")
    bad.write_bytes(bytes(b[:len(b) - 8]))  # truncated raw data
    with pytest.raises(_lib.GPSSError, match="out of the file"):
        sfd.read_h5_dataset(str(bad), "re")
    # a dataspace far larger than the file is refused before any allocation
    dims = (4).to_bytes(8, "little") + (8).to_bytes(8, "little")
    b3 = bytearray(b)
    at = b3.index(dims)
    b3[at:at + 8] = (1 << 40).to_bytes(8, "little")
    bad.write_bytes(bytes(b3))
    with pytest.raises(_lib.GPSSError, match="larger than the file"):
        sfd.read_h5_dataset(str(bad), "im")


def test_reads_float32_big_endian_and_user_block(L, sfd, tmp_path):
    """Other forms the HDF5 library writes: the writer's file re-typed as
    big-endian float32 (same storage, half of it used) behind a 512-byte user
    block (the superblock's base address then points past it)."""
    g = sfd.Grid((8, 4), ((0, 1), (0, 1)))
    f = sfd.Field(g)
    f.phi = np.arange(32, dtype=np.float64).reshape(8, 4, order="F") * (1 + 0.5j)
    sfd.WriterSave(f).write(prefix=str(tmp_path / "b"), istep=1)
    b = bytearray(open(tmp_path / "b-1.h5", "rb").read())
    # re-type the first dataset header's float64 datatype message
    sig = bytes([0x11, 0x20, 63, 0]) + (8).to_bytes(4, "little")
    p = b.index(sig)
    b[p:p + 20] = bytes([0x11, 0x21, 31, 0]) + (4).to_bytes(4, "little") + struct.pack("<HHBBBBI", 0, 32, 23, 8,
                                                                                      0, 23, 127)
    q = b.index(sig)  # the second dataset keeps float64
    assert q > p
    ub = bytes(512) + bytes(b)
    ub = bytearray(ub)
    ub[512 + 24:512 + 32] = (512).to_bytes(8, "little")  # base address
    path = tmp_path / "ub.h5"
    path.write_bytes(bytes(ub))
    # the names are stored sorted and the headers in that order: "im" was re-typed
    got_re = sfd.read_h5_dataset(str(path), "re")
    got_im = sfd.read_h5_dataset(str(path), "im")
    assert np.array_equal(got_re, f.phi.real.T)
    raw = np.ascontiguousarray(f.phi.imag.T).astype("<f8").tobytes()
    want = np.frombuffer(raw, dtype=">f4", count=32).astype(np.float64).reshape(4, 8)
    assert np.array_equal(got_im, want, equal_nan=True)
