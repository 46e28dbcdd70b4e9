"""The HDF5 snapshot writer (fv_h5_save, IOManager::saveSolution's file
layout, IOManager.h:88-192) and the h5py-like reader of fv3d_gb300.snapshots.

The reader is first checked on a file libhdf5 itself wrote (a MATLAB 7.3
test file shipped with scipy, when present), then reads back what the writer
made: every save's fields and time, the root attributes and vertex
coordinates the reference writes, saves that replace one of the same number,
and root groups large enough for several symbol-table nodes and a two-level
B-tree.  The writer's structures follow the conventions of the libhdf5 file
(superblock 0, version-1 object headers, the same datatype encoding)."""
import ctypes as C
import os
import struct

import numpy as np
import pytest

import fv3d_gb300 as fv
from fv3d_gb300 import _abi, snapshots

_dp = C.POINTER(C.c_double)
FIELDS = ("rho", "u", "v", "w", "prs")
LIBHDF5_FILE = os.path.join(os.path.dirname(__import__("scipy").__file__), "io", "matlab", "tests", "data",
                            "testhdf5_7.4_GLNX86.mat")


def _lib():
    lib = fv.load_library()
    lib.fv_h5_save.argtypes = [C.POINTER(_abi.FvParams), C.c_char_p, C.c_int, C.c_double] + [_dp] * 5
    return lib


def _save(lib, p, path, it, t, q):
    q = [np.ascontiguousarray(a, dtype=np.float64) for a in q]
    return lib.fv_h5_save(C.byref(p), str(path).encode(), it, t, *[a.ctypes.data_as(_dp) for a in q])


@pytest.mark.skipif(not os.path.exists(LIBHDF5_FILE), reason="no libhdf5-written file here")
def test_reader_reads_a_libhdf5_file():
    h = snapshots.H5File(LIBHDF5_FILE)  # a 512-byte user block before the superblock
    root = snapshots._H5Group(h, h.root)
    assert root.keys() == ["testdouble"]
    np.testing.assert_allclose(root["testdouble"].ravel(), np.arange(9) * np.pi / 4, rtol=1e-15)
    assert h.attributes(root._members["testdouble"]) == {"MATLAB_class": b"double"}
    # the writer's dataset messages use the same encodings as this file's
    msgs = dict(h.messages(root._members["testdouble"]))
    lib_dtype, lib_space = msgs[0x3], msgs[0x1]
    assert lib_dtype[:20] == _double_type_of_written_file() and lib_space[:4] == b"\x01\x02\x00\x00"


def _double_type_of_written_file(tmp=[]):
    if not tmp:
        import tempfile
        p = fv.parse_ini("[mesh]\nNx=2\nNy=1\nNz=1\n")
        path = os.path.join(tempfile.mkdtemp(), "t.h5")
        assert _save(_lib(), p, path, 0, 0.0, [np.zeros((1, 1, 2))] * 5) == 0
        h = snapshots.H5File(path)
        tmp.append(dict(h.messages(snapshots._H5Group(h, h.root)._members["x"]))[0x3][:20])
    return tmp[0]


def test_writer_layout_and_round_trip(tmp_path):
    lib = _lib()
    p = fv.parse_ini("[mesh]\nNx=5\nNy=3\nNz=2\nxmax=2.0\n[physics]\nproblem=blast\n")
    path = tmp_path / "run.h5"
    rng = np.random.default_rng(3)
    saved = []
    for it in range(40):  # 43 root members: several symbol-table nodes
        q = rng.standard_normal((5, 2, 3, 5))
        assert _save(lib, p, path, it, 0.1 * it, q) == fv._abi.FV_OK
        saved.append(q)
    raw = path.read_bytes()
    assert raw[:8] == b"\x89HDF\r\n\x1a\n" and raw[8] == 0  # superblock version 0
    eof = struct.unpack_from("<Q", raw, 40)[0]
    assert eof == len(raw)
    f = snapshots.File(str(path))
    assert f.keys() == sorted(["x", "y", "z"] + ["ite_%d" % i for i in range(40)])
    want = {"Ntx": 9, "Nty": 7, "Ntz": 6, "Nx": 5, "Ny": 3, "Nz": 2, "ibeg": 2, "iend": 7, "jbeg": 2, "jend": 5,
            "kbeg": 2, "kend": 4}
    for k, v in want.items():
        assert f.attrs[k] == v and f.attrs[k].dtype == np.int32
    assert f.attrs["problem"] == b"blast"
    # vertex coordinates as IOManager.h:115-124: (i - ibeg) dx, k/j/i order
    kk, jj, ii = np.meshgrid(np.arange(3), np.arange(4), np.arange(6), indexing="ij")
    np.testing.assert_array_equal(f["x"], (ii * p.dx).ravel())
    np.testing.assert_array_equal(f["y"], (jj * p.dy).ravel())
    np.testing.assert_array_equal(f["z"], (kk * p.dz).ravel())
    for it in range(40):
        g = f["ite_%d" % it]
        assert g.attrs["time"] == 0.1 * it
        assert sorted(g.keys()) == sorted(FIELDS)
        for k, name in enumerate(FIELDS):
            got = f["ite_%d/%s" % (it, name)]
            assert got.shape == (2, 3, 5)
            np.testing.assert_array_equal(got, saved[it][k])


def test_writer_two_level_tree_and_replaced_save(tmp_path):
    lib = _lib()
    p = fv.parse_ini("[mesh]\nNx=4\nNy=1\nNz=3\n[physics]\nproblem=sod_x\n")
    path = tmp_path / "run.h5"
    for it in range(300):  # > 32 symbol-table nodes: the root B-tree gets a second level
        assert _save(lib, p, path, it, 0.5 * it, [np.full((3, 1, 4), it + 0.25 * k) for k in range(5)]) == 0
    assert _save(lib, p, path, 7, -1.0, [np.full((3, 1, 4), -7.0)] * 5) == 0  # replaces ite_7
    h = snapshots.H5File(str(path))
    stab = [b for t, b in h.messages(h.root) if t == 0x11][0]
    assert h._m[struct.unpack("<QQ", stab)[0] + 5] == 1  # root B-tree level
    f = snapshots.File(str(path))
    assert len(f.keys()) == 303
    for it in range(300):
        u = f["ite_%d/u" % it]
        assert u[0, 0, 0] == (-7.0 if it == 7 else it + 0.25)
    assert f["ite_7"].attrs["time"] == -1.0


def test_writer_refuses(tmp_path):
    lib = _lib()
    p = fv.parse_ini("[mesh]\nNx=2\nNy=2\nNz=1\n")
    q = [np.zeros((1, 2, 2))] * 5
    not_h5 = tmp_path / "x.h5"
    not_h5.write_bytes(b"plain text, not HDF5" * 10)
    assert _save(lib, p, not_h5, 1, 0.0, q) == fv._abi.FV_ERR_IO  # a later save needs a file it made
    assert _save(lib, p, tmp_path / "missing.h5", 3, 0.0, q) == fv._abi.FV_ERR_IO
    assert _save(lib, p, tmp_path / "no_dir" / "a.h5", 0, 0.0, q) == fv._abi.FV_ERR_IO
    assert _save(lib, p, tmp_path / "a.h5", -1, 0.0, q) == fv._abi.FV_ERR_PARAM


def test_python_save_solution(tmp_path):
    p = fv.parse_ini("[mesh]\nNx=3\nNy=2\nNz=1\n[physics]\nproblem=sod_y\n")
    q = [np.arange(6.0).reshape(1, 2, 3) + k for k in range(5)]
    fv.save_solution(p, tmp_path / "a.h5", 0, 0.0, q)
    fv.save_solution(p, tmp_path / "a.h5", 1, 0.5, [-a for a in q])
    with snapshots.File(str(tmp_path / "a")) as f:
        np.testing.assert_array_equal(f["ite_1/prs"], -q[4])
        assert f["ite_1"].attrs["time"] == 0.5
    with pytest.raises(fv.FvError):
        fv.save_solution(p, tmp_path / "b.h5", 2, 0.0, q)


def test_root_table_region_is_reused(tmp_path):
    """The root group's symbol table is rewritten in its reserved region
    (moved to a twice-larger one when full), so the file grows linearly with
    the saves and a reopened file keeps using the region."""
    p = fv.parse_ini("[mesh]\nNx=4\nNy=1\nNz=3\n[physics]\nproblem=sod_x\n")
    path = tmp_path / "run.h5"
    sizes = {}
    for it in range(800):
        fv.save_solution(p, path, it, float(it), [np.full((3, 1, 4), it + 0.5 * k) for k in range(5)])
        if it + 1 in (200, 400, 800):
            sizes[it + 1] = os.path.getsize(path)
    # per-save growth stays flat (a fresh table per save would grow with the entries)
    g1 = (sizes[400] - sizes[200]) / 200.0
    g2 = (sizes[800] - sizes[400]) / 400.0
    assert g2 < 1.25 * g1, sizes
    f = snapshots.File(str(path))
    assert len(f.keys()) == 803
    for it in (0, 1, 399, 400, 799):
        np.testing.assert_array_equal(f["ite_%d/v" % it], np.full((3, 1, 4), it + 1.0))
        assert f["ite_%d" % it].attrs["time"] == float(it)
    h = snapshots.H5File(str(path))
    stab = [b for t, b in h.messages(h.root) if t == 0x11][0]
    heap = struct.unpack("<QQ", stab)[1]
    dsize, free_head, daddr = struct.unpack_from("<QQQ", h._m, heap + 8)
    assert daddr == heap + 32 and free_head != 1 and free_head < dsize  # a free tail: room for more entries
