"""PETSc binary Vec files (the reference's vfield/pfield/nvfield/ufield):
int32 class id 1211214, int32 length, big-endian doubles.  The reader and
writer of the C ABI are host-only; a file built byte by byte from the
format's definition is the known answer."""
import struct

import numpy as np
import pytest

from vfs_v3p2_gb300 import capi

CLASSID = 1211214


def _file(tmp_path, name, payload: bytes):
    p = tmp_path / name
    p.write_bytes(payload)
    return str(p)


def test_read_known_answer(tmp_path):
    vals = [1.0, -2.5, 3.141592653589793, 0.0, -0.0, 1e-310, 6.02e23]
    path = _file(tmp_path, "v.dat", struct.pack(">ii", CLASSID, len(vals)) + struct.pack(f">{len(vals)}d", *vals))
    got = capi.petsc_vec_read(path)
    assert got.tobytes() == np.array(vals).tobytes()


def test_write_matches_format_and_round_trips(tmp_path):
    rng = np.random.default_rng(3)
    a = rng.standard_normal(3 * 7 * 5 * 4) * 1e3
    a[:4] = [np.inf, -np.inf, -0.0, 5e-324]
    path = str(tmp_path / "w.dat")
    capi.petsc_vec_write(path, a)
    raw = open(path, "rb").read()
    assert raw == struct.pack(">ii", CLASSID, a.size) + struct.pack(f">{a.size}d", *a)
    assert capi.petsc_vec_read(path).tobytes() == a.tobytes()
    nan = np.array([np.nan])
    capi.petsc_vec_write(path, nan)
    assert np.isnan(capi.petsc_vec_read(path)[0])


def test_empty_vec(tmp_path):
    path = str(tmp_path / "e.dat")
    capi.petsc_vec_write(path, np.zeros(0))
    assert capi.petsc_vec_read(path).size == 0


def test_errors(tmp_path):
    L = capi.load()
    bad = _file(tmp_path, "bad.dat", struct.pack(">ii", 1211216, 2) + struct.pack(">2d", 1, 2))  # a Mat id
    with pytest.raises(capi.VfsError) as e:
        capi.petsc_vec_read(bad)
    assert e.value.code == capi.VFS_ERR_IO
    short = _file(tmp_path, "short.dat", struct.pack(">ii", CLASSID, 4) + struct.pack(">2d", 1, 2))
    with pytest.raises(capi.VfsError) as e:
        capi.petsc_vec_read(short)
    assert e.value.code == capi.VFS_ERR_IO
    with pytest.raises(capi.VfsError) as e:
        capi.petsc_vec_read(str(tmp_path / "missing.dat"))
    assert e.value.code == capi.VFS_ERR_IO
    ok = _file(tmp_path, "ok.dat", struct.pack(">ii", CLASSID, 2) + struct.pack(">2d", 1, 2))
    out = np.zeros(3)
    assert L.vfs_petsc_vec_read(ok.encode(), capi.dptr(out), 3, None) == capi.VFS_ERR_ARG  # length mismatch
