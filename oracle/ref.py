"""ctypes wrapper of oracle/_ref/libvfsref.so: the reference's own
pressure-path functions compiled unmodified from its sources (oracle/ref.mk)
against single-rank PETSc/HYPRE/MPI stand-ins (oracle/ref_stub/).

TEST INFRASTRUCTURE ONLY: it checks the oracle restatement (vfs_oracle.c)
and generates the committed golden fixtures (tests/golden/make_golden.py).
It needs the reference's sources, so it is built and used only where they
are present; nothing of the product loads it.
"""
from __future__ import annotations

import contextlib
import ctypes
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libvfsref.so")
DEFAULT_REF = "/root/reference"


def source_dir():
    return os.environ.get("VFS_REFERENCE_DIR", DEFAULT_REF)


def available() -> bool:
    """True when the reference's sources are present (the checker can be built)."""
    return os.path.exists(os.path.join(source_dir(), "poisson.c"))


def build():
    subprocess.run(["make", "-s", "-f", "ref.mk", "-j8", f"REF={source_dir()}"], cwd=HERE, check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.vfs_ref_create.argtypes = [ctypes.c_int] * 6 + [dp, dp, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                          ctypes.c_char_p]
        L.vfs_ref_create.restype = ctypes.c_void_p
        L.vfs_ref_destroy.argtypes = [ctypes.c_void_p]
        L.vfs_ref_form_metrics.argtypes = [ctypes.c_void_p, dp]
        L.vfs_ref_lhs.argtypes = [ctypes.c_void_p, ip, ip, dp, ctypes.c_longlong, dp]
        L.vfs_ref_lhs.restype = ctypes.c_longlong
        L.vfs_ref_volume_flux.argtypes = [ctypes.c_void_p, dp, dp]
        L.vfs_ref_rhs.argtypes = [ctypes.c_void_p, dp, dp, ctypes.c_int]
        L.vfs_ref_rhs.restype = ctypes.c_int
        L.vfs_ref_phi2_to_phi.argtypes = [ctypes.c_void_p, dp, dp]
        L.vfs_ref_update_and_project.argtypes = [ctypes.c_void_p, dp, dp, dp, dp]
        L.vfs_ref_remove_nullspace.argtypes = [ctypes.c_void_p, dp]
        L.vfs_ref_rhs2.argtypes = [ctypes.c_void_p, dp, dp, ctypes.c_int]
        L.vfs_ref_rhs2.restype = ctypes.c_int
        L.vfs_ref_link.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 4
        L.vfs_ref_nvert_restrict.argtypes = [ctypes.c_void_p, ctypes.c_void_p, dp]
        L.vfs_ref_restrict.argtypes = [ctypes.c_void_p, dp, dp]
        L.vfs_ref_interpolate.argtypes = [ctypes.c_void_p, dp, dp]
        L.vfs_ref_divergence.argtypes = [ctypes.c_void_p, dp]
        L.vfs_ref_divergence.restype = ctypes.c_double
        _lib = L
    return _lib


@contextlib.contextmanager
def _quiet_stdout():
    """The reference prints progress with printf (setup_lidx2): drop it."""
    sys.stdout.flush()
    saved = os.dup(1)
    null = os.open(os.devnull, os.O_WRONLY)
    try:
        os.dup2(null, 1)
        yield
    finally:
        libc = ctypes.CDLL(None)
        libc.fflush(None)
        os.dup2(saved, 1)
        os.close(saved)
        os.close(null)


def _p(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class RefGrid:
    """One level of the reference's UserCtx (see ref_harness.cpp)."""

    def __init__(self, grid, immersed=0, dt=0.04, st=1.0):
        self.grid = grid
        mx, my, mz = grid.dims
        self.shape = (mz, my, mx)
        self._coor = np.ascontiguousarray(grid.coor, dtype=np.float64)
        self._nv = np.ascontiguousarray(grid.nvert, dtype=np.float64)
        self._dir = tempfile.mkdtemp(prefix="vfsref_")
        self.h = lib().vfs_ref_create(mx, my, mz, grid.i_periodic, grid.j_periodic, grid.k_periodic, _p(self._coor),
                                      _p(self._nv), int(immersed), dt, st, self._dir.encode())
        self.n_fluid = None
        self.gid = None

    def form_metrics(self):
        N = int(np.prod(self.shape))
        M = np.zeros(43 * N)
        lib().vfs_ref_form_metrics(self.h, _p(M))
        return M

    def lhs(self):
        """(rows, cols, vals, gid) of the entries PoissonLHSNew sets, in (row, col) order."""
        N = int(np.prod(self.shape))
        cap = 19 * N
        rows = np.zeros(cap, dtype=np.int32)
        cols = np.zeros(cap, dtype=np.int32)
        vals = np.zeros(cap)
        gid = np.zeros(N)
        ip = ctypes.POINTER(ctypes.c_int)
        with _quiet_stdout():
            n = lib().vfs_ref_lhs(self.h, rows.ctypes.data_as(ip), cols.ctypes.data_as(ip), _p(vals), cap, _p(gid))
        self.gid = gid.reshape(self.shape)
        self.n_fluid = int(gid.max()) + 1
        return rows[:n], cols[:n], vals[:n], self.gid

    def volume_flux(self, ucont):
        u = np.array(ucont, dtype=np.float64, copy=True, order="C")
        out = np.zeros(2)
        lib().vfs_ref_volume_flux(self.h, _p(u), _p(out))
        return u, out

    def rhs(self, ucont):
        """b by compact fluid index (call lhs() first: it numbers the fluid)."""
        u = np.ascontiguousarray(ucont, dtype=np.float64)
        b = np.zeros(self.n_fluid)
        n = lib().vfs_ref_rhs(self.h, _p(u), _p(b), self.n_fluid)
        assert n == self.n_fluid
        return b

    def rhs2(self, ucont):
        """PoissonRHS2: b with the compatibility fix, by compact fluid index."""
        u = np.ascontiguousarray(ucont, dtype=np.float64)
        b = np.zeros(self.n_fluid)
        n = lib().vfs_ref_rhs2(self.h, _p(u), _p(b), self.n_fluid)
        assert n == self.n_fluid
        return b

    def remove_nullspace(self, phi2):
        """Remove_Nullspace of a compact solution (returns a copy)."""
        out = np.array(phi2, dtype=np.float64, copy=True, order="C")
        lib().vfs_ref_remove_nullspace(self.h, _p(out))
        return out

    def phi2_to_phi(self, phi2):
        phi = np.zeros(self.shape)
        lib().vfs_ref_phi2_to_phi(self.h, _p(np.ascontiguousarray(phi2, dtype=np.float64)), _p(phi))
        return phi

    def update_and_project(self, phi, p, ucont):
        p = np.array(p, dtype=np.float64, copy=True, order="C")
        u = np.array(ucont, dtype=np.float64, copy=True, order="C")
        ucat = np.zeros(u.shape)
        lib().vfs_ref_update_and_project(self.h, _p(np.ascontiguousarray(phi, dtype=np.float64)), _p(p), _p(u),
                                         _p(ucat))
        return p, u, ucat

    def link_coarse(self, coarse, semi=(0, 0, 0), coarse_level=0):
        """Link this (fine) level and `coarse` as MG_Initial does."""
        lib().vfs_ref_link(self.h, coarse.h, semi[0], semi[1], semi[2], coarse_level)
        self.coarse, coarse.fine = coarse, self

    def nvert_restrict(self):
        """MyNvertRestriction onto the linked coarse level: its nvert."""
        out = np.zeros(self.coarse.shape)
        lib().vfs_ref_nvert_restrict(self.h, self.coarse.h, _p(out))
        return out

    def restrict(self, xf):
        """MyRestriction of a fine vector onto the linked coarse level."""
        out = np.zeros(self.coarse.shape)
        lib().vfs_ref_restrict(self.coarse.h, _p(np.ascontiguousarray(xf, dtype=np.float64)), _p(out))
        return out

    def interpolate(self, xc):
        """MyInterpolation of a coarse vector onto this level."""
        out = np.zeros(self.shape)
        lib().vfs_ref_interpolate(self.h, _p(np.ascontiguousarray(xc, dtype=np.float64)), _p(out))
        return out

    def divergence(self, ucont):
        return lib().vfs_ref_divergence(self.h, _p(np.ascontiguousarray(ucont, dtype=np.float64)))
