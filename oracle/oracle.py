"""ctypes wrapper of the CPU oracle (vfs_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference arm of bench.py, never by the product package.
Pinned to the reference's own code (oracle/ref.mk, tests/test_ref_oracle.py): see
the header of vfs_oracle.c.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

NSTENCIL = 19
M_TOTAL = 43
# offsets of the metric pack (units of N doubles), vfs_oracle.c enum
M_OFF = dict(csi=0, eta=3, zet=6, aj=9, icsi=10, ieta=13, izet=16, iaj=19, jcsi=20, jeta=23, jzet=26, jaj=29,
             kcsi=30, keta=33, kzet=36, kaj=39, cent=40)
VEC_FIELDS = ("csi", "eta", "zet", "icsi", "ieta", "izet", "jcsi", "jeta", "jzet", "kcsi", "keta", "kzet", "cent")


class Dims(ctypes.Structure):
    _fields_ = [("mx", ctypes.c_int), ("my", ctypes.c_int), ("mz", ctypes.c_int),
                ("ip", ctypes.c_int), ("jp", ctypes.c_int), ("kp", ctypes.c_int)]


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "vfs_oracle.c")):
            build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        D = ctypes.POINTER(Dims)
        L.orc_form_metrics.argtypes = [D, dp, dp]
        L.orc_fluid_regions.argtypes = [D, dp, ctypes.POINTER(ctypes.c_int)]
        L.orc_fluid_regions.restype = ctypes.c_int
        L.orc_gtensor.argtypes = [D, dp, dp]
        L.orc_gid.argtypes = [D, dp, ctypes.POINTER(ctypes.c_int)]
        L.orc_gid.restype = ctypes.c_int
        L.orc_lhs.argtypes = [D, dp, dp, dp]
        L.orc_matvec.argtypes = [D, dp, dp, dp]
        L.orc_csr.argtypes = [D, dp, dp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), dp,
                              ctypes.POINTER(ctypes.c_int)]
        L.orc_csr.restype = ctypes.c_int
        L.orc_rhs.argtypes = [D, dp, dp, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, dp]
        L.orc_rhs.restype = ctypes.c_double
        L.orc_volume_flux.argtypes = [D, ctypes.c_int, dp, dp, dp, dp]
        L.orc_remove_mean.argtypes = [D, dp, dp]
        L.orc_remove_mean.restype = ctypes.c_double
        L.orc_phi_finish.argtypes = [D, dp, dp]
        L.orc_update_pressure.argtypes = [D, dp, dp, dp]
        L.orc_projection.argtypes = [D, dp, dp, dp, ctypes.c_double, ctypes.c_double, ctypes.c_double, dp]
        L.orc_divergence.argtypes = [D, dp, dp, dp, dp]
        L.orc_divergence.restype = ctypes.c_double
        L.orc_contra2cart.argtypes = [D, dp, dp, dp, dp]
        L.orc_coarse_dims.argtypes = [D, ctypes.c_int, ctypes.c_int, ctypes.c_int, D]
        L.orc_coarse_coords.argtypes = [D, D, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp]
        L.orc_nvert_restrict.argtypes = [D, D, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp]
        L.orc_restrict.argtypes = [D, D, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp, dp]
        L.orc_prolong.argtypes = [D, D, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp, dp]
        L.orc_mg_create.argtypes = [D, dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_mg_create.restype = ctypes.c_void_p
        L.orc_mg_destroy.argtypes = [ctypes.c_void_p]
        L.orc_mg_set_params.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_double]
        L.orc_mg_level_dims.argtypes = [ctypes.c_void_p, ctypes.c_int, D]
        L.orc_mg_level_array.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.orc_mg_level_array.restype = dp
        L.orc_mg_apply.argtypes = [ctypes.c_void_p, dp, dp]
        L.orc_mg_matvec.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, dp]
        L.orc_mg_restrict.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, dp]
        L.orc_mg_prolong.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, dp]
        L.orc_mg_smooth.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, dp, ctypes.c_int, ctypes.c_double]
        L.orc_fgmres.argtypes = [ctypes.c_void_p, dp, dp, ctypes.c_double, ctypes.c_int, ctypes.c_int, dp]
        L.orc_fgmres.restype = ctypes.c_int
        L.orc_fgmres_ex.argtypes = [ctypes.c_void_p, dp, dp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    dp]
        L.orc_fgmres_ex.restype = ctypes.c_int
        L.orc_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def dims_of(grid) -> Dims:
    mx, my, mz = grid.dims
    return Dims(mx, my, mz, grid.i_periodic, grid.j_periodic, grid.k_periodic)


def _shape(d: Dims):
    return (d.mz, d.my, d.mx)


def form_metrics(d: Dims, coor: np.ndarray) -> np.ndarray:
    N = d.mx * d.my * d.mz
    M = np.zeros(N * M_TOTAL)
    lib().orc_form_metrics(ctypes.byref(d), _p(np.ascontiguousarray(coor, dtype=np.float64)), _p(M))
    return M


def metric(M: np.ndarray, d: Dims, name: str) -> np.ndarray:
    N = d.mx * d.my * d.mz
    off = M_OFF[name] * N
    if name in VEC_FIELDS:
        return M[off:off + 3 * N].reshape(_shape(d) + (3,))
    return M[off:off + N].reshape(_shape(d))


def gtensor(d: Dims, M: np.ndarray) -> np.ndarray:
    N = d.mx * d.my * d.mz
    g = np.zeros(9 * N)
    lib().orc_gtensor(ctypes.byref(d), _p(M), _p(g))
    return g.reshape((9,) + _shape(d))


def lhs(d: Dims, g: np.ndarray, nvert: np.ndarray) -> np.ndarray:
    N = d.mx * d.my * d.mz
    coef = np.zeros(19 * N)
    lib().orc_lhs(ctypes.byref(d), _p(np.ascontiguousarray(g)), _p(np.ascontiguousarray(nvert, dtype=np.float64)),
                  _p(coef))
    return coef.reshape((19,) + _shape(d))


def matvec(d: Dims, coef: np.ndarray, x: np.ndarray) -> np.ndarray:
    y = np.zeros(_shape(d))
    lib().orc_matvec(ctypes.byref(d), _p(np.ascontiguousarray(coef)), _p(np.ascontiguousarray(x, dtype=np.float64)),
                     _p(y))
    return y


def gid(d: Dims, nvert: np.ndarray):
    N = d.mx * d.my * d.mz
    out = np.zeros(N, dtype=np.int32)
    n = lib().orc_gid(ctypes.byref(d), _p(np.ascontiguousarray(nvert, dtype=np.float64)),
                      out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return n, out.reshape(_shape(d))


def csr(d: Dims, coef: np.ndarray, nvert: np.ndarray):
    """The operator as scipy CSR over the compact fluid numbering."""
    import scipy.sparse as sp
    N = d.mx * d.my * d.mz
    n, _ = gid(d, nvert)
    rowptr = np.zeros(n + 1, dtype=np.int32)
    col = np.zeros(19 * n, dtype=np.int32)
    val = np.zeros(19 * n)
    gidv = np.zeros(N, dtype=np.int32)
    ip = ctypes.POINTER(ctypes.c_int)
    nnz = lib().orc_csr(ctypes.byref(d), _p(np.ascontiguousarray(coef)), _p(np.ascontiguousarray(nvert, dtype=np.float64)),
                        rowptr.ctypes.data_as(ip), col.ctypes.data_as(ip), _p(val), gidv.ctypes.data_as(ip))
    A = sp.csr_matrix((val[:nnz], col[:nnz], rowptr), shape=(n, n))
    return A, gidv.reshape(_shape(d))


def rhs(d: Dims, ucont, nvert, dt=0.04, st=1.0, coeff=1.0, meanfix=True):
    b = np.zeros(_shape(d))
    s = lib().orc_rhs(ctypes.byref(d), _p(np.ascontiguousarray(ucont, dtype=np.float64)),
                      _p(np.ascontiguousarray(nvert, dtype=np.float64)), dt, st, coeff, int(meanfix), _p(b))
    return b, s


def volume_flux(d: Dims, mode: int, ucont: np.ndarray, nvert, M):
    """In place on ucont; returns (flux, area, flux_after, area_after)."""
    out = np.zeros(4)
    assert ucont.flags.c_contiguous and ucont.dtype == np.float64
    lib().orc_volume_flux(ctypes.byref(d), mode, _p(ucont), _p(np.ascontiguousarray(nvert, dtype=np.float64)), _p(M),
                          _p(out))
    return out


def fluid_regions(d: Dims, nvert):
    """(K, labels): connected fluid regions through shared faces, periodic
    wrap included; labels 0..K-1 (in the order of each region's first cell),
    -1 on other cells."""
    lab = np.zeros(_shape(d), dtype=np.int32)
    K = lib().orc_fluid_regions(ctypes.byref(d), _p(np.ascontiguousarray(nvert, dtype=np.float64)),
                                lab.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return K, lab


def remove_mean(d: Dims, nvert, phi):
    return lib().orc_remove_mean(ctypes.byref(d), _p(np.ascontiguousarray(nvert, dtype=np.float64)), _p(phi))


def phi_finish(d: Dims, nvert, phi):
    lib().orc_phi_finish(ctypes.byref(d), _p(np.ascontiguousarray(nvert, dtype=np.float64)), _p(phi))


def update_pressure(d: Dims, nvert, phi, p):
    lib().orc_update_pressure(ctypes.byref(d), _p(np.ascontiguousarray(nvert, dtype=np.float64)),
                              _p(np.ascontiguousarray(phi)), _p(p))


def projection(d: Dims, M, nvert, phi, ucont, dt=0.04, st=1.0, coeff=1.0):
    lib().orc_projection(ctypes.byref(d), _p(M), _p(np.ascontiguousarray(nvert, dtype=np.float64)),
                         _p(np.ascontiguousarray(phi)), dt, st, coeff, _p(ucont))


def divergence(d: Dims, ucont, aj, nvert, field=False):
    div = np.zeros(_shape(d)) if field else None
    v = lib().orc_divergence(ctypes.byref(d), _p(np.ascontiguousarray(ucont)), _p(np.ascontiguousarray(aj)),
                             _p(np.ascontiguousarray(nvert, dtype=np.float64)), _p(div) if field else None)
    return (v, div) if field else v


def contra2cart(d: Dims, M, nvert, ucont, ucat=None):
    ucat = np.zeros(_shape(d) + (3,)) if ucat is None else ucat
    lib().orc_contra2cart(ctypes.byref(d), _p(M), _p(np.ascontiguousarray(nvert, dtype=np.float64)),
                          _p(np.ascontiguousarray(ucont)), _p(ucat))
    return ucat


class MG:
    """Oracle multigrid hierarchy + FGMRES (FP64, OpenMP)."""

    def __init__(self, d: Dims, coor, nvert, levels, semi=(0, 0, 0)):
        self.d = d
        self.levels = levels
        self._coor = np.ascontiguousarray(coor, dtype=np.float64)
        self._nv = np.ascontiguousarray(nvert, dtype=np.float64)
        self.h = lib().orc_mg_create(ctypes.byref(d), _p(self._coor), _p(self._nv), levels, *semi)
        if not self.h:
            raise ValueError("orc_mg_create failed")

    def close(self):
        if self.h:
            lib().orc_mg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, nu1=2, nu2=2, ncoarse=32, omega=0.8, omega_c=0.8):
        lib().orc_mg_set_params(self.h, nu1, nu2, ncoarse, omega, omega_c)

    def level_dims(self, l) -> Dims:
        d = Dims()
        lib().orc_mg_level_dims(self.h, l, ctypes.byref(d))
        return d

    def level_array(self, l, which):
        """which: coor, nvert, M, g, coef, lc, linv."""
        d = self.level_dims(l)
        N = d.mx * d.my * d.mz
        idx = dict(coor=0, nvert=1, M=2, g=3, coef=4, lc=5, linv=6, mcoef=7)[which]
        cnt = dict(coor=3 * N, nvert=N, M=M_TOTAL * N, g=9 * N, coef=19 * N, lc=N, linv=N, mcoef=19 * N)[which]
        ptr = lib().orc_mg_level_array(self.h, l, idx)
        return np.ctypeslib.as_array(ptr, shape=(cnt,)).copy()

    def apply(self, v):
        z = np.zeros(_shape(self.d))
        lib().orc_mg_apply(self.h, _p(np.ascontiguousarray(v, dtype=np.float64)), _p(z))
        return z

    def restrict(self, l, x):
        dc = self.level_dims(l - 1)
        y = np.zeros(_shape(dc))
        lib().orc_mg_restrict(self.h, l, _p(np.ascontiguousarray(x, dtype=np.float64)), _p(y))
        return y

    def prolong(self, l, x):
        df = self.level_dims(l)
        y = np.zeros(_shape(df))
        lib().orc_mg_prolong(self.h, l, _p(np.ascontiguousarray(x, dtype=np.float64)), _p(y))
        return y

    def smooth(self, l, b, x, nsweep, omega):
        lib().orc_mg_smooth(self.h, l, _p(np.ascontiguousarray(b, dtype=np.float64)), _p(x), nsweep, omega)

    def matvec(self, l, x):
        d = self.level_dims(l)
        y = np.zeros(_shape(d))
        lib().orc_mg_matvec(self.h, l, _p(np.ascontiguousarray(x, dtype=np.float64)), _p(y))
        return y

    def fgmres(self, b, x0=None, rtol=1e-12, maxit=200, restart=30, orth=2):
        x = np.zeros(_shape(self.d)) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
        info = np.zeros(3)
        rc = lib().orc_fgmres_ex(self.h, _p(np.ascontiguousarray(b, dtype=np.float64)), _p(x), rtol, maxit, restart,
                                 orth, _p(info))
        return x, dict(converged=(rc == 0), iterations=int(info[0]), relres=float(info[1]), bnorm=float(info[2]))


def projection_step(grid, ucont, levels=3, dt=0.04, st=1.0, coeff=1.0, immersed=0, rtol=1e-12, maxit=400,
                    restart=30, p=None, mg=None, orth=2, div_tol=0.0, max_rounds=4):
    """The whole CPU pressure-projection step, in the reference's order
    (poisson_hypre.c:580-771, solvers.c:874-930): flux balance, RHS with the
    compatibility fix, FGMRES+GMG solve, null-space removal, phi finish,
    UpdatePressure, Projection, Contra2Cart, Divergence.

    div_tol > 0 applies the CUDA path's stopping rule: while the projected
    fluxes leave max |div u| above div_tol, the solve continues from its phi
    with a ten times tighter rtol (at most max_rounds further rounds) and the
    projection is redone from the balanced fluxes."""
    d = dims_of(grid)
    M = form_metrics(d, grid.coor)
    u0 = np.array(ucont, dtype=np.float64, copy=True)
    fa = volume_flux(d, 1 if immersed else 0, u0, grid.nvert, M)
    b, _ = rhs(d, u0, grid.nvert, dt, st, coeff, True)
    own = mg is None
    if own:
        mg = MG(d, grid.coor, grid.nvert, levels)
    aj = metric(M, d, "aj")
    phi, info = mg.fgmres(b, rtol=rtol, maxit=maxit, restart=restart, orth=orth)
    rounds, its = 0, info["iterations"]
    while True:
        ph = phi.copy()
        remove_mean(d, grid.nvert, ph)
        phi_finish(d, grid.nvert, ph)
        u = u0.copy()
        projection(d, M, grid.nvert, ph, u, dt, st, coeff)
        divmax = divergence(d, u, aj, grid.nvert)
        if div_tol <= 0 or divmax <= div_tol or rounds >= max_rounds:
            break
        rounds += 1
        rtol *= 0.1
        phi, info = mg.fgmres(b, x0=phi, rtol=rtol, maxit=maxit, restart=restart, orth=orth)
        its += info["iterations"]
    if own:
        mg.close()
    info = dict(info, iterations=its, rounds=rounds)
    pp = np.zeros(_shape(d)) if p is None else np.array(p, dtype=np.float64, copy=True)
    update_pressure(d, grid.nvert, ph, pp)
    ucat = contra2cart(d, M, grid.nvert, u)
    return dict(phi=ph, p=pp, ucont=u, ucat=ucat, b=b, info=info, divmax=divmax, flux=fa, M=M)
