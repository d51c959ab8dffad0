"""ctypes binding of the C ABI in include/vfs_gpu.h.

This is the reference-side binding a Python caller uses; a C or C++ caller
links libvfs_gb300.so and includes vfs_gpu.h directly.  There is no CPU
fallback: if the CUDA library cannot be built or loaded, every entry point
raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

VFS_OK = 0
VFS_ERR_ARG = 1
VFS_ERR_CUDA = 2
VFS_ERR_NOMEM = 3
VFS_ERR_NOTCONV = 4
VFS_ERR_STATE = 5
VFS_ERR_NUMERIC = 6
VFS_ERR_BUSY = 7

VFS_FP64 = 0
VFS_MIXED = 1
ORTH_CGS, ORTH_CGS2 = 1, 2
SMOOTH_JACOBI, SMOOTH_CHEBYSHEV = 0, 1

FIELD_UCONT = 0
FIELD_P = 1
FIELD_PHI = 2
FIELD_RHS = 3
FIELD_UCAT = 4
FIELD_NVERT = 5
FIELD_USTAR = 6

VFS_ERR_IO = 8
ERRNAMES = {8: "VFS_ERR_IO", 1: "VFS_ERR_ARG", 2: "VFS_ERR_CUDA", 3: "VFS_ERR_NOMEM", 4: "VFS_ERR_NOTCONV", 5: "VFS_ERR_STATE",
            6: "VFS_ERR_NUMERIC", 7: "VFS_ERR_BUSY"}


class VfsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRNAMES.get(code, code)}: {msg}")
        self.code = code


class Config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_ulonglong), ("max_inflight", ctypes.c_int)]


class GridDesc(ctypes.Structure):
    _fields_ = [("mx", ctypes.c_int), ("my", ctypes.c_int), ("mz", ctypes.c_int),
                ("i_periodic", ctypes.c_int), ("j_periodic", ctypes.c_int), ("k_periodic", ctypes.c_int),
                ("mg_levels", ctypes.c_int), ("semi_i", ctypes.c_int), ("semi_j", ctypes.c_int),
                ("semi_k", ctypes.c_int), ("immersed", ctypes.c_int),
                ("coor", ctypes.POINTER(ctypes.c_double)), ("nvert", ctypes.POINTER(ctypes.c_double))]


class SolveParams(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("rtol", ctypes.c_double), ("maxit", ctypes.c_int),
                ("restart", ctypes.c_int), ("nu1", ctypes.c_int), ("nu2", ctypes.c_int),
                ("omega", ctypes.c_double), ("warm_start", ctypes.c_int), ("div_tol", ctypes.c_double),
                ("orth", ctypes.c_int), ("smooth_cols", ctypes.c_int), ("nu1_coarse", ctypes.c_int),
                ("nu2_coarse", ctypes.c_int), ("mg_half", ctypes.c_int), ("smoother", ctypes.c_int),
                ("cheb_hi", ctypes.c_double), ("cheb_ratio", ctypes.c_double), ("proj_exact", ctypes.c_int),
                ("mg_grouped", ctypes.c_int), ("mg_stage", ctypes.c_int)]


class SolveInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("converged", ctypes.c_int), ("relres", ctypes.c_double),
                ("bnorm", ctypes.c_double), ("time_ms", ctypes.c_double), ("div_limited", ctypes.c_int),
                ("mg_half_used", ctypes.c_int)]

    def as_dict(self):
        return dict(iterations=self.iterations, converged=bool(self.converged), relres=self.relres,
                    bnorm=self.bnorm, time_ms=self.time_ms, div_limited=bool(self.div_limited),
                    mg_half_used=bool(self.mg_half_used))


class Request(ctypes.Structure):
    _fields_ = [("grid", ctypes.c_int), ("ucont_in", ctypes.c_void_p), ("ucont_out", ctypes.c_void_p),
                ("p_in", ctypes.c_void_p), ("p_out", ctypes.c_void_p), ("dt", ctypes.c_double), ("st", ctypes.c_double),
                ("coeff", ctypes.c_double), ("params", SolveParams)]


class Result(ctypes.Structure):
    _fields_ = [("ticket", ctypes.c_longlong), ("status", ctypes.c_int), ("info", SolveInfo),
                ("divmax", ctypes.c_double)]


# Every symbol include/vfs_gpu.h declares, with its ctypes signature.
_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
SIGNATURES = {
    "vfs_create": ([ctypes.POINTER(Config), ctypes.POINTER(_P)], _I),
    "vfs_destroy": ([_P], None),
    "vfs_last_error": ([_P], ctypes.c_char_p),
    "vfs_default_params": ([ctypes.POINTER(SolveParams)], None),
    "vfs_grid_create": ([_P, ctypes.POINTER(GridDesc), _IP], _I),
    "vfs_grid_destroy": ([_P, _I], _I),
    "vfs_grid_bytes": ([_P, _I, ctypes.POINTER(ctypes.c_ulonglong)], _I),
    "vfs_grid_estimate": ([ctypes.POINTER(GridDesc), _I, ctypes.POINTER(ctypes.c_ulonglong)], _I),
    "vfs_poisson_lhs": ([_P, _I], _I),
    "vfs_set_field": ([_P, _I, _I, _DP], _I),
    "vfs_get_field": ([_P, _I, _I, _DP], _I),
    "vfs_volume_flux": ([_P, _I, _DP], _I),
    "vfs_poisson_rhs": ([_P, _I, _D, _D, _D, _I, _DP], _I),
    "vfs_poisson_solve": ([_P, _I, ctypes.POINTER(SolveParams), ctypes.POINTER(SolveInfo)], _I),
    "vfs_update_pressure": ([_P, _I], _I),
    "vfs_projection": ([_P, _I, _D, _D, _D], _I),
    "vfs_projection_faces": ([_P, _I, _D, _D, _D], _I),
    "vfs_divergence_max": ([_P, _I, _DP], _I),
    "vfs_divergence_max_noalloc": ([_I, _I, _I, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, ctypes.c_char_p, _I], _I),
    "vfs_projection_step": ([_P, _I, _DP, _DP, _D, _D, _D, ctypes.POINTER(SolveParams), ctypes.POINTER(SolveInfo),
                             _DP], _I),
    "vfs_get_metrics": ([_P, _I, _I, _DP], _I),
    "vfs_get_coef": ([_P, _I, _I, _I, _DP], _I),
    "vfs_get_mg_half": ([_P, _I, _I, _DP, _DP, _DP], _I),
    "vfs_get_level_dims": ([_P, _I, _I, _IP], _I),
    "vfs_get_level_nvert": ([_P, _I, _I, _DP], _I),
    "vfs_apply_op": ([_P, _I, _I, _I, _DP, _DP], _I),
    "vfs_apply_precond": ([_P, _I, _I, ctypes.POINTER(SolveParams), _DP, _DP], _I),
    "vfs_mg_restrict": ([_P, _I, _I, _DP, _DP], _I),
    "vfs_mg_prolong": ([_P, _I, _I, _DP, _DP], _I),
    "vfs_mg_smooth": ([_P, _I, _I, _DP, _DP, _D], _I),
    "vfs_projection_step_batch": ([_P, _I, _IP, _D, _D, _D, ctypes.POINTER(SolveParams), _I,
                                   ctypes.POINTER(SolveInfo), _DP], _I),
    "vfs_sync": ([_P], _I),
    "vfs_grid_update_nvert": ([_P, _I, _DP], _I),
    "vfs_grid_update_coords": ([_P, _I, _DP], _I),
    "vfs_petsc_vec_read": ([ctypes.c_char_p, _DP, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)], _I),
    "vfs_petsc_vec_write": ([ctypes.c_char_p, _DP, ctypes.c_longlong], _I),
    "vfs_submit": ([_P, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_longlong)], _I),
    "vfs_poll": ([_P, _I, ctypes.POINTER(Result)], _I),
    "vfs_inflight": ([_P], _I),
    "vfs_memory": ([_P, ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_ulonglong)], _I),
    "vfs_probe_begin": ([_P, _I], _I),
    "vfs_probe_end": ([_P, ctypes.POINTER(ctypes.c_ulonglong), _DP, _DP], _I),
    "vfs_launch_count": ([ctypes.POINTER(ctypes.c_ulonglong)], _I),
    "vfs_mark": ([_P, _I, _I], _I),
    "vfs_elapsed": ([_P, _I, _I, _DP], _I),
    "vfs_grid_components": ([_P, _I, ctypes.POINTER(_I), ctypes.POINTER(_I)], _I),
    "vfs_probe_record": ([_P, _I, ctypes.c_char_p, _I, ctypes.POINTER(_I), _DP, _DP], _I),
    "vfs_sweep_damping": ([ctypes.POINTER(SolveParams), _I, _I, _DP, _I], _I),
    "vfs_debug_tma_drop": ([_I], _I),
    "vfs_host_register": ([_P, ctypes.c_ulonglong], _I),
    "vfs_host_unregister": ([_P], _I),
    "vfs_host_alloc": ([ctypes.POINTER(_P), ctypes.c_ulonglong], _I),
    "vfs_host_free": ([_P], _I),
}

PROBE_SMOOTH = 1
PROBE_APPLY64 = 2
PROBE_ALL = 3


def launch_count() -> int:
    n = ctypes.c_ulonglong()
    load().vfs_launch_count(ctypes.byref(n))
    return n.value

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libvfs_gb300.so (building it first when missing or stale)."""
    global _lib
    if _lib is None:
        if build_if_missing:
            _build.build()
        if not os.path.exists(_build.LIB):
            raise RuntimeError(f"CUDA library {_build.LIB} is missing; run vfs_v3p2_gb300/build.py")
        L = ctypes.CDLL(_build.LIB)
        for name, (args, res) in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def dptr(a: np.ndarray):
    if a is None:
        return None
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise ValueError("arrays passed to the C ABI must be C-contiguous float64")
    return a.ctypes.data_as(_DP)


def sweep_damping(params: SolveParams, finest: bool, post: bool) -> np.ndarray:
    """Damping of each smoothing sweep the V-cycle launches under params."""
    nu1c = params.nu1_coarse if params.nu1_coarse >= 0 else params.nu1
    nu2c = params.nu2_coarse if params.nu2_coarse >= 0 else params.nu2
    n = (params.nu2 if post else params.nu1) if finest else (nu2c if post else nu1c)
    w = np.zeros(max(n, 1))
    rc = load().vfs_sweep_damping(ctypes.byref(params), int(finest), int(post), dptr(w), n)
    if rc:
        raise VfsError(rc, "vfs_sweep_damping: invalid parameters")
    return w[:n]


def default_params(**kw) -> SolveParams:
    p = SolveParams()
    load().vfs_default_params(ctypes.byref(p))
    names = {f[0] for f in SolveParams._fields_}
    for k, v in kw.items():
        if k not in names:
            raise AttributeError(f"vfs_solve_params has no field {k!r}")
        if k == "precision" and isinstance(v, str):
            v = {"fp64": VFS_FP64, "mixed": VFS_MIXED}[v]
        if k == "orth" and isinstance(v, str):
            v = {"cgs": ORTH_CGS, "cgs2": ORTH_CGS2}[v]
        if k == "smoother" and isinstance(v, str):
            v = {"jacobi": SMOOTH_JACOBI, "chebyshev": SMOOTH_CHEBYSHEV}[v]
        setattr(p, k, v)
    return p


class Context:
    """One vfs_ctx (a device and its resident grids)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0, max_inflight: int = 0):
        self.L = load()
        cfg = Config(device, hbm_budget_bytes, max_inflight)
        h = _P()
        rc = self.L.vfs_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc:
            raise VfsError(rc, "vfs_create failed (no usable CUDA device?)")
        self.h = h

    def check(self, rc):
        if rc:
            raise VfsError(rc, self.L.vfs_last_error(self.h).decode())
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.L.vfs_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- grids --
    def grid_create(self, coor: np.ndarray, nvert: np.ndarray, levels: int, immersed: int = 0,
                    periodic=(1, 0, 1), semi=(0, 0, 0)) -> int:
        coor = np.ascontiguousarray(coor, dtype=np.float64)
        nvert = np.ascontiguousarray(nvert, dtype=np.float64)
        mz, my, mx = nvert.shape
        if coor.shape != (mz, my, mx, 3):
            raise ValueError("coor must be [mz, my, mx, 3]")
        d = GridDesc(mx, my, mz, periodic[0], periodic[1], periodic[2], levels, semi[0], semi[1], semi[2], immersed,
                     dptr(coor), dptr(nvert))
        gid = ctypes.c_int()
        self.check(self.L.vfs_grid_create(self.h, ctypes.byref(d), ctypes.byref(gid)))
        return gid.value

    def grid_destroy(self, g: int):
        self.check(self.L.vfs_grid_destroy(self.h, g))

    def grid_bytes(self, g: int) -> int:
        b = ctypes.c_ulonglong()
        self.check(self.L.vfs_grid_bytes(self.h, g, ctypes.byref(b)))
        return b.value

    def grid_components(self, g: int):
        """(finest, coarsest): connected fluid regions found by poisson_lhs."""
        f, c = _I(), _I()
        self.check(self.L.vfs_grid_components(self.h, g, ctypes.byref(f), ctypes.byref(c)))
        return f.value, c.value

    def level_dims(self, g: int, level: int):
        d = (ctypes.c_int * 3)()
        self.check(self.L.vfs_get_level_dims(self.h, g, level, d))
        return tuple(d)

    def poisson_lhs(self, g: int):
        self.check(self.L.vfs_poisson_lhs(self.h, g))

    def set_field(self, g: int, field: int, a: np.ndarray):
        self.check(self.L.vfs_set_field(self.h, g, field, dptr(np.ascontiguousarray(a, dtype=np.float64))))

    def get_field(self, g: int, field: int, shape) -> np.ndarray:
        out = np.zeros(shape)
        self.check(self.L.vfs_get_field(self.h, g, field, dptr(out)))
        return out

    def volume_flux(self, g: int):
        out = np.zeros(4)
        self.check(self.L.vfs_volume_flux(self.h, g, dptr(out)))
        return out

    def poisson_rhs(self, g: int, dt=0.04, st=1.0, coeff=1.0, meanfix=True) -> float:
        s = ctypes.c_double()
        self.check(self.L.vfs_poisson_rhs(self.h, g, dt, st, coeff, int(meanfix), ctypes.byref(s)))
        return s.value

    def poisson_solve(self, g: int, params: SolveParams, allow_notconv=False):
        info = SolveInfo()
        rc = self.L.vfs_poisson_solve(self.h, g, ctypes.byref(params), ctypes.byref(info))
        if rc and not (allow_notconv and rc == VFS_ERR_NOTCONV):
            self.check(rc)
        return info.as_dict()

    def update_pressure(self, g: int):
        self.check(self.L.vfs_update_pressure(self.h, g))

    def projection(self, g: int, dt=0.04, st=1.0, coeff=1.0, faces: bool = False):
        fn = self.L.vfs_projection_faces if faces else self.L.vfs_projection
        self.check(fn(self.h, g, dt, st, coeff))

    def divergence_max(self, g: int) -> float:
        v = ctypes.c_double()
        self.check(self.L.vfs_divergence_max(self.h, g, ctypes.byref(v)))
        return v.value

    def projection_step(self, g: int, params: SolveParams, ucont: np.ndarray = None, p: np.ndarray = None, dt=0.04,
                        st=1.0, coeff=1.0):
        info = SolveInfo()
        dm = ctypes.c_double()
        self.check(self.L.vfs_projection_step(self.h, g, dptr(ucont), dptr(p), dt, st, coeff, ctypes.byref(params),
                                              ctypes.byref(info), ctypes.byref(dm)))
        return info.as_dict(), dm.value

    def projection_step_ptr(self, g: int, params: SolveParams, ucont_ptr: int, p_ptr: int, dt=0.04, st=1.0,
                            coeff=1.0):
        """Same as projection_step with raw host addresses (e.g. pinned buffers)."""
        info = SolveInfo()
        dm = ctypes.c_double()
        self.check(self.L.vfs_projection_step(self.h, g, ctypes.cast(ucont_ptr, _DP) if ucont_ptr else None,
                                              ctypes.cast(p_ptr, _DP) if p_ptr else None, dt, st, coeff,
                                              ctypes.byref(params), ctypes.byref(info), ctypes.byref(dm)))
        return info.as_dict(), dm.value

    def projection_step_batch(self, grids, params, dt=0.04, st=1.0, coeff=1.0):
        """params: one SolveParams for all grids or a sequence of one per grid."""
        n = len(grids)
        ids = (ctypes.c_int * n)(*grids)
        infos = (SolveInfo * n)()
        dm = np.zeros(n)
        if isinstance(params, SolveParams):
            parr, npar = (SolveParams * 1)(params), 1
        else:
            parr, npar = (SolveParams * n)(*params), n
        self.check(self.L.vfs_projection_step_batch(self.h, n, ids, dt, st, coeff, parr, npar, infos, dptr(dm)))
        return [i.as_dict() for i in infos], dm

    def sync(self):
        self.check(self.L.vfs_sync(self.h))

    # ---- serving ----
    def submit(self, grid: int, params: SolveParams, ucont_in=0, ucont_out=0, p_in=0, p_out=0, dt=0.04, st=1.0,
               coeff=1.0):
        # Admit one projection step (host buffers as raw addresses, 0 = resident).
        # Returns the ticket, or None when no slot is free or the grid is busy.
        req = Request(grid, ucont_in or None, ucont_out or None, p_in or None, p_out or None, dt, st, coeff, params)
        t = ctypes.c_longlong()
        rc = self.L.vfs_submit(self.h, ctypes.byref(req), ctypes.byref(t))
        if rc == VFS_ERR_BUSY:
            return None
        self.check(rc)
        return t.value

    def poll(self, wait: bool = False):
        # One finished request as (ticket, status, info, divmax), or None.
        r = Result()
        rc = self.L.vfs_poll(self.h, 1 if wait else 0, ctypes.byref(r))
        if rc in (VFS_ERR_BUSY, VFS_ERR_STATE):
            return None
        self.check(rc)
        return r.ticket, r.status, r.info.as_dict(), r.divmax

    def inflight(self) -> int:
        return self.L.vfs_inflight(self.h)

    def memory(self):
        u, b = ctypes.c_ulonglong(), ctypes.c_ulonglong()
        self.check(self.L.vfs_memory(self.h, ctypes.byref(u), ctypes.byref(b)))
        return u.value, b.value

    def mark(self, g: int, slot: int):
        self.check(self.L.vfs_mark(self.h, g, slot))

    def elapsed(self, a: int, b: int) -> float:
        ms = ctypes.c_double()
        self.check(self.L.vfs_elapsed(self.h, a, b, ctypes.byref(ms)))
        return ms.value

    def probe_begin(self, kernel: int):
        self.check(self.L.vfs_probe_begin(self.h, kernel))

    def probe_end(self):
        n = ctypes.c_ulonglong()
        ms = ctypes.c_double()
        by = ctypes.c_double()
        self.check(self.L.vfs_probe_end(self.h, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(by)))
        return n.value, ms.value, by.value

    def probe_records(self, n: int):
        """The last probe's records: (kernel, level, ms, algorithmic bytes)."""
        out = []
        buf = ctypes.create_string_buffer(64)
        lv, ms, by = _I(), ctypes.c_double(), ctypes.c_double()
        for i in range(n):
            self.check(self.L.vfs_probe_record(self.h, i, buf, 64, ctypes.byref(lv), ctypes.byref(ms),
                                               ctypes.byref(by)))
            out.append((buf.value.decode(), lv.value, ms.value, by.value))
        return out

    def host_register(self, a: np.ndarray):
        rc = self.L.vfs_host_register(a.ctypes.data_as(_P), a.nbytes)
        if rc:
            raise VfsError(rc, "cudaHostRegister failed")

    def host_unregister(self, a: np.ndarray):
        self.L.vfs_host_unregister(a.ctypes.data_as(_P))

    def host_alloc(self, shape, dtype=np.float64) -> np.ndarray:
        """A numpy array over page-locked memory from vfs_host_alloc; release
        it with host_free (the array must not be used afterwards)."""
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = _P()
        rc = self.L.vfs_host_alloc(ctypes.byref(p), n)
        if rc:
            raise VfsError(rc, "cudaHostAlloc failed")
        return np.frombuffer((ctypes.c_char * n).from_address(p.value), dtype=dtype).reshape(shape)

    def host_free(self, a: np.ndarray):
        self.check(self.L.vfs_host_free(a.ctypes.data_as(_P)))

    # -- hooks --
    def update_nvert(self, g: int, nvert: np.ndarray):
        self.check(self.L.vfs_grid_update_nvert(self.h, g, dptr(np.ascontiguousarray(nvert, dtype=np.float64))))

    def update_coords(self, g: int, coor: np.ndarray):
        self.check(self.L.vfs_grid_update_coords(self.h, g, dptr(np.ascontiguousarray(coor, dtype=np.float64))))

    def metrics(self, g: int, level: int) -> np.ndarray:
        mx, my, mz = self.level_dims(g, level)
        out = np.zeros(43 * mx * my * mz)
        self.check(self.L.vfs_get_metrics(self.h, g, level, dptr(out)))
        return out

    def coef(self, g: int, level: int, which: int = 0) -> np.ndarray:
        mx, my, mz = self.level_dims(g, level)
        out = np.zeros(19 * mx * my * mz)
        self.check(self.L.vfs_get_coef(self.h, g, level, which, dptr(out)))
        return out.reshape((19, mz, my, mx))

    def mg_half(self, g: int, level: int):
        """The FP16 diagonal-normalised multigrid operator of a level: the 19
        slots (centre slot: the row-sum correction), the y-line pivots and the
        restriction weights, as float64 arrays."""
        mx, my, mz = self.level_dims(g, level)
        coef = np.zeros((19, mz, my, mx))
        lf = np.zeros((mz, my, mx))
        rw = np.zeros((mz, my, mx))
        self.check(self.L.vfs_get_mg_half(self.h, g, level, dptr(coef), dptr(lf), dptr(rw)))
        return coef, lf, rw

    def level_nvert(self, g: int, level: int) -> np.ndarray:
        mx, my, mz = self.level_dims(g, level)
        out = np.zeros((mz, my, mx))
        self.check(self.L.vfs_get_level_nvert(self.h, g, level, dptr(out)))
        return out

    def apply_op(self, g: int, level: int, which: int, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        self.check(self.L.vfs_apply_op(self.h, g, level, which, dptr(x), dptr(y)))
        return y

    def apply_precond(self, g: int, precision: int, params: SolveParams, v: np.ndarray) -> np.ndarray:
        v = np.ascontiguousarray(v, dtype=np.float64)
        z = np.zeros_like(v)
        self.check(self.L.vfs_apply_precond(self.h, g, precision, ctypes.byref(params), dptr(v), dptr(z)))
        return z

    def mg_restrict(self, g: int, level: int, x: np.ndarray) -> np.ndarray:
        mx, my, mz = self.level_dims(g, level - 1)
        y = np.zeros((mz, my, mx))
        self.check(self.L.vfs_mg_restrict(self.h, g, level, dptr(np.ascontiguousarray(x, dtype=np.float64)), dptr(y)))
        return y

    def mg_prolong(self, g: int, level: int, x: np.ndarray) -> np.ndarray:
        mx, my, mz = self.level_dims(g, level)
        y = np.zeros((mz, my, mx))
        self.check(self.L.vfs_mg_prolong(self.h, g, level, dptr(np.ascontiguousarray(x, dtype=np.float64)), dptr(y)))
        return y

    def mg_smooth(self, g: int, level: int, b: np.ndarray, x: np.ndarray, omega: float) -> np.ndarray:
        x = np.array(x, dtype=np.float64, copy=True, order="C")
        self.check(self.L.vfs_mg_smooth(self.h, g, level, dptr(np.ascontiguousarray(b, dtype=np.float64)), dptr(x),
                                        omega))
        return x


def petsc_vec_read(path: str) -> np.ndarray:
    """A PETSc binary Vec file (the reference's field files) as a float64 array."""
    L = load()
    n = ctypes.c_longlong()
    rc = L.vfs_petsc_vec_read(path.encode(), None, 0, ctypes.byref(n))
    if rc:
        raise VfsError(rc, f"cannot read PETSc Vec header of {path}")
    out = np.zeros(n.value)
    rc = L.vfs_petsc_vec_read(path.encode(), dptr(out), n.value, None)
    if rc:
        raise VfsError(rc, f"cannot read PETSc Vec {path}")
    return out


def petsc_vec_write(path: str, a: np.ndarray):
    """Write a float64 array as a PETSc binary Vec file."""
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
    rc = load().vfs_petsc_vec_write(path.encode(), dptr(a), a.size)
    if rc:
        raise VfsError(rc, f"cannot write PETSc Vec {path}")
