"""Host logic of the autotuner and the bench (no GPU): candidates map onto
the solve parameters (and back from a cached table entry), a precision copy
keeps every smoothing setting, and the bench's per-kernel table aggregates
probe records by kernel and level class."""
import importlib.util
import os

import numpy as np
import pytest

from vfs_v3p2_gb300 import autotune, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.mark.parametrize("cand", autotune.CANDIDATES)
def test_candidate_roundtrip(cand):
    p = capi.default_params(rtol=1e-7, div_tol=1e-8, warm_start=1)
    autotune.apply_candidate(p, cand)
    assert (p.nu1, p.nu2, p.smooth_cols) == cand[:2] + (cand[3],)
    assert p.omega == pytest.approx(cand[2])
    assert p.nu1_coarse == p.nu2_coarse == cand[4]
    assert p.smoother == autotune.SMOOTHERS[cand[5]]
    assert p.cheb_ratio == pytest.approx(cand[6])
    # untouched: the caller's tolerances and warm start
    assert (p.rtol, p.div_tol, p.warm_start) == (1e-7, 1e-8, 1)
    assert autotune.entry_candidate(autotune.candidate_entry(cand)) == cand
    # every candidate is a valid parameter set for the library
    for finest in (True, False):
        for post in (False, True):
            w = capi.sweep_damping(p, finest, post)
            assert np.all(np.isfinite(w)) and np.all(w > 0)


def test_entry_without_smoother_is_jacobi():
    e = {"nu1": 3, "nu2": 3, "omega": 0.9, "smooth_cols": 0, "nu_coarse": 5}
    assert autotune.entry_candidate(e) == (3, 3, 0.9, 0, 5, "jacobi", 6.0)


def test_with_precision_keeps_settings():
    p = capi.default_params(precision="mixed", nu1=4, nu2=2, nu1_coarse=3, smoother="jacobi", omega=0.8,
                            cheb_hi=1.9, cheb_ratio=7.0, mg_half=1, smooth_cols=16)
    q = autotune.with_precision(p, capi.VFS_FP64)
    assert q.precision == capi.VFS_FP64 and p.precision == capi.VFS_MIXED
    for name, _ in capi.SolveParams._fields_:
        if name != "precision":
            assert getattr(q, name) == getattr(p, name), name


def test_kernel_table_aggregates():
    b = _bench()
    recs = [("k_smooth", 4, 0.05, 2.0e8), ("k_smooth", 4, 0.07, 2.0e8), ("k_smooth", 2, 0.01, 1.0e6),
            ("k_multidot", 4, 0.08, 1.6e8), ("k_arnoldi_finish", 4, 0.01, 0.0)]
    t = b.kernel_table(recs, top=4)
    rows = {(r["kernel"], r["levels"]): r for r in t}
    fin = rows[("k_smooth", "finest")]
    assert fin["launches"] == 2 and fin["ms"] == pytest.approx(0.12) and fin["alg_gb"] == pytest.approx(0.4)
    assert fin["achieved_gbs"] == pytest.approx(0.4 / 0.12e-3)
    assert rows[("k_smooth", "coarser levels")]["launches"] == 1
    assert rows[("k_arnoldi_finish", "finest")]["achieved_gbs"] == 0.0
    assert [r["ms"] for r in t] == sorted((r["ms"] for r in t), reverse=True)


def test_bench_smoother_defaults():
    b = _bench()

    class A:
        nu_coarse = None
        smoother = "chebyshev"
        cheb_hi = 2.0
        cheb_ratio = 6.0
        omega = 0.9

    a = A()
    assert b.nu_coarse(a) == "-1,-1"
    assert b.smoother_config(a) == {"smoother": "chebyshev", "cheb_interval": [2.0 / 6.0, 2.0]}
    a.smoother = "jacobi"
    assert b.nu_coarse(a) == "5,5" and b.smoother_config(a) == {"smoother": "jacobi", "omega": 0.9}
    a.nu_coarse = "4,4"
    assert b.nu_coarse(a) == "4,4"
