"""The measurement probe (VFS_PROBE_ALL): one CUDA-event record per
instrumented launch of a projection step, with its kernel, level and
algorithmic bytes.  Probing runs the iterations uncaptured and checks
convergence after each one, so the probed step does exactly the work of an
unprobed one: the same iterations and bit-identical results."""
import numpy as np
import pytest

from vfs_v3p2_gb300 import capi, synth

pytestmark = pytest.mark.gpu

STEP_KERNELS = {"k_smooth", "k_smooth (zero guess)", "k_resrestrict", "k_prolong", "k_coarse_gemv",
                "k_apply64_krylov", "k_multidot", "k_cgs_update", "k_arnoldi_finish", "k_x_update",
                "k_vflux (2 passes)", "k_rhs + k_meanfix", "k_update_p", "k_projection_fast", "k_contra2cart",
                "k_divergence", "k_fluid_sum + k_sub_mean", "k_phi_zero + ghosts", "k_apply64 (residual)",
                "k_norm2 + k_masked_absmax"}


def test_probe_all_records_a_step(gpu_ctx):
    case = synth.c2_sphere(scale=4)
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
    try:
        gpu_ctx.poisson_lhs(gid)
        params = capi.default_params(rtol=1e-9, div_tol=1e-8)
        out = []
        for probe in (False, True, False):
            gpu_ctx.set_field(gid, capi.FIELD_USTAR, case.ucont)
            gpu_ctx.set_field(gid, capi.FIELD_P, np.zeros(g.nvert.shape))
            if probe:
                gpu_ctx.probe_begin(capi.PROBE_ALL)
            info, dm = gpu_ctx.projection_step(gid, params)
            recs = None
            if probe:
                n, ms, by = gpu_ctx.probe_end()
                recs = gpu_ctx.probe_records(n)
                assert n == len(recs) and ms > 0 and by == pytest.approx(sum(r[3] for r in recs))
            out.append((info, dm, gpu_ctx.get_field(gid, capi.FIELD_UCONT, case.ucont.shape), recs))
        (i0, d0, u0, _), (i1, d1, u1, recs), (i2, d2, u2, _) = out
        assert i1["iterations"] == i0["iterations"] == i2["iterations"]
        assert d1 == d0 and np.array_equal(u1, u0) and np.array_equal(u2, u0)
        names = {r[0] for r in recs}
        assert STEP_KERNELS <= names, STEP_KERNELS - names
        its = i1["iterations"]
        top = case.levels - 1
        assert sum(1 for r in recs if r[0] == "k_apply64_krylov") == its
        assert sum(1 for r in recs if r[0] == "k_smooth (zero guess)" and r[1] == top) == its
        # a finest full sweep streams the face form (5 FP32 face weights and
        # aj with the code bits: 24 bytes), x, b and 1/m and writes x
        ni, nj, nk = g.ni, g.nj, g.nk
        sweeps = [r for r in recs if r[0] == "k_smooth" and r[1] == top]
        assert len(sweeps) == its * (params.nu1 + params.nu2 - 1)
        assert all(r[3] == ni * nj * nk * (24 + 16) for r in sweeps)
        assert all(r[2] > 0 for r in recs if r[3] > 0)
    finally:
        gpu_ctx.grid_destroy(gid)


def test_probe_kinds_rejected(gpu_ctx):
    with pytest.raises(capi.VfsError):
        gpu_ctx.probe_begin(7)


def test_probe_smooth_counts_real_sweeps(gpu_ctx):
    """VFS_PROBE_SMOOTH brackets each run of consecutive full finest sweeps
    with one event pair; it counts every real sweep and none of an iteration
    past convergence."""
    case = synth.c2_sphere(scale=4)
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
    try:
        gpu_ctx.poisson_lhs(gid)
        params = capi.default_params(rtol=1e-9, div_tol=1e-8)
        gpu_ctx.set_field(gid, capi.FIELD_USTAR, case.ucont)
        gpu_ctx.set_field(gid, capi.FIELD_P, np.zeros(g.nvert.shape))
        gpu_ctx.probe_begin(capi.PROBE_SMOOTH)
        info, _ = gpu_ctx.projection_step(gid, params)
        n, ms, by = gpu_ctx.probe_end()
        sweeps = info["iterations"] * (params.nu1 - 1 + params.nu2)
        assert n == sweeps and ms > 0
        assert by == sweeps * g.ni * g.nj * g.nk * (24 + 16)  # face form (24 bytes), x, b, 1/m read, x written
        runs = gpu_ctx.probe_records(2 * info["iterations"])
        assert all(r[0] == "k_smooth (run)" for r in runs)
    finally:
        gpu_ctx.grid_destroy(gid)


def test_probe_open_across_a_batch(gpu_ctx):
    """A probe open during a batched call skips the launches captured into
    the batch graph (their events would become graph nodes) and times the
    rest; the batch's results are those of an unprobed batch."""
    cases = [synth.c2_sphere(scale=8), synth.c1_channel(scale=4)]
    ids = []
    try:
        for c in cases:
            gid = gpu_ctx.grid_create(c.grid.coor, c.grid.nvert, c.levels, c.immersed)
            gpu_ctx.poisson_lhs(gid)
            ids.append(gid)
        params = capi.default_params(rtol=1e-9, div_tol=1e-8)
        out = []
        for probe in (False, True):
            for gid, c in zip(ids, cases):
                gpu_ctx.set_field(gid, capi.FIELD_USTAR, c.ucont)
                gpu_ctx.set_field(gid, capi.FIELD_P, np.zeros(c.grid.nvert.shape))
            if probe:
                gpu_ctx.probe_begin(capi.PROBE_ALL)
            infos, dm = gpu_ctx.projection_step_batch(ids, params)
            if probe:
                n, ms, by = gpu_ctx.probe_end()
                recs = gpu_ctx.probe_records(n)
                assert all(np.isfinite(r[2]) and r[2] >= 0 for r in recs)
            out.append(([i["iterations"] for i in infos], dm.copy(),
                        [gpu_ctx.get_field(gid, capi.FIELD_UCONT, c.ucont.shape) for gid, c in zip(ids, cases)]))
        (it0, dm0, u0), (it1, dm1, u1) = out
        assert it0 == it1 and np.array_equal(dm0, dm1)
        assert all(np.array_equal(a, b) for a, b in zip(u0, u1))
    finally:
        for gid in ids:
            gpu_ctx.grid_destroy(gid)
