"""Batched projection steps (one CUDA graph launch per FGMRES iteration for
all grids of the batch) against the same steps run one grid at a time.

Each grid's kernels and their order are the same in both modes; only the
launch grouping differs (and with mg_grouped = 1 the V-cycles of same-size
grids run as grouped launches, operation i of every V-cycle in one launch
with a table of per-grid items), so pressure, phi and the corrected fluxes
must agree bit for bit, and every solve must reach max |div u| < 1e-8."""
import numpy as np
import pytest

from vfs_v3p2_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _cases():
    return synth.c4_batch(count=6, seed=77, lo=(16, 16, 16), hi=(48, 32, 32))


def _load(ctx, cases):
    ids = []
    for c in cases:
        g = c.grid
        gid = ctx.grid_create(g.coor, g.nvert, c.levels, c.immersed)
        ctx.poisson_lhs(gid)
        ids.append(gid)
    return ids


def _reset(ctx, gid, case):
    ctx.set_field(gid, capi.FIELD_USTAR, case.ucont)
    ctx.set_field(gid, capi.FIELD_P, np.zeros(case.grid.nvert.shape))


def _fields(ctx, gid, case):
    shp = case.grid.nvert.shape
    return (ctx.get_field(gid, capi.FIELD_PHI, shp), ctx.get_field(gid, capi.FIELD_P, shp),
            ctx.get_field(gid, capi.FIELD_UCONT, shp + (3,)))


@pytest.mark.parametrize("precision", ["mixed", "mixed_fp16_operator", "mixed_fp32_assembled", "fp64"])
def test_batch_equals_one_at_a_time(gpu_ctx, precision):
    cases = _cases()
    ids = _load(gpu_ctx, cases)
    try:
        half = {"mixed_fp16_operator": 1, "mixed_fp32_assembled": 2}.get(precision, 0)
        params = capi.default_params(precision=precision.split("_")[0], rtol=1e-9, div_tol=1e-8, mg_half=half)
        for gid, c in zip(ids, cases):
            _reset(gpu_ctx, gid, c)
        infos, dm = gpu_ctx.projection_step_batch(ids, params)
        batch = [_fields(gpu_ctx, gid, c) for gid, c in zip(ids, cases)]
        assert all(i["converged"] for i in infos), infos
        assert (dm < 1e-8).all(), dm
        for q, (gid, c) in enumerate(zip(ids, cases)):
            _reset(gpu_ctx, gid, c)
            info, d1 = gpu_ctx.projection_step(gid, params)
            alone = _fields(gpu_ctx, gid, c)
            assert info["iterations"] == infos[q]["iterations"], (q, info, infos[q])
            assert d1 == dm[q]
            for a, b in zip(alone, batch[q]):
                assert np.array_equal(a, b), (q, np.abs(a - b).max())
    finally:
        for gid in ids:
            gpu_ctx.grid_destroy(gid)


def test_batch_per_grid_parameters(gpu_ctx):
    """Per-grid solve parameters (as an autotuner picks them) in one batch."""
    cases = _cases()[:3]
    ids = _load(gpu_ctx, cases)
    try:
        plist = [capi.default_params(rtol=1e-9, div_tol=1e-8, nu1=n, nu2=n) for n in (1, 2, 3)]
        for gid, c in zip(ids, cases):
            _reset(gpu_ctx, gid, c)
        infos, dm = gpu_ctx.projection_step_batch(ids, plist)
        assert all(i["converged"] for i in infos) and (dm < 1e-8).all()
        for q, (gid, c) in enumerate(zip(ids, cases)):
            _reset(gpu_ctx, gid, c)
            info, d1 = gpu_ctx.projection_step(gid, plist[q])
            assert info["iterations"] == infos[q]["iterations"] and d1 == dm[q]
    finally:
        for gid in ids:
            gpu_ctx.grid_destroy(gid)


@pytest.mark.parametrize("precision,half", [("mixed", 1), ("mixed", 0), ("mixed", 2), ("fp64", 0)])
def test_smoother_tile_does_not_change_results(gpu_ctx, precision, half):
    """The y-line smoother's tile (i-columns per block) only regroups
    independent column solves: every tile gives the same bits."""
    c = _cases()[1]
    gid = _load(gpu_ctx, [c])[0]
    try:
        out = []
        for cols in (0, 8, 16, 32):
            _reset(gpu_ctx, gid, c)
            info, dm = gpu_ctx.projection_step(gid, capi.default_params(precision=precision, rtol=1e-9, div_tol=1e-8,
                                                                        smooth_cols=cols, mg_half=half))
            out.append((info["iterations"], dm, _fields(gpu_ctx, gid, c)[0]))
        for it, dm, phi in out[1:]:
            assert it == out[0][0] and dm == out[0][1] and np.array_equal(phi, out[0][2])
    finally:
        gpu_ctx.grid_destroy(gid)


def test_autotune_picks_a_converging_candidate(gpu_ctx):
    from vfs_v3p2_gb300 import autotune
    cases = _cases()[:2]
    base = capi.default_params(rtol=1e-9, div_tol=1e-8)
    plist, table = autotune.tuned_params(gpu_ctx, cases, base, steps=1)
    assert len(plist) == 2 and all(autotune.size_class(c) in table for c in cases)
    for e in table.values():
        assert autotune.entry_candidate(e) in autotune.CANDIDATES
        assert 0 < e["ms_per_step"] < float("inf")


def test_autotune_batch_objective(gpu_ctx):
    from vfs_v3p2_gb300 import autotune
    cases = _cases()[:3]
    ids = _load(gpu_ctx, cases)
    try:
        for gid, c in zip(ids, cases):
            _reset(gpu_ctx, gid, c)
        base = capi.default_params(rtol=1e-9, div_tol=1e-8)
        plist, table = autotune.tuned_params_batch(gpu_ctx, ids, cases, base, steps=1)
        assert len(plist) == 3 and all(p is not None for p in plist)
        infos, dm = gpu_ctx.projection_step_batch(ids, plist)
        assert all(i["converged"] for i in infos) and (dm < 1e-8).all()
    finally:
        for gid in ids:
            gpu_ctx.grid_destroy(gid)


def test_autotune_per_grid(gpu_ctx):
    """Every grid tuned alone: each picks a candidate of the list, and the
    batch with the per-grid schedules converges to the divergence target."""
    from vfs_v3p2_gb300 import autotune
    cases = _cases()[:3]
    ids = _load(gpu_ctx, cases)
    try:
        for gid, c in zip(ids, cases):
            _reset(gpu_ctx, gid, c)
        base = capi.default_params(rtol=1e-9, div_tol=1e-8)
        plist, table = autotune.tuned_params_grids(gpu_ctx, ids, cases, base, steps=1)
        assert set(table) == {c.name for c in cases}
        for e in table.values():
            assert autotune.entry_candidate(e) in autotune.CANDIDATES and e["ms_per_step"] < float("inf")
        infos, dm = gpu_ctx.projection_step_batch(ids, plist)
        assert all(i["converged"] for i in infos) and (dm < 1e-8).all()
    finally:
        for gid in ids:
            gpu_ctx.grid_destroy(gid)


@pytest.mark.parametrize("members", ["uniform", "mixed_kinds"])
def test_grouped_vcycles_equal_per_grid_launches(gpu_ctx, members):
    """mg_grouped 1 (grouped V-cycles) against 0 (each grid's own launches)
    on the same batch, bit for bit; with mixed_kinds the batch also holds
    grids that are not grouped (the FP16 operator) and FP64 grids, whose
    grouped stages run separately."""
    cases = _cases()
    ids = _load(gpu_ctx, cases)
    try:
        out = {}
        for grouped in (0, 1):
            plist = []
            for q in range(len(cases)):
                prec, half = "mixed", 0
                if members == "mixed_kinds":
                    prec = "fp64" if q % 3 == 2 else "mixed"
                    half = 1 if q % 3 == 1 else 0
                plist.append(capi.default_params(precision=prec, rtol=1e-9, div_tol=1e-8, mg_half=half,
                                                 mg_grouped=grouped, cheb_ratio=6.0 + 4 * (q % 2)))
            for gid, c in zip(ids, cases):
                _reset(gpu_ctx, gid, c)
            infos, dm = gpu_ctx.projection_step_batch(ids, plist)
            assert all(i["converged"] for i in infos) and (dm < 1e-8).all()
            out[grouped] = ([i["iterations"] for i in infos], dm.copy(),
                            [_fields(gpu_ctx, gid, c) for gid, c in zip(ids, cases)])
        assert out[0][0] == out[1][0]
        assert np.array_equal(out[0][1], out[1][1])
        for f0, f1 in zip(out[0][2], out[1][2]):
            for a, b in zip(f0, f1):
                assert np.array_equal(a, b)
    finally:
        for gid in ids:
            gpu_ctx.grid_destroy(gid)
