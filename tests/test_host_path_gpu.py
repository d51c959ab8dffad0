"""The projection step through host buffers (vfs_projection_step with the
fluxes and the pressure in host memory) returns what the same step on the
resident fields leaves on the device, bit for bit.  The fluxes go down in
k-plane slabs, one per 4 MiB of AoS fluxes (1 to 8), each slab converted and
copied while the next one is projected, the two k ghost planes after the
last slab; the pressure upload follows the flux upload."""
import numpy as np
import pytest

from vfs_v3p2_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _slabs(shape):
    mz, my, mx = shape
    return max(1, min(8, (3 * mx * my * mz * 8) >> 22))


CASES = [
    # (case, periodic flags, expected slab count)
    (lambda: synth.c2_sphere(scale=2), (1, 0, 1), 3),
    (lambda: synth.c2_sphere(scale=2), (0, 0, 0), 3),
    (lambda: synth.channel_case(40, 24, 20, seed=31, levels=2), (1, 0, 1), 1),
    (lambda: synth.c2_sphere(scale=1), (1, 0, 1), 8),
]


@pytest.mark.parametrize("memory", ["pageable", "registered", "host_alloc"])
@pytest.mark.parametrize("which", range(len(CASES)))
def test_host_buffers_match_resident(gpu_ctx, which, memory):
    make, periodic, nslab = CASES[which]
    case = make()
    g = case.grid
    assert min(nslab, g.nvert.shape[0] - 2) == min(_slabs(g.nvert.shape), g.nvert.shape[0] - 2)
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed, periodic=periodic)
    try:
        gpu_ctx.poisson_lhs(gid)
        params = capi.default_params(precision="mixed", rtol=1e-9, div_tol=1e-8)
        rng = np.random.default_rng(7)
        p0 = rng.standard_normal(g.nvert.shape)
        # resident: U* and p set on the device, outputs read back after the step
        gpu_ctx.set_field(gid, capi.FIELD_USTAR, case.ucont)
        gpu_ctx.set_field(gid, capi.FIELD_P, p0)
        info_r, dm_r = gpu_ctx.projection_step(gid, params)
        u_r = gpu_ctx.get_field(gid, capi.FIELD_UCONT, case.ucont.shape)
        p_r = gpu_ctx.get_field(gid, capi.FIELD_P, p0.shape)
        # host buffers: a plane left out of the download keeps its U* values
        if memory == "host_alloc":
            u, p = gpu_ctx.host_alloc(case.ucont.shape), gpu_ctx.host_alloc(p0.shape)
            u[...], p[...] = case.ucont, p0
        else:
            u, p = np.ascontiguousarray(case.ucont.copy()), p0.copy()
            if memory == "registered":
                gpu_ctx.host_register(u)
                gpu_ctx.host_register(p)
        try:
            info_h, dm_h = gpu_ctx.projection_step(gid, params, u, p)
            assert info_r["converged"] and info_h["converged"]
            assert info_h["iterations"] == info_r["iterations"]
            assert not np.array_equal(u_r, case.ucont)
            assert np.array_equal(u, u_r)
            assert np.array_equal(p, p_r)
            assert dm_h == dm_r
        finally:
            if memory == "host_alloc":
                gpu_ctx.host_free(u)
                gpu_ctx.host_free(p)
            elif memory == "registered":
                gpu_ctx.host_unregister(u)
                gpu_ctx.host_unregister(p)
    finally:
        gpu_ctx.grid_destroy(gid)
