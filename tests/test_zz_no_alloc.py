"""The allocation-free divergence check (vfs_divergence_max_noalloc, static
device scratch) against the context entry point vfs_divergence_max on the
same fluxes: two calls in a row, each equal bit for bit to the context's
result (a maximum does not depend on the block partition).  Inputs are
caller-owned device arrays (torch CUDA tensors); the entry point itself
allocates nothing.  Kept in its own file, collected last, so it runs both
alone and after every other GPU test in one process."""
import ctypes
import math

import numpy as np
import pytest

from vfs_v3p2_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch has no CUDA device")
    return torch


def test_noalloc_divergence_matches_context_entry(gpu_ctx):
    torch = _torch_cuda()
    case = synth.channel_case(32, 16, 16, seed=31, spheres=[(math.pi, 0.0, math.pi / 2, 0.6)], sigma=0.5, levels=3)
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
    try:
        gpu_ctx.set_field(gid, capi.FIELD_UCONT, case.ucont)
        ref = gpu_ctx.divergence_max(gid)
        mz, my, mx = g.nvert.shape
        n = mx * my * mz
        aj = gpu_ctx.metrics(gid, case.levels - 1)[9 * n:10 * n]
        dev = torch.device("cuda", 0)
        ux = torch.from_numpy(np.ascontiguousarray(case.ucont[..., 0]).reshape(-1)).to(dev)
        uy = torch.from_numpy(np.ascontiguousarray(case.ucont[..., 1]).reshape(-1)).to(dev)
        uz = torch.from_numpy(np.ascontiguousarray(case.ucont[..., 2]).reshape(-1)).to(dev)
        ajd = torch.from_numpy(np.ascontiguousarray(aj)).to(dev)
        nvd = torch.from_numpy(np.ascontiguousarray(g.nvert).reshape(-1)).to(dev)
        out = torch.full((2,), -1.0, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        L = capi.load()
        err = ctypes.create_string_buffer(256)
        stream = torch.cuda.current_stream().cuda_stream
        for call in range(2):
            rc = L.vfs_divergence_max_noalloc(0, mx, my, mz, 1, 0, 1, ux.data_ptr(), uy.data_ptr(), uz.data_ptr(),
                                              ajd.data_ptr(), nvd.data_ptr(), out.data_ptr() + 8 * call, stream, err,
                                              256)
            assert rc == 0, err.value.decode()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert got[0] == ref and got[1] == ref, (got, ref)
    finally:
        gpu_ctx.grid_destroy(gid)


def test_noalloc_rejects_oversized_grid(gpu_ctx):
    torch = _torch_cuda()
    dev = torch.device("cuda", 0)
    buf = torch.zeros(8, dtype=torch.float64, device=dev)
    p = buf.data_ptr()
    err = ctypes.create_string_buffer(256)
    # 2048^3 cells exceed the kernel's 32-bit cell index: rejected before any launch
    rc = capi.load().vfs_divergence_max_noalloc(0, 2048, 2048, 2048, 0, 0, 0, p, p, p, p, p, p, 0, err, 256)
    assert rc == capi.VFS_ERR_ARG
    assert b"2^31" in err.value


def test_noalloc_periodic_flags_do_not_fill_ghosts(gpu_ctx):
    """Current behaviour: the periodic flags are accepted but unused.  Like the
    reference's Divergence (main.c:1279-1349) the check reads each cell's west,
    south and back faces at index - 1, so with the periodic ghost faces left
    unfilled the result is the same with and without the flags, and equals
    the oracle's divergence of those (unfilled) fluxes."""
    torch = _torch_cuda()
    import oracle as O
    case = synth.channel_case(16, 12, 16, seed=32, levels=2)
    g = case.grid
    u = case.ucont.copy()
    u[:, :, 0, 0] = 0.0  # periodic ghost faces left unfilled
    u[0, :, :, 2] = 0.0
    d = O.dims_of(g)
    M = O.form_metrics(d, g.coor)
    aj = O.metric(M, d, "aj")
    ref = O.divergence(d, u, aj, g.nvert)
    mz, my, mx = g.nvert.shape
    dev = torch.device("cuda", 0)
    comps = [torch.from_numpy(np.ascontiguousarray(u[..., c]).reshape(-1)).to(dev) for c in range(3)]
    ajd = torch.from_numpy(np.ascontiguousarray(aj).reshape(-1)).to(dev)
    nvd = torch.from_numpy(np.ascontiguousarray(g.nvert).reshape(-1)).to(dev)
    out = torch.full((2,), -1.0, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    err = ctypes.create_string_buffer(256)
    stream = torch.cuda.current_stream().cuda_stream
    L = capi.load()
    for call, flags in enumerate(((1, 0, 1), (0, 0, 0))):
        rc = L.vfs_divergence_max_noalloc(0, mx, my, mz, *flags, comps[0].data_ptr(), comps[1].data_ptr(),
                                          comps[2].data_ptr(), ajd.data_ptr(), nvd.data_ptr(),
                                          out.data_ptr() + 8 * call, stream, err, 256)
        assert rc == 0, err.value.decode()
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert got[0] == got[1] == ref, (got, ref)
