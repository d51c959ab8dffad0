"""CPU-side checks of the C ABI: the library builds, loads and exports every
function include/vfs_gpu.h declares (no compute calls; no GPU here)."""
import ctypes
import os
import re

from vfs_v3p2_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "vfs_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vfs_\w+)\s*\(", src)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for n in ["vfs_create", "vfs_poisson_lhs", "vfs_poisson_rhs", "vfs_poisson_solve", "vfs_update_pressure",
              "vfs_projection", "vfs_divergence_max", "vfs_projection_step"]:
        assert n in names


def test_library_exports_every_declared_symbol():
    L = capi.load()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    # the binding covers the whole header
    assert set(declared_functions()) <= set(capi.SIGNATURES)


def test_library_is_built_for_sm103a():
    path = capi.lib_path()
    assert os.path.exists(path)
    assert "sm_103a" in " ".join(capi._build.ARCH)
    ctypes.CDLL(path)


def test_default_params_and_unknown_fields():
    """vfs_default_params (host only) and the binding's refusal of a field
    vfs_solve_params does not have (a misspelt option would otherwise be
    set on the Python object and ignored by the library)."""
    import pytest

    p = capi.default_params(precision="mixed")
    assert p.precision == capi.VFS_MIXED and p.mg_stage == 0 and p.mg_grouped == 0 and p.mg_half == 0
    assert capi.default_params(mg_stage=1).mg_stage == 1
    with pytest.raises(AttributeError):
        capi.default_params(mg_tma=1)
