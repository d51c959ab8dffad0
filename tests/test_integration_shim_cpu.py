"""The reference-side shim printed in INTEGRATION.md (the file a maintainer
adds next to poisson.c) compiles: extracted from the document as it stands,
it is compiled as the reference's sources are (C++, gnu++17) against
include/vfs_gpu.h, the reference's own variables.h (UserCtx fields and the
run-option globals) and the single-rank PETSc 3.2 / HYPRE / MPI stand-ins
of oracle/ref_stub.  A signature change of the C ABI, or a shim line that
names something the reference does not have, fails here.  Needs the
reference's sources; skipped where they are absent."""
import os
import re
import shutil
import subprocess

import pytest

import ref as R

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _shim_source() -> str:
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    sec = doc[doc.index("## Reference-side shim"):]
    m = re.search(r"```c\n(.*?)```", sec, re.S)
    assert m, "no C block in the shim section"
    return m.group(1)


@pytest.mark.skipif(not R.available(), reason="the reference's sources are not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_integration_shim_compiles(tmp_path):
    src = tmp_path / "vfs_pressure_gb300.c"
    src.write_text(_shim_source())
    cmd = ["g++", "-std=gnu++17", "-w", "-fsyntax-only", "-x", "c++", "-I", os.path.join(ROOT, "oracle", "ref_stub"),
           "-I", R.source_dir(), "-I", os.path.join(ROOT, "include"), str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_shim_calls_declared_entry_points():
    """Every vfs_* function the shim calls is declared in include/vfs_gpu.h."""
    hdr = open(os.path.join(ROOT, "include", "vfs_gpu.h")).read()
    declared = set(re.findall(r"\b(vfs_\w+)\s*\(", hdr))
    called = set(re.findall(r"\b(vfs_\w+)\s*\(", _shim_source()))
    assert called and called <= declared, called - declared
