"""The reference-side adapter of INTEGRATION.md (simp_gb300.cpp) compiles
against the reference's own headers and this library's C header, so its layout
static_asserts (DirichletBC / NodalLoad against the C structs, one-byte
VoxelTag) hold.  CPU only; skipped where the reference tree is absent."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def adapter_source():
    md = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    sec = md[md.index("## The binding a maintainer adds on the reference side"):]
    m = re.search(r"```cpp\n(.*?)```", sec, re.S)
    assert m, "no C++ block in the adapter section"
    return m.group(1)


def test_adapter_compiles_against_reference_headers(tmp_path):
    from oracle.oracle import reference_path
    inc = reference_path("core", "include")
    if not os.path.isdir(os.path.join(inc, "topopt")):
        pytest.skip("reference tree not present")
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    src = tmp_path / "simp_gb300.cpp"
    src.write_text(adapter_source())
    res = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wall", "-I", inc,
                          "-I", os.path.join(ROOT, "include"), str(src)],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-4000:]
