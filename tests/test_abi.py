"""CPU checks of the drop-in boundary: the C-ABI library exports every entry
point include/mdsgpu.h declares (no compute call is made here), the ctypes
binding covers them, and the tools keep the reference's option handling."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "mdsgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mds_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def built():
    from mdsctk_gb300 import build

    build.build()
    return build


def test_library_exports_header_symbols(built):
    out = subprocess.run(["nm", "-D", "--defined-only", built.LIB], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (mds_[a-z0-9_]+)\b", out))
    missing = [s for s in _declared() if s not in exported]
    assert not missing, missing


def test_ctypes_binding_covers_header(built):
    from mdsctk_gb300 import _lib

    assert set(_declared()) <= set(_lib.SIGNATURES)


def _tool(built, name, *args):
    return subprocess.run([os.path.join(built.BINDIR, name), *args], capture_output=True, text=True)


def test_tools_help_and_missing_options(built):
    for t in built.TOOLS:
        r = _tool(built, t, "-h")
        assert r.returncode == 1, (t, r.stdout)
        assert "usage:" in r.stdout
    assert _tool(built, "make_sysparse").returncode == 255
    assert "ERROR: --knn not supplied." in _tool(built, "make_sysparse").stdout
    assert _tool(built, "knn_data", "-k", "5").returncode == 255  # no -v
    r = _tool(built, "make_sysparse", "-k", "3", "-n", "5")
    assert r.returncode == 255 and "is not less than the input k" in r.stdout
    r = _tool(built, "decomp_sparse", "-n", "4")
    assert r.returncode == 255 and "ERROR: --sigma not supplied." in r.stdout
    r = _tool(built, "knn_rms", "--sort", "maybe", "-k", "3")
    assert r.returncode == 255
