"""The host dense symmetric eigensolver of the Lanczos restarts
(mdsctk_gb300/csrc/sym_eig.h) against numpy's eigh, on CPU.

The projected matrices it meets are arrowhead + tridiagonal (thick restart),
with clusters of nearly equal Ritz values; the cases below cover those, plus
dense random matrices, a diagonal matrix, exact multiplicities and m = 1, 2.
"""
import ctypes
import os
import shutil
import subprocess
import zlib

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "mdsctk_gb300", "csrc")


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("symeig") / "libsymeig.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I" + CSRC,
                    os.path.join(HERE, "native", "sym_eig_shim.cpp"), "-o", out], check=True)
    lib = ctypes.CDLL(out)
    lib.symeig_shim.restype = ctypes.c_int
    return lib


def _solve(lib, a):
    m = a.shape[0]
    a = np.ascontiguousarray(a, dtype=np.float64)
    w = np.zeros(m)
    z = np.zeros((m, m))
    dp = ctypes.POINTER(ctypes.c_double)
    rc = lib.symeig_shim(m, a.ctypes.data_as(dp), w.ctypes.data_as(dp), z.ctypes.data_as(dp))
    assert rc == 0
    return w, z


def _arrowhead(rng, m, k, cluster=False):
    t = np.zeros((m, m))
    theta = np.sort(rng.uniform(0.5, 1.0, k))
    if cluster:
        theta = 1.0 - np.sort(rng.uniform(0, 1e-9, k))  # Ritz values crowded at 1
    s = rng.normal(0, 1e-3, k)
    for i in range(k):
        t[i, i] = theta[i]
        t[i, k] = t[k, i] = s[i]
    alpha = rng.uniform(-0.5, 1.0, m - k)
    beta = rng.uniform(0.01, 0.3, m - k - 1)
    for j in range(k, m):
        t[j, j] = alpha[j - k]
        if j + 1 < m:
            t[j, j + 1] = t[j + 1, j] = beta[j - k]
    return t


CASES = ["dense20", "dense201", "arrow60", "arrow_cluster60", "arrow101", "diag", "multiple", "m1", "m2", "zero_col"]


@pytest.mark.parametrize("case", CASES)
def test_sym_eig_vs_eigh(shim, case):
    rng = np.random.default_rng(zlib.crc32(case.encode()))
    if case.startswith("dense"):
        m = int(case[5:])
        g = rng.normal(size=(m, m))
        a = (g + g.T) / 2
    elif case == "arrow60":
        a = _arrowhead(rng, 60, 30)
    elif case == "arrow_cluster60":
        a = _arrowhead(rng, 60, 30, cluster=True)
    elif case == "arrow101":
        a = _arrowhead(rng, 101, 50)
    elif case == "diag":
        a = np.diag(rng.normal(size=17))
    elif case == "multiple":
        q, _ = np.linalg.qr(rng.normal(size=(12, 12)))
        a = q @ np.diag([1.0] * 4 + [0.5] * 3 + list(np.linspace(-1, 0, 5))) @ q.T
        a = (a + a.T) / 2
    elif case == "m1":
        a = np.array([[3.5]])
    elif case == "m2":
        a = np.array([[1.0, 2.0], [2.0, -1.0]])
    else:  # a zero sub-column: the reflector of that column is skipped
        a = np.diag(np.arange(8.0))
        a[5, 6] = a[6, 5] = 0.25
    w, z = _solve(shim, a)
    ew = np.linalg.eigvalsh(a)
    scale = max(1.0, np.abs(ew).max())
    m = a.shape[0]
    assert np.all(np.diff(w) >= 0)
    assert np.max(np.abs(w - ew)) <= 1e-13 * scale * max(1, m / 10)
    # orthonormal vectors with small residuals
    assert np.max(np.abs(z.T @ z - np.eye(m))) <= 1e-12 * max(1, m / 10)
    assert np.max(np.abs(a @ z - z * w)) <= 1e-12 * scale * max(1, m / 10)
