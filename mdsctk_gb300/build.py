"""Build recipe of libmdsgpu (CUDA kernels + C ABI) and the drop-in tools.

Every translation unit is compiled by nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, into
``mdsctk_gb300/_build``; the shared library goes to ``mdsctk_gb300/lib``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libmdsgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-Wall", "--expt-relaxed-constexpr",
           "-I" + os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(ROOT, "include", "mdsgpu.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [_nvcc()] + ARCH + NVFLAGS + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    extra = extra or []
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), sources()))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    build_tools()
    if verbose:
        print("built", LIB)
    return LIB


TOOLS = ("knn_rms", "knn_data", "knn_data_sparse", "contact_profile", "make_sysparse", "make_gesparse",
         "decomp_sparse", "decomp_sparse_nystrom", "auto_decomp_sparse", "auto_decomp_sparse_nystrom")
BINDIR = os.path.join(HERE, "bin")


def build_tools() -> None:
    """The drop-in command-line tools: C++ mains linked against libmdsgpu."""
    os.makedirs(BINDIR, exist_ok=True)
    tdir = os.path.join(CSRC, "tools")
    headers = [os.path.join(tdir, f) for f in os.listdir(tdir) if f.endswith(".h")]
    cxx = shutil.which("g++") or "g++"

    def one(name):
        src = os.path.join(tdir, name + ".cpp")
        out = os.path.join(BINDIR, name)
        deps = [src, LIB] + headers
        if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
            return
        cmd = [cxx, "-O2", "-std=c++17", "-Wall", src, "-o", out, "-L" + LIBDIR, "-lmdsgpu",
               "-Wl,-rpath,$ORIGIN/../lib"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"tool build failed for {name}:\n{r.stdout}\n{r.stderr}")

    with cf.ThreadPoolExecutor(max_workers=len(TOOLS)) as ex:
        list(ex.map(one, TOOLS))


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
