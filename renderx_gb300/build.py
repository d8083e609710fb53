"""Builds librenderx_gb300.so from renderx_gb300/csrc for sm_103a.

Each CUDA translation unit is compiled by nvcc with
``-gencode arch=compute_103a,code=sm_103a -lineinfo``, host C++ by g++, in parallel;
objects go to renderx_gb300/_build/, the library beside this file. No fast-math: the
closest-hit arithmetic must stay IEEE round-to-nearest.

    python -m renderx_gb300.build [--verbose-ptxas]
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librenderx_gb300.so")
CLI = os.path.join(HERE, "rx_render")  # command-line renderer over the library (cli/rx_render.cpp)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _compile(src: str, ptxas_verbose: bool) -> tuple[str, str]:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if src.endswith(".cu"):
        cmd = [_nvcc(), "-std=c++17", "-O3", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC,-O3",
               "-I", os.path.join(HERE, "..", "include"), "-c", src, "-o", obj]
        if ptxas_verbose:
            cmd[3:3] = ["-Xptxas", "-v"]
    else:
        cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-pthread", "-ffp-contract=off", "-I", "/usr/local/cuda/include",
               "-I", os.path.join(HERE, "..", "include"), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(HERE, "..", "include", "*.h"))
    deps += glob.glob(os.path.join(HERE, "cli", "*"))
    return not os.path.exists(CLI) or any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, ptxas_verbose: bool = False, quiet: bool = True) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, ptxas_verbose), srcs))
    objs = [o for o, _ in results]
    if not quiet or ptxas_verbose:
        for _, log in results:
            if log.strip():
                print(log, file=sys.stderr)
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), "-shared", *ARCH, "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(HERE, "..", "include"), os.path.join(HERE, "cli", "rx_render.cpp"),
           "-o", CLI + ".tmp", "-L", HERE, "-lrenderx_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"cli build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(CLI + ".tmp", CLI)
    return LIB


if __name__ == "__main__":
    print(build(force=True, ptxas_verbose="--verbose-ptxas" in sys.argv, quiet=False))
