"""Build recipe for libbitruss.so and the ``coh`` front end.

Compiles every CUDA source for sm_103a (GB300) only, in parallel, into
``gpu_bitruss_gb300/_build/`` and links ``gpu_bitruss_gb300/libbitruss.so``
(CUDA runtime linked statically) and ``gpu_bitruss_gb300/coh``.  Host code is
portable C++ (no architecture flags), so the same recipe builds on x86_64 and
aarch64 hosts.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libbitruss.so")
COH = os.path.join(PKG, "coh")

CUDA_SOURCES = ["bt_ctx.cu", "bt_count.cu", "bt_msp.cu", "bt_hidx.cu", "bt_noalloc.cu"]
CXX_SOURCES = ["bt_graph.cpp", "bt_batch.cpp", "bt_server.cpp"]
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(home, "bin", "nvcc")
    return path if os.path.exists(path) else (shutil.which("nvcc") or "nvcc")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False) -> str:
    """Compile (if stale) and return the path of libbitruss.so."""
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers += [os.path.join(PKG, "..", "include", "bitruss.h"),
                os.path.join(PKG, "..", "include", "bitruss.hpp")]
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append([nvcc(), GENCODE, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                         "-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp",
                         "-I", os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include"),
                         "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for j in jobs:
            if verbose:
                print(" ".join(j))
        list(ex.map(_run, jobs))
    if _stale(LIB, objs):
        _run([nvcc(), GENCODE, "-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"])
    coh_src = os.path.join(CSRC, "coh.cpp")
    coh_obj = os.path.join(BUILD, "coh.cpp.o")
    if _stale(coh_obj, [coh_src] + headers):
        _run(["g++", "-O3", "-std=c++17",
              "-I", os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include"),
              "-c", coh_src, "-o", coh_obj])
    if _stale(COH, [coh_obj, LIB]):
        _run([nvcc(), GENCODE, "-o", COH, coh_obj, "-L", PKG, "-lbitruss",
              "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
