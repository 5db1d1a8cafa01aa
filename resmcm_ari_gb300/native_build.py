"""Build recipe for the native parts (nvcc + g++, no cmake).

Outputs, all under ``resmcm_ari_gb300/_build/``:

* ``libresmcm_gpu.so`` — the C-ABI library (``include/resmcm_gpu.h``): CUDA
  kernels for sm_103a plus the host executor;
* ``resmcm_gpu`` — the command-line drop-in for the reference ``resmcm``.

Every translation unit is compiled in parallel; a unit is rebuilt when its
source, a header or the flags changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import json
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libresmcm_gpu.so")
CLI = os.path.join(BUILD, "resmcm_gpu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc") if os.path.exists(os.path.join(CUDA_HOME, "bin", "nvcc")) else "nvcc"
CU_SOURCES = ["spgemm.cu", "estimator.cu", "chain_dp.cu", "dense_gemm.cu", "tc_gemm.cu", "batch_fused.cu"]
CPP_SOURCES = ["api.cpp", "server.cpp"]
HEADERS = ["internal.h"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
                     "-I" + INCLUDE, "-I" + CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-fopenmp", "-I" + INCLUDE, "-I" + CSRC,
             "-I" + os.path.join(CUDA_HOME, "include")]


def _digest(paths, flags) -> str:
    h = hashlib.sha256(" ".join(flags).encode())
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def _stamp_ok(obj: str, digest: str) -> bool:
    stamp = obj + ".stamp"
    return os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == digest


def _compile(src: str, verbose: bool) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    deps = [path, os.path.join(INCLUDE, "resmcm_gpu.h")] + [os.path.join(CSRC, h) for h in HEADERS]
    if src.endswith(".cu"):
        cmd = [NVCC] + NVCC_FLAGS + ["-c", path, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-c", path, "-o", obj]
    digest = _digest(deps, cmd)
    if _stamp_ok(obj, digest):
        return obj
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    with open(obj + ".stamp", "w") as f:
        f.write(digest)
    return obj


def build(verbose: bool = False) -> str:
    """Compile every translation unit for sm_103a and link the library + CLI."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = CU_SOURCES + CPP_SOURCES
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    link = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lgomp", "-lpthread"]
    link_digest = _digest(objs, link)
    if not _stamp_ok(LIB, link_digest):
        if verbose:
            print(" ".join(link), flush=True)
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
        with open(LIB + ".stamp", "w") as f:
            f.write(link_digest)
    cli_src = os.path.join(CSRC, "cli.cpp")
    cli_cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-I" + INCLUDE, cli_src, "-o", CLI, "-L" + BUILD,
               "-lresmcm_gpu", "-Wl,-rpath,$ORIGIN"]
    cli_digest = _digest([cli_src, os.path.join(INCLUDE, "resmcm_gpu.h"), LIB], cli_cmd)
    if not _stamp_ok(CLI, cli_digest):
        r = subprocess.run(cli_cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed\n{r.stdout}\n{r.stderr}")
        with open(CLI + ".stamp", "w") as f:
            f.write(cli_digest)
    return LIB


def ptxas_report() -> str:
    """Registers / spills / shared memory of every kernel (``-Xptxas -v``)."""
    out = []
    for src in CU_SOURCES:
        cmd = [NVCC] + NVCC_FLAGS + ["-Xptxas", "-v", "-c", os.path.join(CSRC, src), "-o", os.devnull]
        r = subprocess.run(cmd, capture_output=True, text=True)
        out.append(r.stderr)
    return "\n".join(out)


if __name__ == "__main__":
    print(build(verbose=True))
