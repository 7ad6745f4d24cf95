"""Build the in-tree CUDA library ``libpstd_gb300.so`` for sm_103a.

Every translation unit is compiled with nvcc in parallel into
``openpstd_gb300/_build/`` and linked into ``openpstd_gb300/libpstd_gb300.so``
(both git-ignored).  Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpstd_gb300.so")
CLI = os.path.join(HERE, "pstd-cli")

SOURCES = ["scene.cpp", "stage_fused_s.cu", "stage_fused_m.cu", "stage_fused_l.cu", "stage_fused_h.cu", "stage_tma_a.cu", "stage_tma_b.cu", "stage_small.cu", "stage_mid.cu", "stage_large.cu", "stage_huge.cu", "stage_direct.cu", "stage_toeplitz.cu", "stage_all.cu", "stage_serve.cu", "misc.cu", "solver.cu", "server.cu",
           "gpu_pstd_kernel.cpp", "pstdfile.cpp"]
HEADERS = ["scene.hpp", "device.cuh", "launch.hpp", "stage_kernel.cuh", "stage_fused.cuh", "stage_tma.cuh", "stage_tc5.cuh",
           "transform_gain.hpp", "spectral_receivers.hpp", "kernel_state.hpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")


def _flags(src: str):
    f = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-lineinfo", "-I" + os.path.join(ROOT, "include")]
    if src.endswith(".cu"):
        f += ARCH + ["-Xptxas", "-v"] if os.environ.get("PSTD_PTXAS_V") else ARCH
    else:
        f += ["-x", "cu"] + ARCH if src.endswith(".cu") else []
    return f


def _compile(src: str) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    deps = [path] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "pstd_gb300.h"),
                                                                 os.path.join(ROOT, "include", "pstd_kernel.hpp")]
    newest = max(os.path.getmtime(d) for d in deps if os.path.exists(d))
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    cmd = [NVCC, "-c", path, "-o", obj + ".tmp"] + _flags(src)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and os.environ.get("PSTD_PTXAS_V"):
        sys.stderr.write(r.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(_compile, srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC, "-shared", "-o", LIB + ".tmp"] + objs + ARCH + ["-lcudart", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    # the command line (CLI/main.cpp's create / run), linked against the library
    cli_src = os.path.join(CSRC, "pstd_cli.cpp")
    hdr = os.path.join(ROOT, "include", "pstd_kernel.hpp")
    if not os.path.exists(CLI) or os.path.getmtime(CLI) < max(os.path.getmtime(LIB), os.path.getmtime(cli_src),
                                                              os.path.getmtime(hdr)):
        cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-o", CLI + ".tmp", cli_src,
               "-I" + os.path.join(ROOT, "include"), "-L" + HERE, "-lpstd_gb300", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"pstd-cli build failed:\n{r.stdout}\n{r.stderr}")
        os.replace(CLI + ".tmp", CLI)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
