"""In-tree build of the native libraries (no cmake, no pip install).

    python -m sarsolver_gb300.build

produces
    _build/libsargpu.so        CUDA kernels + C ABI (include/sargpu.h), sm_103a only
    _build/libsargeom_host.so  host build of the kernels' range geometry (precision checks)

Translation units compile in parallel; outputs are rebuilt only when a source is newer.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-fast-math"]
CUDA_UNITS = ["sar_kernels.cu", "sar_api.cu", "sar_noalloc.cu", "sar_cgls.cu", "sar_unet.cu"]
HEADERS = ["sar_geom.cuh", "sar_host_prep.h", "sar_kernels.cuh", "unet_tc.cuh"]

GPU_LIB = os.path.join(BUILD, "libsargpu.so")
HOST_LIB = os.path.join(BUILD, "libsargeom_host.so")


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale(target: str, sources) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _run_parallel(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for c in cmds]
    errors = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(" ".join(c) + "\n" + out)
    if errors:
        raise RuntimeError("native build failed:\n" + "\n".join(errors))


def build(verbose: bool = False) -> dict:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "sargpu.h")]
    nvcc = _nvcc()
    objs, cmds = [], []
    for unit in CUDA_UNITS:
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
        objs.append(obj)
        if _stale(obj, [src] + headers):
            cmds.append([nvcc] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj])
    host_src = os.path.join(CSRC, "geom_host.cpp")
    if _stale(HOST_LIB, [host_src] + headers):
        cmds.append(["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-fno-fast-math", "-ffp-contract=off",
                     "-o", HOST_LIB, host_src])
    if cmds:
        if verbose:
            for c in cmds:
                print(" ".join(c))
        _run_parallel(cmds)
    if _stale(GPU_LIB, objs):
        _run_parallel([[nvcc] + ARCH + ["-shared", "-o", GPU_LIB] + objs + ["-cudart", "shared", "-lcufft"]])
    return {"gpu": GPU_LIB, "host": HOST_LIB}


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
