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
CUDA_UNITS = ["sar_kernels.cu", "sar_api.cu", "sar_noalloc.cu", "sar_cgls.cu", "sar_unet.cu", "sar_resample.cu", "sar_cphd.cu", "sar_pdhg.cu", "sar_probe.cu"]
HEADERS = ["sar_geom.cuh", "sar_host_prep.h", "sar_kernels.cuh", "unet_tc.cuh", "sar_fft_cb.h", "sar_solver_common.cuh"]
# cuFFT load/store callbacks: compiled to LTO-IR, embedded in the library as a byte array and
# handed to cufftXtSetJITCallback at plan creation.
CALLBACK_UNIT = "sar_fft_callbacks.cu"
CALLBACK_ARCH = ["-gencode", "arch=compute_103a,code=lto_103a"]

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
    cb_src = os.path.join(CSRC, CALLBACK_UNIT)
    cb_fatbin = os.path.join(BUILD, "sar_fft_callbacks.fatbin")
    if _stale(cb_fatbin, [cb_src, os.path.join(CSRC, "sar_fft_cb.h")]):
        cmds.append([nvcc] + CALLBACK_ARCH + ["-O3", "-std=c++17", "-rdc=true", "-fatbin", "-o", cb_fatbin, cb_src])
    host_src = os.path.join(CSRC, "geom_host.cpp")
    if _stale(HOST_LIB, [host_src] + headers):
        cmds.append(["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-fno-fast-math", "-ffp-contract=off",
                     "-o", HOST_LIB, host_src])
    if cmds:
        if verbose:
            for c in cmds:
                print(" ".join(c))
        _run_parallel(cmds)
    blob_src = os.path.join(BUILD, "sar_fft_callbacks_blob.cpp")
    blob_obj = os.path.join(BUILD, "sar_fft_callbacks_blob.o")
    if _stale(blob_obj, [cb_fatbin]):
        data = open(cb_fatbin, "rb").read()
        body = ",".join(str(b) for b in data)
        with open(blob_src, "w") as f:
            f.write("#include <cstddef>\n"
                    f"extern \"C\" const unsigned char sar_fft_cb_fatbin[{len(data)}] = {{{body}}};\n"
                    f"extern \"C\" const size_t sar_fft_cb_fatbin_size = {len(data)};\n")
        _run_parallel([["g++", "-O1", "-fPIC", "-c", blob_src, "-o", blob_obj]])
    objs.append(blob_obj)
    if _stale(GPU_LIB, objs):
        _run_parallel([[nvcc] + ARCH + ["-shared", "-o", GPU_LIB] + objs +
                       ["-cudart", "shared", "-lcufft", "-lnvJitLink"]])
    return {"gpu": GPU_LIB, "host": HOST_LIB}


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
