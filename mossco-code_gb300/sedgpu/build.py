"""Build recipe of the CUDA library (libsedgpu.so) for sm_103a.

Each translation unit is compiled by nvcc in parallel and linked into one
shared library under ``mossco-code_gb300/sedgpu/_build`` (git-ignored).  No
cmake: the same recipe runs on the x86 build host and on the aarch64 GPU
host.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_NAME = "libsedgpu.so"
LIB_PATH = os.path.join(BUILD_DIR, LIB_NAME)

SOURCES = ["sed_kernels_f32.cu", "sed_kernels_f64.cu", "sed_kernels_f32_bio3.cu",
           "sed_kernels_f64_bio3.cu", "sed_kernels_warp.cu", "sed_kernels_warp_bio3.cu",
           "sed_capi.cu", "sed_noalloc.cu", "sur_kernels.cu", "sur_capi.cu", "sur_loop.cu",
           "sed_kernels_warp_ens.cu", "sed_kernels_warp_ens_bio3.cu", "pel_capi.cu",
           "cpl_capi.cu", "sur_tc.cu", "sed_kernels_deep_f32.cu",
           "sed_kernels_deep_f32_bio3.cu", "sed_kernels_deep_f64_tile.cu",
           "sed_kernels_deep_f64_warp.cu", "sed_kernels_deep_f64_bio3_tile.cu",
           "sed_kernels_deep_f64_bio3_warp.cu"]
# The FP64 kernels evaluate the reference's arithmetic operation by
# operation: no multiply-add contraction.
# The FP32 kernels write every fused multiply-add explicitly (fmaf): without
# automatic contraction their rounding is the same in every kernel that
# inlines the code, so results do not depend on the launch tuning.
EXTRA_FLAGS = {"sed_kernels_f64.cu": ["-fmad=false"],
               "sed_kernels_f64_bio3.cu": ["-fmad=false"],
               "sed_kernels_f32.cu": ["-fmad=false"],
               "sed_kernels_f32_bio3.cu": ["-fmad=false"],
               "sed_kernels_warp.cu": ["-fmad=false"],
               "sed_kernels_warp_bio3.cu": ["-fmad=false"],
               "sed_kernels_warp_ens.cu": ["-fmad=false"],
               "sed_kernels_warp_ens_bio3.cu": ["-fmad=false"],
               "pel_capi.cu": ["-fmad=false"],
               "cpl_capi.cu": ["-fmad=false"],
               "sed_kernels_deep_f32.cu": ["-fmad=false"],
               "sed_kernels_deep_f32_bio3.cu": ["-fmad=false"],
               "sed_kernels_deep_f64_tile.cu": ["-fmad=false"],
               "sed_kernels_deep_f64_warp.cu": ["-fmad=false"],
               "sed_kernels_deep_f64_bio3_tile.cu": ["-fmad=false"],
               "sed_kernels_deep_f64_bio3_warp.cu": ["-fmad=false"]}
HEADERS = ["sed_device.cuh", "sed_kernels.cuh", "sed_launch.h", "sed_params.h",
           "sur_kernels.h", "sur_internal.h", "sur_loop.h", "cpl_internal.h",
           "cpl_map.cuh", "sur_tc.h", "sur_gelu.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no multiply-add contraction either (aarch64 g++ contracts by
# default), so host-side FP64 forcing rows match the CPU restatement's
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fno-strict-aliasing",
              "-Xcompiler", "-ffp-contract=off"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    files = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    files.append(os.path.join(INCLUDE, "mossco_sed.h"))
    files.append(os.path.join(INCLUDE, "mossco_pel.h"))
    files.append(os.path.join(INCLUDE, "mossco_cpl.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if needed) and return the path of libsedgpu.so."""
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    cc = nvcc()
    tag = f"{os.getpid()}"

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, src.replace(".cu", f".{tag}.o"))
        cmd = [cc, *ARCH, *NVCC_FLAGS, *EXTRA_FLAGS.get(src, []), "-I", INCLUDE, "-c",
               os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH + f".{tag}.tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    for o in objs:
        os.remove(o)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
