"""Builds the sm_103a C-ABI library `libdenrim_cuda.so` in-tree with nvcc.

The library is plain CUDA C++ (no PyTorch types): `csrc/dk_kernels.cu` holds
the kernels, `csrc/dk_host.cu` the C ABI of include/denrim_cuda.h.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB_PATH = os.path.join(OUT_DIR, "libdenrim_cuda.so")
SOURCES = ("dk_kernels.cu", "dk_host.cu", "dk_bvh.cu", "dk_sdf.cu", "dk_noalloc.cu", "dk_server.cu", "dk_denoise.cu", "dk_unet.cu", "dk_image.cu", "dk_svgf.cu", "dk_probe.cu")
ARCH = ("-gencode", "arch=compute_103a,code=sm_103a")


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the sm_103a library cannot be built")


def _newest_input() -> float:
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    paths.append(os.path.join(HERE, "..", "include", "denrim_cuda.h"))
    return max(os.path.getmtime(p) for p in paths)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles the library if any source is newer than it; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= _newest_input():
        return LIB_PATH
    cc = nvcc()
    # Host code without FMA contraction: the host builders restate the
    # reference's arithmetic operation by operation, like the oracle.
    flags = [*ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-pthread",
             "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]
    # Tuning knobs, e.g. DK_NVCC_DEFINES="DK_SHADE_MIN_BLOCKS=6 DK_LAYERS_MIN_BLOCKS=4".
    flags += [f"-D{d}" for d in os.environ.get("DK_NVCC_DEFINES", "").split()]

    def compile_one(src: str) -> str:
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [cc, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
        if verbose:
            sys.stderr.write(res.stderr)
        return obj

    with ThreadPoolExecutor(len(SOURCES)) as pool:
        objs = list(pool.map(compile_one, SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-Xcompiler", "-pthread", *objs, "-o", tmp]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
