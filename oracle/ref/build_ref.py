"""Test infrastructure: builds the reference-shader oracle.

Where the reference sources are present, rewrites the reference's own
PathTrace.metal and Denoise.metal into C++ (metal2cpp.py) under oracle/_ref/;
then, wherever those generated files exist (it travels with the repository copy to machines without
the reference), compiles it with the host driver into
oracle/_ref/libref_pathtrace.so.  Outputs go to oracle/_ref/ only.

The FP32 build uses the same IEEE discipline as the CPU restatement
(-ffp-contract=off -fno-fast-math).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
# The reference checkout: DENRIM_REFERENCE, else its location in the build container.
REFERENCE = os.environ.get("DENRIM_REFERENCE", "/root/reference")
SHADERS = os.path.join(REFERENCE, "Sources", "DenrimRendererKit", "Resources", "Shaders")
# (reference shader, kernels kept, generated file)
UNITS = (("PathTrace.metal", ("pathTraceKernel", "flatPreviewKernel", "interactiveMaterialKernel"), "pathtrace_ref.cpp"),
         ("Denoise.metal", ("simpleSpatialDenoiseKernel", "packSVGFDepthNormalKernel", "copySVGFOutputKernel"),
          "denoise_ref.cpp"))
GENERATED = os.path.join(OUT, "pathtrace_ref.cpp")
LIB = os.path.join(OUT, "libref_pathtrace.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    for shader, kernels, name in UNITS:
        path = os.path.join(SHADERS, shader)
        out = os.path.join(OUT, name)
        if os.path.exists(path):
            sys.path.insert(0, HERE)
            import metal2cpp
            text = metal2cpp.convert(path, kernels)
            old = open(out).read() if os.path.exists(out) else None
            if old != text:
                with open(out, "w") as f:
                    f.write(text)
        if not os.path.exists(out):
            raise FileNotFoundError(f"reference shader {shader} not available and no generated copy in oracle/_ref")
    deps = [os.path.join(OUT, name) for _, _, name in UNITS] + [
        os.path.join(HERE, f) for f in ("ref_driver.cpp", "ref_denoise.cpp", "metal_shim.hpp")] + [
        os.path.join(ORACLE, "oracle_params.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["g++", "-O2", "-std=c++20", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-fno-fast-math",
           "-Wno-attributes", "-I", HERE, "-I", OUT, os.path.join(HERE, "ref_driver.cpp"),
           os.path.join(HERE, "ref_denoise.cpp"), "-o", LIB + ".tmp"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference-shader oracle build failed:\n" + res.stderr[-4000:])
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
