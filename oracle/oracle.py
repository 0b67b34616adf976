"""Test infrastructure: ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may import
this module.  It restates the reference algorithm on the CPU; it is the checker,
never the thing measured or shipped.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

# Counter slots of pathtrace_oracle.cpp (query kinds: 0 extension, 1 shadow,
# 2 subsurface walk, 3 AOV).
COUNTERS = ("paths", "material_fetch", "light_samples", "env_samples", "env_search_steps", "miss_env",
            "shadow_queries", "bounces", "env_lookups", "queries_ext", "queries_shadow", "queries_sss",
            "queries_aov", "nodes_ext", "nodes_shadow", "nodes_sss", "nodes_aov", "tris_ext", "tris_shadow",
            "tris_sss", "tris_aov", "grid_cells", "macro_skips", "brick_tests", "brick_marches", "march_steps",
            "brick_hits", "brick_samples", "range_culls")

_lib = None


def build() -> str:
    res = subprocess.run(["make", "-C", HERE, "-j3"], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stdout + res.stderr)
    return LIB


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        lib = C.CDLL(LIB)
        P, u32 = C.c_void_p, C.c_uint32
        for prefix in ("oracle32_", "oracle64_"):
            getattr(lib, prefix + "render").argtypes = [P, P, u32, u32, P, u32, C.c_int, P, P, P]
            getattr(lib, prefix + "render").restype = C.c_int
            getattr(lib, prefix + "intersect").argtypes = [P, P, P, P]
            getattr(lib, prefix + "hash").argtypes = [u32]
            getattr(lib, prefix + "hash").restype = u32
            getattr(lib, prefix + "random_sequence").argtypes = [u32, u32, P]
            getattr(lib, prefix + "counter_count").restype = u32
        lib.oracle_build_bvh.argtypes = [P, u32, u32, P, P]
        lib.oracle_build_bvh.restype = u32
        lib.oracle_build_lights.argtypes = [P, u32, P, u32, P]
        lib.oracle_build_lights.restype = u32
        lib.oracle_build_environment_samples.argtypes = [P, u32, u32, C.c_float, C.c_float, P]
        lib.oracle_build_environment_samples.restype = u32
        assert lib.oracle32_counter_count() == len(COUNTERS)
        _lib = lib
    return _lib


def build_bvh(triangles: np.ndarray, max_leaf: int = 4):
    from denrimrendererkit_gb300 import abi
    n = len(triangles)
    nodes = np.zeros(max(2 * n, 1), abi.NODE_DTYPE)
    prim = np.zeros(max(n, 1), np.uint32)
    tris = np.ascontiguousarray(triangles)
    count = load().oracle_build_bvh(tris.ctypes.data, n, max_leaf, nodes.ctypes.data, prim.ctypes.data)
    return nodes[:count].copy(), prim[:n].copy()


def build_lights(triangles: np.ndarray, materials: np.ndarray):
    """Returns (tagged triangle copy, light records)."""
    from denrimrendererkit_gb300 import abi
    tris = np.ascontiguousarray(triangles).copy()
    lights = np.zeros(max(len(tris), 1), abi.LIGHT_DTYPE)
    mats = np.ascontiguousarray(materials)
    n = load().oracle_build_lights(tris.ctypes.data, len(tris), mats.ctypes.data, len(mats), lights.ctypes.data)
    return tris, lights[:n].copy()


def build_environment_samples(pixels: np.ndarray, width: int, height: int, intensity: float, max_radiance: float):
    from denrimrendererkit_gb300 import abi
    px = np.ascontiguousarray(np.asarray(pixels, np.float32).reshape(-1, 4))
    out = np.zeros(max(width * height, 1), abi.ENVIRONMENT_SAMPLE_DTYPE)
    n = load().oracle_build_environment_samples(px.ctypes.data, width, height, intensity, max_radiance,
                                                out.ctypes.data)
    return out[:n].copy()


class HostBuilders:
    """compile_scene(host_builders=...) hook: the restatements of the Swift
    builders (BVHBuilder + BVHFlattener, lightRecordsAndTaggedTriangles,
    environmentSamples) in place of the GB300 library's."""

    @staticmethod
    def build_bvh(triangles, max_leaf=4):
        return build_bvh(triangles, max_leaf)

    @staticmethod
    def build_lights(triangles, materials):
        tagged, lights = build_lights(triangles, materials)
        triangles["padding2"] = tagged["padding2"]
        return lights

    @staticmethod
    def build_environment_samples(texture, intensity, max_radiance):
        return build_environment_samples(texture.pixels, texture.width, texture.height, intensity, max_radiance)


def make_params(settings, camera, tile=None):
    """oracle_params from RenderSettings + Camera (GPURenderConstants fields)."""
    from denrimrendererkit_gb300 import abi
    p = abi.OracleParams()
    p.width, p.height = settings.width, settings.height
    p.max_bounces = max(1, settings.max_bounces)
    p.transparent_background = int(settings.transparent_background)
    p.shows_environment_background = int(settings.shows_environment_background)
    for i in range(3):
        p.background_color[i] = float(settings.background_color[i])
    p.sample_radiance_clamp = settings.resolved_sample_radiance_clamp
    p.frame_seed = settings.frame_seed & 0xFFFFFFFF
    from denrimrendererkit_gb300.renderer import aov_ray_enabled
    p.denoiser_enabled = aov_ray_enabled(settings.denoise)
    tx, ty, tw, th = tile or (0, 0, settings.width, settings.height)
    p.tile_x, p.tile_y, p.tile_w, p.tile_h = tx, ty, tw, th
    p.camera = camera.gpu_camera(settings.width, settings.height)
    p.previous_camera = (settings.previous_camera or camera).gpu_camera(settings.width, settings.height)
    return p


class OracleRender:
    """Running-mean accumulation + last-sample AOVs of the CPU oracle."""

    def __init__(self, build, settings, camera, fp64: bool = False, tile=None):
        self.build = build
        self.settings = settings
        self.params = make_params(settings, camera, tile)
        self.scene_struct = build.as_struct()
        self.prefix = "oracle64_" if fp64 else "oracle32_"
        w, h = settings.width, settings.height
        self.accum = np.zeros((h, w, 4), np.float64)
        self.aov = np.zeros((6, h, w, 4), np.float32)
        self.aov[1, ..., :3] = 0.5
        self.counters = np.zeros(len(COUNTERS), np.uint64)
        self.sample_count = 0

    def render(self, samples: int, pixel_list=None, threads: int = 0) -> None:
        fn = getattr(load(), self.prefix + "render")
        pl = None if pixel_list is None else np.ascontiguousarray(pixel_list, np.uint32)
        rc = fn(C.byref(self.scene_struct), C.byref(self.params), self.sample_count, samples,
                None if pl is None else pl.ctypes.data, 0 if pl is None else len(pl), threads,
                self.accum.ctypes.data, self.aov.ctypes.data, self.counters.ctypes.data)
        if rc != 0:
            raise RuntimeError(f"oracle render failed with {rc}")
        self.sample_count += samples

    def counter_dict(self):
        return {k: int(v) for k, v in zip(COUNTERS, self.counters)}


def intersect(build, origin, direction, fp64: bool = False):
    s = build.as_struct()
    o = np.asarray(origin, np.float32)
    d = np.asarray(direction, np.float32)
    out = np.zeros(14, np.float64)
    getattr(load(), ("oracle64_" if fp64 else "oracle32_") + "intersect")(
        C.byref(s), o.ctypes.data, d.ctypes.data, out.ctypes.data)
    keys = ("hit", "t", "px", "py", "pz", "nx", "ny", "nz", "u", "v", "material_id", "object_id", "primitive_id",
            "front_facing")
    return dict(zip(keys, out.tolist()))


def random_sequence(state: int, n: int, fp64: bool = False):
    out = np.zeros(n, np.float64)
    getattr(load(), ("oracle64_" if fp64 else "oracle32_") + "random_sequence")(state, n, out.ctypes.data)
    return out


def hash_u32(v: int) -> int:
    return load().oracle32_hash(v)


# ------------------------------------------------ reference-shader oracle ---
# oracle/_ref/libref_pathtrace.so: the reference's own PathTrace.metal compiled
# as C++ (oracle/ref/build_ref.py).  Present only where it could be built.
REF_LIB = os.path.join(HERE, "_ref", "libref_pathtrace.so")
REF_SDF_COUNTERS = ("dense_volume_tests", "dense_march_steps", "grid_cells", "macro_skips", "brick_tests",
                    "brick_invalid", "range_culls", "brick_marches", "march_steps", "brick_hits",
                    "primary_queries", "bounce_queries", "shadow_queries")
_ref_lib = None


def reference_available() -> bool:
    return os.path.exists(REF_LIB) or os.path.exists(os.path.join(HERE, "_ref", "pathtrace_ref.cpp"))


def load_reference() -> C.CDLL:
    global _ref_lib
    if _ref_lib is None:
        import importlib.util
        spec = importlib.util.spec_from_file_location("build_ref", os.path.join(HERE, "ref", "build_ref.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
        lib = C.CDLL(REF_LIB)
        P, u32 = C.c_void_p, C.c_uint32
        lib.ref_render.argtypes = [P, P, u32, u32, P, u32, C.c_int, P, P, P]
        lib.ref_render.restype = C.c_int
        lib.ref_render_quality.argtypes = [C.c_int, P, P, u32, u32, P, u32, C.c_int, P, P, P]
        lib.ref_render_quality.restype = C.c_int
        lib.ref_sdf_counter_count.restype = u32
        assert lib.ref_sdf_counter_count() == len(REF_SDF_COUNTERS)
        _ref_lib = lib
    return _ref_lib


class ReferenceRender:
    """The reference kernel for the settings' quality (pathTraceKernel,
    flatPreviewKernel or interactiveMaterialKernel) run on the host: RGBA32F
    accumulation texture and last-sample AOV planes, exactly as the kernel
    writes them."""

    def __init__(self, build, settings, camera, tile=None, collect_sdf_counters: bool = False):
        self.build = build
        self.settings = settings
        self.params = make_params(settings, camera, tile)
        self.scene_struct = build.as_struct()
        w, h = settings.width, settings.height
        self.accum = np.zeros((h, w, 4), np.float32)
        self.aov = np.zeros((6, h, w, 4), np.float32)
        self.aov[1, ..., :3] = 0.5
        self.sdf_counters = np.zeros(len(REF_SDF_COUNTERS), np.uint32) if collect_sdf_counters else None
        self.sample_count = 0

    def render(self, samples: int, pixel_list=None, threads: int = 0) -> None:
        pl = None if pixel_list is None else np.ascontiguousarray(pixel_list, np.uint32)
        rc = load_reference().ref_render_quality(
            int(self.settings.quality), C.byref(self.scene_struct), C.byref(self.params), self.sample_count, samples,
            None if pl is None else pl.ctypes.data, 0 if pl is None else len(pl), threads,
            self.accum.ctypes.data, self.aov.ctypes.data,
            None if self.sdf_counters is None else self.sdf_counters.ctypes.data)
        if rc != 0:
            raise RuntimeError(f"reference render failed with {rc}")
        self.sample_count += samples

    def sdf_counter_dict(self):
        return {k: int(v) for k, v in zip(REF_SDF_COUNTERS, self.sdf_counters)}
