"""ctypes binding of the in-tree sm_103a library (include/denrim_cuda.h).

The library is the only compute path: there is no CPU fallback.  Loading fails
loudly when the shared object is missing (run `__graft_entry__.build()` or
`python -m denrimrendererkit_gb300.build`).
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from typing import Tuple

import numpy as np

from . import abi

_LIB = None
_LOCK = threading.Lock()


class DenrimError(RuntimeError):
    """A non-zero dk_status.  `code` maps onto DenrimRendererError
    (Sources/DenrimRendererKit/Renderer/DenrimRenderer.swift:5-26)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{abi.STATUS_NAMES.get(code, code)}: {message}")
        self.code = code


def lib_path() -> str:
    from .build import LIB_PATH
    return LIB_PATH


def load(build_if_missing: bool = False) -> C.CDLL:
    """Loads libdenrim_cuda.so and declares every exported signature."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = lib_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(
                    f"{path} is missing: the sm_103a library must be built first "
                    "(python -m denrimrendererkit_gb300.build); there is no CPU fallback")
            from .build import build
            build()
        lib = C.CDLL(path)
        P = C.c_void_p
        u32, i32, sz = C.c_uint32, C.c_int, C.c_size_t
        sig = {
            "dk_device_open": (i32, [i32]),
            "dk_device_count": (i32, [C.POINTER(i32)]),
            "dk_session_create": (i32, [C.POINTER(abi.Scene), C.POINTER(abi.Settings), C.POINTER(P)]),
            "dk_session_render": (i32, [P, u32]),
            "dk_session_render_tile": (i32, [P, u32, u32, u32, u32, i32]),
            "dk_session_update_camera": (i32, [P, C.POINTER(abi.Camera), C.POINTER(abi.Camera)]),
            "dk_session_reset": (i32, [P]),
            "dk_session_read_output": (i32, [P, i32, P, sz]),
            "dk_session_read_rgba8": (i32, [P, i32, P, sz]),
            "dk_session_copy_output": (i32, [P, i32, P, sz, P]),
            "dk_session_write_png": (i32, [P, i32, C.c_char_p]),
            "dk_encode_rgba8": (i32, [P, u32, u32, i32, P, P, P]),
            "dk_write_png": (i32, [C.c_char_p, P, u32, u32]),
            "dk_session_sample_count": (i32, [P, C.POINTER(u32)]),
            "dk_session_stats": (i32, [P, C.POINTER(abi.Stats)]),
            "dk_session_reset_sdf_stats": (i32, [P]),
            "dk_session_destroy": (i32, [P]),
            "dk_last_error_message": (C.c_char_p, []),
            "dk_build_bvh": (i32, [P, u32, u32, P, C.POINTER(u32), P]),
            "dk_build_lights": (i32, [P, u32, P, u32, P, C.POINTER(u32)]),
            "dk_build_environment_samples": (i32, [P, u32, u32, C.c_float, C.c_float, P, C.POINTER(u32)]),
            "dk_build_environment_samples_noalloc": (i32, [P, u32, u32, C.c_float, C.c_float, P,
                                                             C.POINTER(u32), P]),
            "dk_build_sparse_sphere_volume": (i32, [P, u32, C.POINTER(abi.SparseVolumeSettings), C.POINTER(P)]),
            "dk_bake_sparse_sphere_volume": (i32, [P, u32, C.POINTER(abi.SparseVolumeSettings), C.POINTER(P)]),
            "dk_sparse_volume_view": (i32, [P, C.POINTER(abi.Scene)]),
            "dk_sparse_volume_destroy": (i32, [P]),
            "dk_version": (C.c_char_p, []),
            "dk_probe_bandwidth": (i32, [C.c_uint64, u32, C.POINTER(C.c_double), P]),
            "dk_server_create": (i32, [C.POINTER(abi.Scene), C.POINTER(abi.ServerConfig), C.POINTER(P)]),
            "dk_server_add_scene": (i32, [P, C.POINTER(abi.Scene), C.POINTER(u32)]),
            "dk_server_submit": (i32, [P, C.POINTER(abi.JobDesc), C.POINTER(C.c_uint64)]),
            "dk_server_step": (i32, [P, C.POINTER(u32)]),
            "dk_server_start": (i32, [P]),
            "dk_server_stop": (i32, [P]),
            "dk_server_wait": (i32, [P, C.c_uint64, u32]),
            "dk_server_job_status": (i32, [P, C.c_uint64, C.POINTER(abi.JobStatus)]),
            "dk_server_read_output": (i32, [P, C.c_uint64, i32, P, sz]),
            "dk_server_copy_output": (i32, [P, C.c_uint64, i32, P, sz, P]),
            "dk_server_copy_outputs": (i32, [P, P, sz, i32, P, sz, sz, P]),
            "dk_server_release": (i32, [P, C.c_uint64]),
            "dk_server_get_stats": (i32, [P, C.POINTER(abi.ServerStats)]),
            "dk_server_destroy": (i32, [P]),
            "dk_denoise_spatial": (i32, [P, P, P, P, P, P, u32, u32, C.POINTER(abi.SpatialDenoiseSettings), P]),
            "dk_denoise_error_terms": (i32, [P, P, P, P, P, P, u32, u32, u32, P, P]),
            "dk_average_planes": (i32, [P, P, P, sz, C.c_float, P]),
            "dk_svgf_create": (i32, [u32, u32, P]),
            "dk_svgf_reset": (i32, [P]),
            "dk_svgf_denoise": (i32, [P, P, P, P, P, P, C.POINTER(abi.SpatialDenoiseSettings), P]),
            "dk_svgf_read_state": (i32, [P, i32, P, sz, P]),
            "dk_svgf_destroy": (i32, [P]),
            "dk_svgf_pack_depth_normal": (i32, [P, P, P, u32, u32, P]),
            "dk_svgf_copy_output": (i32, [P, P, P, u32, u32, P]),
            "dk_unet_conv3x3": (i32, [P, u32, u32, u32, u32, u32, P, P, u32, P, u32, u32, i32, i32, P]),
            "dk_unet_conv3x3_avgpool2": (i32, [P, u32, u32, u32, u32, u32, P, P, u32, P, u32, u32, i32, P, u32, P]),
            "dk_unet_conv3x3_wgrad": (i32, [P, u32, P, u32, u32, u32, u32, u32, u32, P, P]),
            "dk_unet_relu_backward": (i32, [P, u32, P, u32, P, u32, u32, u32, P]),
            "dk_unet_bias_grad": (i32, [P, u32, u32, u32, P, P]),
            "dk_unet_avgpool2": (i32, [P, u32, P, u32, u32, u32, u32, u32, u32, P]),
            "dk_unet_avgpool2_backward": (i32, [P, u32, P, u32, u32, u32, u32, u32, i32, P]),
            "dk_unet_upsample2": (i32, [P, u32, P, u32, u32, u32, u32, u32, u32, P]),
            "dk_unet_upsample2_backward": (i32, [P, u32, u32, P, u32, u32, u32, u32, u32, P]),
            "dk_unet_copy_channels": (i32, [P, u32, u32, P, u32, u32, u32, u32, i32, P]),
            "dk_unet_pack_input": (i32, [P, P, P, P, u32, u32, u32, u32, P, u32, u32, u32, P]),
            "dk_unet_l1_loss": (i32, [P, u32, P, u32, P, u32, P, P]),
            "dk_unet_unpack_output": (i32, [P, u32, u32, u32, P, u32, u32, u32, u32, P, P]),
            "dk_unet_l1_loss_residual": (i32, [P, u32, P, u32, P, u32, P, u32, P, P]),
            "dk_unet_unpack_output_residual": (i32, [P, u32, P, u32, u32, u32, P, u32, u32, u32, u32, P, P]),
            "dk_unet_adam": (i32, [P, P, P, P, u32, C.c_float, C.c_float, C.c_float, C.c_float, u32, P, P, u32, u32,
                                   P]),
            "dk_unet_weights_to_bf16": (i32, [P, u32, P, P, u32, u32, P]),
            "dk_unet_set_conv_path": (i32, [i32]),
            "dk_unet_error": (i32, [C.POINTER(i32)]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
        return lib


def check(rc: int) -> None:
    if rc != 0:
        msg = load().dk_last_error_message()
        raise DenrimError(rc, msg.decode() if msg else "")


def device_count() -> int:
    n = C.c_int(0)
    check(load().dk_device_count(C.byref(n)))
    return n.value


def build_bvh(triangles: np.ndarray, max_leaf: int = 4) -> Tuple[np.ndarray, np.ndarray]:
    """dk_build_bvh: BVHBuilder + BVHFlattener (BVHBuilder.swift, FlatBVH.swift)."""
    n = len(triangles)
    if n == 0:
        return np.zeros(0, abi.NODE_DTYPE), np.zeros(0, np.uint32)
    tris = np.ascontiguousarray(triangles)
    nodes = np.zeros(2 * n, abi.NODE_DTYPE)
    prim = np.zeros(n, np.uint32)
    count = C.c_uint32(0)
    check(load().dk_build_bvh(tris.ctypes.data, n, max_leaf, nodes.ctypes.data, C.byref(count), prim.ctypes.data))
    return nodes[: count.value].copy(), prim


def build_lights(triangles: np.ndarray, materials: np.ndarray) -> np.ndarray:
    """dk_build_lights: emissive-triangle records; tags `triangles` in place."""
    n = len(triangles)
    lights = np.zeros(max(n, 1), abi.LIGHT_DTYPE)
    count = C.c_uint32(0)
    if n == 0 or len(materials) == 0:
        return lights[:0].copy()
    assert triangles.flags["C_CONTIGUOUS"] and materials.flags["C_CONTIGUOUS"]
    check(load().dk_build_lights(triangles.ctypes.data, n, materials.ctypes.data, len(materials),
                                 lights.ctypes.data, C.byref(count)))
    return lights[: count.value].copy()


def build_environment_samples(texture, intensity: float, max_radiance: float) -> np.ndarray:
    """dk_build_environment_samples: the HDRI importance table (FP64 prefix sum on the GPU)."""
    px = np.ascontiguousarray(np.asarray(texture.pixels, np.float32).reshape(-1, 4))
    n = texture.width * texture.height
    out = np.zeros(max(n, 1), abi.ENVIRONMENT_SAMPLE_DTYPE)
    count = C.c_uint32(0)
    check(load().dk_build_environment_samples(px.ctypes.data, texture.width, texture.height, float(intensity),
                                              float(max_radiance), out.ctypes.data, C.byref(count)))
    return out[: count.value].copy()


class _VolumeHandle:
    """Owns a dk_sparse_volume; destroyed when the last array viewing it goes."""

    def __init__(self, handle: C.c_void_p):
        self.handle = handle

    def __del__(self):
        try:
            if self.handle:
                load().dk_sparse_volume_destroy(self.handle)
                self.handle = C.c_void_p()
        except Exception:
            pass


class SparseVolume:
    """A sparse distance volume built by dk_bake_sparse_sphere_volume on the GPU
    (`on_device` None: when a CUDA device is present) or by the host build
    dk_build_sparse_sphere_volume (the two are bit-identical); the arrays are
    numpy views of the library-owned buffers, each of which keeps them alive.
    `fp16_distances` stores every sample distance rounded to half precision
    (the renderer then marches over 2-byte samples)."""

    def __init__(self, spheres, resolution, bounds_min, bounds_max, brick_size, narrow_band, volume_material=0,
                 object_id=0, primitive_id=0, on_device=None, fp16_distances=False):
        lib = load()
        if on_device is None:
            n = C.c_int(0)
            on_device = lib.dk_device_count(C.byref(n)) == 0 and n.value > 0
        arr = (abi.SdfSphere * len(spheres))()
        for i, s in enumerate(spheres):
            arr[i].center[:] = [float(x) for x in s["center"]]
            arr[i].radius = float(s["radius"])
            arr[i].material = int(s["material"])
            arr[i].smooth_union_radius = float(s.get("smooth_union_radius", 0.0))
        st = abi.SparseVolumeSettings()
        st.resolution[:] = list(resolution)
        st.bounds_min[:] = list(bounds_min)
        st.bounds_max[:] = list(bounds_max)
        self.bounds_min, self.bounds_max = tuple(bounds_min), tuple(bounds_max)  # world space
        st.brick_size[:] = list(brick_size)
        st.narrow_band = narrow_band
        st.volume_material = volume_material
        st.object_id, st.primitive_id = object_id, primitive_id
        st.fp16_distances = 1 if fp16_distances else 0
        build = lib.dk_bake_sparse_sphere_volume if on_device else lib.dk_build_sparse_sphere_volume
        handle = C.c_void_p()
        check(build(arr, len(spheres), C.byref(st), C.byref(handle)))
        self._owner = _VolumeHandle(handle)
        view = abi.Scene()
        check(lib.dk_sparse_volume_view(handle, C.byref(view)))
        owner = self._owner

        def arr_of(ptr, count, dtype):
            if not count:
                return np.zeros(0, dtype)
            buf = (C.c_uint8 * (count * dtype.itemsize)).from_address(ptr)
            # Every view holds the library handle: the buffers stay alive
            # while any array over them does, even after this object is gone.
            buf._owner = owner
            return np.frombuffer(buf, dtype=dtype, count=count)

        self.volumes = arr_of(view.volumes, view.volume_count, abi.VOLUME_DTYPE)
        self.bricks = arr_of(view.volume_bricks, view.volume_brick_count, abi.BRICK_DTYPE)
        self.samples = arr_of(view.volume_brick_samples, view.volume_brick_sample_count, abi.BRICK_SAMPLE_DTYPE)
        self.grids = arr_of(view.volume_brick_grids, view.volume_brick_grid_count, abi.BRICK_GRID_DTYPE)
        self.grid_indices = arr_of(view.volume_brick_grid_indices, view.volume_brick_grid_index_count, np.dtype(np.uint32))


def probe_bandwidth(nbytes: int, passes: int = 20) -> float:
    """dk_probe_bandwidth: measured read GB/s over an `nbytes` buffer (L2-sized or HBM-sized)."""
    out = C.c_double(0.0)
    check(load().dk_probe_bandwidth(int(nbytes), int(passes), C.byref(out), None))
    return out.value
