"""The C-ABI library: it loads, exports every symbol of include/denrim_cuda.h,
its host-side scene-compile helpers match the oracle bit for bit, and its
validation errors map onto DenrimRendererError.  No GPU compute is called."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from denrimrendererkit_gb300 import abi, library, scenes
from denrimrendererkit_gb300.scene import compile_scene

ROOT = Path(__file__).resolve().parents[1]


def test_exports_every_declared_symbol(dk_lib):
    header = (ROOT / "include" / "denrim_cuda.h").read_text()
    declared = set(re.findall(r"^\s*(?:int|const char\*)\s+(dk_\w+)\s*\(", header, re.M))
    assert declared == set(abi.EXPORTED_SYMBOLS)
    for name in declared:
        assert hasattr(dk_lib, name), name


def test_struct_sizes_match_header():
    assert C.sizeof(abi.Camera) == 80
    assert abi.TRIANGLE_DTYPE.itemsize == 192 and abi.MATERIAL_DTYPE.itemsize == 272


@pytest.mark.parametrize("maker", [scenes.cornell_small, scenes.cornell_box_reference,
                                   scenes.reused_mesh_instance_scene])
def test_library_bvh_matches_oracle(dk_lib, oracle_lib, maker):
    b = compile_scene(maker().scene)
    nodes, prim = oracle_lib.build_bvh(b.triangles, 4)
    assert np.array_equal(nodes.view(np.uint8), b.nodes.view(np.uint8))
    assert np.array_equal(prim, b.primitive_indices)


def test_library_bvh_matches_oracle_large(dk_lib, oracle_lib):
    # 40 displaced subdivision-4 spheres (204,802 tris): exercises the parallel top levels.
    wl = scenes.spheres_large(width=64, height=36, subdivisions=4, hdri_size=(8, 4))
    wl.scene.mesh_instances = wl.scene.mesh_instances[:41]
    tris = np.concatenate([inst.mesh.gpu_triangles(inst.material, inst.transform, i)
                           for i, inst in enumerate(wl.scene.mesh_instances)])
    nodes, prim = library.build_bvh(tris, 4)
    onodes, oprim = oracle_lib.build_bvh(tris, 4)
    assert len(tris) > 65536 * 2
    assert np.array_equal(nodes.view(np.uint8), onodes.view(np.uint8))
    assert np.array_equal(prim, oprim)


def test_library_lights_match_oracle(dk_lib, oracle_lib):
    wl = scenes.spheres_large(width=64, height=36, subdivisions=1, hdri_size=(8, 4))
    tris = np.concatenate([inst.mesh.gpu_triangles(inst.material, inst.transform, i)
                           for i, inst in enumerate(wl.scene.mesh_instances)])
    mats = np.array([m.gpu_material() for m in wl.scene.materials], abi.MATERIAL_DTYPE)
    t1 = tris.copy()
    lights = library.build_lights(t1, mats)
    t2, olights = oracle_lib.build_lights(tris, mats)
    assert len(lights) == 16
    assert np.array_equal(lights.view(np.uint8), olights.view(np.uint8))
    assert np.array_equal(t1["padding2"], t2["padding2"])


def _settings_struct(width=8, height=8, quality=2):
    s = abi.Settings()
    s.width, s.height, s.max_bounces, s.quality = width, height, 1, quality
    return s


def _scene_struct(b):
    return b.as_struct()


def test_validation_errors_map_to_reference(dk_lib):
    # RenderSession.init validation (RenderSession.swift:304-327)
    b = compile_scene(scenes.parity_quad_scene().scene)
    h = C.c_void_p()
    sc = b.as_struct()
    st = _settings_struct(0, 8)
    assert dk_lib.dk_session_create(C.byref(sc), C.byref(st), C.byref(h)) == 3
    assert b"dimensions" in dk_lib.dk_last_error_message()
    st = _settings_struct()
    empty = abi.Scene()
    empty.materials, empty.material_count = sc.materials, sc.material_count
    assert dk_lib.dk_session_create(C.byref(empty), C.byref(st), C.byref(h)) == 3
    assert b"no renderable geometry" in dk_lib.dk_last_error_message()
    nomat = b.as_struct()
    nomat.material_count = 0
    assert dk_lib.dk_session_create(C.byref(nomat), C.byref(st), C.byref(h)) == 3
    assert b"no materials" in dk_lib.dk_last_error_message()
    st = _settings_struct(quality=3)  # not a RenderQuality
    assert dk_lib.dk_session_create(C.byref(sc), C.byref(st), C.byref(h)) == 6
    assert dk_lib.dk_session_create(None, C.byref(st), C.byref(h)) == 6


def test_no_device_is_reported(dk_lib):
    n = C.c_int(-1)
    assert dk_lib.dk_device_count(C.byref(n)) == 0
    if n.value == 0:
        assert dk_lib.dk_device_open(0) == 1  # DK_ERROR_NO_DEVICE (noMetalDevice)


def test_product_fails_loudly_without_library(monkeypatch, tmp_path):
    from denrimrendererkit_gb300 import build
    monkeypatch.setattr(library, "_LIB", None)
    monkeypatch.setattr(build, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        library.load()


def test_denoise_settings_map_to_the_aov_ray_flag():
    # GPURenderConstants.denoiserEnabled = denoise.denoiser != .none (RenderSession.swift:941);
    # the presets are DenoiseSettings.none / .simpleSpatial / .appleSVGF (Denoiser.swift:62-76).
    from denrimrendererkit_gb300.renderer import (DenoiseSettings, RenderDenoiser, RenderSettings, denoise_filter,
                                                  make_settings_struct)
    from denrimrendererkit_gb300.scene import Camera
    cam = Camera((0, 0, 3), (0, 0, 0))
    cases = [(False, 0, None), (True, 1, None), (DenoiseSettings.NONE, 0, None),
             (DenoiseSettings.SIMPLE_SPATIAL, 1, RenderDenoiser.SIMPLE_SPATIAL),
             (DenoiseSettings.APPLE_SVGF, 1, RenderDenoiser.APPLE_SVGF)]
    for denoise, flag, filt in cases:
        s = make_settings_struct(RenderSettings(width=8, height=8, denoise=denoise), cam)
        assert s.denoiser_enabled == flag
        f = denoise_filter(denoise)
        assert (f.denoiser if f else None) == filt
    svgf = DenoiseSettings.APPLE_SVGF
    assert (svgf.radius, svgf.normal_sigma, svgf.depth_sigma, svgf.albedo_sigma, svgf.color_sigma,
            svgf.iterations) == (2, 0.18, 0.08, 0.25, 4.0, 5)
    sp = DenoiseSettings.SIMPLE_SPATIAL
    assert (sp.radius, sp.normal_sigma, sp.depth_sigma, sp.albedo_sigma, sp.color_sigma, sp.iterations) == \
        (2, 0.18, 0.03, 0.25, 1.0, 3)
