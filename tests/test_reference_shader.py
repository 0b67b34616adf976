"""The CPU oracle against the reference's own shader.

oracle/_ref holds the reference's PathTrace.metal rewritten mechanically into
C++ (oracle/ref/metal2cpp.py: swizzles, attributes, hardware-RT functions
dropped, random draws hoisted into left-to-right order) and compiled against a
Metal-subset shim with the restatement's IEEE conventions.  These tests run
the reference kernel `pathTraceKernel` (PathTrace.metal:5167-5586) and the
restatement on the same scenes and require identical bits: accumulation
texture, all six AOV planes, and the reference's own SDF traversal counters
(PathTrace.metal:191-214).  They pin the oracle, which then judges the CUDA
kernels, to the reference's code.
"""
import numpy as np
import pytest

from denrimrendererkit_gb300 import compile_scene, scenes
from denrimrendererkit_gb300.scene import Camera

orc = pytest.importorskip("oracle.oracle")

pytestmark = pytest.mark.skipif(not orc.reference_available(), reason="reference shader sources not available")


@pytest.fixture(scope="module")
def ref_lib(oracle_lib):
    return orc.load_reference()


def _pixels(width, height, step):
    return np.array([y * width + x for y in range(0, height, step) for x in range(0, width, step)], np.uint32)


def _render_both(wl, spp, pixel_list=None, tile=None, fp_build=None, settings=None, camera=None, sdf=False):
    b = fp_build or compile_scene(wl.scene, host_builders=orc.HostBuilders)
    settings = settings or wl.settings
    camera = camera or wl.scene.camera
    o = orc.OracleRender(b, settings, camera, tile=tile)
    r = orc.ReferenceRender(b, settings, camera, tile=tile, collect_sdf_counters=sdf)
    o.render(spp, pixel_list)
    r.render(spp, pixel_list)
    return o, r


def _assert_bits_equal(o, r, mask=None):
    acc = o.accum.astype(np.float32)
    if mask is None:
        mask = np.ones(acc.shape[:2], bool)
    for i, name in enumerate(("depth", "normal", "albedo", "material_id", "object_id", "motion_vector")):
        a, c = o.aov[i][mask], r.aov[i][mask]
        assert np.array_equal(a.view(np.uint32), c.view(np.uint32)), f"{name} AOV differs from the reference"
    a, c = acc[mask], r.accum[mask]
    diff = (a.view(np.uint32) != c.view(np.uint32)).any(-1)
    assert not diff.any(), f"{int(diff.sum())} of {diff.size} accumulation texels differ from the reference"


def test_reference_kernel_cornell_small(ref_lib):
    wl = scenes.cornell_small(width=64, height=36)
    o, r = _render_both(wl, 8)
    _assert_bits_equal(o, r)
    assert r.accum[..., :3].mean() > 0.05


def test_reference_kernel_material_features(ref_lib):
    # thin film, sheen, anisotropy, clearcoat, subsurface walk, rough and
    # thin-walled transmission, interior scattering, cut-out, textures, normal
    # map, rotated and clipped HDRI, emissive quads, radiance clamp
    wl = scenes.material_zoo(width=96, height=64)
    o, r = _render_both(wl, 8)
    _assert_bits_equal(o, r)


def test_reference_kernel_large_scene_sample(ref_lib):
    wl = scenes.spheres_large(width=480, height=270, subdivisions=3, hdri_size=(512, 256))
    pl = _pixels(480, 270, 8)
    o, r = _render_both(wl, 4, pixel_list=pl)
    mask = np.zeros((270, 480), bool)
    mask.flat[pl] = True
    _assert_bits_equal(o, r, mask)


def test_reference_kernel_sparse_volume_and_counters(ref_lib):
    wl = scenes.sdf_spheres(width=64, height=64, resolution=192)
    o, r = _render_both(wl, 4, sdf=True)
    _assert_bits_equal(o, r)
    mine, ref = o.counter_dict(), r.sdf_counter_dict()
    for key in ("grid_cells", "macro_skips", "brick_tests", "range_culls", "brick_marches", "march_steps",
                "brick_hits"):
        assert mine[key] == ref[key], f"{key}: oracle {mine[key]} reference {ref[key]}"
    assert ref["brick_hits"] > 0 and ref["primary_queries"] == 64 * 64 * 4


@pytest.mark.parametrize("maker", [scenes.cornell_box_reference, scenes.parity_quad_scene,
                                   scenes.reused_mesh_instance_scene])
def test_reference_kernel_parity_scenes(ref_lib, maker):
    wl = maker()
    o, r = _render_both(wl, 2)
    _assert_bits_equal(o, r)


def test_reference_kernel_tiles_background_denoiser_motion(ref_lib):
    wl = scenes.material_zoo(width=48, height=32)
    s = wl.settings
    s.transparent_background = True
    s.shows_environment_background = False
    s.background_color = (0.2, 0.3, 0.4)
    s.denoise = True
    cam = wl.scene.camera
    s.previous_camera = Camera((0.3, 2.5, 6.0), (0.0, 0.5, 0.0), vertical_field_of_view_degrees=38.0)
    o, r = _render_both(wl, 3, tile=(8, 4, 24, 20), settings=s, camera=cam)
    _assert_bits_equal(o, r)
    assert np.abs(r.aov[5][4:24, 8:32, :2]).max() > 0  # motion vectors present
