"""The 8-wide traversal tree with 8-bit quantised child boxes (DK_BVH_WIDTH=8)
on the GPU.

Child boxes are rounded outwards, so a box test never drops a triangle the
exact boxes keep, and the leaf test is the same Möller-Trumbore with the same
(t, reference slot) tie-break: renders through the 8-wide tree must meet the
same bar against the CPU oracle as the default 4-wide FP32 tree (AOVs
bit-exact, beauty within the parity tolerance), and its primary-hit AOVs must
equal the 4-wide tree's bit for bit.
"""
import os

import numpy as np
import pytest

from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput, compile_scene, scenes
from test_gpu_parity import AOVS, assert_aovs_bit_exact, beauty_stats, run_pair

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def renderer(dk_lib):
    return DenrimRenderer(0)


@pytest.fixture()
def wide8():
    old = os.environ.get("DK_BVH_WIDTH")
    os.environ["DK_BVH_WIDTH"] = "8"
    yield
    if old is None:
        del os.environ["DK_BVH_WIDTH"]
    else:
        os.environ["DK_BVH_WIDTH"] = old


@pytest.mark.parametrize("maker", [scenes.parity_quad_scene, scenes.cornell_box_reference,
                                   scenes.reused_mesh_instance_scene])
def test_reference_parity_scenes_wide8(renderer, oracle_lib, wide8, maker):
    s, o, _ = run_pair(renderer, oracle_lib, maker(), 1)
    assert_aovs_bit_exact(s, o)
    rel, g, c = beauty_stats(s, o)
    assert rel <= 1e-3
    assert np.array_equal(g[:, 3], c[:, 3])


@pytest.mark.parametrize("maker,samples,tol", [(scenes.cornell_small, 16, 1e-3), (scenes.material_zoo, 16, 5e-2)])
def test_oracle_parity_wide8(renderer, oracle_lib, wide8, maker, samples, tol):
    s, o, _ = run_pair(renderer, oracle_lib, maker(), samples)
    assert_aovs_bit_exact(s, o)
    rel, g, c = beauty_stats(s, o)
    assert rel <= tol
    assert abs(g[:, :3].mean() - c[:, :3].mean()) <= 0.01 * c[:, :3].mean()


def test_spheres_large_pixel_sample_wide8(renderer, oracle_lib, wide8):
    wl = scenes.spheres_large()
    rng = np.random.default_rng(0)
    pl = np.sort(rng.choice(1920 * 1080, 4096, replace=False)).astype(np.uint32)
    s, o, _ = run_pair(renderer, oracle_lib, wl, 2, pixel_list=pl)
    assert_aovs_bit_exact(s, o, pl)
    rel, g, c = beauty_stats(s, o, pl)
    assert rel <= 2e-2


def test_wide8_equals_wide4(renderer):
    # Large scene at 480x270: primary-hit AOVs identical, beauty statistically equal.
    wl = scenes.spheres_large(width=480, height=270)
    b = compile_scene(wl.scene)
    out = {}
    for width in ("4", "8"):
        os.environ["DK_BVH_WIDTH"] = width
        try:
            with renderer.make_session(wl.scene, wl.settings, build=b) as s:
                s.render(8)
                out[width] = {k: s.pixels(k) for k in AOVS + (RenderOutput.BEAUTY,)}
        finally:
            del os.environ["DK_BVH_WIDTH"]
    for kind in AOVS:
        assert np.array_equal(out["4"][kind].view(np.uint32), out["8"][kind].view(np.uint32)), kind.name
    g4 = out["4"][RenderOutput.BEAUTY][..., :3].astype(np.float64)
    g8 = out["8"][RenderOutput.BEAUTY][..., :3].astype(np.float64)
    assert np.isfinite(g8).all()
    assert abs(g8.mean() - g4.mean()) <= 0.01 * g4.mean()
