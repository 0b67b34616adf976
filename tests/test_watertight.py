"""The watertight ray-triangle test (RenderSettings.watertight) beside the
reference's Moller-Trumbore (PathTrace.metal:1801-1852), which stays the
default and the parity mode.

* On a finely tessellated plane seen through pixel centres that fall on its
  grid lines (the unjittered AOV ray), the watertight test leaves no pixel
  without a hit: no ray slips through a shared edge or vertex.
* On the small and the large configurations, the two tests hit the same
  surface except on a few pixels whose primary ray grazes an edge (the counts
  are printed and bounded), the depths of the same surface agree to rounding,
  and the beauty images agree within the parity tolerance of each
  configuration.
"""
import dataclasses

import numpy as np
import pytest

from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput, compile_scene, scenes
from denrimrendererkit_gb300.renderer import RenderQuality, RenderSettings
from denrimrendererkit_gb300.scene import Camera, Material, Mesh, RenderScene

pytestmark = pytest.mark.gpu

IDS = (RenderOutput.DEPTH, RenderOutput.NORMAL, RenderOutput.MATERIAL_ID, RenderOutput.OBJECT_ID)


def grid_plane(n: int, half: float) -> Mesh:
    """An n x n grid of quads (two triangles each) over [-half, half]^2 at z = 0."""
    xs = np.linspace(-half, half, n + 1, dtype=np.float32)
    vx, vy = np.meshgrid(xs, xs, indexing="xy")
    verts = np.stack([vx.ravel(), vy.ravel(), np.zeros(vx.size, np.float32)], axis=1).astype(np.float32)
    idx = []
    for j in range(n):
        for i in range(n):
            a = j * (n + 1) + i
            b, c, d = a + 1, a + n + 2, a + n + 1
            idx += [a, b, c, a, c, d]
    return Mesh(verts, np.array(idx, np.uint32))


def render(wl, spp, watertight, pixel_list=None):
    st = dataclasses.replace(wl.settings, watertight=watertight)
    b = compile_scene(wl.scene)
    with DenrimRenderer(0).make_session(wl.scene, st, build=b) as s:
        s.render(spp)
        return {k: s.pixels(k).copy() for k in (RenderOutput.BEAUTY,) + IDS}


def test_watertight_plane_has_no_cracks(dk_lib):
    # 64 x 64 pixel centres over a 128 x 128 quad grid: every centre lies on a
    # grid line (and most on a vertex) of the plane, up to the camera's rounding.
    w = 64
    scene = RenderScene(camera=Camera((0.0, 0.0, 2.0), (0.0, 0.0, 0.0), orthographic_scale=2.0))
    m = scene.add_material(Material(base_color=(0.6, 0.6, 0.6)))
    scene.add(grid_plane(2 * w, 1.0), m)
    settings = RenderSettings(width=w, height=w, max_bounces=1, quality=RenderQuality.FINAL, denoise=True)
    wl = scenes.Workload("grid-plane", scene, settings, 1)
    wt = render(wl, 1, True)
    mt = render(wl, 1, False)
    hit_wt = wt[RenderOutput.DEPTH][..., 3] > 0
    hit_mt = mt[RenderOutput.DEPTH][..., 3] > 0
    print(f"grid plane: pixels without a hit: watertight {int((~hit_wt).sum())}, "
          f"Moller-Trumbore {int((~hit_mt).sum())} of {w * w}")
    assert hit_wt.all()


@pytest.mark.parametrize("config", ["small", "large"])
def test_watertight_agrees_with_moller_trumbore_off_the_edges(dk_lib, config):
    if config == "small":
        wl, spp, tol, max_frac = scenes.cornell_small(), 16, 1e-2, 2e-3
    else:
        wl, spp, tol, max_frac = scenes.spheres_large(width=480, height=270), 2, 5e-2, 5e-3
    wt = render(wl, spp, True)
    mt = render(wl, spp, False)
    ids_diff = np.zeros(wt[RenderOutput.DEPTH].shape[:2], bool)
    for k in (RenderOutput.MATERIAL_ID, RenderOutput.OBJECT_ID):
        ids_diff |= (wt[k].view(np.uint32) != mt[k].view(np.uint32)).any(axis=-1)
    hit_diff = (wt[RenderOutput.DEPTH][..., 3] > 0) != (mt[RenderOutput.DEPTH][..., 3] > 0)
    same = ~ids_diff & (mt[RenderOutput.DEPTH][..., 3] > 0)
    dw, dm = wt[RenderOutput.DEPTH][..., 0][same], mt[RenderOutput.DEPTH][..., 0][same]
    rel_depth = np.abs(dw - dm) / np.maximum(dm, 1e-6)
    depth_rel = float(np.quantile(rel_depth, 0.999)) if same.any() else 0.0
    # another triangle of the same object (a ray grazing an edge or silhouette)
    other_tri = int((rel_depth > 1e-4).sum())
    g = wt[RenderOutput.BEAUTY][..., :3].astype(np.float64)
    c = mt[RenderOutput.BEAUTY][..., :3].astype(np.float64)
    rel = float(np.sqrt(((g - c) ** 2).mean()) / c.mean())
    print(f"{config}: watertight vs Moller-Trumbore primary hits: another material/object ID on "
          f"{int(ids_diff.sum())} of {ids_diff.size} pixels ({ids_diff.mean():.2e}), hit/miss differs on "
          f"{int(hit_diff.sum())}; depth on the same object within {depth_rel:.1e} relative on 99.9 % of the "
          f"pixels ({other_tri} pixels on another of its triangles); beauty relative RMSE between the two "
          f"{rel:.2e}")
    assert depth_rel <= 1e-4
    assert other_tri <= max_frac * ids_diff.size
    assert np.isfinite(g).all()
    assert ids_diff.mean() <= max_frac
    assert rel <= tol
