"""The reference's TextureMaterialTests
(Tests/DenrimRendererKitTests/TextureMaterialTests.swift:7-150), restated
through the CUDA path at the reference's default quality (preview): a
base-colour checker feeds the albedo AOV, a solid normal map feeds the normal
AOV, linear sampling blends a 2x2 texture; and, in place of the reference's
flat-BVH vs hardware-traversal comparison (:97-126, tolerance 5e-4), the
CUDA albedo and normal AOVs against the reference's own kernel compiled for
the host (oracle/_ref) at the same tolerance."""
import numpy as np
import pytest

from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput, compile_scene
from denrimrendererkit_gb300.renderer import RenderSettings
from denrimrendererkit_gb300.scene import Camera, Material, Mesh, RenderScene, Texture2D

pytestmark = pytest.mark.gpu


def solid(c, mode=0):  # Texture2D.solid (Scene/Texture.swift:137-142)
    return Texture2D(1, 1, np.array([c], np.float32), mode)


def checker(a, b, mode=0):  # Texture2D.checker (Scene/Texture.swift:145-154)
    return Texture2D(2, 2, np.array([a, b, b, a], np.float32), mode)


def textured_quad_scene(material):  # TextureMaterialTests.texturedQuadScene (:128-150)
    scene = RenderScene(camera=Camera((0, 0, 3), (0, 0, 0), vertical_field_of_view_degrees=34.0))
    m = scene.add_material(material)
    scene.add(Mesh.quad((-1, -1, 0), (1, -1, 0), (1, 1, 0), (-1, 1, 0)), m)
    return scene


def first_sample(scene, size, output):
    with DenrimRenderer(0).make_session(scene, RenderSettings(width=size, height=size, max_bounces=1)) as s:
        s.render_next_sample()
        px = s.pixels(output).reshape(-1, 4)
    return px[px[:, 3] > 0]


def test_base_color_texture_feeds_albedo_aov(dk_lib):
    mat = Material(base_color=(1, 1, 1), roughness=0.8, base_color_texture=checker((1, 0, 0, 1), (0, 0, 1, 1)))
    r, g, b, _ = first_sample(textured_quad_scene(mat), 24, RenderOutput.ALBEDO).T
    assert ((r > 0.9) & (g < 0.1) & (b < 0.1)).any()
    assert ((r < 0.1) & (g < 0.1) & (b > 0.9)).any()


def test_normal_map_feeds_normal_aov(dk_lib):
    mat = Material(base_color=(1, 1, 1), roughness=0.8, normal_map=solid((1, 0.5, 0.5, 1)))
    r, g, b, _ = first_sample(textured_quad_scene(mat), 16, RenderOutput.NORMAL).T
    assert ((r > 0.9) & (g > 0.4) & (g < 0.6) & (b > 0.4) & (b < 0.6)).any()


def test_linear_texture_sampling_blends_albedo(dk_lib):
    blended = Texture2D(2, 2, np.array([(1, 0, 0, 1), (0, 0, 1, 1), (1, 0, 0, 1), (0, 0, 1, 1)], np.float32), 1)
    mat = Material(base_color=(1, 1, 1), roughness=0.8, base_color_texture=blended)
    r, g, b, _ = first_sample(textured_quad_scene(mat), 32, RenderOutput.ALBEDO).T
    assert ((r > 0.25) & (r < 0.75) & (g < 0.05) & (b > 0.25) & (b < 0.75)).any()


def test_textured_materials_match_the_reference_kernel(dk_lib):
    from oracle import oracle as orc
    if not orc.reference_available():
        pytest.skip("reference shaders not built")
    mat = Material(base_color=(1, 1, 1), roughness=0.8, base_color_texture=checker((1, 0, 0, 1), (0, 0, 1, 1)),
                   normal_map=solid((1, 0.5, 0.5, 1)))
    scene = textured_quad_scene(mat)
    settings = RenderSettings(width=16, height=16, max_bounces=1)
    b = compile_scene(scene)
    with DenrimRenderer(0).make_session(scene, settings, build=b) as s:
        s.render_next_sample()
        got = {k: s.pixels(k) for k in (RenderOutput.ALBEDO, RenderOutput.NORMAL)}
    ref = orc.ReferenceRender(b, settings, scene.camera)
    ref.render(1)
    for k, px in got.items():
        assert np.abs(px - ref.aov[int(k) - 1]).max() <= 0.0005, k.name
