"""The reference's OpacityTransportTests
(Tests/DenrimRendererKitTests/OpacityTransportTests.swift:7-100), restated
through the CUDA path: a fully transparent (opacity 0) red quad in front of
an emissive green quad; at final quality the primary AOVs and the beauty
show the rear surface."""
import numpy as np
import pytest

from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput
from denrimrendererkit_gb300.renderer import RenderQuality, RenderSettings
from denrimrendererkit_gb300.scene import Camera, Material, Mesh, RenderScene

pytestmark = pytest.mark.gpu


def cutout_scene():  # OpacityTransportTests.cutoutScene (:58-99)
    scene = RenderScene(camera=Camera((0, 0, 3), (0, 0, 0), vertical_field_of_view_degrees=34.0))
    cutout = scene.add_material(Material(base_color=(1, 0, 0), roughness=0.8, opacity=0.0))
    rear = scene.add_material(Material(base_color=(0, 1, 0), emission=(0, 1, 0), emission_strength=1.0, roughness=0.8))
    scene.add(Mesh.quad((-0.9, -0.9, 0), (0.9, -0.9, 0), (0.9, 0.9, 0), (-0.9, 0.9, 0)), cutout)
    scene.add(Mesh.quad((-0.9, -0.9, -0.25), (0.9, -0.9, -0.25), (0.9, 0.9, -0.25), (-0.9, 0.9, -0.25)), rear)
    return scene


def render(output):
    settings = RenderSettings(width=24, height=24, max_bounces=2, quality=RenderQuality.FINAL)
    with DenrimRenderer(0).make_session(cutout_scene(), settings) as s:
        s.render_next_sample()
        return s.pixels(output).reshape(-1, 4)


def test_fully_transparent_primary_surface_reveals_rear_surface_aov(dk_lib):
    albedo = render(RenderOutput.ALBEDO)
    albedo = albedo[albedo[:, 3] > 0]
    r, g, b, a = albedo.T
    assert ((r < 0.1) & (g > 0.8) & (b < 0.1) & (a > 0.99)).any()
    assert not ((r > 0.8) & (g < 0.1) & (b < 0.1) & (a < 0.01)).any()


def test_fully_transparent_primary_surface_reveals_rear_emission(dk_lib):
    r, g, b, _ = render(RenderOutput.BEAUTY).T
    assert ((g > 0.8) & (r < 0.2) & (b < 0.2)).any()
