"""Host scene API against the reference's own known answers (APITests.swift):
the Cornell box scene, an empty scene, the quad-light helper through the
scene compile (triangles, light list, emissive material), clearcoat
attenuation packing and the render settings' defaults and radiance clamp."""
import numpy as np

from denrimrendererkit_gb300 import QuadLight, RenderScene, compile_scene, scenes
from denrimrendererkit_gb300.renderer import RenderDenoiser, RenderQuality, RenderSettings
from denrimrendererkit_gb300.scene import Material


def test_cornell_box_scene_compiles():
    # APITests.testCornellBoxSceneCompiles
    scene = scenes.cornell_box_reference().scene
    assert len(scene.materials) == 4 and len(scene.mesh_instances) == 6
    build = compile_scene(scene)
    assert len(build.triangles) == 12 and len(build.lights) == 2


def test_empty_render_scene_creates_no_default_lights():
    # APITests.testEmptyRenderSceneDoesNotCreateDefaultLights
    scene = RenderScene()
    assert not scene.materials and not scene.mesh_instances and not scene.sparse_volumes


def test_quad_light_adds_an_app_authored_emissive_light():
    # APITests.testQuadLightAPIAddsAppAuthoredEmissiveLight
    scene = RenderScene()
    scene.add_quad_light(QuadLight((-1, 2, -1), (1, 2, -1), (1, 2, 1), (-1, 2, 1), color=(1, 0.8, 0.6), intensity=12))
    build = compile_scene(scene, build_bvh=False)
    assert len(scene.materials) == 1 and len(scene.mesh_instances) == 1
    assert len(build.triangles) == 2 and len(build.lights) == 2
    assert (build.lights["material_index"] == 0).all()
    em = build.materials[0]["emission"]
    assert np.allclose(em, [12, 9.6, 7.2, 0], atol=1e-4)


def test_clearcoat_attenuation_defaults_to_clearcoat_color():
    # APITests.testClearcoatAttenuationDefaultsToClearcoatColor
    m = Material(base_color=(0.4, 0.5, 0.6), clearcoat=0.7, clearcoat_color=(0.72, 0.86, 1), clearcoat_thickness=0.4)
    assert m.clearcoat_attenuation_color is None
    assert np.allclose(m.gpu_material()["clearcoat_attenuation"], [0.72, 0.86, 1, 0.4], atol=1e-4)


def test_settings_defaults_are_small_and_progressive():
    # APITests.testSettingsDefaultsAreSmallAndProgressive
    s = RenderSettings()
    assert (s.width, s.height, s.max_bounces) == (512, 512, 4) and s.quality == RenderQuality.PREVIEW
    assert not s.transparent_background and s.shows_environment_background
    assert tuple(s.background_color) == (0, 0, 0)
    assert not s.denoise or getattr(s.denoise, "denoiser", RenderDenoiser.NONE) == RenderDenoiser.NONE
    assert s.sample_radiance_clamp is None
    assert s.resolved_sample_radiance_clamp == RenderQuality.PREVIEW.default_sample_radiance_clamp


def test_settings_override_or_disable_the_sample_radiance_clamp():
    # APITests.testSettingsCanOverrideOrDisableSampleRadianceClamp
    assert RenderQuality.PREVIEW.default_sample_radiance_clamp == 10
    assert RenderQuality.INTERACTIVE.default_sample_radiance_clamp == 24
    assert RenderSettings(quality=RenderQuality.FINAL).resolved_sample_radiance_clamp == 64
    assert RenderSettings(sample_radiance_clamp=0).resolved_sample_radiance_clamp == 0
    assert RenderSettings(sample_radiance_clamp=18).resolved_sample_radiance_clamp == 18


def test_scene_world_bounds_include_transformed_meshes():
    # APITests.testSceneWorldBoundsIncludeTransformedMeshesAndVolumes (a box at +2; the reference's second
    # object, a dense volume, is a box of the same extent at -2 here: dense volumes are not part of this path)
    from denrimrendererkit_gb300 import Mesh, Transform
    scene = RenderScene()
    m = scene.add_material(Material(base_color=(0.8, 0.8, 0.8)))
    assert scene.world_bounds() is None
    scene.add(Mesh.box(size=(2, 2, 2)), m, Transform.translation((2, 0, 0)))
    scene.add(Mesh.box(size=(1, 1, 1)), m, Transform.translation((-2.5, 0, 0)))
    b = scene.world_bounds()
    assert np.allclose(b.minimum, (-3, -1, -1), atol=1e-4) and np.allclose(b.maximum, (3, 1, 1), atol=1e-4)


def test_camera_frames_perspective_bounds_with_offset():
    # APITests.testCameraFramesPerspectiveBoundsWithOffset
    from denrimrendererkit_gb300.scene import Camera, SceneBounds
    cam = Camera.framing(SceneBounds.of((-1, -1, -1), (1, 1, 1)), aspect_ratio=1, view_direction=(0, 0, -1),
                         padding=1, center_offset=(0.5, 0), vertical_field_of_view_degrees=90)
    assert abs(cam.origin[0] + 0.5) < 1e-4 and abs(cam.origin[2] - 2.5) < 1e-4
    assert abs(cam.target[0] + 0.5) < 1e-4 and abs(cam.focus_distance - 2.5) < 1e-4


def test_camera_frames_orthographic_bounds():
    # APITests.testCameraFramesOrthographicBounds
    from denrimrendererkit_gb300.scene import Camera, SceneBounds
    cam = Camera.framing(SceneBounds.of((-1, -1, -1), (1, 1, 1)), aspect_ratio=1, view_direction=(0, 0, -1),
                         padding=1, orthographic=True)
    assert cam.orthographic_scale is not None and abs(cam.orthographic_scale - 2) < 1e-4
    assert abs(cam.origin[2] - 2) < 1e-4 and abs(cam.target[2]) < 1e-4
