"""The reference's AOV tests (Tests/DenrimRendererKitTests/AOVTests.swift), restated.

They run at the reference's default quality, preview (flatPreviewKernel):
* testPNGVisualizationUsesOutputSpecificEncoding (:161-203): known answers of
  PNGWriter.visualizedRGBA8Pixels, checked on the oracle encoder (CPU) and on
  the device encoder through `dk_encode_rgba8` (GPU);
* testAOVTexturesReceivePrimarySurfaceData, testPublicOutputPixelReadback,
  testMotionVectorOutputUsesPreviousCamera, testAlbedoOutputPreservesMaterialOpacity,
  testAlbedoPNGPreservesMaterialOpacity (:24-160): the same scenes, settings and
  predicates through the CUDA path (GPU).
"""
import ctypes as C

import numpy as np
import pytest

from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput, image, library, scenes
from denrimrendererkit_gb300.renderer import RenderQuality, RenderSettings
from denrimrendererkit_gb300.scene import Camera, Material, Mesh, RenderScene

BEAUTY_PIXELS = np.array([[0, 0, 0, 0.5], [1, 1, 1, 1], [16, 16, 16, 1]], np.float32)
DEPTH_PIXELS = np.array([[0, 0, 0, 0], [2, 2, 2, 1], [4, 4, 4, 1]], np.float32)
ID_PIXELS = np.array([[0, 0, 0, 0], [1, 1, 1, 1], [2, 2, 2, 1]], np.float32)
MOTION_PIXELS = np.array([[0, 0, 0, 1], [2, -2, 0, 1]], np.float32)


def check_encoding_known_answers(encode):
    beauty = encode(BEAUTY_PIXELS, RenderOutput.BEAUTY)
    assert beauty[0].tolist() == [0, 0, 0, 127]
    assert beauty[1, 0] > 200 and beauty[2, 0] > beauty[1, 0]
    depth = encode(DEPTH_PIXELS, RenderOutput.DEPTH)
    assert depth[0].tolist() == [0, 0, 0, 255]
    assert 0 < depth[1, 0] < depth[2, 0]
    ids = encode(ID_PIXELS, RenderOutput.MATERIAL_ID)
    assert ids[0].tolist() == [0, 0, 0, 255]
    assert ids[1, :3].tolist() != ids[2, :3].tolist() and ids[1, :3].tolist() != [255, 255, 255]
    motion = encode(MOTION_PIXELS, RenderOutput.MOTION_VECTOR)
    assert motion[0].tolist() == [127, 127, 128, 255]
    assert motion[1, 0] > motion[1, 1]


def test_png_visualization_known_answers_oracle():
    from oracle import image_oracle as io
    check_encoding_known_answers(lambda px, kind: io.visualized_rgba8(px[None], int(kind))[0])


def opacity_scene(opacity):  # AOVTests.opacityScene
    scene = RenderScene(camera=Camera((0, 0, 3), (0, 0, 0), vertical_field_of_view_degrees=34.0))
    m = scene.add_material(Material(base_color=(0.7, 0.2, 0.1), roughness=0.8, opacity=opacity))
    scene.add(Mesh.quad((-1, -1, 0), (1, -1, 0), (1, 1, 0), (-1, 1, 0)), m)
    return scene


def unique_albedo(px):  # uniqueAlbedoEstimate
    px = px.reshape(-1, 4)
    px = px[px[:, 3] > 0]
    q = np.clip(px[:, :3] * 7, 0, 7).astype(np.int64)
    return len(set((q[:, 0] << 16 | q[:, 1] << 8 | q[:, 2]).tolist()))


def unique_ids(px):  # uniqueIDEstimate: Int(r.rounded()) > 0
    r = px.reshape(-1, 4)[:, 0].astype(np.float64)
    ids = np.sign(r) * np.floor(np.abs(r) + 0.5)
    return len(set(ids[ids > 0].tolist()))


@pytest.fixture(scope="module")
def renderer(dk_lib):
    return DenrimRenderer(0)


@pytest.mark.gpu
def test_png_visualization_known_answers_device(renderer):
    import torch
    lib = library.load()
    ws = torch.zeros(4, dtype=torch.int32, device="cuda")

    def encode(px, kind):
        dev = torch.from_numpy(np.ascontiguousarray(px)).cuda()
        out = torch.zeros((len(px), 4), dtype=torch.uint8, device="cuda")
        library.check(lib.dk_encode_rgba8(C.c_void_p(dev.data_ptr()), len(px), 1, int(kind),
                                          C.c_void_p(out.data_ptr()), C.c_void_p(ws.data_ptr()), None))
        torch.cuda.synchronize()
        return out.cpu().numpy()

    check_encoding_known_answers(encode)


@pytest.mark.gpu
def test_aovs_receive_primary_surface_data(renderer):
    wl = scenes.material_reference()
    settings = RenderSettings(width=32, height=32, max_bounces=1)
    assert settings.quality == RenderQuality.PREVIEW
    with renderer.make_session(wl.scene, settings) as s:
        s.render_next_sample()
        depth, normal, albedo = (s.pixels(k) for k in (RenderOutput.DEPTH, RenderOutput.NORMAL, RenderOutput.ALBEDO))
    assert (depth[..., 0] > 0).any()
    n = normal.reshape(-1, 4)
    assert ((n[:, 3] > 0) & (n[:, :3] >= 0).all(1) & (n[:, :3] <= 1).all(1)).any()
    assert unique_albedo(albedo) > 3


@pytest.mark.gpu
def test_public_output_pixel_readback(renderer):
    wl = scenes.material_reference()
    with renderer.make_session(wl.scene, RenderSettings(width=24, height=24, max_bounces=1)) as s:
        s.render_next_sample()
        out = {k: s.pixels(k) for k in RenderOutput}
    assert all(v.shape == (24, 24, 4) for v in out.values())
    assert (out[RenderOutput.DEPTH][..., 0] > 0).any()
    assert unique_albedo(out[RenderOutput.ALBEDO]) > 3
    assert unique_ids(out[RenderOutput.MATERIAL_ID]) > 3 and unique_ids(out[RenderOutput.OBJECT_ID]) > 3


@pytest.mark.gpu
def test_motion_vectors_use_previous_camera(renderer):
    wl = scenes.material_reference()
    cam = wl.scene.camera
    prev = Camera(tuple(np.add(cam.origin, (0.15, 0, 0))), tuple(np.add(cam.target, (0.15, 0, 0))), up=cam.up,
                  vertical_field_of_view_degrees=cam.vertical_field_of_view_degrees)
    settings = RenderSettings(width=32, height=32, max_bounces=1, previous_camera=prev)
    with renderer.make_session(wl.scene, settings) as s:
        s.render_next_sample()
        motion = s.pixels(RenderOutput.MOTION_VECTOR).reshape(-1, 4)
    assert ((np.abs(motion[:, 0]) > 0.01) | (np.abs(motion[:, 1]) > 0.01)).any()
    assert (motion[:, 3] > 0).any()


@pytest.mark.gpu
def test_albedo_output_and_png_preserve_material_opacity(renderer, tmp_path):
    with renderer.make_session(opacity_scene(0.35), RenderSettings(width=16, height=16, max_bounces=1)) as s:
        s.render_next_sample()
        albedo = s.pixels(RenderOutput.ALBEDO).reshape(-1, 4)
        path = str(tmp_path / "albedo.png")
        s.write_png(path, RenderOutput.ALBEDO)
    albedo = albedo[albedo[:, 3] > 0]
    assert (np.abs(albedo[:, 3] - 0.35) < 0.02).any()
    alphas = image.read_png(path)[..., 3].reshape(-1).astype(int)
    assert (np.abs(alphas - 89) <= 3).any()
