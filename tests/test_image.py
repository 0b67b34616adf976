"""Display encoding, PNG export and the reference's image-metric baselines.

* CPU: the library's PNG writer (`dk_write_png`, host code) round-trips through
  `image.read_png` (zlib checks the Adler-32, the reader every chunk CRC); the
  metric readers on images with known answers; the oracle encoder's fixed
  points of the reference's curves.
* CPU, against the reference's own test baselines
  (Tests/RenderReferenceTests/ReferenceMetrics/*.json, values restated below
  with their tolerances): the CPU oracle renders the reference scenes with the
  reference tests' settings, the oracle encoder turns the beauty into the PNG
  bytes, and ImageMetricReader's metrics must land within the baseline's
  tolerances -- CornellBoxRenderTests.swift:7-33, MaterialReferenceRenderTests.swift:7-27,
  TransparentExportRenderTests.swift:8-30 (at final quality: the test's default quality is preview, but its
  stored baseline is a jittered path-traced render -- the reference's own preview kernel misses it).
* GPU: the same scenes through the CUDA path and `RenderSession.render(samples, to=png)`
  against the same baselines; and the device encoder against the oracle
  encoder on every output kind of rendered scenes: bit-exact for depth, IDs,
  motion vectors and alpha; colour bytes behind the gamma curve's `pow` within
  one step on at most 0.2 % of the bytes (a last-bit difference of powf).
"""
import ctypes as C
import os

import numpy as np
import pytest

from denrimrendererkit_gb300 import image, scenes
from denrimrendererkit_gb300.renderer import RenderQuality, RenderSettings

# ReferenceMetrics/CornellBox.json, MaterialReference.json, TransparentExport.json
BASELINES = {
    "cornell": ({"width": 48, "height": 48, "averageBrightness": 94.0, "maxBrightness": 255.0,
                 "uniqueColorEstimate": 68, "topCenterMaxBrightness": 255.0, "bottomCenterMaxBrightness": 244.0},
                {"averageBrightness": 20.0, "maxBrightness": 20.0, "uniqueColorEstimate": 35,
                 "regionalBrightness": 80.0}),
    "materials": ({"width": 56, "height": 56, "averageBrightness": 115.76, "maxBrightness": 191.0,
                   "uniqueColorEstimate": 70, "topCenterMaxBrightness": 210.0, "bottomCenterMaxBrightness": 180.0},
                  {"averageBrightness": 18.0, "maxBrightness": 35.0, "uniqueColorEstimate": 40,
                   "regionalBrightness": 100.0}),
}
ALPHA_BASELINE = ({"width": 32, "height": 32, "minAlpha": 0, "maxAlpha": 255, "transparentPixels": 778,
                   "opaquePixels": 246}, {"transparentPixels": 4, "opaquePixels": 4})


def cornell_workload():
    wl = scenes.cornell_box_reference(48, 48)
    wl.settings = RenderSettings(width=48, height=48, max_bounces=2, quality=RenderQuality.FINAL)
    wl.samples = 4
    return wl


WORKLOADS = {"cornell": cornell_workload, "materials": scenes.material_reference}


def assert_metrics(m, name):
    base, tol = BASELINES[name]
    assert (m["width"], m["height"]) == (base["width"], base["height"])
    assert abs(m["averageBrightness"] - base["averageBrightness"]) <= tol["averageBrightness"], m
    assert abs(m["maxBrightness"] - base["maxBrightness"]) <= tol["maxBrightness"], m
    assert abs(m["uniqueColorEstimate"] - base["uniqueColorEstimate"]) <= tol["uniqueColorEstimate"], m
    assert abs(m["topCenterMaxBrightness"] - base["topCenterMaxBrightness"]) <= tol["regionalBrightness"], m
    assert abs(m["bottomCenterMaxBrightness"] - base["bottomCenterMaxBrightness"]) <= tol["regionalBrightness"], m


def assert_alpha_metrics(m):
    base, tol = ALPHA_BASELINE
    assert (m["width"], m["height"], m["minAlpha"], m["maxAlpha"]) == (32, 32, base["minAlpha"], base["maxAlpha"]), m
    assert abs(m["transparentPixels"] - base["transparentPixels"]) <= tol["transparentPixels"], m
    assert abs(m["opaquePixels"] - base["opaquePixels"]) <= tol["opaquePixels"], m


# ------------------------------------------------------------------ CPU ----
def test_png_writer_round_trip(dk_lib, tmp_path):
    rng = np.random.default_rng(3)
    for h, w in ((1, 1), (7, 13), (300, 97)):  # 300 x 97 x 4 + rows > one 64 KiB stored block
        img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
        path = str(tmp_path / f"img_{h}x{w}.png")
        assert dk_lib.dk_write_png(os.fsencode(path), img.ctypes.data_as(C.c_void_p), w, h) == 0
        assert np.array_equal(image.read_png(path), img)
    bad = str(tmp_path / "missing-dir" / "x.png")
    assert dk_lib.dk_write_png(os.fsencode(bad), img.ctypes.data_as(C.c_void_p), w, h) == 5  # DK_ERROR_EXPORT_FAILED


def test_metric_readers_known_answers():
    img = np.zeros((8, 16, 4), np.uint8)
    img[..., :3] = 96
    img[..., 3] = 255
    img[0, 7] = (255, 255, 255, 255)  # top-centre band: x in [6, 10], y < 2
    img[7, 8] = (30, 60, 90, 255)     # bottom-centre band: y > 6
    m = image.image_metrics(img)
    assert m["maxBrightness"] == 255.0 and m["topCenterMaxBrightness"] == 255.0
    assert m["bottomCenterMaxBrightness"] == 96.0  # (30 + 60 + 90) / 3 = 60 < 96
    assert m["uniqueColorEstimate"] == 3
    assert abs(m["averageBrightness"] - (126 * 96 + 255 + 60) / 128) < 1e-12
    img[..., 3] = 0
    img[:2, :, 3] = 255
    am = image.alpha_metrics(img)
    assert (am["minAlpha"], am["maxAlpha"], am["transparentPixels"], am["opaquePixels"]) == (0, 255, 96, 32)


def test_oracle_encoder_fixed_points():
    from oracle import image_oracle as io
    f = np.float32
    assert io.tonemap(np.array([0.0, -1.0, np.nan, 1e30], f)).tolist() == [0, 0, 0, 255]
    assert io.display_linear(np.array([0.0, 1.0, 2.0], f)).tolist() == [0, 255, 255]
    assert io.signed(np.array([-1.0, 0.0, 1.0], f)).tolist() == [0, 127, 255]
    c = io.color_for_id(np.array([1, 2, 1000], np.uint32))
    assert c.min() >= 64 and c.max() <= 191 and len({tuple(x) for x in c}) == 3
    depth = np.zeros((2, 2, 4), f)
    depth[..., 0] = [[1.0, 2.0], [np.inf, 0.0]]
    d = io.visualized_rgba8(depth, io.DEPTH)
    assert d[0, 0, 0] == 25 and d[0, 1, 0] == 255 and d[1, 0].tolist() == [0, 0, 0, 255]


@pytest.mark.parametrize("name", ["cornell", "materials"])
def test_oracle_render_meets_reference_metric_baseline(oracle_lib, name):
    from denrimrendererkit_gb300 import compile_scene
    from oracle import image_oracle as io
    from oracle.oracle import HostBuilders
    wl = WORKLOADS[name]()
    b = compile_scene(wl.scene, host_builders=HostBuilders())
    o = oracle_lib.OracleRender(b, wl.settings, wl.scene.camera)
    o.render(wl.samples)
    beauty = o.accum.reshape(wl.settings.height, wl.settings.width, 4).astype(np.float32)
    assert_metrics(image.image_metrics(io.visualized_rgba8(beauty, io.BEAUTY)), name)


def test_oracle_transparent_export_meets_alpha_baseline(oracle_lib):
    from denrimrendererkit_gb300 import compile_scene
    from oracle import image_oracle as io
    from oracle.oracle import HostBuilders
    wl = scenes.transparent_export_scene()
    b = compile_scene(wl.scene, host_builders=HostBuilders())
    o = oracle_lib.OracleRender(b, wl.settings, wl.scene.camera)
    o.render(wl.samples)
    beauty = o.accum.reshape(32, 32, 4).astype(np.float32)
    assert_alpha_metrics(image.alpha_metrics(io.visualized_rgba8(beauty, io.BEAUTY)))


def test_transparent_export_baseline_is_a_jittered_render():
    # The reference test leaves the quality at its default, preview; the
    # reference's own flatPreviewKernel (pixel-centre rays) leaves exactly the
    # 16 x 16 quad pixels opaque, 10 more than the stored baseline's 246 allow
    # (tolerance 4): the baseline was recorded with the path tracer.
    from denrimrendererkit_gb300 import compile_scene
    from oracle import image_oracle as io
    from oracle import oracle as orc
    from oracle.oracle import HostBuilders
    if not orc.reference_available():
        pytest.skip("reference shaders not built")
    wl = scenes.transparent_export_scene()
    wl.settings = RenderSettings(width=32, height=32, max_bounces=1, transparent_background=True)
    assert wl.settings.quality == RenderQuality.PREVIEW
    b = compile_scene(wl.scene, host_builders=HostBuilders())
    o = orc.ReferenceRender(b, wl.settings, wl.scene.camera)
    o.render(1)
    m = image.alpha_metrics(io.visualized_rgba8(o.accum.astype(np.float32), io.BEAUTY))
    assert (m["transparentPixels"], m["opaquePixels"]) == (768, 256)


# ------------------------------------------------------------------ GPU ----
@pytest.fixture(scope="module")
def renderer(dk_lib):
    from denrimrendererkit_gb300 import DenrimRenderer
    return DenrimRenderer(0)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cornell", "materials"])
def test_cuda_render_png_meets_reference_metric_baseline(renderer, tmp_path, name):
    wl = WORKLOADS[name]()
    path = str(tmp_path / f"{name}.png")
    with renderer.make_session(wl.scene, wl.settings) as s:
        s.render(wl.samples, to=path)
        assert s.sample_count == wl.samples
        direct = s.rgba8()
    assert os.path.getsize(path) > 0
    decoded = image.read_png(path)
    assert np.array_equal(decoded, direct)
    m = image.image_metrics(decoded)
    assert m["averageBrightness"] > 3 and m["uniqueColorEstimate"] > 3
    if name == "cornell":  # CornellBoxRenderTests.swift:27-30
        assert m["topCenterMaxBrightness"] > m["bottomCenterMaxBrightness"]
    else:  # MaterialReferenceRenderTests.swift:22-24
        assert m["uniqueColorEstimate"] > 6 and m["maxBrightness"] > 120
    assert_metrics(m, name)


@pytest.mark.gpu
def test_cuda_transparent_export_meets_alpha_baseline(renderer, tmp_path):
    wl = scenes.transparent_export_scene()
    path = str(tmp_path / "transparent.png")
    with renderer.make_session(wl.scene, wl.settings) as s:
        s.render(wl.samples, to=path)
    m = image.alpha_metrics(image.read_png(path))
    assert m["transparentPixels"] > 0 and m["opaquePixels"] > 0
    assert_alpha_metrics(m)


@pytest.mark.gpu
@pytest.mark.parametrize("maker,spp", [(scenes.cornell_small, 8), (scenes.material_zoo, 8)])
def test_device_encoder_matches_oracle_encoder(renderer, maker, spp):
    from denrimrendererkit_gb300 import RenderOutput
    from oracle import image_oracle as io
    wl = maker()
    with renderer.make_session(wl.scene, wl.settings) as s:
        s.render(spp)
        for kind in RenderOutput:
            dev = s.rgba8(kind)
            ref = io.visualized_rgba8(s.pixels(kind), int(kind))
            diff = np.abs(dev.astype(np.int16) - ref.astype(np.int16))
            if kind in (RenderOutput.BEAUTY, RenderOutput.NORMAL, RenderOutput.ALBEDO):
                assert diff[..., :3].max() <= 1 and (diff[..., :3] > 0).mean() <= 2e-3, (kind, diff.max())
                assert np.array_equal(dev[..., 3], ref[..., 3]), kind
            else:
                assert np.array_equal(dev, ref), (kind, int((diff > 0).sum()))
