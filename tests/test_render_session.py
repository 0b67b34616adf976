"""Cases of the reference's RenderSessionTests
(Tests/DenrimRendererKitTests/RenderSessionTests.swift) on the session's
denoised beauty and deep paths, restated through the CUDA path:
* testSimpleSpatialDenoiserFiltersBeautyOutput (:1971-2023) and
  testAppleSVGFDenoiserFiltersBeautyOutput (:2025-2070): with
  `RenderSettings.denoise` set, the beauty output is the filtered image --
  finite, and different from the raw beauty on average;
* testDeepFlatBVHRenderUsesEnergyPreservingTerminationPath (:1890-1909): the
  Cornell box at 6 bounces renders finite, non-black pixels after one sample.
Beyond the reference: the session's filtered beauty equals the standalone
filter over the session's own planes bit for bit, PNG export and display
bytes use it, and a new sample makes it stale.
"""
import numpy as np
import pytest

from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput, compile_scene, image, scenes
from denrimrendererkit_gb300.renderer import DenoiseSettings, RenderDenoiser, RenderQuality, RenderSettings

pytestmark = pytest.mark.gpu


def raw_and_denoised(denoise):
    wl = scenes.material_reference()
    b = compile_scene(wl.scene)
    r = DenrimRenderer(0)
    with r.make_session(wl.scene, RenderSettings(width=32, height=32, max_bounces=2), build=b) as raw, \
            r.make_session(wl.scene, RenderSettings(width=32, height=32, max_bounces=2, denoise=denoise),
                           build=b) as den:
        raw.render_next_sample()
        den.render_next_sample()
        return raw.pixels(RenderOutput.BEAUTY).reshape(-1, 4), den.pixels(RenderOutput.BEAUTY).reshape(-1, 4)


SPATIAL = DenoiseSettings(RenderDenoiser.SIMPLE_SPATIAL, radius=2, normal_sigma=0.25, depth_sigma=0.04,
                          albedo_sigma=0.35, color_sigma=8.0)


@pytest.mark.parametrize("denoise", [SPATIAL, DenoiseSettings.APPLE_SVGF], ids=["simple-spatial", "svgf"])
def test_denoiser_filters_beauty_output(dk_lib, denoise):
    raw, den = raw_and_denoised(denoise)
    assert raw.shape == den.shape
    assert np.isfinite(den).all()
    assert np.abs(raw[:, :3] - den[:, :3]).sum() / max(1, raw.shape[0] * 3) > 0.000001


def test_deep_render_uses_energy_preserving_termination(dk_lib):
    wl = scenes.cornell_box_reference()
    with DenrimRenderer(0).make_session(wl.scene, RenderSettings(width=20, height=20, max_bounces=6)) as s:
        s.render_next_sample()
        px = s.pixels(RenderOutput.BEAUTY).reshape(-1, 4)
        assert s.sample_count == 1
    ok = np.isfinite(px[:, :3]).all(1) & (px[:, :3] > 0).any(1)
    assert ok.any()


def test_session_filtered_beauty_is_the_filter_over_its_planes(dk_lib, tmp_path):
    import torch
    from denrimrendererkit_gb300.denoiser import spatial_denoise
    wl = scenes.material_reference()
    # final quality: each sample adds to the image (preview overwrites it identically)
    settings = RenderSettings(width=40, height=24, max_bounces=2, quality=RenderQuality.FINAL, denoise=SPATIAL)
    with DenrimRenderer(0).make_session(wl.scene, settings) as s:
        s.render(2)
        got = s.pixels(RenderOutput.BEAUTY)
        planes = {k: s.copy_output(k, torch.empty(24, 40, 4, device="cuda"))
                  for k in (RenderOutput.BEAUTY, RenderOutput.DEPTH, RenderOutput.NORMAL, RenderOutput.ALBEDO)}
        want = torch.empty(24, 40, 4, device="cuda")
        spatial_denoise(planes[RenderOutput.BEAUTY], planes[RenderOutput.DEPTH], planes[RenderOutput.NORMAL],
                        planes[RenderOutput.ALBEDO], want, 40, 24, radius=2, normal_sigma=0.25, depth_sigma=0.04,
                        albedo_sigma=0.35, color_sigma=8.0, iterations=3)
        assert np.array_equal(got.view(np.uint32), want.cpu().numpy().view(np.uint32))
        # PNG export and display bytes show the filtered image
        path = str(tmp_path / "beauty.png")
        s.write_png(path)
        assert np.array_equal(image.read_png(path), s.rgba8())
        # stale after a new sample
        s.render(1)
        assert not np.array_equal(s.pixels(RenderOutput.BEAUTY), got)
