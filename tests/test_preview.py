"""RenderQuality.preview and .interactive: the flat preview
(flatPreviewKernel, PathTrace.metal:4728-4868) and the direct-light material
preview (interactiveMaterialKernel, :4870-5165), against the reference's own
kernels compiled for the host (oracle/_ref).

Bar: primary-hit AOVs (depth, normal, albedo, material/object ID, motion)
bit-exact -- camera ray, traversal and the normal/albedo encodings use
correctly rounded operations on both sides; beauty within relative RMSE
1e-4 (preview) and 2e-3 (interactive: `pow`, the environment's `atan2`/`acos`
and FMA contraction in the light loop differ in the last bits, and a light or
occlusion probe sitting exactly on a threshold can flip), 5x that on the
large scene, whose HDRI holds a 1e4x sun; image means within 0.5 %.
"""
import numpy as np
import pytest

from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput, compile_scene, scenes
from denrimrendererkit_gb300.renderer import RenderQuality, RenderSettings

AOVS = (RenderOutput.DEPTH, RenderOutput.NORMAL, RenderOutput.ALBEDO, RenderOutput.MATERIAL_ID,
        RenderOutput.OBJECT_ID, RenderOutput.MOTION_VECTOR)


def reference_or_skip():
    from oracle import oracle as orc
    if not orc.reference_available():
        pytest.skip("reference shaders not built")
    return orc


def with_quality(wl, quality, width=None, height=None):
    st = wl.settings
    wl.settings = RenderSettings(width=width or st.width, height=height or st.height, max_bounces=st.max_bounces,
                                 quality=quality, transparent_background=st.transparent_background,
                                 shows_environment_background=st.shows_environment_background,
                                 background_color=st.background_color)
    return wl


@pytest.mark.parametrize("quality", [RenderQuality.PREVIEW, RenderQuality.INTERACTIVE])
def test_reference_preview_kernels_overwrite_each_sample(quality):
    # The reference previews write (not accumulate) the image and ignore the
    # sample index: 1 and 3 samples give the same bytes (what lets the GPU
    # path run one pass for any sample count).
    orc = reference_or_skip()
    from oracle.oracle import HostBuilders
    wl = with_quality(scenes.material_reference(24, 24), quality)
    b = compile_scene(wl.scene, host_builders=HostBuilders())
    r1 = orc.ReferenceRender(b, wl.settings, wl.scene.camera)
    r1.render(1)
    r3 = orc.ReferenceRender(b, wl.settings, wl.scene.camera)
    r3.render(3)
    assert np.array_equal(r1.accum, r3.accum) and np.array_equal(r1.aov, r3.aov)
    assert np.isfinite(r1.accum).all() and r1.accum[..., :3].mean() > 0.01


CASES = [
    ("cornell", lambda: scenes.cornell_box_reference(48, 40)),
    ("materials", lambda: scenes.material_reference()),
    ("zoo", lambda: scenes.material_zoo()),
    ("large", lambda: scenes.spheres_large(width=160, height=90)),
    ("sdf", lambda: scenes.sdf_spheres(width=64, height=64, resolution=192)),
    ("transparent", lambda: scenes.transparent_export_scene()),
]


@pytest.mark.gpu
@pytest.mark.parametrize("quality", [RenderQuality.PREVIEW, RenderQuality.INTERACTIVE])
@pytest.mark.parametrize("name,maker", CASES, ids=[c[0] for c in CASES])
def test_cuda_preview_matches_reference_kernel(dk_lib, quality, name, maker):
    orc = reference_or_skip()
    wl = with_quality(maker(), quality)
    b = compile_scene(wl.scene)
    renderer = DenrimRenderer(0)
    with renderer.make_session(wl.scene, wl.settings, build=b) as s:
        s.render(2)
        assert s.sample_count == 2
        got = {k: s.pixels(k) for k in (RenderOutput.BEAUTY,) + AOVS}
    ref = orc.ReferenceRender(b, wl.settings, wl.scene.camera)
    ref.render(1)
    for kind in AOVS:
        g = got[kind].view(np.uint32)
        c = ref.aov[int(kind) - 1].view(np.uint32)
        bad = (g != c).any(axis=-1)
        assert not bad.any(), f"{name} {quality.name} {kind.name}: {int(bad.sum())} pixels differ"
    g = got[RenderOutput.BEAUTY].astype(np.float64)
    c = ref.accum.astype(np.float64)
    assert np.isfinite(g).all()
    assert np.array_equal(g[..., 3], c[..., 3])
    rel = np.sqrt(((g[..., :3] - c[..., :3]) ** 2).mean()) / max(c[..., :3].mean(), 1e-12)
    tol = 1e-4 if quality == RenderQuality.PREVIEW else 2e-3
    if name == "large":  # a 1e4x sun in the HDRI magnifies last-bit atan2/acos differences of env lookups
        tol *= 5.0
    assert rel <= tol, (name, quality.name, rel)
    assert abs(g[..., :3].mean() - c[..., :3].mean()) <= 5e-3 * c[..., :3].mean()
