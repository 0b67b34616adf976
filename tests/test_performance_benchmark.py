"""The reference's PerformanceBenchmarkTests
(Tests/DenrimRendererKitTests/PerformanceBenchmarkTests.swift:6-96): session
creation and render time and pixel-samples/s for the Cornell box (128^2,
4 bounces, 8 samples), the material reference (128^2, 4 bounces, 8 samples)
and a distance-volume scene (128^2, 3 bounces, 4 samples), printed as the
reference's PERF lines and asserted positive.  The reference gates them
behind DENRIM_RUN_PERFORMANCE_TESTS=1; they are cheap here and always run.
The reference's distance-volume scene is a dense volume (out of scope for
the CUDA path); the sparse-brick sphere scene stands in for it."""
import time

import pytest

from denrimrendererkit_gb300 import DenrimRenderer, scenes
from denrimrendererkit_gb300.renderer import RenderSettings

pytestmark = pytest.mark.gpu

CASES = [
    ("cornell", lambda: scenes.cornell_box_reference().scene, 4, 8),
    ("materials", lambda: scenes.material_reference().scene, 4, 8),
    ("distance-volume", lambda: scenes.sdf_spheres(width=128, height=128, resolution=192).scene, 3, 4),
]


@pytest.mark.parametrize("name,make,bounces,samples", CASES, ids=[c[0] for c in CASES])
def test_render_throughput(dk_lib, name, make, bounces, samples):
    renderer = DenrimRenderer(0)
    scene = make()
    start = time.perf_counter()
    session = renderer.make_session(scene, RenderSettings(width=128, height=128, max_bounces=bounces))
    session_seconds = time.perf_counter() - start
    render_start = time.perf_counter()
    session.render(samples)
    render_seconds = time.perf_counter() - render_start
    session.close()
    pixel_samples_per_second = 128 * 128 * samples / max(render_seconds, 1e-9)
    print(f"PERF {name} device=GB300 sessionSeconds={session_seconds} renderSeconds={render_seconds} "
          f"pixelSamplesPerSecond={pixel_samples_per_second}")
    assert session_seconds > 0 and render_seconds > 0 and pixel_samples_per_second > 0
