"""The sparse distance-volume build on the GPU (dk_bake_sparse_sphere_volume)
against the host build (dk_build_sparse_sphere_volume, itself pinned by the
oracle tests of the reference's sparse-build cases): every output array --
volume descriptor, brick descriptors, packed samples (distance, materials,
blend), brick grid, grid + macro-occupancy indices -- equal byte for byte, on
small seeded models (ragged brick edges, hard and smooth unions, a single
sphere, a band that keeps nothing) and on the full 768^3 configuration.
"""
import time

import numpy as np
import pytest

from denrimrendererkit_gb300.library import SparseVolume

pytestmark = pytest.mark.gpu


def model(seed, count, smooth=0.05):
    rng = np.random.default_rng(seed)
    return [dict(center=rng.uniform(-0.85, 0.85, 3), radius=float(rng.uniform(0.03, 0.15)), material=i % 3,
                 smooth_union_radius=smooth if i % 4 else 0.0) for i in range(count)]


CASES = [
    ("ragged", model(1, 12), (50, 37, 29), (8, 8, 8), 0.05),
    ("hard-union", model(2, 9, smooth=0.0), (64, 64, 64), (8, 8, 8), 0.03),
    ("one-sphere", model(3, 1), (33, 33, 33), (4, 4, 4), 0.1),
    ("empty-band", [dict(center=(5.0, 5.0, 5.0), radius=0.1, material=0, smooth_union_radius=0.0)],
     (40, 40, 40), (8, 8, 8), 0.01),
    ("config-768", model(5, 32), (768, 768, 768), (8, 8, 8), 0.012),
]


@pytest.mark.parametrize("name,spheres,res,brick,band", CASES, ids=[c[0] for c in CASES])
def test_gpu_bake_equals_host_build(dk_lib, name, spheres, res, brick, band):
    from denrimrendererkit_gb300 import DenrimRenderer
    DenrimRenderer(0)
    args = (spheres, res, (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0), brick, band)
    t0 = time.perf_counter()
    host = SparseVolume(*args, on_device=False)
    t1 = time.perf_counter()
    dev = SparseVolume(*args, on_device=True)
    t2 = time.perf_counter()
    print(f"{name}: {len(host.bricks)} bricks, {len(host.samples)} samples; host {t1 - t0:.3f} s, "
          f"GPU bake {t2 - t1:.3f} s")
    for field in ("volumes", "bricks", "samples", "grids", "grid_indices"):
        a, b = getattr(host, field), getattr(dev, field)
        assert a.shape == b.shape, field
        assert a.tobytes() == b.tobytes(), field
    if name == "empty-band":
        assert len(host.bricks) == 0
    else:
        assert len(host.bricks) > 0
