"""The oracle against the reference's own known-answer tests for this path.

Each case restates an assertion of the reference XCTests (file:line cited) and
checks the CPU oracle against it, so that the oracle is pinned before it judges
the CUDA kernels.
"""
import math

import numpy as np
import pytest

from denrimrendererkit_gb300 import abi, scenes
from denrimrendererkit_gb300.scene import Environment, Material, Mesh, RenderScene, Texture2D, Transform


def quad_tris(a, b, c, d, material=0):
    return Mesh.quad(a, b, c, d).gpu_triangles(material)


def test_bvh_empty(oracle_lib):
    # BVHBuilderTests.testEmptyBVHBuildsWithoutNodes (BVHBuilderTests.swift:6-11)
    nodes, prim = oracle_lib.build_bvh(np.zeros(0, abi.TRIANGLE_DTYPE))
    assert len(nodes) == 0 and len(prim) == 0


def test_bvh_single_leaf_and_flatten(oracle_lib):
    # BVHBuilderTests.swift:13-27 and BVHFlattenerTests.swift:7-26
    tris = quad_tris((-1, -1, 0), (1, -1, 0), (1, 1, 0), (-1, 1, 0))
    nodes, prim = oracle_lib.build_bvh(tris, 4)
    assert len(nodes) == 1
    assert list(prim) == [0, 1]
    assert list(nodes[0]["metadata"]) == [0, 0, 0, 2]
    assert nodes[0]["bounds_min"][0] == pytest.approx(-1, abs=1e-4)
    assert nodes[0]["bounds_max"][0] == pytest.approx(1, abs=1e-4)


def test_bvh_splits_large_set(oracle_lib):
    # BVHBuilderTests.testBVHSplitsLargePrimitiveSet (BVHBuilderTests.swift:29-48)
    tris = np.concatenate([quad_tris((x, 0, 0), (x + 0.5, 0, 0), (x + 0.5, 0.5, 0), (x, 0.5, 0)) for x in range(8)])
    nodes, prim = oracle_lib.build_bvh(tris, 2)
    assert nodes[0]["metadata"][3] == 0 and len(nodes) > 1
    assert sorted(prim.tolist()) == list(range(len(tris)))
    assert max(n["metadata"][3] for n in nodes) <= 2
    assert nodes[0]["bounds_min"][0] == pytest.approx(0, abs=1e-4)
    assert nodes[0]["bounds_max"][0] == pytest.approx(7.5, abs=1e-4)


def test_bvh_interior_children(oracle_lib):
    # BVHFlattenerTests.testFlattenedInteriorStoresChildIndices (:28-47)
    tris = np.concatenate([quad_tris((x, 0, 0), (x + 0.5, 0, 0), (x + 0.5, 0.5, 0), (x, 0.5, 0)) for x in range(4)])
    nodes, prim = oracle_lib.build_bvh(tris, 2)
    assert len(nodes) > 1
    assert nodes[0]["metadata"][3] == 0
    left, right = int(nodes[0]["metadata"][0]), int(nodes[0]["metadata"][1])
    assert left == 1 and right > left  # pre-order numbering
    assert sorted(prim.tolist()) == list(range(8))


def test_cornell_build_bounds(oracle_lib):
    # BVHFlattenerTests.testAccelerationBackendBuildsFlatBVH (:49-58)
    from denrimrendererkit_gb300.scene import compile_scene
    wl = scenes.cornell_box_reference()
    tris = np.concatenate([inst.mesh.gpu_triangles(inst.material, inst.transform, i)
                           for i, inst in enumerate(wl.scene.mesh_instances)])
    nodes, prim = oracle_lib.build_bvh(tris, 4)
    assert len(wl.scene.mesh_instances) == 6
    assert len(prim) == len(tris)
    assert nodes[0]["bounds_min"][0] == pytest.approx(-1, abs=1e-4)
    assert nodes[0]["bounds_max"][1] == pytest.approx(2, abs=1e-4)


def _materials(*mats):
    return np.array([m.gpu_material() for m in mats], abi.MATERIAL_DTYPE)


def test_light_list(oracle_lib):
    # BVHFlattenerTests.testAccelerationBackendBuildsEmissiveTriangleLightList (:60-94)
    mats = _materials(Material(base_color=(0.8, 0.8, 0.8)),
                      Material(base_color=(1, 1, 1), emission=(1, 0.8, 0.6), emission_strength=4))
    tris = np.concatenate([quad_tris((-1, 0, 1), (1, 0, 1), (1, 0, -1), (-1, 0, -1), 0),
                           quad_tris((-0.5, 1, -0.5), (0.5, 1, -0.5), (0.5, 1, 0.5), (-0.5, 1, 0.5), 1)])
    tagged, lights = oracle_lib.build_lights(tris, mats)
    assert len(tagged) == 4
    assert lights["triangle_index"].tolist() == [2, 3]
    assert all(mats[l["material_index"]]["emission"][0] > 0 for l in lights)
    assert np.allclose(lights["area"], 0.5, atol=1e-4)
    assert (lights["normal"][:, 1] < -0.99).all()
    assert tagged["padding2"][2] == 1 and tagged["padding2"][3] == 2
    assert lights["selection_cdf"][-1] == pytest.approx(1, abs=1e-4)


def test_light_power_cdf(oracle_lib):
    # BVHFlattenerTests.testAccelerationBackendBuildsPowerWeightedLightSelectionCDF (:96-134)
    mats = _materials(Material(base_color=(1, 1, 1), emission=(1, 1, 1), emission_strength=1),
                      Material(base_color=(1, 1, 1), emission=(1, 1, 1), emission_strength=3))
    tris = np.concatenate([quad_tris((-1, 0, 1), (0, 0, 1), (0, 0, 0), (-1, 0, 0), 0),
                           quad_tris((0, 0, 1), (1, 0, 1), (1, 0, 0), (0, 0, 0), 1)])
    tagged, lights = oracle_lib.build_lights(tris, mats)
    assert len(lights) == 4
    assert lights["selection_cdf"][-1] == pytest.approx(1, abs=1e-4)
    assert (np.diff(lights["selection_cdf"]) > 0).all()
    assert lights["selection_cdf"][1] == pytest.approx(0.25, abs=1e-4)
    assert tagged["padding2"].tolist() == [1, 2, 3, 4]


def test_light_list_empty_without_emission(oracle_lib):
    # BVHFlattenerTests.testAccelerationBackendLeavesLightListEmptyWithoutEmission (:136-151)
    mats = _materials(Material(base_color=(0.8, 0.8, 0.8)))
    tagged, lights = oracle_lib.build_lights(quad_tris((-1, -1, 0), (1, -1, 0), (1, 1, 0), (-1, 1, 0)), mats)
    assert len(tagged) == 2 and len(lights) == 0


def test_environment_distribution(oracle_lib):
    # BVHFlattenerTests.testAccelerationBackendBuildsEnvironmentImportanceDistribution (:153-183)
    px = np.array([[1, 1, 1, 1], [3, 3, 3, 1]], np.float32)
    env = oracle_lib.build_environment_samples(px, 2, 1, 1.0, 0.0)
    assert len(env) == 2
    assert env["cdf"][0] == pytest.approx(0.25, abs=1e-4)
    assert env["cdf"][1] == pytest.approx(1.0, abs=1e-4)
    assert env["pdf_solid_angle"][1] > env["pdf_solid_angle"][0]


def _single_quad_build(material=7, transform=None):
    scene = RenderScene()
    for _ in range(material + 1):
        scene.add_material(Material(base_color=(0.8, 0.8, 0.8)))
    tris = Mesh.quad((-1, -1, 0), (1, -1, 0), (1, 1, 0), (-1, 1, 0)).gpu_triangles(material, transform, 0)
    from oracle import oracle as orc
    nodes, prim = orc.build_bvh(tris)
    from denrimrendererkit_gb300.scene import AccelerationBuild
    mats = np.array([m.gpu_material() for m in scene.materials], abi.MATERIAL_DTYPE)
    z = lambda dt: np.zeros(0, dt)  # noqa: E731
    return AccelerationBuild(tris, mats, nodes, prim, z(abi.TEXTURE_DESCRIPTOR_DTYPE), np.zeros((0, 4), np.float32),
                             z(abi.LIGHT_DTYPE), z(abi.ENVIRONMENT_SAMPLE_DTYPE), 0, 1.0, 0.0, 16.0)


def test_intersect_quad_hit(oracle_lib):
    # CPUIntersectorTests.testRayHitsQuad (CPUIntersectorTests.swift:6-28)
    b = _single_quad_build(7)
    h = oracle_lib.intersect(b, (0, 0, 2), (0, 0, -1))
    assert h["hit"] == 1 and h["material_id"] == 7
    assert h["t"] == pytest.approx(2, abs=1e-4)
    assert (h["px"], h["py"], h["pz"]) == pytest.approx((0, 0, 0), abs=1e-4)
    assert h["nz"] == pytest.approx(1, abs=1e-4)


def test_intersect_quad_miss(oracle_lib):
    # CPUIntersectorTests.testRayMissesQuad (:30-47)
    h = oracle_lib.intersect(_single_quad_build(0), (2, 0, 2), (0, 0, -1))
    assert h["hit"] == 0


def test_intersect_translated_quad(oracle_lib):
    # CPUIntersectorTests.testRayHitsTranslatedQuad (:49-71)
    b = _single_quad_build(1, Transform.translation((2, 0, 0)))
    h = oracle_lib.intersect(b, (2, 0, 2), (0, 0, -1))
    assert h["hit"] == 1
    assert h["t"] == pytest.approx(2, abs=1e-4)
    assert h["px"] == pytest.approx(2, abs=1e-4) and h["pz"] == pytest.approx(0, abs=1e-4)


def test_rng_hash_chain(oracle_lib):
    # hash / randomFloat (PathTrace.metal:255-268): known values of the
    # xorshift-multiply hash and the 24-bit uniform.
    def ref_hash(v):
        v &= 0xFFFFFFFF
        v ^= v >> 16
        v = (v * 0x7FEB352D) & 0xFFFFFFFF
        v ^= v >> 15
        v = (v * 0x846CA68B) & 0xFFFFFFFF
        v ^= v >> 16
        return v

    for v in (0, 1, 2, 0x1234ABCD, 0xFFFFFFFF, 123456789):
        assert oracle_lib.hash_u32(v) == ref_hash(v)
    state = 1 ^ ref_hash(5 + 7 * 320) ^ ref_hash(3 + 1)
    seq = oracle_lib.random_sequence(state, 8)
    s = state
    for x in seq:
        s = ref_hash(s)
        assert x == (s & 0xFFFFFF) / 16777216.0
    assert np.array_equal(seq, oracle_lib.random_sequence(state, 8, fp64=True))


def test_oracle_fp32_vs_fp64_small(oracle_lib):
    """The FP32 build and the FP64 build agree on a converging statistic
    (mean radiance of the small Cornell configuration at 2 spp), and the
    integer AOVs (IDs) of the two builds are identical."""
    from denrimrendererkit_gb300.scene import compile_scene
    wl = scenes.cornell_small(width=64, height=36)
    b = compile_scene(wl.scene)
    r32 = oracle_lib.OracleRender(b, wl.settings, wl.scene.camera)
    r64 = oracle_lib.OracleRender(b, wl.settings, wl.scene.camera, fp64=True)
    r32.render(2)
    r64.render(2)
    assert np.array_equal(r32.aov[3], r64.aov[3]) and np.array_equal(r32.aov[4], r64.aov[4])
    m32, m64 = r32.accum[..., :3].mean(), r64.accum[..., :3].mean()
    assert abs(m32 - m64) / m64 < 0.05


# ------------------------------------------------------------ sparse bricks --
def _sdf_build(spheres, resolution, brick, band, camera, settings=None):
    from denrimrendererkit_gb300 import library
    from denrimrendererkit_gb300.scene import compile_scene
    scene = RenderScene(camera=camera)
    scene.add_material(Material(base_color=(0.2, 0.65, 0.9), roughness=0.55))
    scene.sparse_volumes.append(library.SparseVolume(spheres, (resolution,) * 3, (-1, -1, -1), (1, 1, 1),
                                                     (brick,) * 3, band, volume_material=0))
    return scene, compile_scene(scene)


def test_sparse_sphere_known_hit(oracle_lib, dk_lib):
    # The geometry of CPUIntersectorTests.testRayHitsDistanceVolumeSphere
    # (CPUIntersectorTests.swift:73-89): r = 0.5 sphere on a 24^3 grid over
    # [-1, 1]^3, ray from z = 2 towards -z hits at t = 1.5 +- 0.08, normal +z.
    from denrimrendererkit_gb300.scene import Camera
    _, b = _sdf_build([dict(center=(0, 0, 0), radius=0.5, material=0)], 24, 8, 0.3, Camera((0, 0, 3), (0, 0, 0)))
    h = oracle_lib.intersect(b, (0, 0, 2), (0, 0, -1))
    assert h["hit"] == 1
    assert h["t"] == pytest.approx(1.5, abs=0.08)
    assert h["pz"] == pytest.approx(0.5, abs=0.08)
    assert h["nz"] == pytest.approx(1.0, abs=0.08)
    assert oracle_lib.intersect(b, (2, 2, 2), (0, 0, -1))["hit"] == 0


def test_sparse_volume_only_scene_uses_brick_path(oracle_lib, dk_lib):
    # RenderSessionTests.testSparseVolumeOnlySceneRendersThroughBrickPathOnFlatPath
    # (RenderSessionTests.swift:806-860): sphere r = 0.55, resolution 20, brick 5,
    # band 0.3, orthographic camera (scale 2.4), 20x20, 1 bounce.
    from denrimrendererkit_gb300.renderer import RenderQuality, RenderSettings
    from denrimrendererkit_gb300.scene import Camera
    cam = Camera((0, 0, 3), (0, 0, 0), orthographic_scale=2.4)
    scene, b = _sdf_build([dict(center=(0, 0, 0), radius=0.55, material=0)], 20, 5, 0.3, cam)
    settings = RenderSettings(width=20, height=20, max_bounces=1, quality=RenderQuality.FINAL)
    r = oracle_lib.OracleRender(b, settings, cam)
    r.render(1)
    c = r.counter_dict()
    assert c["grid_cells"] > 0 and c["brick_tests"] > 0 and c["brick_marches"] > 0
    assert c["march_steps"] > 0 and c["brick_hits"] > 0
    albedo = r.aov[2].reshape(-1, 4)
    assert ((albedo[:, 0] < 0.35) & (albedo[:, 1] > 0.45) & (albedo[:, 2] > 0.65) & (albedo[:, 3] > 0.9)).any()


def test_sparse_brick_without_zero_crossing_is_culled(oracle_lib):
    # RenderSessionTests.testSparseBrickWithoutZeroCrossingIsCulledBeforeMarch
    # (RenderSessionTests.swift:862-919): one 3^3 brick, all distances 0.05.
    from denrimrendererkit_gb300.renderer import RenderQuality, RenderSettings
    from denrimrendererkit_gb300.scene import AccelerationBuild, Camera
    cam = Camera((0, 0, 3), (0, 0, 0), orthographic_scale=2.0)
    mats = _materials(Material(base_color=(0.8, 0.2, 0.2)))
    vol = np.zeros(1, abi.VOLUME_DTYPE)
    vol["world_bounds_min"][0] = vol["local_bounds_min"][0] = (-1, -1, -1, 0)
    vol["world_bounds_max"][0] = vol["local_bounds_max"][0] = (1, 1, 1, 0)
    vol["dimensions"][0] = (3, 3, 3, 0)
    vol["metadata"][0] = (0, 0, 0, 1)
    vol["material_program"][0] = (0xFFFFFFFF, 0, 0, 0)
    vol["world_to_local"][0] = np.eye(4)
    vol["normal_transform"][0] = np.eye(4)
    brick = np.zeros(1, abi.BRICK_DTYPE)
    brick["world_bounds_min"][0] = brick["local_bounds_min"][0] = (-1, -1, -1, 0)
    brick["world_bounds_max"][0] = brick["local_bounds_max"][0] = (1, 1, 1, 0)
    brick["sample_bounds_min"][0] = (-1, -1, -1, 0.05)
    brick["sample_bounds_max"][0] = (1, 1, 1, 0.05)
    brick["dimensions_and_sample_offset"][0] = (3, 3, 3, 0)
    samples = np.zeros(27, abi.BRICK_SAMPLE_DTYPE)
    samples["distance"] = 0.05
    grid = np.zeros(1, abi.BRICK_GRID_DTYPE)
    grid["dimensions_and_index_offset"][0] = (1, 1, 1, 0)
    grid["brick_size_and_volume"][0] = (3, 3, 3, 0)
    grid["macro_dimensions_and_index_offset"][0] = (1, 1, 1, 1)
    grid["macro_size_and_reserved"][0] = (4, 4, 4, 0)
    gidx = np.array([0, 1], np.uint32)
    z = lambda dt: np.zeros(0, dt)  # noqa: E731
    b = AccelerationBuild(z(abi.TRIANGLE_DTYPE), mats, z(abi.NODE_DTYPE), z(np.uint32), z(abi.TEXTURE_DESCRIPTOR_DTYPE),
                          np.zeros((0, 4), np.float32), z(abi.LIGHT_DTYPE), z(abi.ENVIRONMENT_SAMPLE_DTYPE), 0, 1.0, 0.0,
                          16.0, volumes=vol, volume_bricks=brick, volume_brick_samples=samples,
                          volume_brick_grids=grid, volume_brick_grid_indices=gidx)
    r = oracle_lib.OracleRender(b, RenderSettings(width=8, height=8, max_bounces=1, quality=RenderQuality.FINAL), cam)
    r.render(1)
    c = r.counter_dict()
    assert c["grid_cells"] > 0 and c["brick_tests"] > 0 and c["range_culls"] > 0
    assert c["brick_marches"] == 0 and c["march_steps"] == 0 and c["brick_hits"] == 0
