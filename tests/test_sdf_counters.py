"""The reference's SDF traversal counters (PathTrace.metal:191-214, read by
RenderSession.sdfTraversalStats, RenderSession.swift:808-831) on the GPU:
collected only when the session asks for them, against the CPU oracle's
counts of the same walk (the oracle's counters are pinned against the
reference shader itself, tests/test_reference_shader.py), and the cases of
RenderSessionTests.swift:806-860 (cells visited >= empty cells + brick tests,
marches, march steps and hits on a sparse scene; reset to zero)."""
import numpy as np
import pytest

from denrimrendererkit_gb300 import DenrimRenderer, compile_scene, scenes

pytestmark = pytest.mark.gpu

PAIRS = (("sparse_grid_cells_visited", "grid_cells"), ("sparse_grid_macro_skips", "macro_skips"),
         ("sparse_brick_tests", "brick_tests"), ("sparse_brick_range_culls", "range_culls"),
         ("sparse_brick_marches", "brick_marches"), ("sparse_brick_march_steps", "march_steps"),
         ("sparse_brick_hits", "brick_hits"))


@pytest.fixture(scope="module")
def renderer(dk_lib):
    return DenrimRenderer(0)


def sdf_workload(bounces):
    wl = scenes.sdf_spheres(width=64, height=64, resolution=192)
    wl.settings.collects_traversal_stats = True
    wl.settings.max_bounces = bounces
    return wl


def gpu_and_oracle_counts(renderer, oracle_lib, wl, spp):
    b = compile_scene(wl.scene)
    with renderer.make_session(wl.scene, wl.settings, build=b) as s:
        s.render(spp)
        gpu = s.sdf_traversal_stats()
    o = oracle_lib.OracleRender(b, wl.settings, wl.scene.camera)
    o.render(spp)
    return gpu, o.counter_dict()


def test_primary_walk_counts_equal_the_oracle(renderer, oracle_lib):
    # One bounce: every ray is a camera ray, bit-exact with the oracle's, so
    # every grid cell, macro skip, brick test, cull, march step and hit is the same.
    wl = sdf_workload(1)
    gpu, ref = gpu_and_oracle_counts(renderer, oracle_lib, wl, 4)
    for mine, theirs in PAIRS:
        assert gpu[mine] == ref[theirs], f"{mine}: GPU {gpu[mine]} oracle {ref[theirs]}"
    assert gpu["primary_scene_queries"] == 64 * 64 * 4
    assert gpu["sparse_brick_hits"] > 0 and gpu["sparse_brick_range_culls"] > 0
    assert gpu["sparse_grid_cells_visited"] >= gpu["sparse_grid_empty_cells"] + gpu["sparse_brick_tests"]
    assert gpu["dense_volume_tests"] == 0 and gpu["dense_march_steps"] == 0 and gpu["sparse_brick_invalid"] == 0


def test_full_path_counts_track_the_oracle(renderer, oracle_lib):
    # Eight bounces: the bounce directions agree with the oracle's to rounding,
    # so a few walks may differ; the totals agree within 1 %.
    wl = sdf_workload(8)
    gpu, ref = gpu_and_oracle_counts(renderer, oracle_lib, wl, 4)
    for mine, theirs in PAIRS:
        assert abs(gpu[mine] - ref[theirs]) <= 0.01 * max(ref[theirs], 100), f"{mine}: GPU {gpu[mine]} oracle {ref[theirs]}"
    assert gpu["primary_scene_queries"] == 64 * 64 * 4
    assert gpu["bounce_scene_queries"] > 0


def test_counters_need_the_setting_accumulate_and_reset(renderer):
    wl = scenes.sdf_spheres(width=32, height=32, resolution=192)
    wl.settings.max_bounces = 1
    b = compile_scene(wl.scene)
    with renderer.make_session(wl.scene, wl.settings, build=b) as s:
        s.render(2)
        assert all(v == 0 for v in s.sdf_traversal_stats().values())
    wl.settings.collects_traversal_stats = True
    with renderer.make_session(wl.scene, wl.settings, build=b) as s:
        s.render(2)
        first = s.sdf_traversal_stats()
        s.render(2)
        second = s.sdf_traversal_stats()
        assert first["primary_scene_queries"] == 32 * 32 * 2 and second["primary_scene_queries"] == 32 * 32 * 4
        assert second["sparse_grid_cells_visited"] > first["sparse_grid_cells_visited"] > 0
        s.reset_sdf_traversal_stats()
        assert all(v == 0 for v in s.sdf_traversal_stats().values())


def test_triangle_scene_counts_queries(renderer):
    wl = scenes.cornell_box_reference(32, 32)
    wl.settings.collects_traversal_stats = True
    wl.settings.max_bounces = 3
    b = compile_scene(wl.scene)
    with renderer.make_session(wl.scene, wl.settings, build=b) as s:
        s.render(2)
        st = s.sdf_traversal_stats()
    assert st["primary_scene_queries"] == 32 * 32 * 2
    assert st["bounce_scene_queries"] > 0 and st["shadow_scene_queries"] > 0
    assert st["sparse_grid_cells_visited"] == 0 and st["sparse_brick_tests"] == 0
