"""Serving (dk_server_*): jobs packed into shared waves render exactly what
each renders alone, admission honours the HBM budget, and invalid jobs are
refused at submission.

The equality bar is bit-exactness: a path depends only on its pixel, sample
index, frame seed and the job's own materials and settings, and every pixel
accumulates its samples in sample order whatever the wave composition."""
import dataclasses
import threading
import time

import numpy as np
import pytest

from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput, abi, compile_scene, library, scenes
from denrimrendererkit_gb300.presets import PRESETS
from denrimrendererkit_gb300.renderer import RenderQuality, RenderSettings
from denrimrendererkit_gb300.scene import Camera, Material
from denrimrendererkit_gb300.serving import RenderServer, ServerConfig

pytestmark = pytest.mark.gpu

OUTPUTS = (RenderOutput.BEAUTY, RenderOutput.DEPTH, RenderOutput.NORMAL, RenderOutput.ALBEDO,
           RenderOutput.MATERIAL_ID, RenderOutput.OBJECT_ID, RenderOutput.MOTION_VECTOR)


@pytest.fixture(scope="module")
def preview(dk_lib):
    DenrimRenderer(0)
    scene = scenes.material_preview(hdri=scenes.synthetic_hdri(512, 256))
    return scene, compile_scene(scene)


def _table(build, sphere: Material):
    t = build.materials.copy()
    t[1] = sphere.gpu_material()
    return t


def _jobs():
    glass = Material(base_color=(0.92, 0.98, 0.98), roughness=0.01, index_of_refraction=1.45, transmission=1.0,
                     transmission_color=(0.96, 1.0, 1.0), transmission_roughness=0.01)
    cam2 = Camera((0.4, 0.9, 2.4), (0.0, 0.45, 0.0), vertical_field_of_view_degrees=40.0)
    return [
        (96, 96, 16, PRESETS["metal.gold"], None),
        (256, 256, 24, PRESETS["subsurface.skin-warm"], None),
        (128, 64, 40, PRESETS["coating.iridescent-amber"], cam2),
        (200, 150, 8, PRESETS["fabric.velvet-purple"], None),
        (64, 64, 20, glass, None),  # transmissive: the shadow layer walk under the job's own opacity mask
    ]


def _settings(w, h, **kw):
    return RenderSettings(width=w, height=h, max_bounces=8, quality=RenderQuality.FINAL, frame_seed=1, **kw)


def _solo(scene, build, w, h, spp, table, cam):
    b2 = dataclasses.replace(build, materials=table)
    with DenrimRenderer(0).make_session(scene, _settings(w, h), build=b2) as s:
        if cam is not None:
            s.update_camera(cam, cam)
        s.render(spp)
        return {o: s.pixels(o) for o in OUTPUTS}


def _assert_same(a, b, what):
    for o in OUTPUTS:
        assert np.array_equal(a[o].view(np.uint32), b[o].view(np.uint32)), f"{what}: {o.name} differs"


def test_jobs_in_a_mix_equal_their_solo_renders(preview):
    scene, build = preview
    jobs = _jobs()
    # Small waves: every job is split over several waves and shares each with others.
    with RenderServer(build, ServerConfig(wave_paths=1 << 19, samples_per_wave=8)) as srv:
        ids = [srv.submit(_settings(w, h), cam or scene.camera, spp, _table(build, m)) for w, h, spp, m, cam in jobs]
        steps = 0
        while any(srv.status(i).state != abi.JOB_DONE for i in ids):
            assert srv.step() > 0
            steps += 1
        stats = srv.stats()
        assert stats["max_jobs_in_wave"] >= 3 and stats["waves"] == steps
        assert max(srv.status(i).waves for i in ids) > 1  # split over waves
        for jid, (w, h, spp, m, cam) in zip(ids, jobs):
            st = srv.status(jid)
            assert st.samples_done == spp and st.waves >= 1
            got = {o: srv.pixels(jid, o) for o in OUTPUTS}
            _assert_same(got, _solo(scene, build, w, h, spp, _table(build, m), cam), f"job {jid}")
            assert np.isfinite(got[RenderOutput.BEAUTY]).all() and got[RenderOutput.BEAUTY][..., :3].mean() > 0


def test_background_loop_with_arrivals_and_budget(preview):
    scene, build = preview
    jobs = _jobs() * 2
    per_job = max(w * h for w, h, *_ in jobs) * 164
    budget = int(per_job * 2.5)  # at most two or three resident jobs: admission must wait for releases
    results = {}
    with RenderServer(build, ServerConfig(hbm_budget_bytes=budget, wave_paths=1 << 20, samples_per_wave=16)) as srv:
        srv.start()
        ids = []
        lock = threading.Lock()

        def drain():
            pending = list(range(len(jobs)))
            while pending:
                for k in list(pending):
                    with lock:
                        if k >= len(ids):
                            continue
                        jid = ids[k]
                    if srv.status(jid).state == abi.JOB_DONE:
                        results[k] = srv.pixels(jid, RenderOutput.BEAUTY)
                        srv.release(jid)
                        pending.remove(k)
                time.sleep(0.002)

        t = threading.Thread(target=drain)
        t.start()
        for w, h, spp, m, cam in jobs:
            jid = srv.submit(_settings(w, h), cam or scene.camera, spp, _table(build, m))
            with lock:
                ids.append(jid)
            time.sleep(0.005)
        t.join(timeout=300)
        assert not t.is_alive()
        stats = srv.stats()
        srv.stop()
    assert stats["jobs_done"] == len(jobs) and stats["budget_peak_bytes"] <= budget
    for k, (w, h, spp, m, cam) in enumerate(jobs[:len(_jobs())]):
        solo = _solo(scene, build, w, h, spp, _table(build, m), cam)[RenderOutput.BEAUTY]
        assert np.array_equal(results[k].view(np.uint32), solo.view(np.uint32))
        assert np.array_equal(results[k + len(_jobs())].view(np.uint32), solo.view(np.uint32))


def test_invalid_jobs_are_refused(preview):
    scene, build = preview
    with RenderServer(build, ServerConfig(wave_paths=1 << 16)) as srv:
        t = _table(build, PRESETS["metal.gold"])
        with pytest.raises(library.DenrimError):
            srv.submit(_settings(64, 64), scene.camera, 4, t[:1])  # wrong material count
        bad = t.copy()
        bad[1]["emission"] = (1.0, 1.0, 1.0, 0.0)
        with pytest.raises(library.DenrimError):
            srv.submit(_settings(64, 64), scene.camera, 4, bad)  # emission changes the light list
        with pytest.raises(library.DenrimError):
            srv.submit(_settings(512, 512), scene.camera, 4, t)  # a frame exceeds the 65,536-path wave
        with pytest.raises(library.DenrimError):
            srv.submit(_settings(64, 64), scene.camera, 0, t)
        jid = srv.submit(_settings(64, 64), scene.camera, 2, t)
        with pytest.raises(library.DenrimError):
            srv.release(jid)  # not finished
        while srv.status(jid).state != abi.JOB_DONE:
            srv.step()
        srv.release(jid)
        with pytest.raises(library.DenrimError):
            srv.pixels(jid)


def test_jobs_across_resident_scenes_equal_their_solo_renders(preview):
    # Two resident scenes in one server: the preview scene and the small
    # Cornell box (another BVH, light list and environment).  Jobs of both
    # scenes share every step -- one packed wave per scene, the two waves on
    # their own streams -- and each renders what it renders alone.
    scene, build = preview
    box = scenes.cornell_small(width=64, height=48)
    box_build = compile_scene(box.scene)
    with RenderServer(build, ServerConfig(wave_paths=1 << 18, samples_per_wave=6)) as srv:
        b_idx = srv.add_scene(box_build)
        assert b_idx == 1
        jobs = [(0, 96, 96, 12, PRESETS["metal.gold"]), (1, 64, 48, 10, None), (0, 128, 64, 9,
                PRESETS["fabric.velvet-purple"]), (1, 80, 60, 7, None)]
        ids = []
        for sc, w, h, spp, m in jobs:
            if sc == 0:
                ids.append(srv.submit(_settings(w, h), scene.camera, spp, _table(build, m)))
            else:
                ids.append(srv.submit(_settings(w, h), box.scene.camera, spp, scene=1))
        while any(srv.status(i).state != abi.JOB_DONE for i in ids):
            assert srv.step() > 0
        stats = srv.stats()
        assert stats["waves"] > 2
        for jid, (sc, w, h, spp, m) in zip(ids, jobs):
            got = {o: srv.pixels(jid, o) for o in OUTPUTS}
            if sc == 0:
                want = _solo(scene, build, w, h, spp, _table(build, m), None)
            else:
                want = _solo(box.scene, box_build, w, h, spp, box_build.materials, None)
            _assert_same(got, want, f"scene {sc} job {jid}")
        with pytest.raises(ValueError):
            srv.submit(_settings(32, 32), scene.camera, 1, scene=2)  # no such scene
