"""One-wave renders replayed as CUDA graphs, and the device-side output copy.

A render whose samples fit one wave is captured once per (tile, samples,
bounces) key and replayed on later calls; everything that changes between
calls (camera, sample index, accumulation) lives in the device job table and
the accumulation planes, not in the captured launches. The replayed renders
must equal plain launches (DK_RENDER_GRAPHS=0, in a child process) bit for
bit, across a camera change and an accumulation reset between replays.

`RenderSession.copy_output` (texture(for:), RenderSession.swift:1072-1094)
must hand over the same pixels as the host readback `pixels(for:)`.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SEQUENCE = r"""
import sys
import numpy as np
from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput, compile_scene, scenes
from denrimrendererkit_gb300.scene import Camera

def run(out_path):
    wl = scenes.cornell_box_reference(64, 48)
    cam = wl.scene.camera
    moved = Camera(tuple(np.add(cam.origin, (0.2, 0.05, 0))), cam.target, up=cam.up,
                   vertical_field_of_view_degrees=cam.vertical_field_of_view_degrees)
    frames = []
    with DenrimRenderer(0).make_session(wl.scene, wl.settings, build=compile_scene(wl.scene)) as s:
        s.render(4)                       # captured
        frames.append(s.pixels(RenderOutput.BEAUTY))
        s.render(4)                       # replayed, samples 4..7
        frames.append(s.pixels(RenderOutput.BEAUTY))
        s.update_camera(moved, cam)       # replayed with the new camera
        s.render(4)
        frames += [s.pixels(k) for k in RenderOutput]
        s.reset_accumulation()
        s.render(2)                       # another key
        s.render(4)
        frames.append(s.pixels(RenderOutput.BEAUTY))
        frames.append(np.array([s.sample_count], np.float32).reshape(1, 1, 1))
    np.savez(out_path, *frames)

run(sys.argv[1])
"""


def render_sequence(tmp_path, graphs: bool):
    out = tmp_path / f"frames_{int(graphs)}.npz"
    env = dict(os.environ, DK_RENDER_GRAPHS="1" if graphs else "0")
    env["PYTHONPATH"] = ROOT + os.pathsep + env.get("PYTHONPATH", "")
    subprocess.run([sys.executable, "-c", SEQUENCE, str(out)], cwd=ROOT, env=env, check=True, timeout=600)
    with np.load(out) as z:
        return [z[f"arr_{i}"] for i in range(len(z.files))]


def test_graph_replays_equal_plain_launches(dk_lib, tmp_path):
    graphed = render_sequence(tmp_path, True)
    plain = render_sequence(tmp_path, False)
    assert len(graphed) == len(plain)
    for i, (a, b) in enumerate(zip(graphed, plain)):
        assert a.shape == b.shape
        assert a.view(np.uint32).tobytes() == b.view(np.uint32).tobytes(), f"frame {i} differs"
    assert float(graphed[-1].reshape(-1)[0]) == 6.0
    assert graphed[0][..., :3].mean() > 0.01
    assert not np.array_equal(graphed[1], graphed[2])  # the camera move changed the image


def test_copy_output_equals_host_readback(dk_lib):
    import torch
    from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput, compile_scene, scenes
    wl = scenes.material_reference(40, 24)
    with DenrimRenderer(0).make_session(wl.scene, wl.settings, build=compile_scene(wl.scene)) as s:
        s.render(3)
        side = torch.cuda.Stream()
        for k in RenderOutput:
            host = s.pixels(k)
            dev = torch.full((24, 40, 4), -1.0, device="cuda")
            s.copy_output(k, dev)  # ordered on torch's current stream
            assert np.array_equal(dev.cpu().numpy().view(np.uint32), host.view(np.uint32)), k.name
            on_side = torch.full((24 * 40 * 4,), -1.0, device="cuda")
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                s.copy_output(k, on_side)
                got = on_side.view(24, 40, 4).clone()
            side.synchronize()
            assert np.array_equal(got.cpu().numpy().view(np.uint32), host.view(np.uint32)), k.name
        with pytest.raises(ValueError):
            s.copy_output(RenderOutput.BEAUTY, torch.empty(10, device="cuda"))


def test_server_copy_output_equals_host_readback(dk_lib):
    import torch
    from denrimrendererkit_gb300 import RenderOutput, compile_scene, scenes
    from denrimrendererkit_gb300.serving import RenderServer
    wl = scenes.material_reference(32, 16)
    with RenderServer(compile_scene(wl.scene)) as server:
        ids = [server.submit(wl.settings, wl.scene.camera, spp) for spp in (2, 5)]
        while server.step():
            pass
        for j in ids:
            for k in RenderOutput:
                host = server.pixels(j, k)
                dev = torch.full((16, 32, 4), -1.0, device="cuda")
                server.copy_output(j, k, dev)
                assert np.array_equal(dev.cpu().numpy().view(np.uint32), host.view(np.uint32)), k.name
        more = [server.submit(wl.settings, wl.scene.camera, spp) for spp in (1, 3, 4)]
        while server.step():
            pass
        for k in RenderOutput:
            batch = torch.full((3, 16, 32, 4), -1.0, device="cuda")
            server.copy_outputs(more, k, batch)
            for i, j in enumerate(more):
                host = server.pixels(j, k)
                assert np.array_equal(batch[i].cpu().numpy().view(np.uint32), host.view(np.uint32)), k.name
        for j in ids + more:
            server.release(j)


def test_session_created_while_another_renders(dk_lib):
    # Two sessions in flight, as the pipelined end-to-end loop runs them: one
    # is created (host traversal build, uploads) on a second thread while the
    # other renders; both images equal their one-at-a-time renders bit for bit.
    from concurrent.futures import ThreadPoolExecutor
    from denrimrendererkit_gb300 import RenderOutput, compile_scene, scenes
    from denrimrendererkit_gb300.renderer import RenderSession
    wl_a = scenes.spheres_large(width=192, height=108)
    wl_b = scenes.material_zoo()
    ba, bb = compile_scene(wl_a.scene), compile_scene(wl_b.scene)

    def run(build, wl):
        s = RenderSession(build, wl.settings, wl.scene.camera)
        s.render(4)
        img = s.pixels(RenderOutput.BEAUTY)
        ids = s.pixels(RenderOutput.OBJECT_ID)
        s.close()
        return img, ids

    solo_a, solo_b = run(ba, wl_a), run(bb, wl_b)
    with ThreadPoolExecutor(1) as ex:
        for _ in range(2):
            sa = RenderSession(ba, wl_a.settings, wl_a.scene.camera)
            fut = ex.submit(RenderSession, bb, wl_b.settings, wl_b.scene.camera)
            sa.render(4)
            got_a = (sa.pixels(RenderOutput.BEAUTY), sa.pixels(RenderOutput.OBJECT_ID))
            sa.close()
            sb = fut.result()
            sb.render(4)
            got_b = (sb.pixels(RenderOutput.BEAUTY), sb.pixels(RenderOutput.OBJECT_ID))
            sb.close()
            for got, want in ((got_a, solo_a), (got_b, solo_b)):
                for g, w in zip(got, want):
                    assert g.view(np.uint32).tobytes() == w.view(np.uint32).tobytes()
