"""SVGF, the reference's DenoiseSettings.appleSVGF (Denoiser.swift:67-76,
167-300).

Pinned: the reference's own helper kernels, packSVGFDepthNormalKernel and
copySVGFOutputKernel (Denoise.metal:117-154) compiled for the host, against
the numpy restatement (CPU) and the CUDA kernels (GPU), bit for bit,
including pixels without a surface and non-finite filter results.

Unpinned (the reference's filter is Apple's closed MPSSVGFDenoiser): the CUDA
filter against the numpy restatement of the published algorithm over a
rendered moving-camera sequence (relative RMS 1e-3: `exp`/`pow` intrinsics
against libm and contracted multiply-adds; history lengths equal but for
<0.5 % of pixels whose reprojection test sits on a threshold), and properties -- a constant image stays constant, static
frames integrate (history length grows, error falls below the raw frame's),
disoccluded pixels restart their history.
"""
import ctypes as C
import dataclasses

import numpy as np
import pytest

from oracle import svgf_oracle as so

f32 = np.float32


def reference_lib():
    from oracle import oracle as orc
    if not orc.reference_available():
        pytest.skip("reference shaders not built")
    lib = orc.load_reference()
    for name in ("ref_svgf_pack_depth_normal", "ref_svgf_copy_output"):
        fn = getattr(lib, name)
        fn.argtypes = [C.c_void_p] * 3 + [C.c_uint32] * 2
        fn.restype = C.c_int
    return lib


def helper_inputs(seed=4, w=23, h=17):
    rng = np.random.default_rng(seed)
    depth = np.repeat(rng.uniform(0.1, 9.0, (h, w, 1)).astype(f32), 4, -1)
    normal = rng.uniform(0, 1, (h, w, 4)).astype(f32)
    normal[..., 3] = 1.0
    normal[0, :5, 3] = 0.0          # no surface
    depth[1, :3, 0] = np.nan        # non-finite depth
    depth[2, :3, 0] = -1.0          # behind
    normal[3, 0, :3] = 0.5          # zero-length signed normal
    den = rng.normal(0.5, 1.0, (h, w, 4)).astype(f32)
    den[4, :4, 0] = np.nan
    den[5, :4, 1] = np.inf
    orig = rng.uniform(0, 2, (h, w, 4)).astype(f32)
    return depth, normal, den, orig


def ref_helpers(lib, depth, normal, den, orig):
    h, w = depth.shape[:2]
    dn = np.zeros_like(depth)
    out = np.zeros_like(orig)
    assert lib.ref_svgf_pack_depth_normal(depth.ctypes.data, normal.ctypes.data, dn.ctypes.data, w, h) == 0
    assert lib.ref_svgf_copy_output(den.ctypes.data, orig.ctypes.data, out.ctypes.data, w, h) == 0
    return dn, out


def same_bits(a, b):
    """Bit for bit, except that NaNs compare as NaNs (their payload is the
    platform's: libm and the GPU produce different canonical NaNs)."""
    a, b = np.asarray(a, f32), np.asarray(b, f32)
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32))


def test_restated_helpers_equal_reference_kernels():
    lib = reference_lib()
    depth, normal, den, orig = helper_inputs()
    dn, out = ref_helpers(lib, depth, normal, den, orig)
    assert same_bits(so.pack_depth_normal(depth, normal), dn)
    assert same_bits(so.copy_output(den, orig), out)


def test_oracle_constant_image_is_a_fixed_point():
    h, w = 20, 24
    beauty = np.full((h, w, 4), (0.3, 0.5, 0.7, 1.0), f32)
    depth = np.full((h, w, 4), 2.0, f32)
    normal = np.full((h, w, 4), (0.5, 0.5, 1.0, 1.0), f32)
    motion = np.zeros((h, w, 4), f32)
    motion[..., 3] = 1.0
    s = so.Svgf(w, h)
    p = so.params()
    for _ in range(3):
        out = s.denoise(beauty, depth, normal, motion, p)
        assert np.allclose(out, beauty, rtol=1e-6, atol=1e-7)


def test_oracle_integrates_static_frames_and_restarts_disocclusions():
    rng = np.random.default_rng(9)
    h, w = 24, 32
    truth = np.zeros((h, w, 4), f32)
    truth[..., 0] = np.linspace(0.2, 0.8, w)[None, :]
    truth[..., 1] = 0.4
    truth[..., 2] = np.linspace(0.6, 0.1, h)[:, None]
    truth[..., 3] = 1.0
    depth = np.full((h, w, 4), 3.0, f32)
    normal = np.full((h, w, 4), (0.5, 0.5, 1.0, 1.0), f32)
    motion = np.zeros((h, w, 4), f32)
    motion[..., 3] = 1.0
    s = so.Svgf(w, h)
    p = so.params()
    hist_errs = []
    for k in range(8):
        noisy = truth.copy()
        noisy[..., :3] *= rng.exponential(1.0, (h, w, 1)).astype(f32)
        out = s.denoise(noisy, depth, normal, motion, p)
        err = np.sqrt(((out[..., :3] - truth[..., :3]) ** 2).mean())
        raw = np.sqrt(((noisy[..., :3] - truth[..., :3]) ** 2).mean())
        assert err < 0.3 * raw
        hist_errs.append(np.sqrt(((s.prev[1][..., :3] - truth[..., :3]) ** 2).mean()))
    # the temporally integrated history converges (the output's a-trous
    # strength follows the per-frame variance, so it settles instead)
    assert hist_errs[-1] < 0.4 * hist_errs[0]
    assert (s.prev[2][..., 2] == 8).all()
    # a depth jump in the left half: its history restarts
    depth2 = depth.copy()
    depth2[:, : w // 2, :] = 6.0
    s.denoise(truth, depth2, normal, motion, p)
    hist = s.prev[2][..., 2]
    assert (hist[:, : w // 2] == 1).all() and (hist[:, w // 2:] == 9).all()


# ---------------------------------------------------------------- GPU ---
def device(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.gpu
def test_cuda_helpers_equal_reference_kernels(dk_lib):
    import torch
    from denrimrendererkit_gb300 import library
    lib = reference_lib()
    depth, normal, den, orig = helper_inputs(w=37, h=19)
    dn_ref, out_ref = ref_helpers(lib, depth, normal, den, orig)
    h, w = depth.shape[:2]
    dn = torch.zeros(h, w, 4, device="cuda")
    out = torch.zeros(h, w, 4, device="cuda")
    d, n, de, o = (device(a) for a in (depth, normal, den, orig))
    library.check(dk_lib.dk_svgf_pack_depth_normal(C.c_void_p(d.data_ptr()), C.c_void_p(n.data_ptr()),
                                                   C.c_void_p(dn.data_ptr()), w, h, None))
    library.check(dk_lib.dk_svgf_copy_output(C.c_void_p(de.data_ptr()), C.c_void_p(o.data_ptr()),
                                             C.c_void_p(out.data_ptr()), w, h, None))
    torch.cuda.synchronize()
    assert same_bits(dn.cpu().numpy(), dn_ref)
    assert same_bits(out.cpu().numpy(), out_ref)
    # planes are float4: a misaligned pointer is refused before any launch
    rc = dk_lib.dk_svgf_copy_output(C.c_void_p(de.data_ptr() + 4), C.c_void_p(o.data_ptr()),
                                    C.c_void_p(out.data_ptr()), w, h, None)
    assert rc == 6  # DK_ERROR_INVALID_ARGUMENT


def render_frames(count, moves, width=48, height=40, spp=1):
    """Frames of the Cornell box, one frame seed each, the camera sliding by
    `moves[k]` between frames; the motion AOV comes from the previous camera."""
    from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput, compile_scene, scenes
    from denrimrendererkit_gb300.scene import Camera
    wl = scenes.cornell_box_reference(width, height)
    b = compile_scene(wl.scene)
    cam = wl.scene.camera
    r = DenrimRenderer(0)
    frames, prev = [], cam
    for k in range(count):
        dx = moves[k]
        cur = Camera(tuple(np.add(prev.origin, (dx, 0, 0))), tuple(np.add(prev.target, (dx, 0, 0))), up=cam.up,
                     vertical_field_of_view_degrees=cam.vertical_field_of_view_degrees)
        st = dataclasses.replace(wl.settings, frame_seed=100 + k, denoise=True, previous_camera=prev)
        wl.scene.camera = cur
        with r.make_session(wl.scene, st, build=b) as s:
            s.render(spp)
            frames.append({kind: s.pixels(kind) for kind in (RenderOutput.BEAUTY, RenderOutput.DEPTH,
                                                             RenderOutput.NORMAL, RenderOutput.MOTION_VECTOR)})
        prev = cur
    return frames


@pytest.mark.gpu
def test_cuda_svgf_equals_restatement_on_a_moving_camera(dk_lib):
    import torch
    from denrimrendererkit_gb300 import RenderOutput
    from denrimrendererkit_gb300.denoiser import SvgfDenoiser
    frames = render_frames(5, [0.0, 0.03, 0.03, 0.0, 0.05], spp=2)
    h, w = frames[0][RenderOutput.BEAUTY].shape[:2]
    gpu = SvgfDenoiser(w, h)
    cpu = so.Svgf(w, h)
    p = so.params()
    out = torch.empty(h, w, 4, device="cuda")
    for k, f in enumerate(frames):
        b, d, n, m = (f[kind] for kind in (RenderOutput.BEAUTY, RenderOutput.DEPTH, RenderOutput.NORMAL,
                                           RenderOutput.MOTION_VECTOR))
        gpu.denoise(device(b), device(d), device(n), device(m), out)
        want = cpu.denoise(b, d, n, m, p)
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert np.array_equal(got[..., 3], want[..., 3])
        rel = np.sqrt(((got[..., :3] - want[..., :3]) ** 2).mean()) / max(float(want[..., :3].mean()), 1e-9)
        assert rel < 1e-3, (k, rel)
        lengths = gpu.state(1)[..., 2].cpu().numpy()
        # reprojection tests sitting on a threshold may flip between the two
        off = np.abs(lengths - cpu.prev[2][..., 2]) > 1e-3
        assert off.mean() < 0.005, (k, off.mean())
        if k > 0:
            # most surface pixels reprojected through the motion vectors
            surf = d[..., 0] > 0
            assert (lengths[surf] > 1).mean() > 0.8, (k, (lengths[surf] > 1).mean())
    gpu.reset()
    gpu.denoise(device(b), device(d), device(n), device(m), out)
    assert (gpu.state(1)[..., 2] == 1).all()


@pytest.mark.gpu
def test_cuda_svgf_static_frames_converge(dk_lib):
    import torch
    from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput, compile_scene, scenes
    from denrimrendererkit_gb300.denoiser import SvgfDenoiser
    frames = render_frames(8, [0.0] * 8)
    wl = scenes.cornell_box_reference(48, 40)
    with DenrimRenderer(0).make_session(wl.scene, dataclasses.replace(wl.settings, frame_seed=7),
                                        build=compile_scene(wl.scene)) as s:
        s.render(512)
        truth = s.pixels(RenderOutput.BEAUTY)[..., :3]
    h, w = truth.shape[:2]
    gpu = SvgfDenoiser(w, h)
    out = torch.empty(h, w, 4, device="cuda")
    errs, hist_errs = [], []
    for f in frames:
        gpu.denoise(*(device(f[k]) for k in (RenderOutput.BEAUTY, RenderOutput.DEPTH, RenderOutput.NORMAL,
                                             RenderOutput.MOTION_VECTOR)), out)
        errs.append(float(np.sqrt(((out.cpu().numpy()[..., :3] - truth) ** 2).mean())))
        hist_errs.append(float(np.sqrt(((gpu.state(0).cpu().numpy()[..., :3] - truth) ** 2).mean())))
    raw = float(np.sqrt(((frames[-1][RenderOutput.BEAUTY][..., :3] - truth) ** 2).mean()))
    lengths = gpu.state(1)[..., 2].cpu().numpy()
    surf = frames[-1][RenderOutput.DEPTH][..., 0] > 0
    assert (lengths[surf] == 8).mean() > 0.95
    assert max(errs) < 0.7 * raw, (errs, raw)
    # the history's error is mostly the blur across the box's edges: it
    # still falls as frames integrate
    assert hist_errs[-1] < 0.92 * hist_errs[0], hist_errs


def test_oracle_reprojection_follows_the_motion_convention():
    # The motion AOV is previousScreen - currentScreen (PathTrace.metal:5569-5577): content that moved one
    # pixel right has motion (-1, 0), and its history comes from one pixel to the left.  Stripes one pixel
    # wide: with the right convention the blended history equals the new frame exactly; with the sign
    # flipped it would mix the neighbouring stripes.
    h, w = 12, 20
    xs = np.arange(w)
    pattern = np.zeros((h, w, 4), f32)
    pattern[..., 0] = (xs % 2)[None, :] * 0.8 + 0.1
    pattern[..., 1] = 0.3
    pattern[..., 2] = ((xs // 2) % 2)[None, :] * 0.5 + 0.2
    pattern[..., 3] = 1.0
    depth = np.full((h, w, 4), 2.0, f32)
    normal = np.full((h, w, 4), (0.5, 0.5, 1.0, 1.0), f32)
    still = np.zeros((h, w, 4), f32)
    still[..., 3] = 1.0
    s = so.Svgf(w, h)
    p = so.params()
    s.denoise(pattern, depth, normal, still, p)
    moved = np.roll(pattern, 1, axis=1)
    motion = still.copy()
    motion[..., 0] = -1.0
    s.denoise(moved, depth, normal, motion, p)
    length = s.prev[2][..., 2]
    assert (length[:, 1:] == 2).all() and (length[:, 0] == 1).all()
    # the integrated luminance moments of the interior equal the moved frame's (no stripe mixing)
    lum = so.luminance(moved[..., :3])
    assert np.allclose(s.prev[2][:, 1:, 0], lum[:, 1:], rtol=1e-6, atol=1e-7)
