"""The denoisers on rendered images.

* The spatial filter (dk_denoise_spatial) against the reference's own
  simpleSpatialDenoiseKernel (Denoise.metal:39-115) compiled for the host
  (oracle/_ref): the same arithmetic up to the last bits of `exp`, so a
  relative tolerance of 1e-5 per texel.
* The U-Net trained on the GPU by the library's kernels on pairs the tracer
  renders (4 spp + AOVs -> 512 spp): on held-out scene variants it must beat
  both the 4-spp input (by half) and the spatial filter in relative RMSE of
  the displayed image (the reference's PNG tone curve) against the converged
  render -- what the network gains over the method without it.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput, compile_scene, scenes  # noqa: E402
from denrimrendererkit_gb300.denoiser import (UNet, display_relative_rmse, relative_rmse, render_pairs,  # noqa: E402
                                              spatial_denoise, train)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def renderer(dk_lib):
    return DenrimRenderer(0)


def test_spatial_filter_matches_reference_kernel(renderer, oracle_lib):
    from oracle import oracle as orc
    if not orc.reference_available():
        pytest.skip("reference shaders not built")
    lib = orc.load_reference()
    wl = scenes.cornell_variant(5, 96, 64)
    b = compile_scene(wl.scene)
    with renderer.make_session(wl.scene, wl.settings, build=b) as s:
        s.render(4)
        planes = {k: s.pixels(k) for k in (RenderOutput.BEAUTY, RenderOutput.DEPTH, RenderOutput.NORMAL,
                                           RenderOutput.ALBEDO)}
    dev = {k: torch.from_numpy(v).cuda() for k, v in planes.items()}
    for iterations, sigmas in ((1, (0.18, 0.03, 0.25, 1.0)), (3, (0.18, 0.03, 0.25, 1.0)), (5, (0.18, 0.08, 0.25, 4.0))):
        out = torch.empty_like(dev[RenderOutput.BEAUTY])
        spatial_denoise(dev[RenderOutput.BEAUTY], dev[RenderOutput.DEPTH], dev[RenderOutput.NORMAL],
                        dev[RenderOutput.ALBEDO], out, 96, 64, 2, *sigmas, iterations)
        torch.cuda.synchronize()
        ref = np.zeros_like(planes[RenderOutput.BEAUTY])
        import ctypes as C
        lib.ref_denoise_spatial.argtypes = [C.c_void_p] * 5 + [C.c_uint32] * 3 + [C.c_float] * 4 + [C.c_uint32]
        rc = lib.ref_denoise_spatial(planes[RenderOutput.BEAUTY].ctypes.data, planes[RenderOutput.DEPTH].ctypes.data,
                                     planes[RenderOutput.NORMAL].ctypes.data, planes[RenderOutput.ALBEDO].ctypes.data,
                                     ref.ctypes.data, 96, 64, 2, *sigmas, iterations)
        assert rc == 0
        got = out.cpu().numpy()
        assert np.allclose(got, ref, rtol=1e-5, atol=1e-6), float(np.abs(got - ref).max())
        assert not np.array_equal(got, planes[RenderOutput.BEAUTY])


def test_unet_trained_on_rendered_pairs_beats_input_and_spatial_filter(renderer):
    size = 256
    train_set = render_pairs(range(48), size=size, noisy_spp=4, target_spp=512)
    held_out = render_pairs(range(1000, 1004), size=size, noisy_spp=4, target_spp=512)
    net = UNet(seed=1)
    losses = train(net, train_set, steps=1500, batch=16, crop=128, lr=1e-3, log_every=100)
    assert losses[-1] < 0.7 * losses[0], losses
    noisy, spatial, learned, lin = [], [], [], []
    for k in range(held_out.count):
        out = torch.empty_like(held_out.beauty[k])
        net.denoise(held_out.beauty[k], held_out.albedo[k], held_out.normal[k], held_out.depth[k], size, size, out)
        sp = torch.empty_like(out)
        spatial_denoise(held_out.beauty[k], held_out.depth[k], held_out.normal[k], held_out.albedo[k], sp, size, size)
        torch.cuda.synchronize()
        t = held_out.target[k]
        noisy.append(display_relative_rmse(held_out.beauty[k], t))
        spatial.append(display_relative_rmse(sp, t))
        learned.append(display_relative_rmse(out, t))
        lin.append((relative_rmse(held_out.beauty[k], t), relative_rmse(sp, t), relative_rmse(out, t)))
    n, s, l = np.mean(noisy), np.mean(spatial), np.mean(learned)
    print(f"display relative RMSE on held-out variants: 4 spp {n:.4f}, spatial filter {s:.4f}, U-Net {l:.4f}; "
          f"linear: {np.mean(lin, axis=0)}; losses {losses}")
    assert l < 0.5 * n and l < s


def test_error_terms_match_a_float64_reduction(renderer):
    # dk_denoise_error_terms against the same sums in FP64 on the host, for a
    # batch of images of a size that is not a multiple of the block.
    from denrimrendererkit_gb300.denoiser import estimate_errors
    import ctypes as C
    from denrimrendererkit_gb300 import library
    g = torch.Generator(device="cuda").manual_seed(3)
    n, h, w = 3, 37, 53
    planes = [torch.rand(n, h, w, 4, generator=g, device="cuda") + 0.1 * k for k in range(6)]
    terms = torch.empty(n, 5, dtype=torch.float64, device="cuda")
    library.check(library.load().dk_denoise_error_terms(*(C.c_void_p(p.data_ptr()) for p in planes), h * w, n, 0,
                                                        C.c_void_p(terms.data_ptr()), None))
    torch.cuda.synchronize()
    a, b, f, da, db, df = (p[..., :3].double().cpu() for p in planes)
    want = torch.stack([((da - db) ** 2).sum((1, 2, 3)), ((a - b) ** 2).sum((1, 2, 3)), ((f - df) ** 2).sum((1, 2, 3)),
                        df.sum((1, 2, 3)), f.sum((1, 2, 3))], 1)
    assert torch.allclose(terms.cpu(), want, rtol=1e-9, atol=0)
    est = estimate_errors(*planes)
    assert len(est) == n and all(e.denoised >= e.noise >= 0 and e.plain > 0 for e in est)
    # the displayed-image sums: the reference's tone curve applied to every plane first
    from denrimrendererkit_gb300.denoiser import display
    library.check(library.load().dk_denoise_error_terms(*(C.c_void_p(p.data_ptr()) for p in planes), h * w, n, 1,
                                                        C.c_void_p(terms.data_ptr()), None))
    torch.cuda.synchronize()
    a, b, f, da, db, df = (display(p).cpu() for p in planes)
    want = torch.stack([((da - db) ** 2).sum((1, 2, 3)), ((a - b) ** 2).sum((1, 2, 3)), ((f - df) ** 2).sum((1, 2, 3)),
                        df.sum((1, 2, 3)), f.sum((1, 2, 3))], 1)
    assert torch.allclose(terms.cpu(), want, rtol=1e-5, atol=1e-6)


def test_serving_to_an_error_target_falls_back_to_more_samples(renderer):
    # denoiser.serve_to_error_target through the render server: a target every
    # estimate meets returns the denoised images after the first round; one no
    # estimate can meet grows the samples round after round up to max_spp and
    # returns the plain renders (the fallback).
    from denrimrendererkit_gb300.denoiser import UNet, serve_to_error_target
    from denrimrendererkit_gb300.serving import RenderServer, ServerConfig
    wl = scenes.cornell_variant(7, 64, 64)
    b = compile_scene(wl.scene)
    net = UNet(seed=1)
    reqs = [(wl.settings, wl.scene.camera, None, 0), (wl.settings, wl.scene.camera, None, 0)]
    with RenderServer(b, ServerConfig(wave_paths=1 << 20)) as srv:
        loose = serve_to_error_target(srv, net, reqs, 64, 64, target=10.0, start_spp=8)
        assert all(x.denoised and x.spp == 8 and x.rounds == 1 for x in loose)
        tight = serve_to_error_target(srv, net, reqs, 64, 64, target=1e-6, start_spp=8, max_spp=64)
        assert all(not x.denoised and x.spp == 64 and x.rounds == 3 for x in tight)  # 8 -> 32 -> 64
        for x in tight:
            img = x.image.cpu().numpy()
            assert np.isfinite(img).all() and img[..., :3].mean() > 0
            assert x.estimate.plain > 1e-6
        assert srv.stats()["jobs_submitted"] == 2 * 2 + 2 * (2 + 1 + 1)
