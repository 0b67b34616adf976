"""The learned denoiser's kernels against a plain PyTorch FP32 reference on the
CPU: convolution forward (with bias, ReLU, channel slices, accumulation), its
input gradient (tap-flipped transposed weights) and weight gradient, and the
full network's loss gradient w.r.t. every weight and bias.

Tolerances follow from bf16 operands and activations with FP32 accumulation:
a single convolution is compared at relative RMS error <= 1e-2 (bf16 rounding
of the output, 2^-8), whole-network gradients at <= 6e-2."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from denrimrendererkit_gb300 import library  # noqa: E402
from denrimrendererkit_gb300.denoiser import IN_CH, LEVELS, OUT_CH, UNet, _ptr  # noqa: E402

pytestmark = pytest.mark.gpu


def rel_rms(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(((a - b) ** 2).mean()) / max(np.sqrt((b ** 2).mean()), 1e-30))


def to_torch_weight(w):  # [co][9][ci] -> [co][ci][3][3]
    co, _, ci = w.shape
    return w.reshape(co, 3, 3, ci).permute(0, 3, 1, 2).contiguous()


@pytest.fixture(scope="module", params=[3, 2, 1, 0], ids=["halo_tcgen05", "tma_tcgen05", "cpasync_tcgen05",
                                                          "mma_sync"])
def lib(dk_lib, request):
    """Runs every test with each convolution kernel: the halo-row TMA + tcgen05
    kernel where a layer fits it, else the per-tap one (the default), the
    per-tap persistent TMA + tcgen05 kernel alone, cp.async + tcgen05, and
    mma.sync."""
    import ctypes as C
    from denrimrendererkit_gb300 import DenrimRenderer
    DenrimRenderer(0)
    lib = library.load()
    library.check(lib.dk_unet_set_conv_path(request.param))
    yield lib
    err = C.c_int(0)
    library.check(lib.dk_unet_error(C.byref(err)))
    library.check(lib.dk_unet_set_conv_path(3))
    assert err.value == 0, "a tensor-core wait timed out"


@pytest.mark.parametrize("cin,cout,act,ldi_extra,ldo_extra,co_off", [
    (16, 32, 1, 0, 0, 0), (32, 16, 0, 16, 32, 32), (96, 96, 1, 0, 0, 0), (160, 64, 1, 32, 0, 0),
    (288, 128, 1, 0, 64, 32)])
def test_conv3x3_forward(lib, cin, cout, act, ldi_extra, ldo_extra, co_off):
    g = torch.Generator().manual_seed(cin * 7 + cout)
    n, h, w = 2, 13, 37  # not multiples of the tiles: ragged edges
    ldi, ldo = cin + ldi_extra, cout + ldo_extra + co_off
    x = torch.randn(n, h, w, ldi, generator=g).to(torch.bfloat16)
    wt = (torch.randn(cout, 9, cin, generator=g) / (3 * cin ** 0.5)).to(torch.bfloat16)
    b = torch.randn(cout, generator=g) * 0.1
    prior = torch.randn(n, h, w, ldo, generator=g).to(torch.bfloat16)
    for accumulate in (0, 1):
        xd, wd, bd = x.cuda(), wt.cuda(), b.cuda()
        out = prior.clone().cuda()
        library.check(lib.dk_unet_conv3x3(_ptr(xd), n, h, w, cin, ldi, _ptr(wd), _ptr(bd), cout, _ptr(out), ldo,
                                          co_off, act, accumulate, None))
        torch.cuda.synchronize()
        got = out.cpu().float()
        ref = torch.nn.functional.conv2d(x[..., :cin].float().permute(0, 3, 1, 2), to_torch_weight(wt.float()),
                                         b, padding=1).permute(0, 2, 3, 1)
        if act:
            ref = torch.relu(ref)
        if accumulate:
            ref = ref + prior[..., co_off:co_off + cout].float()
        assert rel_rms(got[..., co_off:co_off + cout], ref) <= 1e-2
        untouched = torch.cat([got[..., :co_off], got[..., co_off + cout:]], -1)
        expect = torch.cat([prior[..., :co_off], prior[..., co_off + cout:]], -1).float()
        assert torch.equal(untouched, expect)


@pytest.mark.parametrize("cin,cout,act,ldi_extra,ldo_extra,co_off", [
    (16, 32, 1, 0, 0, 0), (32, 32, 1, 32, 0, 0), (96, 32, 1, 0, 64, 64), (32, 16, 0, 0, 0, 0), (64, 64, 1, 0, 0, 0),
    (64, 96, 1, 0, 0, 0), (128, 32, 1, 0, 0, 0), (48, 32, 1, 0, 0, 0), (80, 16, 1, 0, 0, 0), (112, 64, 1, 0, 0, 0),
    (160, 64, 1, 32, 0, 0), (224, 96, 1, 0, 32, 32), (288, 128, 1, 0, 0, 0), (96, 96, 1, 0, 0, 0),
    (176, 160, 0, 16, 0, 0)])
def test_conv3x3_forward_wide(lib, cin, cout, act, ldi_extra, ldo_extra, co_off):
    # Images at least 128 pixels wide (the halo-row kernel's layers, and the
    # row-tap mode of the per-tap kernel for the layers whose weights do not
    # fit the halo kernel), with a partial last tile column.
    g = torch.Generator().manual_seed(cin * 11 + cout)
    n, h, w = 2, 9, 200
    ldi, ldo = cin + ldi_extra, cout + ldo_extra + co_off
    x = torch.randn(n, h, w, ldi, generator=g).to(torch.bfloat16)
    wt = (torch.randn(cout, 9, cin, generator=g) / (3 * cin ** 0.5)).to(torch.bfloat16)
    b = torch.randn(cout, generator=g) * 0.1
    prior = torch.randn(n, h, w, ldo, generator=g).to(torch.bfloat16)
    ref = torch.nn.functional.conv2d(x[..., :cin].float().permute(0, 3, 1, 2), to_torch_weight(wt.float()), b,
                                     padding=1).permute(0, 2, 3, 1)
    if act:
        ref = torch.relu(ref)
    xd, wd, bd = x.cuda(), wt.cuda(), b.cuda()  # held: the kernel reads them after this statement
    for accumulate in (0, 1):
        out = prior.clone().cuda()
        library.check(lib.dk_unet_conv3x3(_ptr(xd), n, h, w, cin, ldi, _ptr(wd), _ptr(bd), cout, _ptr(out), ldo,
                                          co_off, act, accumulate, None))
        torch.cuda.synchronize()
        got = out.cpu().float()
        want = ref + prior[..., co_off:co_off + cout].float() if accumulate else ref
        assert rel_rms(got[..., co_off:co_off + cout], want) <= 1e-2
        untouched = torch.cat([got[..., :co_off], got[..., co_off + cout:]], -1)
        expect = torch.cat([prior[..., :co_off], prior[..., co_off + cout:]], -1).float()
        assert torch.equal(untouched, expect)


@pytest.mark.parametrize("cin,cout", [(32, 32), (96, 32), (64, 64), (32, 16), (48, 32), (80, 16), (144, 32),
                                       (160, 64)])
def test_conv3x3_forward_tall(lib, cin, cout):
    # About 40 output rows per persistent CTA, crossing tile columns and
    # images: the halo-row ring (up to 16 slots) and the stacked-tap
    # accumulator window (8 to 32 slots) wrap, and the MMAs at a segment's
    # first and last rows and at the window's wrap take the per-tap form.
    # Three input chunks (144, 160): the per-tap kernel's row-tap mode.
    g = torch.Generator().manual_seed(cin + 7 * cout)
    n, h, w = 3, 1000, 136
    x = torch.randn(n, h, w, cin, generator=g).to(torch.bfloat16)
    wt = (torch.randn(cout, 9, cin, generator=g) / (3 * cin ** 0.5)).to(torch.bfloat16)
    b = torch.randn(cout, generator=g) * 0.1
    ref = torch.relu(torch.nn.functional.conv2d(x.float().permute(0, 3, 1, 2), to_torch_weight(wt.float()), b,
                                                padding=1)).permute(0, 2, 3, 1)
    xd, wd, bd = x.cuda(), wt.cuda(), b.cuda()
    out = torch.zeros(n, h, w, cout, dtype=torch.bfloat16, device="cuda")
    library.check(lib.dk_unet_conv3x3(_ptr(xd), n, h, w, cin, cin, _ptr(wd), _ptr(bd), cout, _ptr(out), cout, 0, 1, 0,
                                      None))
    torch.cuda.synchronize()
    assert rel_rms(out.cpu().float(), ref) <= 1e-2


@pytest.mark.parametrize("cin,cout,ldo_extra,co_off,n,h,w", [
    (32, 32, 64, 64, 3, 200, 136),   # the first level's second convolution: 32 of 96 channels at offset 64
    (32, 32, 0, 0, 3, 1000, 136),    # ~40 rows per CTA: rings and accumulator windows wrap
    (64, 64, 96, 96, 2, 34, 130),    # the second level's, ragged right tile, row pairs across images
    (16, 32, 0, 0, 1, 16, 128),      # fewer row pairs than CTAs: CTAs with empty ranges
    (48, 16, 16, 0, 2, 64, 256),
    (96, 96, 0, 0, 1, 32, 160),      # not a tensor-store layer: convolution and pooling run separately
    (32, 32, 0, 0, 2, 8, 48),        # narrower than one 128-pixel tile: the per-tap kernel
])
def test_conv3x3_avgpool2_equals_its_two_steps(lib, cin, cout, ldo_extra, co_off, n, h, w):
    # The fused call writes the convolution's output and the 2x2 average of it;
    # the average must be the pooling kernel's over that output bit for bit,
    # channels outside the slices stay untouched, and the output matches the
    # plain convolution call and FP32.
    g = torch.Generator().manual_seed(cin + 5 * cout + h)
    x = torch.randn(n, h, w, cin, generator=g).to(torch.bfloat16)
    wt = (torch.randn(cout, 9, cin, generator=g) / (3 * cin ** 0.5)).to(torch.bfloat16)
    b = torch.randn(cout, generator=g) * 0.1
    ref = torch.relu(torch.nn.functional.conv2d(x.float().permute(0, 3, 1, 2), to_torch_weight(wt.float()), b,
                                                padding=1)).permute(0, 2, 3, 1)
    xd, wd, bd = x.cuda(), wt.cuda(), b.cuda()
    ldo, pld = cout + ldo_extra, cout + 16
    out = torch.full((n, h, w, ldo), 3.0, dtype=torch.bfloat16, device="cuda")
    pool = torch.full((n, h // 2, w // 2, pld), 7.0, dtype=torch.bfloat16, device="cuda")
    library.check(lib.dk_unet_conv3x3_avgpool2(_ptr(xd), n, h, w, cin, cin, _ptr(wd), _ptr(bd), cout, _ptr(out), ldo,
                                               co_off, 1, _ptr(pool), pld, None))
    plain = torch.zeros(n, h, w, cout, dtype=torch.bfloat16, device="cuda")
    library.check(lib.dk_unet_conv3x3(_ptr(xd), n, h, w, cin, cin, _ptr(wd), _ptr(bd), cout, _ptr(plain), cout, 0, 1,
                                      0, None))
    check = torch.zeros(n, h // 2, w // 2, cout, dtype=torch.bfloat16, device="cuda")
    library.check(lib.dk_unet_avgpool2(_ptr(out, co_off), ldo, _ptr(check), cout, 0, cout, n, h, w, None))
    torch.cuda.synchronize()
    got = out[..., co_off:co_off + cout].cpu()
    assert torch.equal(pool[..., :cout].cpu(), check.cpu())
    assert bool((pool[..., cout:] == 7.0).all()) and bool((out[..., :co_off] == 3.0).all())
    assert bool((out[..., co_off + cout:] == 3.0).all())
    assert rel_rms(got.float(), plain.cpu().float()) <= 1e-3
    assert rel_rms(got.float(), ref) <= 1e-2


def test_conv3x3_avgpool2_rejects_odd_extents(lib):
    t = torch.zeros(64, dtype=torch.bfloat16, device="cuda")
    with pytest.raises(RuntimeError):
        library.check(lib.dk_unet_conv3x3_avgpool2(_ptr(t), 1, 3, 4, 16, 16, _ptr(t), None, 16, _ptr(t), 16, 0, 1,
                                                   _ptr(t), 16, None))


@pytest.mark.parametrize("cin,cout", [(16, 32), (64, 96), (160, 128), (96, 16)])
def test_conv3x3_input_and_weight_gradients(lib, cin, cout):
    g = torch.Generator().manual_seed(cin + 3 * cout)
    n, h, w = 2, 16, 24
    x = torch.randn(n, h, w, cin, generator=g).to(torch.bfloat16)
    wt = (torch.randn(cout, 9, cin, generator=g) / (3 * cin ** 0.5))
    dy = torch.randn(n, h, w, cout, generator=g).to(torch.bfloat16)
    # reference gradients in FP32 from bf16-rounded operands
    xr = x.float().permute(0, 3, 1, 2).requires_grad_(True)
    wr = to_torch_weight(wt.to(torch.bfloat16).float()).requires_grad_(True)
    y = torch.nn.functional.conv2d(xr, wr, padding=1)
    y.backward(dy.float().permute(0, 3, 1, 2))
    gx_ref = xr.grad.permute(0, 2, 3, 1)
    gw_ref = wr.grad.permute(0, 2, 3, 1).reshape(cout, 9, cin)
    # device: flipped weights via the bf16 conversion kernel, dgrad as a forward conv
    wd = wt.cuda().contiguous()
    wbf = torch.empty(cout, 9, cin, dtype=torch.bfloat16, device="cuda")
    wflip = torch.empty(cin, 9, cout, dtype=torch.bfloat16, device="cuda")
    library.check(lib.dk_unet_weights_to_bf16(_ptr(wd), wd.numel(), _ptr(wbf), _ptr(wflip), cout, cin, None))
    dyd, xd = dy.cuda(), x.cuda()
    gx = torch.zeros(n, h, w, cin, dtype=torch.bfloat16, device="cuda")
    library.check(lib.dk_unet_conv3x3(_ptr(dyd), n, h, w, cout, cout, _ptr(wflip), None, cin, _ptr(gx), cin, 0, 0, 0,
                                      None))
    gw = torch.zeros(cout, 9, cin, dtype=torch.float32, device="cuda")
    library.check(lib.dk_unet_conv3x3_wgrad(_ptr(xd), cin, _ptr(dyd), cout, n, h, w, cin, cout, _ptr(gw), None))
    gb = torch.zeros(cout, dtype=torch.float32, device="cuda")
    library.check(lib.dk_unet_bias_grad(_ptr(dyd), cout, cout, n * h * w, _ptr(gb), None))
    torch.cuda.synchronize()
    assert rel_rms(gx.cpu().float(), gx_ref) <= 1e-2
    assert rel_rms(gw.cpu(), gw_ref) <= 1e-3  # FP32 accumulation of exact bf16 products
    assert rel_rms(gb.cpu(), dy.float().sum(dim=(0, 1, 2))) <= 1e-4


def torch_unet(x, weights):
    """The same network in plain PyTorch FP32 (NCHW)."""
    F = torch.nn.functional

    def conv(name, t, act=True):
        w, b = weights[name]
        y = F.conv2d(t, to_torch_weight(w), b, padding=1)
        return torch.relu(y) if act else y

    skips = []
    t = x
    for k in range(4):
        t = conv(f"enc{k}b", conv(f"enc{k}a", t))
        skips.append(t)
        t = F.avg_pool2d(t, 2)
    t = conv("botb", conv("bota", t))
    for k in (3, 2, 1, 0):
        t = F.interpolate(t, scale_factor=2, mode="nearest")
        t = torch.cat([t, skips[k]], 1)
        t = conv(f"dec{k}b", conv(f"dec{k}a", t))
    return conv("out", t, act=False)


def test_network_gradients_match_fp32_reference(lib):
    n, h, w = 2, 32, 48
    net = UNet(seed=3)
    g = torch.Generator().manual_seed(11)
    # biases non-zero so their gradients and the ReLU masks are exercised
    state = {}
    for l in net.layers:
        wv, _ = net.state()[l.name]
        state[l.name] = (wv, (torch.randn(l.cout, generator=g) * 0.05).numpy())
    net.load_state(state)
    x = torch.randn(n, h, w, IN_CH, generator=g)
    x[..., :3] = x[..., :3].abs()  # log(1 + noisy) channels are non-negative
    x = x.to(torch.bfloat16)
    # Targets 0.5..1.5 above the residual's base in log space: the L1 loss's
    # sign stays away from zero, where bf16 rounding would flip gradient terms.
    tl0 = x[..., :3].float() + 0.5 + torch.rand(n, h, w, 3, generator=g)
    target = torch.cat([torch.expm1(tl0), torch.ones(n, h, w, 1)], -1).reshape(n * h * w, 4)
    B = net.grad_buffers(n, h, w)
    B["x"].copy_(x.cuda())
    net.zero_grad()
    B["loss"].zero_()
    net.forward(n, h, w)
    net.loss(target.cuda().contiguous(), n, h, w)
    net.backward(n, h, w)
    torch.cuda.synchronize()
    # FP32 reference on the CPU, same (bf16-rounded) weights
    wts = {}
    for l in net.layers:
        wr = l.wbf.cpu().float().requires_grad_(True)
        br = l.b.cpu().clone().requires_grad_(True)
        wts[l.name] = (wr, br)
    pred = torch_unet(x.float().permute(0, 3, 1, 2), wts)
    tl = torch.log1p(target[:, :3].reshape(n, h, w, 3).permute(0, 3, 1, 2))
    # the network's output is a residual over the input's first 3 channels
    loss = (pred[:, :3] + x.float().permute(0, 3, 1, 2)[:, :3] - tl).abs().mean()
    loss.backward()
    assert abs(B["loss"].item() - loss.item()) <= 2e-2 * loss.item()
    got_pred = B["pred"].cpu().float()[..., :3].permute(0, 3, 1, 2)
    assert rel_rms(got_pred, pred[:, :3].detach()) <= 3e-2
    for l in net.layers:
        wr, br = wts[l.name]
        ew = rel_rms(l.gw.cpu(), wr.grad)
        eb = rel_rms(l.gb.cpu(), br.grad)
        assert ew <= 6e-2, (l.name, ew)
        assert eb <= 6e-2, (l.name, eb)


def test_batched_denoise_equals_single_images(lib):
    # A batch of images through one pass of the network (and its CUDA graph)
    # gives each image's own result bit for bit.
    from denrimrendererkit_gb300.denoiser import GraphedDenoiser
    net = UNet(seed=6)
    g = torch.Generator().manual_seed(3)
    n, w, h = 3, 40, 24
    planes = [torch.rand(n, h, w, 4, generator=g).cuda() for _ in range(4)]
    single = torch.empty(n, h, w, 4, device="cuda")
    for i in range(n):
        net.denoise(*(p[i] for p in planes), w, h, single[i])
    batched = torch.empty_like(single)
    net.denoise_batch(*planes, w, h, batched)
    graphed = GraphedDenoiser(net, w, h, batch=n)
    for dst, src in zip(graphed.inputs, planes):
        dst.copy_(src)
    replayed = graphed.replay().clone()
    torch.cuda.synchronize()
    assert torch.equal(batched, single)
    assert torch.equal(replayed, single)


def test_graphed_denoiser_equals_direct_calls(lib):
    # The CUDA-graph replay runs the same kernels on the same buffers.
    from denrimrendererkit_gb300.denoiser import GraphedDenoiser
    net = UNet(seed=5)
    g = torch.Generator().manual_seed(2)
    w, h = 72, 40  # padded to 80 x 48 inside
    planes = [torch.rand(h, w, 4, generator=g).cuda() for _ in range(4)]
    direct = torch.empty(h, w, 4, device="cuda")
    net.denoise(*planes, w, h, direct)
    graphed = GraphedDenoiser(net, w, h)
    out = torch.empty_like(direct)
    for _ in range(2):
        graphed.denoise(*planes, out)
    torch.cuda.synchronize()
    assert torch.equal(out, direct)


def test_conv_plan_replays_the_forward_convolutions(lib):
    # conv_plan lists forward's convolutions with its buffers: replayed over the
    # buffers forward left (pooled and upsampled inputs in place), every
    # convolution's output -- and so the prediction -- is unchanged.
    net = UNet(seed=4)
    n, h, w = 1, 32, 48
    B = net.buffers(n, h, w)
    g = torch.Generator().manual_seed(8)
    B["x"].copy_(torch.randn(n, h, w, IN_CH, generator=g).to(torch.bfloat16).cuda())
    net.forward(n, h, w)
    torch.cuda.synchronize()
    pred = B["pred"].clone()
    plan = net.conv_plan(n, h, w)
    assert len(plan) == len(net.layers)
    B["pred"].zero_()
    for (l, src, so, ldi, dst, do, ldo, hh, ww) in plan:
        net._conv(l, src, so, ldi, dst, do, ldo, n, hh, ww)
    torch.cuda.synchronize()
    assert torch.equal(B["pred"], pred)
