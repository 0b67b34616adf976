"""Learned denoiser: a 5-level U-Net over the tracer's AOVs, trained on the GPU
by this library's own kernels (dk_unet_* in include/denrim_cuda.h).

The reference's denoisers are a hand-tuned spatial filter
(Sources/DenrimRendererKit/Resources/Shaders/Denoise.metal:39-115, here
`spatial_denoise`) and Apple's SVGF; this network is the learned stage that
replaces them.  Input: log(1 + beauty), albedo, normal, depth (10 of 16
channels); output: log(1 + radiance).  Levels of 32-64-96-128-160 channels,
two 3x3 convolutions + ReLU per level on each side, 2x2 average pooling,
nearest upsampling, skip concatenation.  Activations are NHWC bf16, weights
FP32 masters with bf16 copies, FP32 accumulation; every convolution, its
input and weight gradients, the pooling/upsampling and their gradients, the
loss and Adam run in the library.  PyTorch only owns the device buffers.
The network predicts a residual over the input's log(1 + noisy) channels,
composed in FP32 when the image is written (`UNet.residual`).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import abi, library

LEVELS = (32, 64, 96, 128, 160)
IN_CH = 16
OUT_CH = 16


def _torch():
    import torch
    return torch


def _ptr(t, offset_elems: int = 0) -> int:
    return t.data_ptr() + offset_elems * t.element_size()


@dataclasses.dataclass
class Conv:
    name: str
    cin: int
    cout: int
    act: int  # 1 ReLU, 0 identity
    w: object = None      # fp32 master [cout][9][cin]
    b: object = None      # fp32 [cout]
    wbf: object = None    # bf16 [cout][9][cin]
    wflip: object = None  # bf16 [cin][9][cout], taps flipped
    gw: object = None
    gb: object = None
    mw: object = None
    vw: object = None
    mb: object = None
    vb: object = None

    @property
    def count(self) -> int:
        return self.cout * 9 * self.cin


def layer_plan() -> List[Conv]:
    c = LEVELS
    return [
        Conv("enc0a", IN_CH, c[0], 1), Conv("enc0b", c[0], c[0], 1),
        Conv("enc1a", c[0], c[1], 1), Conv("enc1b", c[1], c[1], 1),
        Conv("enc2a", c[1], c[2], 1), Conv("enc2b", c[2], c[2], 1),
        Conv("enc3a", c[2], c[3], 1), Conv("enc3b", c[3], c[3], 1),
        Conv("bota", c[3], c[4], 1), Conv("botb", c[4], c[4], 1),
        Conv("dec3a", c[4] + c[3], c[3], 1), Conv("dec3b", c[3], c[3], 1),
        Conv("dec2a", c[3] + c[2], c[2], 1), Conv("dec2b", c[2], c[2], 1),
        Conv("dec1a", c[2] + c[1], c[1], 1), Conv("dec1b", c[1], c[1], 1),
        Conv("dec0a", c[1] + c[0], c[0], 1), Conv("dec0b", c[0], c[0], 1),
        Conv("out", c[0], OUT_CH, 0),
    ]


def flops_per_pixel() -> float:
    """Multiply-adds x 2 of one forward pass per full-resolution pixel."""
    total = 0.0
    for layer in layer_plan():
        level = 0
        for k, name in enumerate(("enc0", "enc1", "enc2", "enc3", "bot")):
            if layer.name.startswith(name):
                level = k
        for k, name in enumerate(("dec0", "dec1", "dec2", "dec3")):
            if layer.name.startswith(name):
                level = k
        total += 2.0 * 9 * layer.cin * layer.cout / (4 ** level)
    return total


class UNet:
    """The network, its optimiser state and its activation buffers."""

    def __init__(self, seed: int = 0, device: str = "cuda", stream=None, residual: bool = True):
        torch = _torch()
        self.lib = library.load()
        self.device = device
        # The output is a residual over the input's log(1 + noisy) channels
        # (summed in FP32 when the image is written), so converged pixels --
        # visible lights -- keep their value instead of the bf16 activations'
        # 3 significant digits; False predicts log(1 + radiance) directly.
        self.residual = residual
        self.layers = layer_plan()
        self.by_name = {l.name: l for l in self.layers}
        g = torch.Generator().manual_seed(seed)
        for l in self.layers:
            std = math.sqrt(2.0 / (9 * l.cin)) * (0.1 if l.name == "out" else 1.0)
            w = torch.randn(l.cout, 9, l.cin, generator=g) * std
            l.w = w.to(device).contiguous()
            l.b = torch.zeros(l.cout, device=device)
            for k in ("gw", "mw", "vw"):
                setattr(l, k, torch.zeros_like(l.w))
            for k in ("gb", "mb", "vb"):
                setattr(l, k, torch.zeros_like(l.b))
            l.wbf = torch.empty(l.cout, 9, l.cin, dtype=torch.bfloat16, device=device)
            l.wflip = torch.empty(l.cin, 9, l.cout, dtype=torch.bfloat16, device=device)
        self.step_count = 0
        self.stream = stream
        self._buffers: Dict[Tuple[int, int, int], dict] = {}
        self.refresh_bf16()

    # ----------------------------------------------------------- helpers --
    @property
    def _st(self):
        return None if self.stream is None else C.c_void_p(self.stream)

    def _check(self, rc):
        library.check(rc)

    def refresh_bf16(self) -> None:
        for l in self.layers:
            self._check(self.lib.dk_unet_weights_to_bf16(_ptr(l.w), l.count, _ptr(l.wbf), _ptr(l.wflip), l.cout,
                                                         l.cin, self._st))

    def load_state(self, weights: Dict[str, Tuple[np.ndarray, np.ndarray]]) -> None:
        torch = _torch()
        for name, (w, b) in weights.items():
            l = self.by_name[name]
            l.w.copy_(torch.as_tensor(np.asarray(w, np.float32).reshape(l.cout, 9, l.cin)))
            l.b.copy_(torch.as_tensor(np.asarray(b, np.float32)))
        self.refresh_bf16()

    def state(self) -> Dict[str, Tuple[np.ndarray, np.ndarray]]:
        return {l.name: (l.w.cpu().numpy().copy(), l.b.cpu().numpy().copy()) for l in self.layers}

    def buffers(self, n: int, h: int, w: int) -> dict:
        key = (n, h, w)
        if key in self._buffers:
            return self._buffers[key]
        if h % 16 or w % 16:
            raise ValueError("U-Net input height and width must be multiples of 16")
        torch = _torch()
        c = LEVELS
        bf = dict(dtype=torch.bfloat16, device=self.device)

        def t(level, ch):
            return torch.zeros(n, h >> level, w >> level, ch, **bf)

        B = {
            "x": t(0, IN_CH),
            # concat buffers: [up | skip]; the encoder's second conv of a level writes its skip slice
            "cat0": t(0, c[1] + c[0]), "cat1": t(1, c[2] + c[1]), "cat2": t(2, c[3] + c[2]),
            "cat3": t(3, c[4] + c[3]),
            "e0a": t(0, c[0]), "p1": t(1, c[0]), "e1a": t(1, c[1]), "p2": t(2, c[1]), "e2a": t(2, c[2]),
            "p3": t(3, c[2]), "e3a": t(3, c[3]), "p4": t(4, c[3]), "ba": t(4, c[4]), "bb": t(4, c[4]),
            "d3a": t(3, c[3]), "d3b": t(3, c[3]), "d2a": t(2, c[2]), "d2b": t(2, c[2]), "d1a": t(1, c[1]),
            "d1b": t(1, c[1]), "d0a": t(0, c[0]), "d0b": t(0, c[0]), "pred": t(0, OUT_CH),
        }
        self._buffers[key] = B
        return B

    def grad_buffers(self, n: int, h: int, w: int) -> dict:
        B = self.buffers(n, h, w)
        if "g_pred" in B:
            return B
        torch = _torch()
        for k in list(B.keys()):
            if k == "x" or k.startswith("g_"):
                continue
            B["g_" + k] = torch.zeros_like(B[k])
        B["dpre"] = torch.zeros(n, h, w, 288, dtype=torch.bfloat16, device=self.device)
        B["loss"] = torch.zeros(1, dtype=torch.float32, device=self.device)
        return B

    # ---------------------------------------------------------- forward --
    def conv_plan(self, n: int, h: int, w: int):
        """The forward pass's convolutions in order, as (layer, source, source
        channel offset, source leading dimension, destination, destination
        offset, destination leading dimension, height, width) over buffers(n, h,
        w): what `forward` runs between its pooling and upsampling steps, for
        timing the convolutions alone."""
        B = self.buffers(n, h, w)
        c = LEVELS
        L = self.by_name
        cat = [B["cat0"], B["cat1"], B["cat2"], B["cat3"]]
        catc = [c[1] + c[0], c[2] + c[1], c[3] + c[2], c[4] + c[3]]
        upc = [c[1], c[2], c[3], c[4]]
        firsts = [B["e0a"], B["e1a"], B["e2a"], B["e3a"]]
        srcs = [(B["x"], IN_CH), (B["p1"], c[0]), (B["p2"], c[1]), (B["p3"], c[2])]
        plan = []
        for k in range(4):
            hk, wk = h >> k, w >> k
            plan.append((L[f"enc{k}a"], srcs[k][0], 0, srcs[k][1], firsts[k], 0, c[k], hk, wk))
            plan.append((L[f"enc{k}b"], firsts[k], 0, c[k], cat[k], upc[k], catc[k], hk, wk))
        plan.append((L["bota"], B["p4"], 0, c[3], B["ba"], 0, c[4], h >> 4, w >> 4))
        plan.append((L["botb"], B["ba"], 0, c[4], B["bb"], 0, c[4], h >> 4, w >> 4))
        for k in (3, 2, 1, 0):
            hk, wk = h >> k, w >> k
            plan.append((L[f"dec{k}a"], cat[k], 0, catc[k], B[f"d{k}a"], 0, c[k], hk, wk))
            plan.append((L[f"dec{k}b"], B[f"d{k}a"], 0, c[k], B[f"d{k}b"], 0, c[k], hk, wk))
        plan.append((L["out"], B["d0b"], 0, c[0], B["pred"], 0, OUT_CH, h, w))
        return plan

    def _conv(self, l: Conv, src, src_off, ldi, dst, dst_off, ldo, n, h, w, accumulate=0):
        self._check(self.lib.dk_unet_conv3x3(_ptr(src, src_off), n, h, w, l.cin, ldi, _ptr(l.wbf), _ptr(l.b), l.cout,
                                             _ptr(dst), ldo, dst_off, l.act, accumulate, self._st))

    def forward(self, n: int, h: int, w: int) -> dict:
        """Runs the network on buffers()['x']; the result is buffers()['pred']."""
        B = self.buffers(n, h, w)
        c = LEVELS
        L = self.by_name
        lib, st = self.lib, self._st
        hs = [h >> k for k in range(5)]
        ws = [w >> k for k in range(5)]
        cat = [B["cat0"], B["cat1"], B["cat2"], B["cat3"]]
        catc = [c[1] + c[0], c[2] + c[1], c[3] + c[2], c[4] + c[3]]
        upc = [c[1], c[2], c[3], c[4]]
        # encoder
        src, src_ld = B["x"], IN_CH
        pools = [None, B["p1"], B["p2"], B["p3"], B["p4"]]
        firsts = [B["e0a"], B["e1a"], B["e2a"], B["e3a"]]
        for k in range(4):
            la, lb = L[f"enc{k}a"], L[f"enc{k}b"]
            self._conv(la, src, 0, src_ld, firsts[k], 0, c[k], n, hs[k], ws[k])
            # the second convolution and the 2x2 average of its output (fused where its rows leave by TMA stores)
            self._check(lib.dk_unet_conv3x3_avgpool2(_ptr(firsts[k]), n, hs[k], ws[k], lb.cin, c[k], _ptr(lb.wbf),
                                                     _ptr(lb.b), lb.cout, _ptr(cat[k]), catc[k], upc[k], lb.act,
                                                     _ptr(pools[k + 1]), c[k], st))
            src, src_ld = pools[k + 1], c[k]
        # bottleneck
        self._conv(L["bota"], B["p4"], 0, c[3], B["ba"], 0, c[4], n, hs[4], ws[4])
        self._conv(L["botb"], B["ba"], 0, c[4], B["bb"], 0, c[4], n, hs[4], ws[4])
        low, low_c = B["bb"], c[4]
        # decoder
        for k in (3, 2, 1, 0):
            self._check(lib.dk_unet_upsample2(_ptr(low), low_c, _ptr(cat[k]), catc[k], 0, low_c, n, hs[k + 1],
                                              ws[k + 1], st))
            la, lb = L[f"dec{k}a"], L[f"dec{k}b"]
            da, db = B[f"d{k}a"], B[f"d{k}b"]
            self._conv(la, cat[k], 0, catc[k], da, 0, c[k], n, hs[k], ws[k])
            self._conv(lb, da, 0, c[k], db, 0, c[k], n, hs[k], ws[k])
            low, low_c = db, c[k]
        self._conv(L["out"], B["d0b"], 0, c[0], B["pred"], 0, OUT_CH, n, h, w)
        return B

    # --------------------------------------------------------- backward --
    def _conv_backward(self, l: Conv, x, x_off, ldx, out, out_off, ldo, gout, gout_off, ldg, gin, gin_off, ldgi,
                       n, h, w, gin_accumulate=0):
        """Gradients of one conv layer: relu backward -> dpre; wgrad, bias
        grad; input gradient into `gin` (None: not needed)."""
        lib, st = self.lib, self._st
        B = self._cur
        M = n * h * w
        if l.act:
            dpre, ldp = B["dpre"], l.cout
            self._check(lib.dk_unet_relu_backward(_ptr(out, out_off), ldo, _ptr(gout, gout_off), ldg, _ptr(dpre), ldp,
                                                  l.cout, M, st))
            dsrc, dsrc_off, ldd = dpre, 0, ldp
        else:
            dsrc, dsrc_off, ldd = gout, gout_off, ldg
        self._check(lib.dk_unet_conv3x3_wgrad(_ptr(x, x_off), ldx, _ptr(dsrc, dsrc_off), ldd, n, h, w, l.cin, l.cout,
                                              _ptr(l.gw), st))
        self._check(lib.dk_unet_bias_grad(_ptr(dsrc, dsrc_off), ldd, l.cout, M, _ptr(l.gb), st))
        if gin is not None:
            self._check(lib.dk_unet_conv3x3(_ptr(dsrc, dsrc_off), n, h, w, l.cout, ldd, _ptr(l.wflip), None, l.cin,
                                            _ptr(gin, gin_off), ldgi, 0, 0, gin_accumulate, st))

    def backward(self, n: int, h: int, w: int) -> None:
        """Accumulates weight/bias gradients of the loss whose gradient is in
        grad_buffers()['g_pred'] (filled by `loss`)."""
        B = self.grad_buffers(n, h, w)
        self._cur = B
        c = LEVELS
        L = self.by_name
        lib, st = self.lib, self._st
        hs = [h >> k for k in range(5)]
        ws = [w >> k for k in range(5)]
        cat = [B["cat0"], B["cat1"], B["cat2"], B["cat3"]]
        gcat = [B["g_cat0"], B["g_cat1"], B["g_cat2"], B["g_cat3"]]
        catc = [c[1] + c[0], c[2] + c[1], c[3] + c[2], c[4] + c[3]]
        upc = [c[1], c[2], c[3], c[4]]
        # output layer
        self._conv_backward(L["out"], B["d0b"], 0, c[0], B["pred"], 0, OUT_CH, B["g_pred"], 0, OUT_CH,
                            B["g_d0b"], 0, c[0], n, h, w)
        # decoder, top level first
        for k in (0, 1, 2, 3):
            la, lb = L[f"dec{k}a"], L[f"dec{k}b"]
            da, db = B[f"d{k}a"], B[f"d{k}b"]
            gda, gdb = B[f"g_d{k}a"], B[f"g_d{k}b"]
            self._conv_backward(lb, da, 0, c[k], db, 0, c[k], gdb, 0, c[k], gda, 0, c[k], n, hs[k], ws[k])
            self._conv_backward(la, cat[k], 0, catc[k], da, 0, c[k], gda, 0, c[k], gcat[k], 0, catc[k], n, hs[k],
                                ws[k])
            # the upsampled part of gcat[k] flows to the level below's output
            low = B[f"g_d{k + 1}b"] if k < 3 else B["g_bb"]
            self._check(lib.dk_unet_upsample2_backward(_ptr(gcat[k]), catc[k], 0, _ptr(low), upc[k], upc[k], n,
                                                       hs[k + 1], ws[k + 1], st))
        # bottleneck
        self._conv_backward(L["botb"], B["ba"], 0, c[4], B["bb"], 0, c[4], B["g_bb"], 0, c[4], B["g_ba"], 0, c[4],
                            n, hs[4], ws[4])
        self._conv_backward(L["bota"], B["p4"], 0, c[3], B["ba"], 0, c[4], B["g_ba"], 0, c[4], B["g_p4"], 0, c[3],
                            n, hs[4], ws[4])
        # encoder, deepest level first; the skip gradient (gcat[k] skip slice)
        # gains the pooled path's gradient
        pools = [None, B["p1"], B["p2"], B["p3"], B["p4"]]
        gpools = [None, B["g_p1"], B["g_p2"], B["g_p3"], B["g_p4"]]
        firsts = [B["e0a"], B["e1a"], B["e2a"], B["e3a"]]
        gfirsts = [B["g_e0a"], B["g_e1a"], B["g_e2a"], B["g_e3a"]]
        for k in (3, 2, 1, 0):
            self._check(lib.dk_unet_avgpool2_backward(_ptr(gpools[k + 1]), c[k], _ptr(gcat[k], upc[k]), catc[k], c[k],
                                                      n, hs[k], ws[k], 1, st))
            la, lb = L[f"enc{k}a"], L[f"enc{k}b"]
            self._conv_backward(lb, firsts[k], 0, c[k], cat[k], upc[k], catc[k], gcat[k], upc[k], catc[k],
                                gfirsts[k], 0, c[k], n, hs[k], ws[k])
            src, src_ld = (B["x"], IN_CH) if k == 0 else (pools[k], c[k - 1])
            gsrc = None if k == 0 else gpools[k]
            self._conv_backward(la, src, 0, src_ld, firsts[k], 0, c[k], gfirsts[k], 0, c[k], gsrc, 0,
                                c[k - 1] if k else IN_CH, n, hs[k], ws[k])

    # ------------------------------------------------------------ train --
    def zero_grad(self) -> None:
        for l in self.layers:
            l.gw.zero_()
            l.gb.zero_()

    def loss(self, target, n: int, h: int, w: int) -> None:
        """L1 in log space against `target` (N*H*W RGBA32F, device); the mean
        is added to grad_buffers()['loss']."""
        B = self.grad_buffers(n, h, w)
        if self.residual:
            self._check(self.lib.dk_unet_l1_loss_residual(_ptr(B["pred"]), OUT_CH, _ptr(B["x"]), IN_CH, _ptr(target),
                                                          n * h * w, _ptr(B["g_pred"]), OUT_CH, _ptr(B["loss"]),
                                                          self._st))
            return
        self._check(self.lib.dk_unet_l1_loss(_ptr(B["pred"]), OUT_CH, _ptr(target), n * h * w, _ptr(B["g_pred"]),
                                             OUT_CH, _ptr(B["loss"]), self._st))

    def adam(self, lr: float = 1e-3, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8) -> None:
        self.step_count += 1
        for l in self.layers:
            self._check(self.lib.dk_unet_adam(_ptr(l.w), _ptr(l.gw), _ptr(l.mw), _ptr(l.vw), l.count, lr, beta1, beta2,
                                              eps, self.step_count, _ptr(l.wbf), _ptr(l.wflip), l.cout, l.cin,
                                              self._st))
            self._check(self.lib.dk_unet_adam(_ptr(l.b), _ptr(l.gb), _ptr(l.mb), _ptr(l.vb), l.cout, lr, beta1, beta2,
                                              eps, self.step_count, None, None, 1, 1, self._st))

    # -------------------------------------------------------- inference --
    def pack(self, beauty, albedo, normal, depth, img_w: int, img_h: int, x0: int, y0: int, n: int, h: int, w: int,
             batch_index: int) -> None:
        B = self.buffers(n, h, w)
        self._check(self.lib.dk_unet_pack_input(_ptr(beauty), _ptr(albedo), _ptr(normal), _ptr(depth), img_w, img_h,
                                                x0, y0, _ptr(B["x"]), h, w, batch_index, self._st))

    def denoise(self, beauty, albedo, normal, depth, img_w: int, img_h: int, out) -> None:
        """Denoises one RGBA32F image (device tensors of img_h*img_w*4 floats)
        into `out`, padding the network input to multiples of 16."""
        h = (img_h + 15) // 16 * 16
        w = (img_w + 15) // 16 * 16
        self.pack(beauty, albedo, normal, depth, img_w, img_h, 0, 0, 1, h, w, 0)
        B = self.forward(1, h, w)
        self._unpack(B["pred"], B["x"], h, w, beauty, img_w, img_h, out)

    def _unpack(self, pred, x, h, w, beauty, img_w, img_h, out) -> None:
        if self.residual:
            self._check(self.lib.dk_unet_unpack_output_residual(_ptr(pred), OUT_CH, _ptr(x), IN_CH, h, w, _ptr(beauty),
                                                                img_w, img_h, 0, 0, _ptr(out), self._st))
        else:
            self._check(self.lib.dk_unet_unpack_output(_ptr(pred), OUT_CH, h, w, _ptr(beauty), img_w, img_h, 0, 0,
                                                       _ptr(out), self._st))

    def denoise_batch(self, beauty, albedo, normal, depth, img_w: int, img_h: int, out) -> None:
        """Denoises n images of one size as one batch: every argument is a
        device tensor (n, img_h, img_w, 4) float32.  One pass of the network
        over the batch; each image equals its own `denoise` call."""
        n = beauty.shape[0]
        h = (img_h + 15) // 16 * 16
        w = (img_w + 15) // 16 * 16
        for i in range(n):
            self.pack(beauty[i], albedo[i], normal[i], depth[i], img_w, img_h, 0, 0, n, h, w, i)
        B = self.forward(n, h, w)
        for i in range(n):
            self._unpack(B["pred"][i], B["x"][i], h, w, beauty[i], img_w, img_h, out[i])


class GraphedDenoiser:
    """`UNet.denoise` of one image size as a CUDA graph: the pack, every
    convolution / pooling / upsampling launch and the unpack are captured once
    on a private stream and replayed per image, so a small image pays one graph
    launch instead of ~60 kernel launches and their host calls.  Inputs are
    copied into static device tensors before the replay; the weights are read
    at replay time, so training between replays needs no new capture."""

    def __init__(self, net: "UNet", width: int, height: int, batch: int = 0):
        """batch 0: one image, tensors (height, width, 4); batch n >= 1: n
        images per replay (`UNet.denoise_batch`), tensors (n, height, width, 4)."""
        torch = _torch()
        self.net, self.w, self.h, self.batch = net, width, height, batch
        shape = (batch, height, width, 4) if batch else (height, width, 4)
        run = net.denoise_batch if batch else net.denoise
        self.inputs = [torch.zeros(shape, dtype=torch.float32, device=net.device) for _ in range(4)]
        self.out = torch.zeros(shape, dtype=torch.float32, device=net.device)
        self.stream = torch.cuda.Stream()
        # Pool streams do not order against the default stream: the warm-up
        # reuses the network's activation buffers, so it waits for work
        # already queued on the caller's stream.
        self.stream.wait_stream(torch.cuda.current_stream())
        saved = net.stream
        try:
            net.stream = self.stream.cuda_stream
            with torch.cuda.stream(self.stream):  # warm-up: buffers, tensor-map encoders, lazy loading
                run(*self.inputs, width, height, self.out)
            self.stream.synchronize()
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph, stream=self.stream):
                run(*self.inputs, width, height, self.out)
        finally:
            net.stream = saved

    def denoise(self, beauty, albedo, normal, depth, out) -> None:
        for dst, src in zip(self.inputs, (beauty, albedo, normal, depth)):
            dst.copy_(src)
        self.graph.replay()
        out.copy_(self.out)

    def replay(self):
        """Denoises what is already in `inputs` (beauty, albedo, normal,
        depth -- e.g. filled by `RenderSession.copy_output`) into `out`, on
        torch's current stream; returns `out`."""
        self.graph.replay()
        return self.out


class SvgfDenoiser:
    """DenoiseSettings.appleSVGF (Denoiser.swift:67-76): spatiotemporal
    variance-guided filtering with a temporal history per image size
    (AppleSVGFDenoiser, Denoiser.swift:167-300).  `denoise` takes device
    RGBA32F planes (beauty, depth, encoded normal and motion-vector AOVs) and
    writes the filtered beauty into `out`; `reset` drops the history
    (clearTemporalHistory)."""

    def __init__(self, width: int, height: int):
        self.lib = library.load()
        self.width, self.height = width, height
        self._h = C.c_void_p()
        library.check(self.lib.dk_svgf_create(width, height, C.byref(self._h)))

    def denoise(self, beauty, depth, normal, motion, out, radius: int = 2, normal_sigma: float = 0.18,
                depth_sigma: float = 0.08, color_sigma: float = 4.0, iterations: int = 5, stream=None) -> None:
        torch = _torch()
        s = abi.SpatialDenoiseSettings(radius, normal_sigma, depth_sigma, 0.25, color_sigma, iterations)
        st = torch.cuda.current_stream().cuda_stream if stream is None else stream
        library.check(self.lib.dk_svgf_denoise(self._h, _ptr(beauty), _ptr(depth), _ptr(normal), _ptr(motion),
                                               _ptr(out), C.byref(s), C.c_void_p(st)))

    def reset(self) -> None:
        library.check(self.lib.dk_svgf_reset(self._h))

    def state(self, which: int):
        """0: history colour, 1: (luminance mean, mean square, history length, 0), 2: packed depth + normal."""
        torch = _torch()
        out = torch.empty(self.height, self.width, 4, dtype=torch.float32, device="cuda")
        library.check(self.lib.dk_svgf_read_state(self._h, which, _ptr(out), self.width * self.height,
                                                  C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        return out

    def close(self) -> None:
        if self._h:
            self.lib.dk_svgf_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def spatial_denoise(beauty, depth, normal, albedo, out, width: int, height: int, radius: int = 2,
                    normal_sigma: float = 0.18, depth_sigma: float = 0.03, albedo_sigma: float = 0.25,
                    color_sigma: float = 1.0, iterations: int = 3, stream=None) -> None:
    """The reference's simple spatial denoiser on device RGBA32F planes
    (DenoiseSettings defaults, Denoiser.swift:44-60)."""
    torch = _torch()
    lib = library.load()
    s = abi.SpatialDenoiseSettings(radius, normal_sigma, depth_sigma, albedo_sigma, color_sigma, iterations)
    scratch = torch.empty(2 * width * height * 4, dtype=torch.float32, device=beauty.device)
    library.check(lib.dk_denoise_spatial(_ptr(beauty), _ptr(depth), _ptr(normal), _ptr(albedo), _ptr(out),
                                         _ptr(scratch), width, height, C.byref(s),
                                         None if stream is None else C.c_void_p(stream)))


# ------------------------------------------------------------ training ---
@dataclasses.dataclass
class TrainingSet:
    """Device tensors (K, H, W, 4) float32 of the inputs and targets."""
    beauty: object
    albedo: object
    normal: object
    depth: object
    target: object

    @property
    def count(self) -> int:
        return self.beauty.shape[0]


def render_pairs(seeds, size: int = 256, noisy_spp: int = 4, target_spp: int = 1024) -> TrainingSet:
    """Renders (noisy AOVs, converged beauty) pairs of seeded small-scene
    variants with the tracer; the target uses an independent frame seed."""
    torch = _torch()
    from . import compile_scene, scenes
    from .renderer import DenrimRenderer, RenderOutput
    r = DenrimRenderer(0)
    k = len(seeds)
    planes = {name: torch.empty(k, size, size, 4, dtype=torch.float32, device="cuda")
              for name in ("beauty", "albedo", "normal", "depth", "target")}
    for i, seed in enumerate(seeds):
        wl = scenes.cornell_variant(seed, size, size)
        b = compile_scene(wl.scene)
        with r.make_session(wl.scene, wl.settings, build=b) as s:
            s.render(noisy_spp)
            for name, out in (("beauty", RenderOutput.BEAUTY), ("albedo", RenderOutput.ALBEDO),
                              ("normal", RenderOutput.NORMAL), ("depth", RenderOutput.DEPTH)):
                planes[name][i].copy_(torch.from_numpy(s.pixels(out)))
        tgt = dataclasses.replace(wl.settings, frame_seed=(wl.settings.frame_seed ^ 0x5BD1E995) & 0x7FFFFFFF)
        with r.make_session(wl.scene, tgt, build=b) as s:
            s.render(target_spp)
            planes["target"][i].copy_(torch.from_numpy(s.pixels(RenderOutput.BEAUTY)))
    return TrainingSet(**planes)


def train(net: UNet, data: TrainingSet, steps: int, batch: int = 16, crop: Optional[int] = None, lr: float = 1e-3,
          seed: int = 0, log_every: int = 0) -> List[float]:
    """Adam on random batches of random `crop` x `crop` windows of the
    training images (whole images when `crop` is None); L1 in log space with
    a cosine learning-rate decay to 10 %.  Returns the logged losses."""
    torch = _torch()
    H, W = data.beauty.shape[1], data.beauty.shape[2]
    h = w = crop if crop else None
    if h is None:
        h, w = H, W
    n = batch
    B = net.grad_buffers(n, h, w)
    target = torch.empty(n, h, w, 4, dtype=torch.float32, device="cuda")
    rng = np.random.default_rng(seed)
    losses = []
    for step in range(steps):
        idx = rng.integers(0, data.count, size=n)
        for j, k in enumerate(idx):
            x0 = int(rng.integers(0, W - w + 1))
            y0 = int(rng.integers(0, H - h + 1))
            net.pack(data.beauty[k], data.albedo[k], data.normal[k], data.depth[k], W, H, x0, y0, n, h, w, j)
            target[j].copy_(data.target[k][y0:y0 + h, x0:x0 + w])
        net.zero_grad()
        B["loss"].zero_()
        net.forward(n, h, w)
        net.loss(target, n, h, w)
        net.backward(n, h, w)
        cur = lr * (0.1 + 0.9 * 0.5 * (1.0 + math.cos(math.pi * step / max(steps, 1))))
        net.adam(cur)
        if log_every and (step % log_every == 0 or step == steps - 1):
            losses.append(float(B["loss"].item()))
    return losses


def relative_rmse(image, reference) -> float:
    """sqrt(mean((image - reference)^2)) / mean(reference) over linear RGB."""
    torch = _torch()
    a = image[..., :3].double()
    b = reference[..., :3].double()
    return float(torch.sqrt(((a - b) ** 2).mean()) / b.mean())


def display(image):
    """The reference's PNG tone curve before 8-bit quantisation
    (PNGWriter.tonemap, Sources/DenrimRendererKit/Image/PNGWriter.swift:182-188):
    exposure 0.8, the ACES fit x (2.51 x + 0.03) / (x (2.43 x + 0.59) + 0.14),
    clamp to [0, 1], gamma 1 / 2.2."""
    torch = _torch()
    x = image[..., :3].double().clamp(min=0.0) * 0.8
    mapped = (x * (2.51 * x + 0.03)) / (x * (2.43 * x + 0.59) + 0.14)
    return torch.pow(mapped.clamp(0.0, 1.0), 1.0 / 2.2)


def display_relative_rmse(image, reference) -> float:
    """Relative RMSE of the displayed images: sqrt(mean((d(x) - d(t))^2)) /
    mean(d(t)) with d the reference's PNG tone curve.  The error measure of
    the denoisers: in the linear domain it is dominated by a few fireflies."""
    torch = _torch()
    a, b = display(image), display(reference)
    return float(torch.sqrt(((a - b) ** 2).mean()) / b.mean())


# ------------------------------------------------------ error estimate ---
@dataclasses.dataclass
class ErrorEstimate:
    """Estimated relative RMSE (linear RGB, over the image's mean) of one
    image's denoised full render dF and of its plain full render F."""
    denoised: float
    noise: float     # the variance part of `denoised`
    bias: float      # the bias part of `denoised`
    plain: float


def estimate_errors(half_a, half_b, full, den_a, den_b, den_full, stream=None, display: bool = False,
                    samples=None) -> List[ErrorEstimate]:
    """Per-image error estimates from two independent half-sample renders A and
    B, their full render F = (A + B) / 2 and the three denoised images (device
    tensors (n, H, W, 4) or (H, W, 4) float32), with no reference image:

    * noise: the denoised output's variance, Var(dF) ~ E|dA - dB|^2 / 4 (A and
      B carry half the samples each, so each has twice F's variance);
    * bias: what the denoiser changes beyond F's own noise.  With dF keeping
      a fraction g of F's noise (g^2 ~ E|dA - dB|^2 / E|A - B|^2),
      E|F - dF|^2 ~ (1 - g)^2 Var(F) + bias^2, Var(F) ~ E|A - B|^2 / 4, so
      bias^2 ~ E|F - dF|^2 - (1 - g)^2 Var(F) (clamped at zero);
    * plain: F's own error, sqrt(Var(F)) -- unbiased, the progressive
      renderer's estimate.
    `display`: the same on the displayed images (the reference's PNG tone
    curve, as `display_relative_rmse` measures).  `samples` (per image, or one
    pair for all): the sample counts (n_a, n_b) of A and B when they differ;
    then Var(F) ~ E|A - B|^2 n_a n_b / (n_a + n_b)^2 (1/4 for halves), and
    the same factor for dF.  The sums run on the device
    (dk_denoise_error_terms)."""
    torch = _torch()
    lib = library.load()
    t = [x if x.dim() == 4 else x.unsqueeze(0) for x in (half_a, half_b, full, den_a, den_b, den_full)]
    n, h, w = t[0].shape[0], t[0].shape[1], t[0].shape[2]
    for x in t:
        if not (x.is_cuda and x.dtype == torch.float32 and x.is_contiguous() and tuple(x.shape) == (n, h, w, 4)):
            raise ValueError("estimate_errors needs contiguous float32 CUDA tensors of one shape (n, H, W, 4)")
    terms = torch.empty(n, 5, dtype=torch.float64, device=t[0].device)
    library.check(lib.dk_denoise_error_terms(*(_ptr(x) for x in t), h * w, n, 1 if display else 0, _ptr(terms),
                                             None if stream is None else C.c_void_p(stream)))
    return estimates_from_terms(terms.cpu().numpy().tolist(), h * w, samples)


def estimates_from_terms(terms, pixels: int, samples=None) -> List[ErrorEstimate]:
    """The estimates of `estimate_errors` from its per-image sums over the
    RGB channels of `pixels` pixels: (sum |dA - dB|^2, sum |A - B|^2,
    sum |F - dF|^2, sum dF, sum F) per image."""
    out = []
    m = 3.0 * pixels
    n = len(terms)
    if samples is None:
        weights = [0.25] * n
    else:
        pairs = [samples] * n if isinstance(samples[0], (int, float)) else list(samples)
        weights = [na * nb / float(na + nb) ** 2 for na, nb in pairs]
    for (dd, nn, fd, sd, sf), wgt in zip(terms, weights):
        var_dn = dd * wgt / m
        var_f = nn * wgt / m
        g = min(1.0, math.sqrt(dd / nn)) if nn > 0.0 else 0.0
        bias2 = max(0.0, fd / m - var_f * (1.0 - g) ** 2)
        mean_d = max(sd / m, 1e-12)
        mean_f = max(sf / m, 1e-12)
        out.append(ErrorEstimate(denoised=math.sqrt(var_dn + bias2) / mean_d, noise=math.sqrt(var_dn) / mean_d,
                                 bias=math.sqrt(bias2) / mean_d, plain=math.sqrt(var_f) / mean_f))
    return out


def average_planes(a, b, out, t: float = 0.5, stream=None) -> None:
    """out = (1 - t) a + t b on the device (dk_average_planes): the full render
    of two independent renders of n_a and n_b samples with t = n_b / (n_a +
    n_b); tensors of one size."""
    library.check(library.load().dk_average_planes(_ptr(a), _ptr(b), _ptr(out), a.numel() // 4, float(t),
                                                   None if stream is None else C.c_void_p(stream)))


@dataclasses.dataclass
class ServedImage:
    """One request of `serve_to_error_target`: the image returned, the samples
    it took, its last estimate, and whether it is the denoised image or the
    plain render (the fallback)."""
    image: object
    spp: int
    estimate: ErrorEstimate
    denoised: bool
    rounds: int


def next_sample_count(spp: int, estimate: float, target: float, step: int = 8) -> int:
    """The sample count a progressive render grows to when its error estimate
    is `estimate` at `spp` samples: error ~ 1 / sqrt(spp) predicts
    spp (estimate / target)^2; 10 % more, at least 1.25x and at most 4x the
    current count, rounded up to a multiple of `step`."""
    want = spp * 1.1 * (estimate / target) ** 2 if target > 0 else 4.0 * spp
    want = min(max(want, 1.25 * spp), 4.0 * spp)
    return int(math.ceil(want / step) * step)


def serve_to_error_target(server, net: "UNet", requests, width: int, height: int, target: float = 0.02,
                          start_spp: int = 16, max_spp: int = 8192, denoise: bool = True,
                          seed_base: int = 0x51ED, display: bool = True) -> List[ServedImage]:
    """Renders each request (settings, camera, materials or None, scene index)
    through the render server until its estimated relative RMSE is at most
    `target`, and returns the images.

    Round 0 renders two independent halves A and B of `start_spp` samples per
    request (two jobs with different frame seeds, packed into the same waves
    as every other request's); F is their average.  With `denoise`, the U-Net
    denoises A, B and F of every open request as one batch and
    `estimate_errors` judges dF without a reference: a request whose
    estimate is within the target returns dF.  Otherwise -- and always without
    `denoise` -- F returns once its own (unbiased) estimate is within the
    target.  A request that meets neither grows: its F becomes the next A, a
    new render of as many more samples as `next_sample_count` predicts the
    next B, and F their sample-weighted average.  At `max_spp` the plain
    render returns (the fallback) whatever its estimate.  `display`: the
    error is that of the displayed images (the reference's PNG tone curve),
    else of the linear radiance."""
    torch = _torch()
    import dataclasses as dc
    from .renderer import RenderOutput
    n = len(requests)
    shape = (height, width, 4)
    open_ = list(range(n))
    full = [None] * n          # F of each request (device tensor)
    spp = [0] * n              # samples in F
    grow = [0] * n             # samples of the next render
    aov = [None] * n           # albedo, normal, depth of each request
    result: List[Optional[ServedImage]] = [None] * n
    rounds = 0
    seed = [seed_base + 7919 * k for k in range(n)]

    def submit(k, samples, s):
        settings, camera, materials, scene = requests[k]
        st = dc.replace(settings, frame_seed=s & 0x7FFFFFFF)
        return server.submit(st, camera, samples, materials, scene=scene)

    while open_:
        jobs = {}
        for k in open_:
            if spp[k] == 0:
                jobs[k] = (submit(k, start_spp // 2, seed[k]), submit(k, start_spp - start_spp // 2, seed[k] + 1))
                seed[k] += 2
            else:
                jobs[k] = (None, submit(k, grow[k], seed[k]))
                seed[k] += 1
        while server.step():
            pass
        m = len(open_)
        A = torch.empty((m,) + shape, device="cuda")
        B = torch.empty_like(A)
        F = torch.empty_like(A)
        pairs = []
        for i, k in enumerate(open_):
            ja, jb = jobs[k]
            if ja is None:
                A[i].copy_(full[k])
                na, nb = spp[k], grow[k]
            else:
                server.copy_output(ja, RenderOutput.BEAUTY, A[i])
                aov[k] = [server.copy_output(ja, kind, torch.empty(shape, device="cuda"))
                          for kind in (RenderOutput.ALBEDO, RenderOutput.NORMAL, RenderOutput.DEPTH)]
                server.release(ja)
                na, nb = start_spp // 2, start_spp - start_spp // 2
            server.copy_output(jb, RenderOutput.BEAUTY, B[i])
            server.release(jb)
            average_planes(A[i], B[i], F[i], nb / float(na + nb))
            spp[k] = na + nb
            pairs.append((na, nb))
        if denoise:
            al = torch.stack([aov[k][0] for k in open_]).repeat(3, 1, 1, 1).contiguous()
            no = torch.stack([aov[k][1] for k in open_]).repeat(3, 1, 1, 1).contiguous()
            de = torch.stack([aov[k][2] for k in open_]).repeat(3, 1, 1, 1).contiguous()
            noisy = torch.cat([A, B, F]).contiguous()
            den = torch.empty_like(noisy)
            net.denoise_batch(noisy, al, no, de, width, height, den)
            dA, dB, dF = den[:m].contiguous(), den[m:2 * m].contiguous(), den[2 * m:].contiguous()
        else:
            dA, dB, dF = A, B, F
        est = estimate_errors(A, B, F, dA, dB, dF, display=display, samples=pairs)
        rounds += 1
        still = []
        for i, k in enumerate(open_):
            e = est[i]
            if denoise and e.denoised <= target:
                result[k] = ServedImage(dF[i].clone(), spp[k], e, True, rounds)
            elif e.plain <= target or spp[k] >= max_spp:
                result[k] = ServedImage(F[i].clone(), spp[k], e, False, rounds)
            else:
                full[k] = F[i].clone()
                need = min(e.denoised, e.plain) if denoise else e.plain
                grow[k] = min(next_sample_count(spp[k], need, target), max_spp) - spp[k]
                still.append(k)
        open_ = still
    return result
