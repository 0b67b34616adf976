"""Test infrastructure: a numpy restatement of spatiotemporal variance-guided
filtering (Schied et al., "Spatiotemporal Variance-Guided Filtering", HPG
2017) with the parameters the reference's AppleSVGFDenoiser.configure sets
(Sources/DenrimRendererKit/Denoising/Denoiser.swift:227-237) and the
edge-stopping functions Apple documents for MPSSVGF's depth, normal and
luminance weights -- the checker of the CUDA dk_svgf_* path.

Parity unpinned: the reference's SVGF is Apple's closed MPSSVGFDenoiser, so
no output of the reference exists to pin this restatement; the reference's
own helper kernels around it (packSVGFDepthNormalKernel and
copySVGFOutputKernel, Denoise.metal:117-154) are pinned separately against
the reference kernels compiled for the host.

Stages per frame: pack, temporal reprojection through the motion-vector AOV
(previous pixel = pixel + motion, PathTrace.metal:5569-5577) with an
exponential moving average (0.2, at least 1/history), variance (temporal
moments, or a bilateral spatial estimate for histories shorter than 4),
`iterations` a-trous passes with steps 1, 2, 4, ... (the first pass feeds the
next frame's history), output copy.
"""
import numpy as np

f32 = np.float32
INVALID_DEPTH = f32(1.0e6)
HISTORY_CAP = f32(32.0)
REPROJECT_DEPTH = f32(0.1)
REPROJECT_NORMAL = f32(0.9)
LUMA = (f32(0.2126), f32(0.7152), f32(0.0722))


def params(radius=2, normal_sigma=0.18, depth_sigma=0.08, color_sigma=4.0, iterations=5):
    """AppleSVGFDenoiser.configure(settings:) with DenoiseSettings.appleSVGF defaults (Denoiser.swift:69-76)."""
    r = max(1, min(int(radius), 4))
    return dict(radius=r, variance_radius=r, depth_weight=f32(max(depth_sigma, 1e-4)),
                normal_weight=f32(max(1.0, min(512.0, 1.0 / max(normal_sigma, 1e-4) * 24.0))),
                luminance_weight=f32(max(color_sigma, 1e-4)), bilateral_sigma=f32(1.2), variance_sigma=f32(2.0),
                prefilter_sigma=f32(1.33), alpha=f32(0.2), alpha_moments=f32(0.2),
                iterations=max(1, min(int(iterations), 5)))


def luminance(c):
    return (LUMA[0] * c[..., 0] + LUMA[1] * c[..., 1]) + LUMA[2] * c[..., 2]


def pack_depth_normal(depth, normal):
    """packSVGFDepthNormalKernel (Denoise.metal:117-136)."""
    d = depth[..., 0]
    e = normal
    bad = (e[..., 3] <= f32(0.0001)) | ~np.isfinite(d) | (d <= 0)
    v = e[..., :3] * f32(2.0) - f32(1.0)
    out = np.empty(depth.shape, f32)
    out[..., 0] = d
    with np.errstate(all="ignore"):
        inv = f32(1.0) / np.sqrt((v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1]) + v[..., 2] * v[..., 2])
        out[..., 1:] = v * inv[..., None]
    out[bad] = (INVALID_DEPTH, 0.0, 0.0, 1.0)
    return out


def copy_output(denoised, original):
    """copySVGFOutputKernel (Denoise.metal:138-154)."""
    f = denoised.copy()
    bad = ~np.isfinite(f[..., :3]).all(-1)
    f[bad] = original[bad]
    out = np.empty_like(original)
    out[..., :3] = np.fmax(f[..., :3], f32(0.0))
    out[..., 3] = original[..., 3]
    return out


def shifted(a, dx, dy, fill=0.0):
    """a[y + dy, x + dx] with `fill` outside the image, and the inside mask."""
    h, w = a.shape[:2]
    out = np.full_like(a, fill)
    ok = np.zeros((h, w), bool)
    if abs(dx) >= w or abs(dy) >= h:
        return out, ok
    ys, yd = (slice(dy, h), slice(0, h - dy)) if dy >= 0 else (slice(0, h + dy), slice(-dy, h))
    xs, xd = (slice(dx, w), slice(0, w - dx)) if dx >= 0 else (slice(0, w + dx), slice(-dx, w))
    out[yd, xd] = a[ys, xs]
    ok[yd, xd] = True
    return out, ok


def edge_weight(dp, dq, lp, lq, lum_scale, p):
    with np.errstate(all="ignore"):
        wz = np.exp(-np.abs(dp[..., 0] - dq[..., 0]) / p["depth_weight"])
        cosn = np.maximum(f32(0.0), dp[..., 1] * dq[..., 1] + dp[..., 2] * dq[..., 2] + dp[..., 3] * dq[..., 3])
        wn = np.power(cosn, p["normal_weight"])
        wl = np.exp(-np.abs(lp - lq) * lum_scale)
    return (wz * wn * wl).astype(f32)


class Svgf:
    def __init__(self, width, height):
        self.w, self.h = width, height
        self.reset()

    def reset(self):
        self.prev = None  # (depth-normal, history colour, moments)

    def denoise(self, beauty, depth, normal, motion, p):
        h, w = self.h, self.w
        dn = pack_depth_normal(depth, normal)
        c = beauty[..., :3].astype(f32)
        l = luminance(c)
        sum_c = np.zeros((h, w, 3), f32)
        sum_m = np.zeros((h, w, 3), f32)
        sum_w = np.zeros((h, w), f32)
        if self.prev is not None:
            dn_prev, hist_c, hist_m = self.prev
            ys, xs = np.mgrid[0:h, 0:w]
            px = xs.astype(f32) + motion[..., 0]
            py = ys.astype(f32) + motion[..., 1]
            fx0, fy0 = np.floor(px), np.floor(py)
            fx, fy = px - fx0, py - fy0
            use = (motion[..., 3] > 0) & (dn[..., 0] < INVALID_DEPTH)
            for t in range(4):
                qx = fx0.astype(np.int64) + (t & 1)
                qy = fy0.astype(np.int64) + (t >> 1)
                wt = ((fx if t & 1 else f32(1) - fx) * (fy if t >> 1 else f32(1) - fy)).astype(f32)
                ok = use & (wt > 0) & (qx >= 0) & (qy >= 0) & (qx < w) & (qy < h)
                qxc, qyc = np.clip(qx, 0, w - 1), np.clip(qy, 0, h - 1)
                dq = dn_prev[qyc, qxc]
                ok &= dq[..., 0] < INVALID_DEPTH
                ok &= ~(np.abs(dq[..., 0] - dn[..., 0]) > REPROJECT_DEPTH * np.maximum(dn[..., 0], f32(1e-3)))
                ok &= ~((dq[..., 1] * dn[..., 1] + dq[..., 2] * dn[..., 2]) + dq[..., 3] * dn[..., 3] < REPROJECT_NORMAL)
                wt = np.where(ok, wt, f32(0))
                sum_c += wt[..., None] * hist_c[qyc, qxc, :3]
                sum_m += wt[..., None] * hist_m[qyc, qxc, :3]
                sum_w += wt
        valid = sum_w > f32(1e-4)
        inv = np.where(valid, f32(1) / np.where(valid, sum_w, f32(1)), f32(0))
        length = np.minimum(sum_m[..., 2] * inv + f32(1), HISTORY_CAP)
        a = np.maximum(p["alpha"], f32(1) / length)
        am = np.maximum(p["alpha_moments"], f32(1) / length)
        hc = sum_c * inv[..., None]
        integ = np.where(valid[..., None], hc + (c - hc) * a[..., None], c).astype(f32)
        m1, m2 = sum_m[..., 0] * inv, sum_m[..., 1] * inv
        mom = np.zeros((h, w, 4), f32)
        mom[..., 0] = np.where(valid, m1 + (l - m1) * am, l)
        mom[..., 1] = np.where(valid, m2 + (l * l - m2) * am, l * l)
        mom[..., 2] = np.where(valid, length, f32(1))
        # variance
        var_t = np.maximum(f32(0), mom[..., 1] - mom[..., 0] * mom[..., 0])
        r = p["variance_radius"]
        g = f32(1) / (f32(2) * p["variance_sigma"] * p["variance_sigma"])
        s1 = np.zeros((h, w), f32)
        s2 = np.zeros((h, w), f32)
        sw = np.zeros((h, w), f32)
        for dy in range(-r, r + 1):
            for dx in range(-r, r + 1):
                mq, ok = shifted(mom, dx, dy)
                dq, _ = shifted(dn, dx, dy)
                wt = np.exp(-f32(dx * dx + dy * dy) * g) * edge_weight(dn, dq, mom[..., 0], mq[..., 0], f32(0), p)
                wt = np.where(ok, wt, f32(0))
                s1 += wt * mq[..., 0]
                s2 += wt * mq[..., 1]
                sw += wt
        with np.errstate(all="ignore"):
            invw = np.where(sw > 0, f32(1) / sw, f32(0))
        var_s = np.maximum(f32(0), s2 * invw - (s1 * invw) ** 2) * (f32(4) / np.maximum(mom[..., 2], f32(1)))
        work = np.zeros((h, w, 4), f32)
        work[..., :3] = integ
        work[..., 3] = np.where(mom[..., 2] >= 4, var_t, var_s)
        history = None
        for it in range(p["iterations"]):
            work = self._atrous(work, dn, 1 << it, p)
            if it == 0:
                history = work.copy()
        self.prev = (dn, history, mom)
        return copy_output(work, beauty)

    @staticmethod
    def _atrous(src, dn, step, p):
        h, w = src.shape[:2]
        gpre = f32(1) / (f32(2) * p["prefilter_sigma"] * p["prefilter_sigma"])
        vs = np.zeros((h, w), f32)
        vw = np.zeros((h, w), f32)
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                q, ok = shifted(src, dx, dy)
                wt = np.where(ok, np.exp(-f32(dx * dx + dy * dy) * gpre), f32(0))
                vs += wt * q[..., 3]
                vw += wt
        sigma = np.sqrt(np.maximum(vs / vw, f32(0)))
        lum_scale = f32(1) / (p["luminance_weight"] * sigma + f32(1e-6))
        lp = luminance(src[..., :3])
        gb = f32(1) / (f32(2) * p["bilateral_sigma"] * p["bilateral_sigma"])
        sc = np.zeros((h, w, 3), f32)
        sv = np.zeros((h, w), f32)
        sw = np.zeros((h, w), f32)
        r = p["radius"]
        for ky in range(-r, r + 1):
            for kx in range(-r, r + 1):
                q, ok = shifted(src, kx * step, ky * step)
                dq, _ = shifted(dn, kx * step, ky * step)
                wt = np.exp(-f32(kx * kx + ky * ky) * gb) * edge_weight(dn, dq, lp, luminance(q[..., :3]), lum_scale, p)
                wt = np.where(ok, wt, f32(0)).astype(f32)
                sc += wt[..., None] * q[..., :3]
                sv += wt * wt * q[..., 3]
                sw += wt
        out = src.copy()
        good = sw > 0
        with np.errstate(all="ignore"):
            inv = np.where(good, f32(1) / sw, f32(0))
        out[..., :3] = np.where(good[..., None], sc * inv[..., None], src[..., :3])
        out[..., 3] = np.where(good, sv * inv * inv, src[..., 3])
        return out
