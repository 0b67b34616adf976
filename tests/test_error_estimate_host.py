"""The serving loop's host arithmetic on the CPU: the reference-free error
estimate from its per-image sums (`denoiser.estimates_from_terms`, the sums
being what `dk_denoise_error_terms` computes on the device, checked against
FP64 numpy in tests/test_denoiser.py) against the true error of synthetic
renders, and the sample-count growth (`next_sample_count`)."""
import math

import numpy as np
import pytest

from denrimrendererkit_gb300.denoiser import estimates_from_terms, next_sample_count


def terms_of(a, b, f, da, db, df):
    """The five device sums over the RGB channels."""
    c = slice(0, 3)
    return [float(((da[..., c] - db[..., c]) ** 2).sum()), float(((a[..., c] - b[..., c]) ** 2).sum()),
            float(((f[..., c] - df[..., c]) ** 2).sum()), float(df[..., c].sum()), float(f[..., c].sum())]


def rel_rmse(x, truth):
    return math.sqrt(((x[..., :3] - truth[..., :3]) ** 2).mean()) / truth[..., :3].mean()


def synthetic(rng, n_a, n_b, sigma=0.4, keep=0.3, bias=0.03, size=160):
    """A smooth image T; renders A and B of n_a and n_b samples (per-sample
    noise sigma); F their sample-weighted average; a linear denoiser that keeps
    `keep` of the noise and adds a spatially varying bias."""
    y, x = np.mgrid[0:size, 0:size] / size
    truth = np.zeros((size, size, 4))
    for ch in range(3):
        truth[..., ch] = 0.4 + 0.3 * np.sin(3 * x + ch) * np.cos(2 * y - ch)
    a = truth + rng.normal(0, sigma / math.sqrt(n_a), truth.shape)
    b = truth + rng.normal(0, sigma / math.sqrt(n_b), truth.shape)
    f = (n_a * a + n_b * b) / (n_a + n_b)
    offset = bias * np.sin(7 * x)[..., None] * np.ones(4)

    def denoise(img):
        return (1 - keep) * (truth + offset) + keep * img

    return truth, a, b, f, denoise(a), denoise(b), denoise(f)


@pytest.mark.parametrize("n_a,n_b", [(16, 16), (16, 48), (64, 64)])
def test_estimates_match_the_true_errors(n_a, n_b):
    rng = np.random.default_rng(n_a * 7 + n_b)
    truth, a, b, f, da, db, df = synthetic(rng, n_a, n_b)
    est = estimates_from_terms([terms_of(a, b, f, da, db, df)], truth.shape[0] * truth.shape[1],
                               samples=None if n_a == n_b else (n_a, n_b))[0]
    true_plain, true_denoised = rel_rmse(f, truth), rel_rmse(df, truth)
    assert abs(est.plain - true_plain) <= 0.03 * true_plain, (est.plain, true_plain)
    assert abs(est.denoised - true_denoised) <= 0.05 * true_denoised, (est.denoised, true_denoised)
    assert est.denoised < est.plain and est.bias > 0 and est.noise > 0
    assert math.isclose(est.denoised ** 2, est.noise ** 2 + est.bias ** 2, rel_tol=1e-12)


def test_a_denoiser_that_changes_nothing_has_no_bias():
    rng = np.random.default_rng(3)
    truth, a, b, f, *_ = synthetic(rng, 32, 32)
    est = estimates_from_terms([terms_of(a, b, f, a, b, f)], truth.shape[0] * truth.shape[1])[0]
    assert est.bias == 0.0 and math.isclose(est.denoised, est.plain, rel_tol=1e-9)


def test_next_sample_count_bounds_and_rounding():
    # error ~ 1/sqrt(spp): twice the target wants 4x the samples (+10 %), capped at 4x
    assert next_sample_count(64, 0.04, 0.02) == 256
    assert next_sample_count(64, 0.03, 0.02) == 160  # 64 x 1.1 x 2.25 = 158.4 -> 160
    assert next_sample_count(64, 0.021, 0.02) == 80  # at least 1.25x
    assert next_sample_count(100, 0.5, 0.02) == 400  # at most 4x
    assert next_sample_count(64, 0.03, 0.0) == 256   # no target: 4x
    for spp in (8, 24, 100, 1000):
        for est in (0.019, 0.02, 0.05, 1.0):
            s = next_sample_count(spp, est, 0.02)
            assert s % 8 == 0 and 1.25 * spp <= s <= 4 * spp + 8
