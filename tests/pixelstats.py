"""Per-pixel statistical comparison of two renderers at equal spp.

Each side renders the same image K times with independent random streams (K seeds).
Per pixel and channel, the K images give a mean and a sample variance on each side.
Welch's t statistic is computed from them, with its Welch-Satterthwaite degrees of
freedom.  Each t is then mapped to the standard normal deviate of the same two-sided
tail probability, so that the counts below can be read against the Gaussian tail.

If both renderers estimate the same image, the deviates are close to N(0, 1):
  - their mean is near 0;
  - their standard deviation is near 1;
  - about 6.3e-5 of them exceed 4 in magnitude.

Pixels whose samples are identical on both sides (zero variance, e.g. a pixel that only
sees the constant environment) must have equal means.

The same statistic is applied at two coarser scales, which have more power against a
bias that covers many pixels:
  - the means of 8 x 8-pixel blocks;
  - the mean of the whole image, per channel.
"""
from __future__ import annotations

import numpy as np


def pixel_deviates(a: np.ndarray, b: np.ndarray):
    """a, b: (K, H, W, 3) independent renders of each side.  Returns (deviates of the
    pixels with variance, max relative difference of the means of zero-variance ones)."""
    from scipy import stats

    K = a.shape[0]
    ma, mb = a.mean(0, dtype=np.float64), b.mean(0, dtype=np.float64)
    va, vb = a.var(0, ddof=1, dtype=np.float64) / K, b.var(0, ddof=1, dtype=np.float64) / K
    se2 = va + vb
    live = se2 > 0
    t = (ma - mb)[live] / np.sqrt(se2[live])
    dof = se2[live] ** 2 / (va[live] ** 2 / (K - 1) + vb[live] ** 2 / (K - 1))
    p = 2.0 * stats.t.sf(np.abs(t), dof)
    z = np.sign(t) * stats.norm.isf(np.maximum(p, 1e-300) / 2.0)
    dead = ~live
    flat = float(np.max(np.abs(ma[dead] - mb[dead]) / np.maximum(np.abs(mb[dead]), 1e-12))) if dead.any() else 0.0
    return z, flat


def _blocks(x: np.ndarray, k: int) -> np.ndarray:
    K, H, W, C = x.shape
    return x[:, :H // k * k, :W // k * k].reshape(K, H // k, k, W // k, k, C).mean(axis=(2, 4), dtype=np.float64)


def check_consistent(a: np.ndarray, b: np.ndarray, max_tail: int = 5):
    """Asserts that the two sides' means agree within their noise.
    Pixels: at most `max_tail` deviates beyond 4 (the Gaussian expectation is 6.3e-5 of
    them), a mean deviate within 0.15 of 0 and a standard deviation within [0.9, 1.15].
    8 x 8 blocks: at most one deviate beyond 4.
    Whole image: every channel's deviate within 4."""
    z, flat = pixel_deviates(a, b)
    zb, _ = pixel_deviates(_blocks(a, 8), _blocks(b, 8))
    zi, _ = pixel_deviates(a.mean(axis=(1, 2), dtype=np.float64)[:, None, None, :],
                           b.mean(axis=(1, 2), dtype=np.float64)[:, None, None, :])
    tail = int((np.abs(z) > 4.0).sum())
    expected = 6.334e-5 * z.size
    summary = (f"{z.size} pixel deviates: {tail} beyond 4 (Gaussian expectation {expected:.2f}), mean "
               f"{z.mean():.3f}, std {z.std():.3f}, max |z| {np.abs(z).max():.2f}; zero-variance pixels differ by "
               f"{flat:.1e}; {zb.size} block deviates: mean {zb.mean():.3f}, max |z| {np.abs(zb).max():.2f}; "
               f"image deviates {np.round(zi, 2).tolist()}")
    assert flat <= 1e-5, summary
    assert tail <= max_tail, summary
    assert abs(float(z.mean())) <= 0.15, summary
    assert 0.9 <= float(z.std()) <= 1.15, summary
    assert int((np.abs(zb) > 4.0).sum()) <= 1, summary
    assert float(np.abs(zi).max()) <= 4.0, summary
    return summary
