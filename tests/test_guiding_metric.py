"""The equal-time guiding comparison's error metric (spica_gb300/guiding.py), on CPU
with synthetic images: relMSE against a noisy reference, minus the reference's own noise
term, estimates the error against the converged image."""
import numpy as np

from spica_gb300 import guiding


def test_reference_noise_correction_is_unbiased():
    rng = np.random.default_rng(5)
    H, W = 256, 256
    mu = rng.lognormal(-1.0, 1.0, (H, W, 3))
    ref_var = (0.05 * mu) ** 2            # variance of the reference's per-pixel mean
    img_var = (0.2 * mu) ** 2             # variance of the image under test
    ests, truths = [], []
    for _ in range(8):
        ref = mu + rng.normal(size=mu.shape) * np.sqrt(ref_var)
        img = mu + rng.normal(size=mu.shape) * np.sqrt(img_var)
        ests.append(guiding.relmse(img, ref) - guiding.reference_noise(ref, ref_var))
        truths.append(guiding.relmse(img, mu))
    est, truth = np.mean(ests), np.mean(truths)
    raw = guiding.relmse(img, ref)
    assert abs(est - truth) < 0.03 * truth, (est, truth)
    assert raw > truth * 1.03          # uncorrected, the reference's noise inflates the error
