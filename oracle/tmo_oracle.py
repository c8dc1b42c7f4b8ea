"""Test infrastructure only: a numpy restatement of the reference's tone-mapping
operators, used by tests/ as the checker for the device film output.  Nothing in the
product path imports it.

Each function follows the reference file and lines it names, in float64 as the
reference computes.  The image is resolved first (Film::save, core/film.cc:25-28:
pixel sum / (weight + EPS)); luminance is RGBSpectrum::gray (0.2126 r + 0.7152 g +
0.0722 b).  The reference stores luminances as RGB spectra with three equal channels and
reads them back with gray(), so a stored value v is read as 0.2126 v + 0.7152 v + 0.0722 v
(`_gray_rep`), which is not always v in floating point."""
import numpy as np

EPS = 1.0e-12   # core/common.h:55


def resolve(film):
    """Film::save: (H, W, 4) sums and weights -> (H, W, 3) float64 (core/film.cc:25-28)."""
    f = np.asarray(film, np.float64)
    return f[..., :3] / (f[..., 3:4] + EPS)


def _gray(rgb):
    return 0.2126 * rgb[..., 0] + 0.7152 * rgb[..., 1] + 0.0722 * rgb[..., 2]


def _gray_rep(v):
    return 0.2126 * v + 0.7152 * v + 0.0722 * v


def _log_mean(L):
    """logMean (core/tmo.cc:15-27), summed in the reference's row-major order."""
    s = 0.0
    for v in np.log(L + EPS).ravel():
        s += v
    return np.exp(s / L.size)


def reinhard(film, alpha):
    """ReinhardTmo::apply and whitePoint (core/tmo.cc:81-124)."""
    img = resolve(film)
    L = _gray(img)
    n = L.size
    Ls = np.sort(L.ravel())
    Lmax = Ls[min(int(n * 0.99), n - 1)]
    Lmin = Ls[min(int(n * 0.01), n - 1)]
    Lwhite = 1.5 * 2.0 ** (np.log2(Lmax + EPS) - np.log2(Lmin + EPS) - 5)
    Lwa = _log_mean(L)
    Ls_ = (alpha * L) / Lwa
    Ld = (Ls_ * (1.0 + Ls_ / (Lwhite * Lwhite))) / (1.0 + Ls_)
    return img / (L + EPS)[..., None] * Ld[..., None]


def drago(film, p, Ldmax=100.0):
    """DragoTmo::apply (core/tmo.cc:125-159); lumMax starts from 0 (core/tmo.cc:29-41)."""
    img = resolve(film)
    L = _gray(img)
    Lwa = _log_mean(L) / (1.0 + p - 0.85) ** 5.0
    Lmax_wa = max(0.0, float(L.max())) / Lwa
    c1 = np.log(p) / np.log(0.5)
    c2 = (Ldmax / 100.0) / np.log10(1.0 + Lmax_wa)
    L_wa = L / Lwa
    Ld = c2 * np.log1p(L_wa) / np.log(2.0 + 8.0 * (L_wa / Lmax_wa) ** c1)
    return img / (L + EPS)[..., None] * Ld[..., None]


def domain_transform_filter(img, sigma_s, sigma_r, maxiter=20):
    """domainTransformFilter of one channel (core/birateral.cc:86-135): the recursive
    filter of Gastal and Oliveira's domain transform, horizontal then vertical passes,
    maxiter times with a halving kernel width.  Rows (columns) run in parallel; each
    runs forward then backward along its line."""
    H, W = img.shape
    ratio = sigma_s / sigma_r
    dctx = 1.0 + ratio * np.abs(img[:, 1:] - img[:, :-1])   # (H, W-1)
    dcty = 1.0 + ratio * np.abs(img[1:, :] - img[:-1, :])   # (H-1, W)
    out = img.copy()
    for i in range(maxiter):
        sigma_H = sigma_s * np.sqrt(3.0) * 2.0 ** (maxiter - i - 1) / np.sqrt(4.0 ** maxiter - 1.0)
        a = np.exp(-np.sqrt(2.0) / sigma_H)
        V = a ** dctx   # recursiveFilterHorizontal (core/birateral.cc:50-84)
        for x in range(1, W):
            out[:, x] = out[:, x] + V[:, x - 1] * (out[:, x - 1] - out[:, x])
        for x in range(W - 2, -1, -1):
            out[:, x] = out[:, x] + V[:, x] * (out[:, x + 1] - out[:, x])
        V = a ** dcty   # recursiveFilterVertical (core/birateral.cc:14-48)
        for y in range(1, H):
            out[y] = out[y] + V[y - 1] * (out[y - 1] - out[y])
        for y in range(H - 2, -1, -1):
            out[y] = out[y] + V[y] * (out[y + 1] - out[y])
    return out


def durand(film, target_contrast, sigma_space=0.02, sigma_color=0.4):
    """DurandTMO::apply and birateralSeparation (core/tmo.cc:161-243)."""
    img = resolve(film)
    H, W = img.shape[:2]
    l = _gray(img)
    tmp = img / (l + EPS)[..., None]
    # birateralSeparation: filter log10 luminance, split into base and detail
    logL = np.log10(_gray_rep(l) + 1.0e-6)
    fil = domain_transform_filter(logL, max(W, H) * sigma_space, sigma_color)
    lbase = np.maximum(0.0, 10.0 ** _gray_rep(fil) - 1.0e-6)
    ldetail = l / (lbase + EPS)
    log_base = np.log10(_gray_rep(lbase) + EPS)
    log_detail = np.log10(_gray_rep(ldetail) + EPS)
    cf = np.log(target_contrast) / (log_base.max() - log_base.min())
    log_abs = cf * log_base.max()
    m = 10.0 ** (_gray_rep(log_base) * cf + _gray_rep(log_detail) - log_abs)
    return _clamp01(tmp * m[..., None])


def _clamp01(c):
    """Spectrum::clamp(c, 0, 1) = maximum(lo, minimum(c, hi)) with std::max / std::min per
    channel (core/spectrum.cc:697-713): a NaN channel becomes 0."""
    t = np.where(1.0 < c, 1.0, c)
    return np.where(0.0 < t, t, 0.0)
