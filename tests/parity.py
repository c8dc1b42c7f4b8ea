"""Comparison rules between the GPU (FP32) and the CPU oracle (FP64).

Hit primitives must be identical except for *stated FP32 ties*, decided in double:
  * two different primitives both hit within 1e-6 relative t of each other
    (shared edges / vertices);
  * the ray passes within the FP32 rounding band of an edge of the primitive that
    one side hit and the other did not (the barycentric margin, min(u, v, 1-u-v), is
    below 8 * 2^-24 times the condition number of the Moller-Trumbore terms);
  * for any-hit, the nearest surface lies within 1e-5 relative of tmax.
Hit distances of identical primitives must agree within 1e-5 relative.
Images: per pixel and channel, z = (mean_gpu - mean_ref) / sqrt(var_gpu + var_ref + f^2)
(variances of the means; f = 1e-5 x |mean| absorbs FP32-vs-FP64 rounding where a pixel
sees a constant radiance, e.g. a uniform region of the environment map, and both
variances are zero); at most 1 % of |z| may exceed 3 (a Gaussian gives 0.27 %).
"""
from __future__ import annotations

import numpy as np

EPS32 = 2.0 ** -24
T_REL_TOL = 1e-5
TIE_T_REL = 1e-6


def mt_double(verts, prim, org, dir):
    """Moller-Trumbore in double for ray i against triangle prim[i]: t, u, v, margin tol."""
    v = verts[prim].astype(np.float64)
    v0, v1, v2 = v[:, 0:3], v[:, 3:6], v[:, 6:9]
    o = org.astype(np.float64)
    d = dir.astype(np.float64)
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    e1, e2 = v1 - v0, v2 - v0
    pv = np.cross(d, e2)
    det = np.einsum("ij,ij->i", e1, pv)
    tv = o - v0
    qv = np.cross(tv, e1)
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / det
        u = np.einsum("ij,ij->i", tv, pv) * inv
        w = np.einsum("ij,ij->i", d, qv) * inv
        t = np.einsum("ij,ij->i", e2, qv) * inv
        kappa = (np.linalg.norm(tv, axis=1) * np.linalg.norm(pv, axis=1) +
                 np.linalg.norm(qv, axis=1)) / np.abs(det)
    margin = np.minimum(np.minimum(u, w), 1.0 - u - w)
    tol = 8.0 * EPS32 * (1.0 + np.nan_to_num(kappa, nan=1e30, posinf=1e30))
    return t, u, w, margin, tol


def classify_closest(verts, org, dir, prim_gpu, t_gpu, prim_ref, t_ref):
    """Returns dict with counts: total, equal, ties, fail, t_fail, t_max_rel."""
    n = prim_ref.shape[0]
    same = prim_gpu == prim_ref
    res = {"total": int(n), "equal": int(same.sum())}
    hit = same & (prim_ref >= 0)
    rel = np.abs(t_gpu[hit].astype(np.float64) - t_ref[hit]) / np.maximum(t_ref[hit], 1e-30)
    res["t_max_rel"] = float(rel.max()) if rel.size else 0.0
    res["t_fail"] = int((rel > T_REL_TOL).sum())
    mis = np.nonzero(~same)[0]
    tie = np.zeros(mis.size, bool)
    if mis.size:
        pg, pr = prim_gpu[mis], prim_ref[mis]
        o, d = org[mis], dir[mis]
        # edge band of the reference's primitive (the GPU missed it or chose another)
        ok_r = pr >= 0
        if ok_r.any():
            t_r, _, _, m_r, tol_r = mt_double(verts, pr[ok_r], o[ok_r], d[ok_r])
            tie[ok_r] |= m_r <= tol_r
        ok_g = pg >= 0
        if ok_g.any():
            t_g, _, _, m_g, tol_g = mt_double(verts, pg[ok_g], o[ok_g], d[ok_g])
            tie[ok_g] |= m_g <= tol_g
        both = ok_r & ok_g
        if both.any():
            t_r2, *_ = mt_double(verts, pr[both], o[both], d[both])
            t_g2, *_ = mt_double(verts, pg[both], o[both], d[both])
            tie[both] |= np.abs(t_g2 - t_r2) <= TIE_T_REL * np.abs(t_r2)
    res["ties"] = int(tie.sum())
    res["fail"] = int((~tie).sum())
    res["fail_idx"] = mis[~tie][:20].tolist()
    return res


def classify_any(verts, org, dir, tmax, hit_gpu, hit_ref, prim_near, t_near, prim_gpu_c=None, t_gpu_c=None):
    """Any-hit mismatches are ties when the nearest surface (oracle closest hit
    prim_near/t_near, and the GPU's own closest hit when given) sits within 1e-5
    relative of tmax or in the FP32 edge band."""
    mis = np.nonzero(hit_gpu != hit_ref)[0]
    tie = np.zeros(mis.size, bool)
    if mis.size:
        tm = tmax[mis].astype(np.float64)
        pn, tn = prim_near[mis], t_near[mis]
        ok = pn >= 0
        tie[ok] |= np.abs(tn[ok] - tm[ok]) <= T_REL_TOL * np.maximum(tm[ok], 1e-30)
        if ok.any():
            _, _, _, m, tol = mt_double(verts, pn[ok], org[mis][ok], dir[mis][ok])
            tie[ok] |= m <= tol
        if prim_gpu_c is not None:
            pg, tg = prim_gpu_c[mis], t_gpu_c[mis]
            okg = pg >= 0
            tie[okg] |= np.abs(tg[okg] - tm[okg]) <= T_REL_TOL * np.maximum(tm[okg], 1e-30)
            if okg.any():
                _, _, _, m, tol = mt_double(verts, pg[okg], org[mis][okg], dir[mis][okg])
                tie[okg] |= m <= tol
    return {"total": int(hit_ref.size), "mismatch": int(mis.size), "ties": int(tie.sum()),
            "fail": int((~tie).sum()), "fail_idx": mis[~tie][:20].tolist()}


ROUNDING_FLOOR = 1e-5


def zscores(mean_a, var_a, mean_b, var_b):
    floor = (ROUNDING_FLOOR * np.maximum(np.abs(mean_a), np.abs(mean_b))) ** 2
    v = var_a + var_b + floor
    with np.errstate(divide="ignore", invalid="ignore"):
        z = (mean_a - mean_b) / np.sqrt(v)
    z[(v == 0) & (mean_a == mean_b)] = 0.0
    z[(v == 0) & (mean_a != mean_b)] = np.inf
    return z


# ---------------------------------------------------------------- BSDFs, function by function
BSDF_REL_TOL = 1e-4     # f and pdf, relative to the oracle
WI_ABS_TOL = 1e-5       # sampled unit directions, per component
BSDF_ABS_FLOOR = 1e-7   # values below this fraction of the table's largest are compared absolutely
ULP_STEPS = 4           # input perturbation of the conditioning test, in float32 ulps


def bsdf_mismatch(f, pdf, fr, pr, rel=BSDF_REL_TOL):
    """Rows where f (n, 3) or pdf (n,) differ from the oracle's fr, pr by more than rel
    relative (with an absolute floor of BSDF_ABS_FLOOR times the largest oracle value)."""
    f, pdf, fr, pr = (np.asarray(a, np.float64) for a in (f, pdf, fr, pr))
    fa = BSDF_ABS_FLOOR * max(float(np.abs(fr).max(initial=0.0)), 1e-30)
    pa = BSDF_ABS_FLOOR * max(float(np.abs(pr).max(initial=0.0)), 1e-30)
    bad_f = (np.abs(f - fr) > rel * np.abs(fr) + fa).any(axis=1)
    bad_p = np.abs(pdf - pr) > rel * np.abs(pr) + pa
    return bad_f | bad_p


BECKMANN_CDF_TOL = 1e-6   # the Beckmann slope inversion stops within this of its target (core/microfacet.cc:120)
BECKMANN_TAIL = 1e-4      # first numbers this close to 0 or 1 meet that tolerance and the erfinv clamp


def bsdf_conditioning(oracle, inputs, rows, fr, pr, wr=None, sr=None, trials=8, seed=0, abs_tol=None):
    """Stated FP32 ties among the flagged rows: the oracle's output (f, pdf and, for
    sampling, the direction and type) moves beyond the contract's tolerance when every
    input component moves by up to ULP_STEPS float32 ulps, or by abs_tol[k] (absolute,
    per input k; e.g. BECKMANN_CDF_TOL on the first random number of a Beckmann sampler,
    whose result the reference itself defines only to that tolerance).  oracle(*inputs)
    returns (f, pdf) or (f, pdf, wi, type)."""
    idx = np.nonzero(rows)[0]
    tie = np.zeros(rows.shape[0], bool)
    if idx.size == 0:
        return tie
    rng = np.random.default_rng(seed)
    sub = [np.asarray(x, np.float64)[idx] for x in inputs]
    base_f, base_p = fr[idx], pr[idx]
    for _ in range(trials):
        pert = []
        for k, x in enumerate(sub):
            step = ULP_STEPS * np.spacing(np.abs(x).astype(np.float32)).astype(np.float64)
            if abs_tol is not None and abs_tol[k] is not None:
                step = np.maximum(step, np.asarray(abs_tol[k], np.float64))
            pert.append(x + step * rng.choice([-1.0, 1.0], size=x.shape))
        out = oracle(*pert)
        moved = bsdf_mismatch(out[0], out[1], base_f, base_p)
        if wr is not None:
            both = (out[1] > 0) & (base_p > 0)
            moved |= both & (np.abs(out[2] - wr[idx]).max(axis=1) > WI_ABS_TOL)
            moved |= out[3] != sr[idx]
        tie[idx[moved]] = True
    return tie
