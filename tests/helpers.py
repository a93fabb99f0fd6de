"""Shared test helpers: golden fixture access and the per-pixel error metric."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_cases():
    with open(os.path.join(GOLDEN, "cases.json")) as f:
        return json.load(f)


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


def rel_error(got, ref):
    """Per-pixel relative error |g-r| / max(|r|, tau), tau = 1e-30 * max|r|.

    Non-finite reference pixels must be matched by the same class (NaN by NaN,
    +inf by +inf, -inf by -inf); such pixels get error 0 when matched and inf
    otherwise. Returns (rel array, number of non-finite class mismatches)."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    fin = np.isfinite(ref)
    mism = 0
    rel = np.zeros(ref.shape)
    nf = ~fin
    if nf.any():
        same = (np.isnan(ref) & np.isnan(got)) | ((ref == got) & np.isinf(ref))
        mism = int((nf & ~same).sum())
        rel[nf & ~same] = np.inf
    gf = fin
    tau = 1e-30 * (np.max(np.abs(ref[gf])) if gf.any() else 1.0)
    with np.errstate(invalid="ignore", over="ignore"):
        d = np.abs(got[gf] - ref[gf]) / np.maximum(np.abs(ref[gf]), tau)
    d[~np.isfinite(d)] = np.inf
    rel[gf] = d
    return rel, mism


def params_struct(cs, params):
    """A cs_params filled like the console: defaults, then reference keys."""
    import ctypes
    lib = cs.load_library()
    h = lib.cs_create()
    try:
        for k, v in params.items():
            rc = lib.cs_set_param(h, k.encode(), float(v))
            assert rc == 0, (k, lib.cs_last_error(h))
        p = cs.CsParams()
        lib.cs_get_params(h, ctypes.byref(p))
        return p
    finally:
        lib.cs_destroy(h)


def written_mask(params, shape):
    """Pixels that the reference actually writes. With quadrant expansion the
    mirroring never writes column x = -zmax (Q1, Q2) nor row y = -zmax at
    x < 0 (Q2); the reference leaves whatever the reused image buffer held
    there (Source/sc_calc_generic_cpu.cpp:1246-1269, checkArrays :8201), so
    those pixels are excluded from comparisons."""
    m = np.ones(shape, dtype=bool)
    if params.get("ExpandImage", 0) and not params.get("RadioButtonQ4", 1):
        zmax = int(params["GridPoints"])
        m[:, 0] = False  # x = -zmax
        if params.get("RadioButtonQ2", 0) and not params.get("RadioButtonQ1", 0):
            m[0, :zmax] = False  # y = -zmax, x < 0
    return m


ILL = 1e-12  # a pixel is ill-conditioned when one-ulp libm changes move the reference by more


def compare_to_reference(got, ref, cond, mask=None, tol=1e-10, envelope=100.0):
    """Compares an image with the reference's own image.

    Well-conditioned pixels (cond <= 1e-12) must agree to `tol`. Ill-conditioned
    pixels, whose reference value itself moves by `cond` under one-ulp changes
    of the math library, must agree to envelope*cond (and to tol at least).
    Non-finite pixels must match in class unless the reference's own probe
    turned them finite (cond = inf). Returns a dict of counts and maxima."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    cond = np.asarray(cond, dtype=np.float64)
    if mask is None:
        mask = np.ones(ref.shape, dtype=bool)
    rel, _ = rel_error(got, ref)
    ill = cond > ILL
    allowed = np.maximum(tol, envelope * cond)
    bad = mask & (rel > allowed)
    well = mask & ~ill
    fin_well = well & np.isfinite(rel)
    worst = []
    if bad.any():
        idx = np.flatnonzero(bad.ravel())
        order = np.argsort(-np.nan_to_num(rel.ravel()[idx], nan=np.inf))[:5]
        for j in idx[order]:
            worst.append((int(j), float(rel.ravel()[j]), float(cond.ravel()[j]), float(got.ravel()[j]),
                          float(ref.ravel()[j])))
    return {
        "worst_bad": worst,
        "n": int(mask.sum()),
        "n_ill": int((mask & ill).sum()),
        "n_bad": int(bad.sum()),
        "max_rel_well": float(rel[fin_well].max()) if fin_well.any() else 0.0,
        "median_rel": float(np.median(rel[mask])) if mask.any() else 0.0,
        "max_rel_all": float(np.nanmax(np.where(np.isfinite(rel[mask]), rel[mask], 0))) if mask.any() else 0.0,
        "n_above_tol": int((mask & (rel > tol)).sum()),
    }


HP_SPREAD_FACTOR = 10.0  # multiple of the exact value's own spread allowed where that spread exceeds tol


def compare_with_exact(got, g, mask=None, tol=1e-10, envelope=100.0):
    """Compares an image with a golden record g (the reference's image and
    its one-ulp spread "cond"; where present the quadruple-precision value of
    the reference's algorithm "hp" and that value's spread "hp_cond" under
    4-ulp moves of q and 2-ulp moves of the series coefficients):

    * reference stable (cond <= 1e-12): relative error vs the reference's
      image <= tol;
    * reference ill-conditioned, exact value known: relative error vs hp <=
      max(tol, 10 hp_cond) -- tol wherever the exact value is stable at that
      level; looser only where q or the coefficients alone move it more;
    * reference ill-conditioned, no exact value (the generic pixel function,
      which the oracle does not restate): vs the reference's image within
      max(tol, envelope cond), counted apart.
    Returns a dict of counts and maxima ("n_bad" must be 0)."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(g["image"], dtype=np.float64)
    cond = np.asarray(g["cond"], dtype=np.float64)
    if mask is None:
        mask = np.ones(ref.shape, dtype=bool)
    ill = cond > ILL
    rel_r, _ = rel_error(got, ref)
    allowed = np.full(ref.shape, tol)
    rel = rel_r.copy()
    has_hp = "hp" in g
    if has_hp:
        hp = np.asarray(g["hp"], dtype=np.float64)
        hpc = np.asarray(g["hp_cond"], dtype=np.float64)
        rel_h, _ = rel_error(got, hp)
        rel[ill] = rel_h[ill]
        allowed[ill] = np.maximum(tol, HP_SPREAD_FACTOR * hpc[ill])
        loose = mask & ill & (allowed > tol)
        envelope_px = np.zeros(ref.shape, dtype=bool)
    else:
        allowed[ill] = np.maximum(tol, envelope * cond[ill])
        envelope_px = mask & ill
        loose = envelope_px & (allowed > tol)
    bad = mask & (rel > allowed)
    worst = []
    if bad.any():
        idx = np.flatnonzero(bad.ravel())
        order = np.argsort(-np.nan_to_num(rel.ravel()[idx], nan=np.inf))[:5]
        for j in idx[order]:
            worst.append((int(j), float(rel.ravel()[j]), float(allowed.ravel()[j]), float(got.ravel()[j]),
                          float(ref.ravel()[j])))
    well = mask & ~ill & np.isfinite(rel_r)
    ill_fin = mask & ill & np.isfinite(rel)
    return {
        "worst_bad": worst,
        "n": int(mask.sum()),
        "n_ill": int((mask & ill).sum()),
        "n_checked_vs_exact": int((mask & ill).sum()) if has_hp else 0,
        "n_looser_than_tol": int(loose.sum()),
        "n_envelope": int(envelope_px.sum()),
        "n_bad": int(bad.sum()),
        "max_rel_well": float(rel_r[well].max()) if well.any() else 0.0,
        "max_rel_ill": float(rel[ill_fin].max()) if ill_fin.any() else 0.0,
    }
