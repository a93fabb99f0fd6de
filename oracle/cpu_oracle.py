"""Python access to the CPU test oracle (oracle/_build/liboracle_cs.so).

TEST INFRASTRUCTURE: the checker for the GPU path and the timed CPU baseline.
The parameter set is prepared by the library's host preparation
(cs_prepare_params, no CUDA involved) and then evaluated pixel by pixel by
the oracle's own restatement of the reference's per-pixel functions.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

LIB = os.path.join(HERE, "_build", "liboracle_cs.so")
PROBE = os.path.join(HERE, "_build", "liboracle_cs_probe.so")
_lib = None
_probe = None
# probe modes: bit k set = function k (sin cos atan atan2 pow exp sqrt log acos)
# rounded one ulp up, clear = one ulp down
PROBE_MODES = (0x1FF, 0x100, 0x155, 0x0AA)


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            from oracle import build_oracle
            build_oracle.build()
        lib = ctypes.CDLL(LIB)
        lib.oracle_image_rows.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.oracle_image_rows.restype = ctypes.c_long
        lib.oracle_pixel.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        lib.oracle_pixel.restype = ctypes.c_double
        lib.oracle_supported.argtypes = [ctypes.c_void_p]
        lib.oracle_extents.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        lib.oracle_image_rowlist.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                             ctypes.c_int]
        lib.oracle_image_rowlist.restype = ctypes.c_long
        lib.oracle_fit.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_long),
                                   ctypes.POINTER(ctypes.c_long)]
        lib.oracle_fit.restype = ctypes.c_double
        _lib = lib
    return _lib


def load_probe():
    global _probe
    if _probe is None:
        if not os.path.exists(PROBE):
            from oracle import build_oracle
            build_oracle.build()
        lib = ctypes.CDLL(PROBE)
        lib.oracle_image_rows.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.oracle_image_rows.restype = ctypes.c_long
        lib.oracle_set_probe.argtypes = [ctypes.c_int]
        lib.oracle_image_rowlist.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                             ctypes.c_int]
        lib.oracle_image_rowlist.restype = ctypes.c_long
        _probe = lib
    return _probe


def condition(params, ign_cbs=0, nthreads=None, modes=PROBE_MODES):
    """Per-pixel sensitivity of the reference computation to last-bit libm
    differences: max over probe modes of |I_mode - I| / max(|I|, tau), with the
    unperturbed image I. Non-finite disagreements count as inf."""
    P = prepare(params, ign_cbs)
    base, _ = image_prepared(P, nthreads)
    lib = load_probe()
    cond = np.zeros(base.shape)
    fin = np.isfinite(base)
    tau = 1e-30 * (np.max(np.abs(base[fin])) if fin.any() else 1.0)
    for m in modes:
        out = np.zeros(base.shape, dtype=np.float64)
        lib.oracle_set_probe(int(m))
        lib.oracle_image_rows(ctypes.byref(P), out.ctypes.data, 0, 0, int(nthreads or os.cpu_count() or 1))
        with np.errstate(invalid="ignore", over="ignore"):
            d = np.abs(out - base) / np.maximum(np.abs(base), tau)
        same_nf = (~np.isfinite(base)) & ((np.isnan(base) & np.isnan(out)) | (base == out))
        d[same_nf] = 0.0
        d[~np.isfinite(d)] = np.inf
        cond = np.maximum(cond, d)
    lib.oracle_set_probe(0)
    return cond


def prepare(params, ign_cbs=0):
    """Prepared block (CsPrepared) for a dict of reference keys."""
    import crystalscatter_gb300 as cs
    from crystalscatter_gb300 import prepared
    lib = cs.load_library()
    h = lib.cs_create()
    try:
        for k, v in params.items():
            if lib.cs_set_param(h, k.encode(), float(v)) != 0:
                raise KeyError(k)
        p = cs.CsParams()
        lib.cs_get_params(h, ctypes.byref(p))
    finally:
        lib.cs_destroy(h)
    rc, P, msg = prepared.prepare(p, 0, ign_cbs)
    if rc != 0:
        raise RuntimeError(f"prepare failed ({rc}): {msg}")
    return P


def supported(P):
    """True when the oracle restates the pixel function of prepared block P."""
    return bool(load().oracle_supported(ctypes.byref(P)))


def image(params, ign_cbs=0, nthreads=None, rows=None):
    """The oracle image for a parameter dict (all rows, or ihex rows [r0,r1))."""
    P = prepare(params, ign_cbs)
    lib = load()
    if not lib.oracle_supported(ctypes.byref(P)):
        raise RuntimeError("oracle: combination not covered")
    ny = P.ymax - P.ymin
    nx = P.xmax - P.xmin
    out = np.zeros((ny, nx), dtype=np.float64)
    nt = nthreads or os.cpu_count() or 1
    r0, r1 = rows if rows else (0, 0)
    lib.oracle_image_rows(ctypes.byref(P), out.ctypes.data, int(r0), int(r1), int(nt))
    return out


def image_prepared(P, nthreads=None, rows=None):
    lib = load()
    out = np.zeros((P.ymax - P.ymin, P.xmax - P.xmin), dtype=np.float64)
    r0, r1 = rows if rows else (0, 0)
    n = lib.oracle_image_rows(ctypes.byref(P), out.ctypes.data, int(r0), int(r1), int(nthreads or os.cpu_count() or 1))
    return out, n


def fit(params, target, bstop=0, border=0, nofit=()):
    """doFitCalculation on the CPU: (chi2, cnt, nancnt, fqs)."""
    P = prepare(params)
    target = np.ascontiguousarray(target, dtype=np.float64)
    h, w = target.shape
    P.fit_width = w
    P.fit_height = h
    P.fit_bstop = bstop
    P.fit_border = border
    for i in range(4):
        r = nofit[i] if i < len(nofit) else (-1, -1, -1, -1)
        P.nofit_x0[i], P.nofit_y0[i], P.nofit_x1[i], P.nofit_y1[i] = r
    fqs = np.zeros((h, w), dtype=np.float64)
    cnt = ctypes.c_long()
    nan = ctypes.c_long()
    chi2 = load().oracle_fit(ctypes.byref(P), target.ctypes.data, fqs.ctypes.data, ctypes.byref(cnt), ctypes.byref(nan))
    return chi2, cnt.value, nan.value, fqs


# ------------------------------------------------------ quadruple precision

QUAD = os.path.join(HERE, "_build", "liboracle_cs_quad.so")
_quad = None


def load_quad():
    """The oracle evaluated in quadruple precision (oracle/quad_oracle.cpp)."""
    global _quad
    if _quad is None:
        if not os.path.exists(QUAD):
            from oracle import build_oracle
            build_oracle.build()
        lib = ctypes.CDLL(QUAD)
        lib.quad_image.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        lib.quad_image.restype = ctypes.c_long
        lib.quad_set_qmode.argtypes = [ctypes.c_int, ctypes.c_int]
        _quad = lib
    return _quad


def quad_image(P, nthreads=None):
    """The reference algorithm's value on every pixel of prepared block P
    (ctypes struct or buffer), evaluated in quadruple precision and rounded to
    double."""
    lib = load_quad()
    e = (ctypes.c_int * 9)()
    load().oracle_extents(P if isinstance(P, ctypes.Array) else ctypes.byref(P), e)
    out = np.zeros((e[3] - e[2], e[1] - e[0]), dtype=np.float64)
    lib.quad_image(P if isinstance(P, ctypes.Array) else ctypes.byref(P), out.ctypes.data,
                   int(nthreads or os.cpu_count() or 1))
    return out


# one-ulp input perturbations for the stability of the exact value: q moved by
# 4 double ulps (all up, all down, mixed) and the series coefficients moved by
# 2 ulps (all up, all down, alternating by order either way)
QUAD_Q_MODES = (8, 15, 10, 13)
QUAD_COEFF_MODES = (0, 1, 2, 3)


def _perturb_coefficients(P, mode, steps=2):
    import copy
    Q = copy.deepcopy(P)
    for arr in (Q.carrp, Q.carrf):
        a = np.ctypeslib.as_array(arr)
        n = np.arange(a.shape[1])[None, :]
        if mode == 0:
            up = np.ones(a.shape, dtype=bool)
        elif mode == 1:
            up = np.zeros(a.shape, dtype=bool)
        else:
            up = np.broadcast_to((n % 2) == (mode - 2), a.shape)
        with np.errstate(over="ignore"):
            for _ in range(steps):
                a[...] = np.where(up, np.nextafter(a, np.inf), np.nextafter(a, -np.inf))
    return Q


def _spread(img, base, tau):
    with np.errstate(invalid="ignore", over="ignore", divide="ignore"):
        d = np.abs(img - base) / np.maximum(np.abs(base), tau)
    same = (~np.isfinite(base)) & ((np.isnan(img) & np.isnan(base)) | (img == base))
    d[same] = 0.0
    d[~np.isfinite(d)] = np.inf
    return d


def quad_condition(P, nthreads=None, base=None):
    """(exact value H, its spread): the largest relative change of the
    quadruple-precision value under the input perturbations above (tau =
    1e-30 max|H|). A pixel whose spread is large has no stable answer at
    double-precision inputs: its coefficients or q alone decide the value."""
    lib = load_quad()
    H = quad_image(P, nthreads) if base is None else base
    fin = np.isfinite(H)
    tau = 1e-30 * (np.max(np.abs(H[fin])) if fin.any() else 1.0)
    spread = np.zeros(H.shape)
    try:
        for m in QUAD_Q_MODES:
            lib.quad_set_qmode(m, 4)
            spread = np.maximum(spread, _spread(quad_image(P, nthreads), H, tau))
    finally:
        lib.quad_set_qmode(0, 0)
    for m in QUAD_COEFF_MODES:
        spread = np.maximum(spread, _spread(quad_image(_perturb_coefficients(P, m), nthreads), H, tau))
    return H, spread
