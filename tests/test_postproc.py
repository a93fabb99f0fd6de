"""The r-phi transform against the reference's own (Source/sc_postproc.cpp,
compiled into oracle/_ref/libscpost.so by oracle/build_ref.sh where the
reference sources are present), and size-independent properties."""
import ctypes
import os

import numpy as np
import pytest

from crystalscatter_gb300 import postproc

LIB = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "libscpost.so")


def _ref_rphi(d, x0, x1, y0, y1, xc, yc, s, scale=False, clip=False, clip40=False):
    lib = ctypes.CDLL(LIB)
    lib.ref_rphi.argtypes = [ctypes.c_int] * 7 + [ctypes.c_void_p] + [ctypes.c_int] * 3 + [ctypes.c_void_p]
    a = np.ascontiguousarray(d, dtype=np.float64)
    out = np.empty(s * s)
    assert lib.ref_rphi(x0, x1, y0, y1, xc, yc, s, a.ctypes.data, int(scale), int(clip), int(clip40),
                        out.ctypes.data) == 0
    return out.reshape(s, s)


def _image(n=64, m=None, seed=5):
    m = m or n
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:m, 0:n]
    r = np.hypot(x - n / 2 + 0.3, y - m / 2 - 0.7)
    return (1.0 + np.cos(r / 3.0)) * np.exp(-r / 20.0) + 0.01 * rng.random((m, n))


@pytest.mark.skipif(not os.path.exists(LIB), reason="reference post-processing not built")
@pytest.mark.parametrize("case", [
    dict(n=64, s=40, x0=-32, y0=-32, xc=0, yc=0),
    dict(n=64, s=64, x0=-32, y0=-32, xc=5, yc=-3),
    dict(n=48, m=40, s=33, x0=-24, y0=-20, xc=-2, yc=1),
    dict(n=64, s=50, x0=0, y0=0, xc=20, yc=30),
    dict(n=64, s=40, x0=-32, y0=-32, xc=0, yc=0, scale=True),
    dict(n=64, s=40, x0=-32, y0=-32, xc=0, yc=0, scale=True, clip=True),
    dict(n=64, s=40, x0=-32, y0=-32, xc=0, yc=0, scale=True, clip40=True),
])
def test_rphi_matches_reference(case):
    n, m, s = case["n"], case.get("m", case["n"]), case["s"]
    d = _image(n, m)
    x0, y0 = case["x0"], case["y0"]
    kw = {k: case.get(k, False) for k in ("scale", "clip", "clip40")}
    ref = _ref_rphi(d, x0, x0 + n, y0, y0 + m, case["xc"], case["yc"], s, **kw)
    got = postproc.rphi(d, x0, x0 + n, y0, y0 + m, case["xc"], case["yc"], s, **kw)
    written = ~np.isnan(ref)
    assert written.sum() > 0.8 * s * s
    # entries the reference leaves unwritten are 0 here (after clip: 0 maps to 0)
    assert np.all(got[~written] == 0.0)
    scale = np.max(np.abs(ref[written]))
    assert np.max(np.abs(got[written] - ref[written])) <= 1e-12 * scale


def test_rphi_constant_image():
    d = np.full((30, 30), 2.5)
    out = postproc.rphi(d, -15, 15, -15, 15, 0, 0, 20)
    nz = out != 0
    # inside the image every average of a constant is that constant
    assert np.allclose(out[:, 0][nz[:, 0]], 2.5)
    assert np.allclose(out[nz], 2.5)


def test_rphi_radial_image_is_angle_independent():
    n = 80
    y, x = np.mgrid[0:n, 0:n]
    d = np.exp(-np.hypot(x - n // 2, y - n // 2) / 10.0)
    out = postproc.rphi(d, -n // 2, n // 2, -n // 2, n // 2, 0, 0, 32)
    # columns inside the inscribed circle: every angle sees the same radius
    # (row 0 takes its column index from a float sum without an offset, so a
    # step just below an integer lands one column lower there than in the
    # other rows: it is left out)
    for k in range(1, 10):
        col = out[1:32, k]
        col = col[col > 0]
        assert np.ptp(col) <= 0.05 * np.max(col)


def test_rphi_rejects_positive_minimum():
    with pytest.raises(ValueError):
        postproc.rphi(np.ones((4, 4)), 1, 5, 0, 4, 2, 2, 4)


def test_rphi_matches_reference_golden():
    """postproc.rphi against the reference's own outputs committed in
    tests/golden/rphi.npz (made by tests/golden/make_rphi_golden.py)."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_rphi_golden import CASES, image
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rphi.npz"))
    for k in range(len(CASES)):
        ref = z[f"ref{k}"]
        x0, x1, y0, y1, xc, yc, s, f = (int(v) for v in z[f"args{k}"])
        got = postproc.rphi(image(x1 - x0, y1 - y0, 100 + k), x0, x1, y0, y1, xc, yc, s,
                            scale=bool(f & 1), clip=bool(f & 2), clip40=bool(f & 4))
        written = ~np.isnan(ref)
        assert np.all(got[~written] == 0.0)
        assert np.max(np.abs(got[written] - ref[written])) <= 1e-12 * np.max(np.abs(ref[written]))
