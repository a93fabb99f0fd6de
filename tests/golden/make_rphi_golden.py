"""Writes tests/golden/rphi.npz: r-phi images computed by the reference's
own SasCalc_PostProc::generateRphi (Source/sc_postproc.cpp, compiled into
oracle/_ref/libscpost.so by oracle/build_ref.sh) for seeded test images.
Entries the reference leaves unwritten are NaN. The test images are not
stored: image() regenerates them from their seeds (100 + case index). Run here, where the
reference sources exist:  python tests/golden/make_rphi_golden.py"""
import ctypes
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
LIB = os.path.join(ROOT, "oracle", "_ref", "libscpost.so")

CASES = [
    dict(n=64, m=64, s=40, x0=-32, y0=-32, xc=0, yc=0, flags=0),
    dict(n=96, m=80, s=72, x0=-40, y0=-50, xc=7, yc=-3, flags=0),
    dict(n=64, m=64, s=50, x0=0, y0=0, xc=20, yc=30, flags=0),
    dict(n=128, m=128, s=128, x0=-64, y0=-64, xc=0, yc=0, flags=1),
    dict(n=64, m=64, s=40, x0=-32, y0=-32, xc=3, yc=2, flags=3),
    dict(n=64, m=64, s=40, x0=-32, y0=-32, xc=0, yc=0, flags=5),
]


def image(n, m, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:m, 0:n]
    r = np.hypot(x - n / 2 + 0.3, y - m / 2 - 0.7)
    return (1.0 + np.cos(r / 3.0)) * np.exp(-r / 20.0) + 0.01 * rng.random((m, n))


def main():
    lib = ctypes.CDLL(LIB)
    lib.ref_rphi.argtypes = [ctypes.c_int] * 7 + [ctypes.c_void_p] + [ctypes.c_int] * 3 + [ctypes.c_void_p]
    out = {}
    for k, c in enumerate(CASES):
        d = np.ascontiguousarray(image(c["n"], c["m"], 100 + k))
        s = c["s"]
        r = np.empty(s * s)
        f = c["flags"]
        assert lib.ref_rphi(c["x0"], c["x0"] + c["n"], c["y0"], c["y0"] + c["m"], c["xc"], c["yc"], s,
                            d.ctypes.data, f & 1, (f >> 1) & 1, (f >> 2) & 1, r.ctypes.data) == 0
        out[f"ref{k}"] = r.reshape(s, s)
        out[f"args{k}"] = np.array([c["x0"], c["x0"] + c["n"], c["y0"], c["y0"] + c["m"], c["xc"], c["yc"], s, f])
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "rphi.npz"), **out)


if __name__ == "__main__":
    main()
