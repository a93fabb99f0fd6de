"""Writes tests/golden/simplex_ref.json: the reference's own downhill simplex
(SasCalc_SimplexFit2D::doSimplexFit2D, Source/sc_simplexfit2d.cpp, compiled
into oracle/_ref/libscsimplex.so by oracle/build_ref.sh with a stand-in
calculation class that hands each evaluation's parameter values to an
objective) run on analytic objectives: every evaluated point in order, the
fit results, iterations, evaluation count and abort flag. Run here, where
the reference sources exist:  python tests/golden/make_simplex_golden.py"""
import ctypes
import json
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
LIB = os.path.join(ROOT, "oracle", "_ref", "libscsimplex.so")
OBJ = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_void_p)


def rosen(x):
    return float(sum(100.0 * (x[i + 1] - x[i] ** 2) ** 2 + (1 - x[i]) ** 2 for i in range(len(x) - 1)))


def bowl(x):
    x = np.asarray(x, dtype=np.float64)
    return float(np.sum((x - np.arange(1, len(x) + 1)) ** 2 * (1 + np.arange(len(x)))))


def shifted(x):
    return (x[0] - 10.0) ** 2 + (x[1] - 0.2) ** 2


def nan_after(x):
    # a NaN objective away from the start ends the fit through the
    # reference's rtol = NaN abort
    return float("nan") if x[0] > 1.25 else (x[0] - 2.0) ** 2 + (x[1] + 1.0) ** 2


OBJECTIVES = {"rosen": rosen, "bowl": bowl, "shifted": shifted, "nan_after": nan_after}

# (table, objective, stp, maxit, ftol); table rows: key, min, max, start, used
CASES = {
    "rosen_first_free": ([["a", 0, 360, 1.7, 1], ["b", -5, 5, 1.2, 1], ["c", -5, 5, 0.8, 1],
                          ["d", -5, 5, 1.4, 1]], "rosen", 0.1, 300, 1e-9),
    "bowl_with_fixed": ([["p1", -10, 10, 3.0, 1], ["p2", -10, 10, -1.0, 1], ["p0", -10, 10, 0.5, 0],
                         ["p3", -10, 10, 2.5, 1]], "bowl", 0.1, 300, 1e-9),
    "first_param_bounded": ([["r", 2.0, 30.0, 11.0, 1], ["s", 0.0, 1.0, 0.3, 1]], "shifted", 0.1, 300, 1e-9),
    "bowl_few_iterations": ([["u", -10, 10, 4.0, 1], ["v", -10, 10, -3.0, 1], ["w", -10, 10, 1.0, 1]],
                            "bowl", 0.2, 7, 1e-12),
    "bowl_loose_tolerance": ([["u", -10, 10, 4.0, 1], ["v", -10, 10, -3.0, 1]], "bowl", 0.05, 300, 1e-2),
    "nan_abort": ([["a", -10, 10, 0.6, 1], ["b", -10, 10, 0.4, 1]], "nan_after", 0.3, 300, 1e-9),
}


def table_order(table):
    """the simplex's parameter order: fitted keys sorted, then fixed keys sorted"""
    fit = sorted(r[0] for r in table if r[4])
    fix = sorted(r[0] for r in table if not r[4])
    return fit + fix


def run_reference(table, fn, stp, maxit, ftol):
    lib = ctypes.CDLL(LIB)
    lib.ref_simplex_run.restype = ctypes.c_int
    n = len(table)
    names = (ctypes.c_char_p * n)(*[r[0].encode() for r in table])
    dbl = lambda vals: (ctypes.c_double * n)(*vals)  # noqa: E731
    used = (ctypes.c_int * n)(*[int(r[4]) for r in table])
    points = []

    def cb(vals, m, ctx):
        x = [vals[i] for i in range(m)]
        points.append(x)
        return fn(x)

    cfn = OBJ(cb)
    res = (ctypes.c_double * n)()
    reps, imgs, ab = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    lib.ref_simplex_run(n, names, dbl([r[3] for r in table]), dbl([r[1] for r in table]),
                        dbl([r[2] for r in table]), used, ctypes.c_double(stp), maxit, ctypes.c_double(ftol),
                        cfn, None, res, ctypes.byref(reps), ctypes.byref(imgs), ctypes.byref(ab))
    return {"points": points, "fitres": {table[i][0]: res[i] for i in range(n)}, "repetitions": reps.value,
            "images": imgs.value, "aborted": ab.value}


def main():
    out = {}
    for name, (table, obj, stp, maxit, ftol) in CASES.items():
        out[name] = run_reference(table, OBJECTIVES[obj], stp, maxit, ftol)
        out[name]["order"] = table_order(table)
    # float.hex keeps every bit of the trajectory
    enc = {k: dict(v, points=[[float.hex(x) for x in p] for p in v["points"]],
                   fitres={kk: float.hex(vv) for kk, vv in v["fitres"].items()}) for k, v in out.items()}
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "simplex_ref.json"), "w") as f:
        json.dump(enc, f, indent=0)


if __name__ == "__main__":
    main()
