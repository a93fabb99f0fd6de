"""The library's simplex (cs_simplex_minimize) and the Python restatement
(oracle/simplex_oracle.py) against the reference's own doSimplexFit2D
(Source/sc_simplexfit2d.cpp), whose trajectories on analytic objectives are
committed in tests/golden/simplex_ref.json (tests/golden/make_simplex_golden.py):
every evaluated point bit for bit, the results, iterations, evaluation counts
and the abort flag."""
import ctypes
import json
import os
import sys

import numpy as np
import pytest

import crystalscatter_gb300 as cs
from oracle import simplex_oracle

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_simplex_golden import CASES, LIB, OBJECTIVES, run_reference  # noqa: E402

GOLDEN = os.path.join(HERE, "golden", "simplex_ref.json")


def _golden(name):
    g = json.load(open(GOLDEN))[name]
    g["points"] = [[float.fromhex(x) for x in p] for p in g["points"]]
    g["fitres"] = {k: float.fromhex(v) for k, v in g["fitres"].items()}
    return g


def _table(rows):
    return [{"key": r[0], "min": r[1], "max": r[2], "start": r[3], "used": bool(r[4])} for r in rows]


def _same(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


@pytest.mark.parametrize("name", sorted(CASES))
def test_library_simplex_follows_reference_trajectory(name):
    rows, obj, stp, maxit, ftol = CASES[name]
    g = _golden(name)
    fn = OBJECTIVES[obj]
    points = []

    def f(pts):
        out = []
        for p in pts:
            points.append([float(v) for v in p])
            out.append(fn(list(p)))
        return out

    got, rep = cs.simplex_minimize(f, _table(rows), stp=stp, maxit=maxit, ftol=ftol, schedule=cs.CS_FIT_SEQUENTIAL)
    assert len(points) == len(g["points"])
    assert _same(points, g["points"])
    assert _same([got[k] for k in g["order"]], [g["fitres"][k] for k in g["order"]])
    assert rep["repetitions"] == g["repetitions"]
    assert rep["images"] == g["images"]
    assert rep["aborted"] == g["aborted"]


@pytest.mark.parametrize("name", sorted(CASES))
def test_restatement_matches_reference(name):
    rows, obj, stp, maxit, ftol = CASES[name]
    g = _golden(name)
    fn = OBJECTIVES[obj]
    res, reps, _, n = simplex_oracle.simplex(lambda v: fn(list(v)), _table(rows), stp=stp, maxit=maxit, ftol=ftol)
    assert _same([res[k] for k in g["order"]], [g["fitres"][k] for k in g["order"]])
    assert reps == g["repetitions"]
    assert n == g["images"]


@pytest.mark.skipif(not os.path.exists(LIB), reason="reference simplex not built")
@pytest.mark.parametrize("name", sorted(CASES))
def test_golden_is_current(name):
    rows, obj, stp, maxit, ftol = CASES[name]
    g = _golden(name)
    r = run_reference(rows, OBJECTIVES[obj], stp, maxit, ftol)
    assert _same(r["points"], g["points"])
    assert r["repetitions"] == g["repetitions"] and r["aborted"] == g["aborted"]
