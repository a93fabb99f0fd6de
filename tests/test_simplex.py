"""The library's simplex (cs_simplex_minimize, the same code as cs_simplex_fit
with a caller's objective) against the reference's algorithm restated in
Python (oracle/simplex_oracle.py): identical trajectories, results and
evaluation counts on analytic objectives, for both schedules (the batched
schedule only evaluates more points, speculatively)."""
import math

import numpy as np
import pytest

import crystalscatter_gb300 as cs
from oracle import simplex_oracle


def rosen(v):
    # v in table order; a 4-parameter Rosenbrock-like valley plus offsets
    x = np.asarray(v, dtype=np.float64)
    return float(sum(100.0 * (x[i + 1] - x[i] ** 2) ** 2 + (1 - x[i]) ** 2 for i in range(len(x) - 1)))


def bowl(v):
    x = np.asarray(v, dtype=np.float64)
    return float(np.sum((x - np.arange(1, len(x) + 1)) ** 2 * (1 + np.arange(len(x)))))


TABLES = {
    "rosen_first_free": ([{"key": "a", "min": 0, "max": 360, "start": 1.7, "used": True},
                          {"key": "b", "min": -5, "max": 5, "start": 1.2, "used": True},
                          {"key": "c", "min": -5, "max": 5, "start": 0.8, "used": True},
                          {"key": "d", "min": -5, "max": 5, "start": 1.4, "used": True}], rosen),
    "bowl_with_fixed": ([{"key": "p1", "min": -10, "max": 10, "start": 3.0, "used": True},
                         {"key": "p2", "min": -10, "max": 10, "start": -1.0, "used": True},
                         {"key": "p0", "min": -10, "max": 10, "start": 0.5, "used": False},
                         {"key": "p3", "min": -10, "max": 10, "start": 2.5, "used": True}], bowl),
    "first_param_bounded": ([{"key": "r", "min": 2.0, "max": 30.0, "start": 11.0, "used": True},
                             {"key": "s", "min": 0.0, "max": 1.0, "start": 0.3, "used": True}],
                            lambda v: (v[0] - 10.0) ** 2 + (v[1] - 0.2) ** 2),
}


@pytest.mark.parametrize("name", sorted(TABLES))
@pytest.mark.parametrize("schedule", [cs.CS_FIT_SEQUENTIAL, cs.CS_FIT_BATCHED])
def test_simplex_matches_reference_restatement(name, schedule):
    table, f = TABLES[name]
    ref, rep_ref, y_ref, n_ref = simplex_oracle.simplex(f, table, stp=0.1, maxit=300, ftol=1e-9)
    got, rep = cs.simplex_minimize(lambda pts: [f(p) for p in pts], table, stp=0.1, maxit=300, ftol=1e-9,
                                   schedule=schedule)
    assert got == ref
    assert rep["repetitions"] == rep_ref
    assert rep["chi2"] == y_ref
    if schedule == cs.CS_FIT_SEQUENTIAL:
        assert rep["images"] == n_ref
    else:
        assert rep["images"] >= n_ref


def test_first_parameter_initialisation_quirk():
    # the first parameter of every initial vertex starts at 0 + step; with a
    # lower limit of 2 all those vertices are out of bounds and the simplex
    # reports the start vertex with its first parameter 0
    table, f = TABLES["first_param_bounded"]
    ref, rep_ref, y_ref, _ = simplex_oracle.simplex(f, table, stp=0.1, maxit=50, ftol=1e-9)
    assert ref["r"] == 0.0 and y_ref == f([11.0, 0.3])
