"""Fit evaluation and the simplex fit on the GPU.

* doFitCalculation (cs_fit_chi2) against the reference's own chi^2, count and
  NaN count of every mask variant in the golden fixtures;
* the batch fit (cs_batch_fit_chi2, all vertices in one persistent launch,
  replayed as a CUDA graph) equals the single-set chi^2 bit for bit;
* the simplex fit (cs_simplex_fit): the batched schedule reproduces the
  sequential schedule's trajectory exactly; the fit lowers chi^2 and moves the
  parameters towards the values the target was made with."""
import os

import numpy as np
import pytest

import crystalscatter_gb300 as cs
from crystalscatter_gb300 import configs as C
from helpers import GOLDEN, golden_cases

pytestmark = pytest.mark.gpu


def fit_calc(params, target, v):
    c = cs.SasCalc_GENERIC_calculation()
    c.setParams(params)
    h, w = target.shape
    c.setFitData(w, h, target)
    for i, r in enumerate(v.get("nofit", [])):
        c.setNoFitRect(i, *r)
    chi2, cnt, nan = c.doFitCalculation(0, v["bstop"], v["border"])
    c.cleanup()
    return chi2, cnt, nan


def test_fit_chi2_matches_reference():
    fc = golden_cases()["fit"]
    target = np.load(os.path.join(GOLDEN, "fit_target.npy"))
    for name, v in fc["variants"].items():
        chi2, cnt, nan = fit_calc(fc["params"], target, v)
        assert cnt == v["cnt"] and nan == v["nancnt"], name
        assert abs(chi2 - v["chi2"]) <= 1e-10 * abs(v["chi2"]), (name, chi2, v["chi2"])


@pytest.mark.parametrize("variant", ["plain", "border_bstop", "nofit_rects", "corner_threshold"])
def test_batch_fit_equals_single_set(variant):
    fc = golden_cases()["fit"]
    v = fc["variants"][variant]
    target = np.load(os.path.join(GOLDEN, "fit_target.npy"))
    sets = [dict(fc["params"], EditRadius=fc["params"]["EditRadius"] * f, EditSigma=s)
            for f, s in ((0.9, 0.1), (1.0, 0.12), (1.05, 0.08), (1.2, 0.1), (0.97, 0.15))]
    b = cs.SasCalcBatch()
    b.set_fit(target, bstop=v["bstop"], border=v["border"], nofit=v.get("nofit"))
    for _ in range(2):  # second pass replays the captured graph
        b.prepare(sets)
        chi2, cnt, nan = b.fit_chi2(cs.CS_MODE_FP64)
        for k, p in enumerate(sets):
            c2, n2, z2 = fit_calc(p, target, v)
            assert chi2[k] == c2 and cnt[k] == n2 and nan[k] == z2, (variant, k, chi2[k], c2)
    b.cleanup()


def synthetic_target(params):
    c = cs.SasCalc_GENERIC_calculation()
    c.setParams(params)
    c.doCalculation(0, False, False)
    img = c.data()
    c.cleanup()
    return img


def fit_table(truth):
    # The reference's initialisation zeroes the first parameter (in sorted key
    # order) of every initial vertex; EditAzi sorts first, is not used by a
    # sphere without lattice, and its limits 0..360 are not checked.
    return [
        {"key": "EditAzi", "min": 0.0, "max": 360.0, "start": 5.0, "used": True},
        {"key": "EditRadius", "min": 2.0, "max": 30.0, "start": truth["EditRadius"] * 1.15, "used": True},
        {"key": "EditSigma", "min": 0.02, "max": 0.4, "start": truth["EditSigma"] * 0.85, "used": True},
        {"key": "I0", "min": 0.01, "max": 100.0, "start": 1.3, "used": True},
    ]


@pytest.mark.parametrize("mode", [cs.CS_MODE_FP64, cs.CS_MODE_MIXED])
def test_simplex_batched_equals_sequential(mode):
    truth = C.scaled(C.SPHERE, 24)
    target = synthetic_target(truth)
    out = []
    for sched in (cs.CS_FIT_SEQUENTIAL, cs.CS_FIT_BATCHED):
        res, rep = cs.simplex_fit(truth, target, fit_table(truth), stp=0.1, maxit=40, ftol=1e-6, mode=mode,
                                  schedule=sched)
        out.append((res, rep))
    (r0, p0), (r1, p1) = out
    assert r0 == r1
    assert p0["repetitions"] == p1["repetitions"] and p0["chi2"] == p1["chi2"]
    assert p1["images"] >= p0["images"]


def test_simplex_lowers_chi2_towards_truth():
    truth = C.scaled(C.SPHERE, 24)
    target = synthetic_target(truth)
    table = fit_table(truth)
    start = dict(truth, EditAzi=5.0, EditRadius=table[1]["start"], EditSigma=table[2]["start"], I0=table[3]["start"])
    c0, _, _ = fit_calc(start, target, {"bstop": 0, "border": 0})
    res, rep = cs.simplex_fit(truth, target, table, stp=0.1, maxit=200, ftol=1e-8, schedule=cs.CS_FIT_BATCHED)
    assert rep["chi2"] < 0.05 * c0
    assert abs(res["EditRadius"] / truth["EditRadius"] - 1) < abs(table[1]["start"] / truth["EditRadius"] - 1)


def test_simplex_reproduces_first_parameter_initialisation():
    # With EditRadius first in sorted order and limits 2..30, the reference's
    # zeroing of the first parameter puts every initial vertex but the start
    # values below the limit (chi^2 1e20): the simplex cannot move and reports
    # the start vertex, whose first parameter is 0 (sc_simplexfit2d.cpp:375-380).
    truth = C.scaled(C.SPHERE, 16)
    target = synthetic_target(truth)
    table = fit_table(truth)[1:]
    start = dict(truth, EditRadius=table[0]["start"], EditSigma=table[1]["start"], I0=table[2]["start"])
    c0, _, _ = fit_calc(start, target, {"bstop": 0, "border": 0})
    res, rep = cs.simplex_fit(truth, target, table, stp=0.1, maxit=20, ftol=1e-8, schedule=cs.CS_FIT_SEQUENTIAL)
    assert res["EditRadius"] == 0.0
    assert rep["chi2"] == c0
    assert res["EditSigma"] == table[1]["start"] and res["I0"] == table[2]["start"]


def test_fit_from_saved_target_files(tmp_path):
    """The golden target written as the program's saved image (.dat and
    .csv/.txt) with its no-fit rectangles (.dat.nofit), read back with
    crystalscatter_gb300.readers: the chi^2, count and NaN count are the
    reference's for that mask."""
    from crystalscatter_gb300 import readers

    fc = golden_cases()["fit"]
    v = fc["variants"]["nofit_rects"]
    target = np.load(os.path.join(GOLDEN, "fit_target.npy"))
    h, w = target.shape
    base = str(tmp_path / "target")
    readers.write_sascrystal(readers.Image(target, 0, w, 0, h, {"Comment": "fit target"}), base)
    rects = [list(r) for r in v["nofit"]] + [[-1, -1, -1, -1]] * (4 - len(v["nofit"]))
    with open(base + ".dat.nofit", "w") as f:
        for r in rects:
            f.write(" ".join(str(t) for t in r) + "\n")
    for fn, read in ((base + ".dat", readers.read_sascrystal_dat), (base + ".csv", readers.read_sascrystal_csv)):
        img = read(fn)
        assert np.array_equal(img.data, target)
        c = cs.SasCalc_GENERIC_calculation()
        c.setParams(fc["params"])
        c.setFitData(img.cols, img.rows, img.data)
        readers.apply_nofit(c, readers.read_nofit(fn))
        chi2, cnt, nan = c.doFitCalculation(0, v["bstop"], v["border"])
        c.cleanup()
        assert cnt == v["cnt"] and nan == v["nancnt"], fn
        assert abs(chi2 - v["chi2"]) <= 1e-10 * abs(v["chi2"]), (fn, chi2, v["chi2"])
