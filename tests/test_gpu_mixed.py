"""Mixed-precision path (FP32 bulk, FP64 series/decisions, FP64 redo of
guarded pixels) against the reference and against the FP64 drop-in.

Bar: per-pixel relative error <= 1e-5: vs the reference's image where it is
stable, vs the quadruple-precision value of its algorithm where it is not
(widened only where that exact value itself moves by more under few-ulp input
changes; see test_gpu_golden)."""
import numpy as np
import pytest

import crystalscatter_gb300 as cs
from crystalscatter_gb300 import configs as C
from helpers import compare_with_exact, golden, golden_cases, rel_error, written_mask

CASES = golden_cases()["images"]
TOL = 1e-5

pytestmark = pytest.mark.gpu


def run(params, ign_cbs, mode, ign_new_switch=0):
    c = cs.SasCalc_GENERIC_calculation()
    c.setParams(params)
    c.doCalculation(0, bool(ign_new_switch), bool(ign_cbs), mode=mode)
    img = c.data()
    redo = c.mixed_redo_pixels() if mode == cs.CS_MODE_MIXED else 0
    c.cleanup()
    return img, redo


@pytest.mark.parametrize("name", sorted(CASES))
def test_mixed_matches_reference(name):
    case = CASES[name]
    g = golden(name)
    img, redo = run(case["params"], case["ign_cbs"], cs.CS_MODE_MIXED, case.get("ign_new_switch", 0))
    m = written_mask(case["params"], img.shape)
    r = compare_with_exact(img, g, mask=m, tol=TOL)
    print(name, "redo", redo, r)
    assert r["n_bad"] == 0, r
    assert r["max_rel_well"] <= TOL, r


@pytest.mark.parametrize("workload", ["sphere", "cyl_gauss", "cyl_gauss_x", "sphere_fcc"])
def test_mixed_matches_fp64_full_size(workload):
    params = C.WORKLOADS[workload]
    if workload == "cyl_gauss_x":
        params = C.scaled(params, 128)  # the FP64 nested Romberg takes seconds at full size
    ref, _ = run(params, 0, cs.CS_MODE_FP64)
    img, redo = run(params, 0, cs.CS_MODE_MIXED)
    rel, mism = rel_error(img, ref)
    fin = np.isfinite(rel)
    print(workload, "pixels", img.size, "redo", redo, "max", rel[fin].max(), "p99.99", np.quantile(rel[fin], 0.9999),
          "median", np.median(rel[fin]))
    assert mism == 0
    assert rel[fin].max() <= TOL
