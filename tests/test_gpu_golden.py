"""FP64 GPU drop-in against the reference's own images (golden fixtures).

Bar: per-pixel relative error <= 1e-10 on every pixel the reference computes
stably. Where the reference's own result moves under one-ulp changes of the
math library (the golden "cond" map; e.g. series/asymptote or Romberg stop
decisions near their thresholds, and the catastrophically cancelling cylinder
F(q) series of the BCT case), the GPU must stay within 100x that spread. The
number of such ill-conditioned pixels is part of the report."""
import numpy as np
import pytest

import crystalscatter_gb300 as cs
from helpers import compare_to_reference, golden, golden_cases, written_mask

CASES = golden_cases()["images"]
TOL = 1e-10

pytestmark = pytest.mark.gpu


def run_case(case, mode=cs.CS_MODE_FP64):
    c = cs.SasCalc_GENERIC_calculation()
    c.setParams(case["params"])
    c.doCalculation(0, bool(case.get("ign_new_switch", 0)), bool(case["ign_cbs"]), mode=mode)
    img = c.data()
    dims = [c.minX(), c.maxX(), c.minY(), c.maxY()]
    c.cleanup()
    return img, dims


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp64_image_matches_reference(name):
    case = CASES[name]
    g = golden(name)
    img, dims = run_case(case)
    assert dims == [int(v) for v in g["dims"]]
    m = written_mask(case["params"], img.shape)
    r = compare_to_reference(img, g["image"], g["cond"], mask=m, tol=TOL)
    print(name, r)
    assert r["n_bad"] == 0, r
    assert r["max_rel_well"] <= TOL, r
