"""FP64 GPU drop-in against the reference's own images (golden fixtures).

Bar: max per-pixel relative error <= 1e-10 with matching non-finite classes.
Pixels whose series/asymptote or Romberg decision flips on last-bit
differences of the device math library would exceed that; they are counted
and must stay below 0.1% of the image (none are expected on these cases)."""
import numpy as np
import pytest

import crystalscatter_gb300 as cs
from helpers import golden, golden_cases, rel_error, written_mask

CASES = golden_cases()["images"]
TOL = 1e-10

pytestmark = pytest.mark.gpu


def run_case(case, mode=cs.CS_MODE_FP64):
    c = cs.SasCalc_GENERIC_calculation()
    c.setParams(case["params"])
    c.doCalculation(0, False, bool(case["ign_cbs"]), mode=mode)
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
    rel, mism = rel_error(img[m], g["image"][m])
    assert mism == 0, f"non-finite class mismatches: {mism}"
    bad = int((rel > TOL).sum())
    assert bad <= max(1, img.size // 1000), f"{bad} pixels above {TOL}, max {rel.max():.3e}"
    assert np.median(rel) <= 1e-13
