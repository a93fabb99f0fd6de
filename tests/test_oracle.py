"""The CPU oracle pinned against the reference's own output (golden fixtures,
generated from the reference by tests/golden/make_golden.py) and, when the
reference build is present, against the reference run live."""
import numpy as np
import pytest

from helpers import golden, golden_cases, rel_error, written_mask
from oracle import cpu_oracle

CASES = golden_cases()["images"]


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_golden(name):
    case = CASES[name]
    if case.get("ign_new_switch") or not cpu_oracle.supported(cpu_oracle.prepare(case["params"], case["ign_cbs"])):
        pytest.skip("generic pixel function: pinned on the GPU against the reference's images directly")
    g = golden(name)
    img = cpu_oracle.image(case["params"], ign_cbs=case["ign_cbs"])
    assert img.shape == g["image"].shape
    m = written_mask(case["params"], img.shape)
    rel, mism = rel_error(img[m], g["image"][m])
    assert mism == 0
    assert rel.max() <= 1e-13, f"max rel {rel.max():.3e}"


def test_oracle_fit_matches_reference_golden():
    fitcases = golden_cases()["fit"]
    target = np.load(__import__("os").path.join(__import__("helpers").GOLDEN, "fit_target.npy"))
    for vname, v in fitcases["variants"].items():
        chi2, cnt, nan, fqs = cpu_oracle.fit(fitcases["params"], target, bstop=v["bstop"], border=v["border"],
                                             nofit=[tuple(x) for x in v["nofit"]])
        assert cnt == v["cnt"] and nan == v["nancnt"], vname
        assert abs(chi2 - v["chi2"]) <= 1e-12 * abs(v["chi2"]), (vname, chi2, v["chi2"])
