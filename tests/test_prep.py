"""Host preparation against the reference's own prepared constants.

The golden fixtures hold, per case, the coefficient arrays, series/asymptote
switch points, orientation norm and reflection tables that the reference's
prepareCalculation()/coefficients() produced (tests/golden/make_golden.py).
The library's preparation must reproduce them bit for bit (up to the last
bit of long-double rounding differences between x86 and aarch64)."""
import numpy as np
import pytest

from crystalscatter_gb300 import prepared
import crystalscatter_gb300 as cs
from helpers import golden, golden_cases, params_struct

CASES = golden_cases()["images"]

# The reference's isotropic-ellipsoid coefficients (Source/sc_calc_generic_cpu.cpp:
# 3004-3011) build carr4f from fsum[1..n], which nothing in that case writes:
# its values (and limq4f) are whatever the allocation held. The ellipsoid
# pixel function takes F(q) = P(q) and reads neither.
UNINIT_F = {"carr4f", "limq4f"}


# The orientation-averaged cylinder's F(q) coefficients are formed only for
# lattices, the only pixel functions that read them.
F_ONLY_LATTICE = {"carr1f", "carr2f", "carr4f", "carr5f", "carr6f", "limq1f", "limq4f"}


def _skipped(case, name):
    p = case["params"]
    if p.get("ComboBoxParticle") == 5 and name in UNINIT_F:
        return True
    no_lattice = p.get("LType", 12) == 12
    return no_lattice and p.get("ComboBoxParticle") == 1 and p.get("Ordis", 0) == 0 and name in F_ONLY_LATTICE

ARR = {"carr1p": ("carrp", 0), "carr2p": ("carrp", 1), "carr3p": ("carrp", 2), "carr4p": ("carrp", 3),
       "carr5p": ("carrp", 4), "carr6p": ("carrp", 5), "carr1f": ("carrf", 0), "carr2f": ("carrf", 1),
       "carr4f": ("carrf", 3), "carr5f": ("carrf", 4), "carr6f": ("carrf", 5)}


def _close(a, b, rtol):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    same = (a == b) | (np.isnan(a) & np.isnan(b))
    with np.errstate(invalid="ignore", over="ignore"):
        rel = np.abs(a - b) / np.maximum(np.abs(a), 1e-300)
    return bool(np.all(same | (rel <= rtol)))


@pytest.mark.parametrize("name", sorted(CASES))
def test_prepared_constants_match_reference(name):
    case = CASES[name]
    g = golden(name)
    p = params_struct(cs, case["params"])
    rc, P, msg = prepared.prepare(p, 0, case["ign_cbs"])
    assert rc == 0, msg
    for a, (field, k) in ARR.items():
        if _skipped(case, a) or a not in g:
            continue  # (carr2f is stored for the cases whose pixel function reads it)
        ours = np.array(getattr(P, field)[k][:])
        assert _close(g[a], ours, 1e-15), a
    ours11 = np.array(P.carr11pm).reshape(131, 131)
    assert _close(g["carr11pm"].reshape(131, 131), ours11, 1e-15)
    for s in ("limq1", "limq2", "limq3", "limq4", "limq5", "limq6"):
        assert _close(g["s_" + s], P.limq[int(s[4:])], 1e-15), s
    for s in ("limq1f", "limq4f"):
        if _skipped(case, s):
            continue
        assert _close(g["s_" + s], P.limqf[int(s[4])], 1e-15), s
    assert _close(g["s_norm"], P.norm, 1e-15)
    assert _close(g["s_order"], P.order, 1e-15)
    assert int(g["s_orcase"]) == P.orcase
    if P.lattice:
        assert int(g["s_peakmax1"]) == P.peakmax1
        assert int(g["s_peakmax2"]) == P.peakmax2
        for i in (1, 2, 3):
            assert _close(g[f"s_latpar{i}"], P.latpar[i], 1e-15)
        n = P.peakmax2 + 1
        n1 = P.peakmax1 + 1  # rows beyond peakmax1 are not part of the result
        assert np.array_equal(g["latpar1"][:n1], np.array(P.latpar1)[:n1])
        assert np.array_equal(g["latpar2"][:n], np.array(P.latpar2)[:n])
        assert _close(g["latpar3"][:n], np.array(P.latpar3)[:n], 1e-7)
    # extents
    x0, x1, y0, y1 = [int(v) for v in g["dims"]]
    assert (P.xmin, P.xmax, P.ymin, P.ymax) == (x0, x1, y0, y1)


@pytest.mark.parametrize("name", sorted(golden_cases()["rejected"]))
def test_rejected_parameters_same_message(name):
    case = golden_cases()["rejected"][name]
    p = params_struct(cs, case["params"])
    rc, P, msg = prepared.prepare(p, 0, 0)
    assert rc == cs.CS_ERR_PARAM
    assert msg == case["error"]
