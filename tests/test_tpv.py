"""Training-data parameter randomisation (crystalscatter_gb300.tpv) against
the reference's tpvPerformRandom, run in the reference build
(oracle/_ref/libscref.so, oracle/ref_driver.cpp ref_tpv_run) with the same
seed of the C library's generator: the same log text, and the same image
from the randomised parameters (prepared by this library, evaluated by the
CPU oracle)."""
import ctypes

import numpy as np
import pytest

import crystalscatter_gb300 as cs
from crystalscatter_gb300 import configs as C, prepared, tpv
from oracle import cpu_oracle, refbind
from helpers import rel_error

pytestmark = pytest.mark.skipif(not refbind.available(), reason="reference build not available")


def _params(mapping):
    lib = cs.load_library()
    h = lib.cs_create()
    try:
        for k, v in mapping.items():
            assert lib.cs_set_param(h, k.encode(), float(v)) == 0, k
        p = cs.CsParams()
        lib.cs_get_params(h, ctypes.byref(p))
    finally:
        lib.cs_destroy(h)
    return p


CASES = [
    ("sphere", C.scaled(C.SPHERE, 24), ["I0=0.2", "EditRadius=0.1", "EditSigma=0.3", "Base=0.5"], 7),
    ("sphere_fcc", C.scaled(C.SPHERE_FCC, 16),
     ["EditRadius=0.05", "uca=0.1", "ucb=0.1", "ucc=0.1", "EditDomainSize=0.3", "EditDebyeWaller=0.4",
      "EditAzi=0.2", "phi=1"], 11),
    ("cyl_gauss", C.scaled(C.CYL_GAUSS_X, 12), ["Length=0.2", "SigmaL=0.1", "EditDbeta=0.3", "Unknown=0.5"], 3),
]


@pytest.mark.parametrize("name,params,ids,seed", CASES, ids=[c[0] for c in CASES])
def test_tpv_matches_reference(name, params, ids, seed):
    r = refbind.RefCalc(params)
    try:
        rc, log_ref = r.tpv_run(ids, seed, nthreads=4)
        assert rc == 0
        ref = r.image()
    finally:
        r.close()
    p = _params(params)
    t = tpv.TpvRandom()
    tpv.srand(seed)
    log = t.perform(p, ids)
    assert log == log_ref
    rc, P, msg = prepared.prepare(p, 0, 0)
    assert rc == 0, msg
    got, _ = cpu_oracle.image_prepared(P, nthreads=4)
    rel, mism = rel_error(got, ref)
    assert mism == 0
    assert np.max(rel) <= 1e-10, (name, np.max(rel))


def test_tpv_clear_and_repeat():
    p = _params(C.scaled(C.SPHERE, 8))
    r0 = p.radius
    t = tpv.TpvRandom()
    tpv.srand(1)
    t.perform(p, ["EditRadius=0.5"])
    r1 = p.radius
    # a second call scales the value saved at the first, not the new one
    t.perform(p, ["EditRadius=0.5"])
    assert abs(p.radius / r0 - 1) <= 0.5 and abs(r1 / r0 - 1) <= 0.5
    assert t.perform(p, []) == "TPV: clear" and p.tpv_domain_dev == 0.0


def test_tpv_dw_and_azi_restore_first_values():
    p = _params(C.scaled(C.SPHERE_FCC, 8))
    dw0, azi0 = p.debyewaller, p.azi
    t = tpv.TpvRandom()
    tpv.srand(5)
    t.perform(p, ["EditDebyeWaller=0.4", "EditAzi=0.2"])
    assert p.tpv_dw_dev != 0.0
    # a caller changes both between calls without clearing: the next draw
    # starts again from the values saved at the first call, as the reference's
    # hlp->oldval does
    p.debyewaller, p.azi = 2 * dw0, 3 * azi0
    log = t.perform(p, ["EditDebyeWaller=0.4", "EditAzi=0.2"])
    assert p.debyewaller == dw0 and p.azi == azi0
    v_dw = float(log.split("EditDebyeWaller = ")[1].split()[0])
    assert abs(v_dw / (dw0 * dw0 / 3.0) - 1) <= 0.4 + 1e-6
    # clearing resets both randomised factors
    assert t.perform(p, []) == "TPV: clear"
    assert p.tpv_dw_dev == 0.0 and p.tpv_domain_dev == 0.0


def test_tpv_length_adjustments():
    p = _params(dict(C.scaled(C.SPHERE, 8), ComboBoxParticle=2, EditRadius=10.0, Length=5.0))
    tpv.TpvRandom().perform(p, ["I0=0.0001"])
    assert p.length == 25.0  # disk: length <= 2 radius -> 2 radius + length
