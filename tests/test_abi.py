"""The C-ABI library loads without a GPU and exports every function that
include/crystalscatter.h declares; its exported names carry no C++ types."""
import os
import re
import subprocess

import crystalscatter_gb300 as cs

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "crystalscatter.h")


def declared_functions():
    src = open(HDR).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(cs_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    lib = cs.load_library()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_exports_are_plain_c():
    out = subprocess.run(["nm", "-D", "--defined-only", cs.library_path()], stdout=subprocess.PIPE, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    for n in declared_functions():
        assert n in exported, n  # unmangled C symbol


def test_create_destroy_without_gpu_and_defaults():
    lib = cs.load_library()
    c = cs.SasCalc_GENERIC_calculation()
    p = c.params()
    # console defaults (sc_calcCons.cpp:24-100): the particle default text is
    # not in the combobox list, hence -1; ordis "isotropic" = 7; LType None = 12
    assert (p.particle, p.ordis, p.ltype, p.peak, p.hklmax, p.gridpoints) == (-1, 7, 12, 1, 5, 64)
    assert p.izero == 10000 and p.radius == 1.0 and p.sigma == 0.07 and p.radq4 == 1
    assert lib.cs_prepared_size() > 400000
    c.cleanup()


def test_cpu_thread_count_is_rejected():
    c = cs.SasCalc_GENERIC_calculation()
    c.setParam("ComboBoxParticle", 0)
    try:
        c.doCalculation(4)
        raised = False
    except cs.CrystalScatterError as e:
        raised = e.code == cs.CS_ERR_PARAM
    assert raised
    c.cleanup()


def test_batch_without_gpu_fails_loudly():
    # no CPU path: preparing a batch needs the device (pinned staging, device arena)
    import pytest
    if cs.SasCalc_GENERIC_calculation.gpuAvailable():
        pytest.skip("a GPU is present")
    b = cs.SasCalcBatch()
    with pytest.raises(cs.CrystalScatterError) as e:
        b.prepare([{"ComboBoxParticle": 0, "GridPoints": 8}])
    assert e.value.code == cs.CS_ERR_CUDA
    assert "no CUDA device" in str(e.value)
    b.cleanup()
