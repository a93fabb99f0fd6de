"""The generic FP64 pixel function of the device code, compiled for the host
(tests/host_emu/emu_generic.cpp), against the reference's golden images.

The GPU tests pin the same cases on the device; this one runs the device
code's logic on the CPU, with the host math library (the reference's own), so
that every generic case is checked here too: relative error <= 1e-10 wherever
the reference is stable, within its one-ulp envelope elsewhere, the same
non-finite pixels. Only cases of the generic pixel function (dispatch key
CS_KEY_GENERIC) without the quadrant expansion are run: the specialised
pixel functions and the image mirroring live in other kernels."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import crystalscatter_gb300 as cs
from helpers import compare_with_exact, golden, golden_cases, written_mask
from oracle import cpu_oracle

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CASES = golden_cases()["images"]
KEY_GENERIC = 0x7F000000  # CS_KEY_GENERIC, cs_prepared.h


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    lib = cs.load_library()
    libdir = os.path.dirname(lib._name)
    out = str(tmp_path_factory.mktemp("emu") / "emu_generic.so")
    src = os.path.join(HERE, "host_emu", "emu_generic.cpp")
    inc = os.path.join(ROOT, "crystalscatter_gb300", "csrc")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w", "-I" + inc,
                    "-I" + cuda_inc, src, "-o", out, "-L" + libdir, "-lcrystalscatter", "-Wl,-rpath," + libdir],
                   check=True)
    e = ctypes.CDLL(out)
    e.emu_generic_region.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    return e


def _generic(name):
    case = CASES[name]
    p = case["params"]
    if case.get("ign_new_switch") or p.get("ExpandImage", 0):
        return None
    P = cpu_oracle.prepare(p, case["ign_cbs"])
    return P if P.key == KEY_GENERIC else None


@pytest.mark.parametrize("name", sorted(CASES))
def test_generic_device_code_on_host_matches_reference(emu, name):
    P = _generic(name)
    if P is None:
        pytest.skip("not the generic pixel function")
    g = golden(name)
    nx, ny = P.zzmax - P.zzmin, P.iimax - P.iimin
    region = np.zeros(nx * ny)
    emu.emu_generic_region(ctypes.byref(P), region.ctypes.data)
    img = np.zeros(g["image"].shape)
    img[P.iimin - P.ymin:P.iimax - P.ymin, P.zzmin - P.xmin:P.zzmax - P.xmin] = region.reshape(ny, nx)
    m = written_mask(CASES[name]["params"], img.shape)
    r = compare_with_exact(img, g, mask=m, tol=1e-10)
    assert r["n_bad"] == 0, r
