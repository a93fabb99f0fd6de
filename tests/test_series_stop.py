"""The power series' stop test (cs_series_stop.h) against the reference's own
test fabs((s - old) / s) < 0.0001 (e.g. Source/sc_lib_formpq_partCylinder.h:109-110):
the host build of the same function decides every case as the plain quotient
does, on 20 million pairs concentrated at the threshold and on the special
values (zero, subnormal, infinite, NaN, the ends of the exponent screen)."""
import ctypes
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "crystalscatter_gb300", "csrc")

HARNESS = r"""
#include <cmath>
#include <cstdint>
#include <cstring>
#include "cs_series_stop.h"

static std::uint64_t st = 0x9E3779B97F4A7C15ull;
static std::uint64_t next() { st ^= st << 13; st ^= st >> 7; st ^= st << 17; return st; }
static double unif() { return (double)(next() >> 11) * 0x1p-53; }
static double bits(std::uint64_t u) { double x; std::memcpy(&x, &u, sizeof x); return x; }

static long check(double s, double old) {
    const bool ref = std::fabs((s - old) / s) < 0.0001;
    return cs_series::series_converged(s, old) != ref;
}

extern "C" long run(long n, long *n_close) {
    long bad = 0, close = 0;
    const double specials[] = {0.0, -0.0, 1.0, -1.0, 0x1p-962, -0x1p-962, 0x1.fffffffffffffp-963, 0x1p963,
                               0x1.fffffffffffffp962, 0x1p-1074, 0x1p-1022, 1e-300, 1e300, 1.7e308,
                               INFINITY, -INFINITY, NAN};
    for (double a : specials)
        for (double b : specials) {
            bad += check(a, b);
            bad += check(a, a - b * 1e-4);
            bad += check(a, a * (1 - 1e-4));
        }
    for (long i = 0; i < n; i++) {
        const int e = (int)(next() % 2100) - 1050;
        double s = std::ldexp(1.0 + unif(), e);
        if (next() & 1) s = -s;
        double r;
        const unsigned kind = next() % 4;
        if (kind == 0) r = std::ldexp(1.0 + unif(), -(int)(next() % 40));               /* wide */
        else if (kind == 1) r = 1e-4 * (1.0 + (unif() - 0.5) * 0x1p-40);                 /* at the band */
        else if (kind == 2) r = 1e-4 * (1.0 + (unif() - 0.5) * std::ldexp(1.0, -(int)(next() % 52)));
        else r = std::ldexp(1.0, -13) * (1.0 + (unif() - 0.5) * 1e-6);                   /* at the screen */
        if (next() & 1) r = -r;
        const double old = s - s * r;
        const double q = std::fabs((s - old) / s);
        if (std::isfinite(q) && std::fabs(q - 1e-4) < 1e-4 * 0x1p-48) close++;
        bad += check(s, old);
        /* the same pair with old built from the increment's exponent only */
        bad += check(s, s - std::ldexp(s, -13 + (int)(next() % 3) - 1));
    }
    *n_close = close;
    return bad;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("series_stop")
    src = d / "h.cpp"
    src.write_text(HARNESS)
    so = d / "libh.so"
    subprocess.check_call([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", CSRC,
                           str(src), "-o", str(so)])
    lib = ctypes.CDLL(str(so))
    lib.run.argtypes = [ctypes.c_long, ctypes.POINTER(ctypes.c_long)]
    lib.run.restype = ctypes.c_long
    return lib


def test_stop_test_matches_the_quotient(harness):
    close = ctypes.c_long()
    bad = harness.run(20_000_000, ctypes.byref(close))
    assert bad == 0
    assert close.value > 1000  # the sample does reach the rounding band of the threshold
