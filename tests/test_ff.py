"""The float-pair arithmetic and functions of the mixed kernels
(crystalscatter_gb300/csrc/cs_ff.cuh), built for the host with the same
source, against long double on random arguments: the relative errors of
exp, atan, division and square root, of log1p below 1/64 (its series), the
absolute errors of log and log1p elsewhere (they enter the closed forms only
through exp(-m/2 log(1 + 4a^2)), whose relative error is m/2 times that
absolute error) and the absolute errors of sin and cos (whose arguments reach ~2000 in the closed forms). Results below
~1e-29 lose precision (the low part becomes subnormal); the kernels use them
only as vanishing terms."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "crystalscatter_gb300", "csrc")

HARNESS = r"""
#include <cmath>
#include <cstdint>
#include "cs_ff.cuh"
using namespace csff;
typedef long double L;
static std::uint64_t st = 0x243F6A8885A308D3ull;
static std::uint64_t nx() { st ^= st << 13; st ^= st >> 7; st ^= st << 17; return st; }
static double unif() { return (double)(nx() >> 11) * 0x1p-53; }
static L val(ff a) { return (L)a.hi + (L)a.lo; }
static ff rnd_ff(double lo, double hi) { return from_double(lo + (hi - lo) * unif()); }
static ff logrnd(double e0, double e1) { return from_double(std::exp(e0 + (e1 - e0) * unif())); }
// worst errors: 0 exp, 1 log (absolute below 1), 2 log1p (same), 3 atan, 4 sin/cos (absolute), 5 div,
// 6 sqrt, 7 log within 1e-6 of 1 (relative)
extern "C" void run(long n, double *worst) {
    for (int k = 0; k < 8; k++) worst[k] = 0;
    auto upd = [&](int k, L err) { if (!(err <= worst[k])) worst[k] = (double)err; };
    for (long i = 0; i < n; i++) {
        ff x = rnd_ff(-65.0, 80.0);  // results above ~1e-29: both parts normal floats
        L r = std::exp(val(x));
        upd(0, std::fabs((val(exp_ff(x)) - r) / r));
        x = logrnd(-60.0, 60.0);
        r = std::log(val(x));
        upd(1, std::fabs(val(log_ff(x)) - r) / std::fmax(std::fabs(r), (L)1));
        x = logrnd(-30.0, 3.0);
        if (nx() & 1) x = neg(mul_f(x, 0.5f));
        r = std::log1p(val(x));
        upd(2, std::fabs(val(log1p_ff(x)) - r) / std::fmax(std::fabs(r), (L)(std::fabs(val(x)) < 1.0 / 64 ? 0 : 1)));
        x = (nx() & 1) ? logrnd(-20.0, 14.0) : rnd_ff(-4.0, 4.0);
        r = std::atan(val(x));
        upd(3, std::fabs((val(atan_ff(x)) - r) / r));
        x = rnd_ff(-2000.0, 2000.0);
        ff s, c;
        sincos_ff(x, s, c);
        upd(4, std::fmax(std::fabs(val(s) - std::sin(val(x))), std::fabs(val(c) - std::cos(val(x)))));
        ff a = rnd_ff(-10.0, 10.0), b = logrnd(-20.0, 20.0);
        r = val(a) / val(b);
        upd(5, std::fabs((val(div(a, b)) - r) / r));
        a = logrnd(-40.0, 40.0);
        r = std::sqrt(val(a));
        upd(6, std::fabs((val(sqrt_ff(a)) - r) / r));
        x = add_f(rnd_ff(-1e-6, 1e-6), 1.0f);
        r = std::log(val(x));
        upd(7, std::fabs(val(log_ff(x)) - r) / std::fmax(std::fabs(r), (L)1e-300));
    }
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("no host compiler")
    d = tmp_path_factory.mktemp("ff")
    src = d / "h.cpp"
    src.write_text(HARNESS)
    so = d / "h.so"
    # no contraction: the error-free transformations rely on separate roundings
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-I", CSRC, str(src), "-o",
                    str(so)], check=True)
    return ctypes.CDLL(str(so))


def test_float_pair_functions(lib):
    w = (ctypes.c_double * 8)()
    lib.run(200000, w)
    names = ["exp", "log", "log1p", "atan", "sincos_abs", "div", "sqrt", "log_near_1_rel"]
    got = dict(zip(names, list(w)))
    print(got)
    assert got["exp"] < 5e-14
    assert got["log"] < 5e-14
    assert got["log1p"] < 5e-14
    assert got["atan"] < 5e-14
    assert got["sincos_abs"] < 5e-14
    assert got["div"] < 5e-14
    assert got["sqrt"] < 5e-14
    assert got["log_near_1_rel"] < 2e-13


FORMS = r"""
#include <cmath>
#include <cstdint>
#include "cs_ff.cuh"
typedef long double L;
static std::uint64_t st = 0x13198A2E03707344ull;
static std::uint64_t nx() { st ^= st << 13; st ^= st >> 7; st ^= st << 17; return st; }
static double unif() { return (double)(nx() >> 11) * 0x1p-53; }
// the reference's closed forms, evaluated in long double
static L len_ref(L a, L z) {
    return (1 / (2.0L * z * (z - 1))) * (1 / (a * a)) * (1 - cosl((z - 1) * atanl(2.0L * a)) / powl(1.0L + 4 * a * a, (z - 1) / 2.0L));
}
static L cross_ref(L a, L z) {
    const L p1 = (1 / (z * (z - 1) * (z - 2))) * powl(a, -3);
    const L p2 = p1 * sinl((z - 2) * atanl(2.0L * a)) / powl(1.0L + 4 * a * a, (z - 2) / 2.0L);
    const L p3 = (1 / (z * (z - 1) * (z - 2) * (z - 3))) * powl(a, -4) * cosl((z - 3) * atanl(2.0L * a)) /
                 powl(1.0L + 4 * a * a, (z - 3) / 2.0L);
    return (4.0L / 3.14159265358979323846264338327950288L) * (p1 - p2 - (9.0L / 8.0L) * p3);
}
// worst error / own estimate, and worst error where the estimate is <= 1e-10
extern "C" void run(long n, double *out) {
    for (int k = 0; k < 4; k++) out[k] = 0;
    for (long i = 0; i < n; i++) {
        const double sig = 0.03 + 0.3 * unif();
        const double z = (1 - sig * sig) / (sig * sig);
        double a = std::exp(std::log(0.05 / (z - 1)) + (std::log(200.0) - std::log(0.05 / (z - 1))) * unif());
        if (nx() & 1) a = -a;
        float rel;
        double v = csff::cyl_len_closed(a, z, rel);
        L r = len_ref(a, z);
        double e = (double)fabsl((v - r) / r);
        if (e / rel > out[0]) out[0] = e / rel;
        if (rel <= 1e-10 && e > out[1]) out[1] = e;
        const double ap = std::fabs(a) + 0.2;
        v = csff::cyl_cross_asym(ap, z, rel);
        r = cross_ref(ap, z);
        e = (double)fabsl((v - r) / r);
        if (e / rel > out[2]) out[2] = e / rel;
        if (rel <= 1e-10 && e > out[3]) out[3] = e;
    }
}
"""


def test_float_pair_closed_forms(tmp_path):
    """The cylinder's length factor and cross-section asymptote in float pairs
    against the reference's expressions in long double, over Schulz widths
    0.03..0.33 and arguments from |m a| = 0.05 to 200: every error within the
    function's own estimate, and below 1e-10 wherever the estimate is."""
    if not shutil.which("g++"):
        pytest.skip("no host compiler")
    src = tmp_path / "f.cpp"
    src.write_text(FORMS)
    so = tmp_path / "f.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-I", CSRC, str(src), "-o",
                    str(so)], check=True)
    out = (ctypes.c_double * 4)()
    ctypes.CDLL(str(so)).run(100000, out)
    print(list(out))
    assert out[0] <= 1.0 and out[2] <= 1.0
    assert out[1] <= 1e-10 and out[3] <= 1e-10
