// count_ops.cpp — operation-counting build of the oracle (test and
// measurement infrastructure, not part of the product).
//
// The oracle source (cs_oracle.c) is compiled here as C++ with `double`
// replaced by OpDouble, a value type that behaves like double and tallies
// every floating-point add/subtract, multiply, divide and math-library call it
// takes part in. Comparisons, fabs and conversions are not counted. The one
// difference from the checker build: the orientation integral of an
// identically-zero integrand (orientation case outside 1..4) returns its exact
// +0 without the result-free Romberg work, and sin/cos/exp of quadrature node
// positions (pixel-independent) are evaluated without being counted; both GPU
// paths do the same (exact zero, node tables).
// oracle/count_ops.py calls ops_pixel() on sampled pixels of each workload and
// turns the tallies into algorithmic operations per pixel with a fixed cost
// table. Pixel results are the oracle's own (the arithmetic is unchanged).
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include <cmath>

struct OpTally {
    unsigned long long add, mul, div, sqrt_, exp_, log_, sin_, cos_, tan_, atan_, atan2_, pow_, acos_;
};
static OpTally g_t;

struct OpDouble {
    double v;
    OpDouble() = default;
    OpDouble(double x) : v(x) {}
    operator double() const { return v; }
    OpDouble operator-() const { return OpDouble(-v); }
    OpDouble &operator+=(OpDouble o) { g_t.add++; v += o.v; return *this; }
    OpDouble &operator-=(OpDouble o) { g_t.add++; v -= o.v; return *this; }
    OpDouble &operator*=(OpDouble o) { g_t.mul++; v *= o.v; return *this; }
    OpDouble &operator/=(OpDouble o) { g_t.div++; v /= o.v; return *this; }
};
static_assert(sizeof(OpDouble) == sizeof(double), "layout of the prepared block must not change");

#define OPD_BIN(OP, CNT)                                                                         \
    inline OpDouble operator OP(OpDouble a, OpDouble b) { g_t.CNT++; return OpDouble(a.v OP b.v); } \
    inline OpDouble operator OP(OpDouble a, double b) { g_t.CNT++; return OpDouble(a.v OP b); }     \
    inline OpDouble operator OP(double a, OpDouble b) { g_t.CNT++; return OpDouble(a OP b.v); }     \
    inline OpDouble operator OP(OpDouble a, float b) { g_t.CNT++; return OpDouble(a.v OP b); }      \
    inline OpDouble operator OP(float a, OpDouble b) { g_t.CNT++; return OpDouble(a OP b.v); }      \
    inline OpDouble operator OP(OpDouble a, int b) { g_t.CNT++; return OpDouble(a.v OP b); }        \
    inline OpDouble operator OP(int a, OpDouble b) { g_t.CNT++; return OpDouble(a OP b.v); }        \
    inline OpDouble operator OP(OpDouble a, long b) { g_t.CNT++; return OpDouble(a.v OP b); }       \
    inline OpDouble operator OP(long a, OpDouble b) { g_t.CNT++; return OpDouble(a OP b.v); }
OPD_BIN(+, add)
OPD_BIN(-, add)
OPD_BIN(*, mul)
OPD_BIN(/, div)
#undef OPD_BIN

#define OPD_FN1(F, CNT) \
    inline OpDouble F(OpDouble a) { g_t.CNT++; return OpDouble(std::F(a.v)); }
OPD_FN1(sqrt, sqrt_)
OPD_FN1(exp, exp_)
OPD_FN1(log, log_)
OPD_FN1(sin, sin_)
OPD_FN1(cos, cos_)
OPD_FN1(tan, tan_)
OPD_FN1(atan, atan_)
OPD_FN1(acos, acos_)
#undef OPD_FN1
inline OpDouble fabs(OpDouble a) { return OpDouble(std::fabs(a.v)); }
inline OpDouble atan2(OpDouble a, OpDouble b) { g_t.atan2_++; return OpDouble(std::atan2(a.v, b.v)); }
inline OpDouble pow(OpDouble a, OpDouble b) { g_t.pow_++; return OpDouble(std::pow(a.v, b.v)); }
inline OpDouble pow(OpDouble a, double b) { g_t.pow_++; return OpDouble(std::pow(a.v, b)); }
inline OpDouble pow(double a, OpDouble b) { g_t.pow_++; return OpDouble(std::pow(a, b.v)); }
inline OpDouble pow(OpDouble a, int b) { g_t.pow_++; return OpDouble(std::pow(a.v, b)); }
inline OpDouble modf(OpDouble a, OpDouble *ip) {
    double i;
    const double f = std::modf(a.v, &i);
    ip->v = i;
    return OpDouble(f);
}
inline bool isfinite(OpDouble a) { return std::isfinite(a.v); }
inline bool isnan(OpDouble a) { return std::isnan(a.v); }
inline bool isinf(OpDouble a) { return std::isinf(a.v); }

#define CS_ORACLE_SKIP_ZERO_INTEGRAL
// node positions' sin/cos/exp: evaluated, not counted (pixel-independent)
#define NODE_SIN(x) OpDouble(std::sin((x).v))
#define NODE_COS(x) OpDouble(std::cos((x).v))
#define NODE_EXP(x) OpDouble(std::exp((x).v))
#define double OpDouble
#include "cs_oracle.c"
#undef double

extern "C" {

// One pixel of the oracle with the tallies of that pixel added to *t (13
// counters in the order of OpTally); returns the pixel value.
double ops_pixel(const cs_prepared *P, int ihex, int i, unsigned long long *t) {
    g_t = OpTally{};
    const double v = (double)oracle_pixel(P, ihex, i);
    const unsigned long long *c = &g_t.add;
    for (int k = 0; k < 13; k++) t[k] += c[k];
    return v;
}

size_t ops_prepared_size(void) { return sizeof(cs_prepared); }

}  // extern "C"
