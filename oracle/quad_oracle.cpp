// quad_oracle.cpp — the CPU oracle evaluated in quadruple precision (test
// infrastructure, not part of the product).
//
// The oracle source (cs_oracle.c: the reference's per-pixel algorithm) is
// compiled here as C++ with its working type `double` replaced by __float128
// (113-bit significand) and its math-library calls by libquadmath's; it reads
// the same prepared block (real doubles, and float where the reference keeps
// float). Every operation, branch and stop rule is the reference's, so the
// result is the reference algorithm's value without its FP64 rounding: where
// the reference's FP64 result is ill-conditioned (it moves under one-ulp
// changes of the math library), this is the answer its arithmetic
// approximates. Constants stay the reference's double literals (M_PI
// included): they are part of the algorithm. Used by
// tests/golden/make_golden.py to store a high-precision image per golden case.
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include <cmath>

#include "../crystalscatter_gb300/csrc/cs_prepared.h"

typedef double pdouble_t;  // the prepared block's element type

#if defined(__aarch64__)
// long double is IEEE binary128 on AArch64 Linux: the standard library's
// long-double overloads of the math functions serve as they are
typedef long double Q;
#else
#include <quadmath.h>
typedef __float128 Q;

inline Q sin(Q x) { return sinq(x); }
inline Q cos(Q x) { return cosq(x); }
inline Q tan(Q x) { return tanq(x); }
inline Q atan(Q x) { return atanq(x); }
inline Q acos(Q x) { return acosq(x); }
inline Q atan2(Q y, Q x) { return atan2q(y, x); }
inline Q atan2(Q y, double x) { return atan2q(y, (Q)x); }
inline Q atan2(double y, Q x) { return atan2q((Q)y, x); }
inline Q exp(Q x) { return expq(x); }
inline Q log(Q x) { return logq(x); }
inline Q sqrt(Q x) { return sqrtq(x); }
inline Q fabs(Q x) { return fabsq(x); }
inline Q trunc(Q x) { return truncq(x); }
inline Q pow(Q x, Q y) { return powq(x, y); }
inline Q pow(Q x, double y) { return powq(x, (Q)y); }
inline Q pow(double x, Q y) { return powq((Q)x, y); }
inline Q pow(Q x, int y) { return powq(x, (Q)y); }
inline Q pow(Q x, float y) { return powq(x, (Q)y); }
inline Q pow(int x, Q y) { return powq((Q)x, y); }
inline Q modf(Q x, Q *ip) { return modfq(x, ip); }
inline bool isfinite(Q x) { return finiteq(x); }
inline bool isnan(Q x) { return isnanq(x); }
inline bool isinf(Q x) { return isinfq(x); }
#endif

// q perturbation (quad_set_qmode): each component of q, as the reference
// forms it in double, is moved by `steps` double ulps (up or down per
// component as the mode's bits select) before the exact evaluation. A GPU
// path whose detector geometry differs from the reference's by a few ulps can
// at best reach the value's spread under such moves.
static int g_qmode = 0, g_qsteps = 4;
static double qmove(double v, int up, int steps) {
    for (int k = 0; k < steps; k++) v = nextafter(v, up ? INFINITY : -INFINITY);
    return v;
}
#define CS_ORACLE_Q_HOOK(qx, qy, qz)                                          \
    if (g_qmode) {                                                           \
        qx = qmove((double)qx, (g_qmode >> 0) & 1, g_qsteps);               \
        qy = qmove((double)qy, (g_qmode >> 1) & 1, g_qsteps);               \
        qz = qmove((double)qz, (g_qmode >> 2) & 1, g_qsteps);               \
    }

#define CS_PDOUBLE_T pdouble_t
#define double Q
#include "cs_oracle.c"
#undef double

extern "C" {

// The calculated region of P (all rows, quadrants mirrored as the reference
// does) in quadruple precision with nthreads threads, rounded to double into
// out (the image layout of oracle_image_rows). Returns the pixel count.
long quad_image(const cs_prepared *P, double *out, int nthreads) {
    const long n = (long)(P->xmax - P->xmin) * (long)(P->ymax - P->ymin);
    Q *q = (Q *)calloc((size_t)n, sizeof(Q));
    if (!q) return -1;
    const long r = oracle_image_rows(P, q, 0, 0, nthreads);
    for (long k = 0; k < n; k++) out[k] = (double)q[k];
    free(q);
    return r;
}

// One pixel in quadruple precision, rounded to double.
double quad_pixel(const cs_prepared *P, int ihex, int i) { return (double)oracle_pixel(P, ihex, i); }

size_t quad_prepared_size(void) { return sizeof(cs_prepared); }

// q perturbation mode (0: off; bits 0..2 move qx, qy, qz up when set, down
// when clear) and its size in double ulps.
void quad_set_qmode(int mode, int steps) {
    g_qmode = mode;
    g_qsteps = steps;
}

}  // extern "C"
