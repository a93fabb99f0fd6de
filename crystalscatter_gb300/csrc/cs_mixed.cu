// cs_mixed.cu — mixed-precision pixel kernels (CS_MODE_MIXED).
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so the bulk of the
// per-pixel work runs in FP32 here, with FP64 kept where the reference's
// numerics need it:
//   * FP64: detector geometry q, the small-qR Schulz-Zimm power series of
//     P(q)/F(q) (alternating series with cancellation up to 1e9 near their
//     switch points), the Romberg extrapolation (polint) and every stop/branch
//     decision, the final combination of the structure factor.
//   * FP32: the large-qR asymptotes, the lattice peak sums (compensated
//     accumulation, radial distance from a float-float q), the orientation
//     quadrature integrand (with a Taylor form where its closed form cancels)
//     and the trapezoid sums (compensated).
// A pixel whose FP64 decision lies within a guard band of its threshold (where
// FP32 rounding could flip the reference's discrete choice: series vs.
// asymptote, Romberg convergence) is flagged; a second kernel recomputes the
// flagged pixels with the FP64 drop-in functions. The image written is then
// within ~1e-6 of the FP64 path everywhere (bar <= 1e-5).
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "cs_ff.cuh"
#include "cs_fp64.cuh"
#include "cs_launch.h"
#include "cs_batch.cuh"
#include "cs_mixed.h"

namespace csm {

using cs64::Ctx;

#define LOG2E_F 1.4426950408889634f


// Relative error estimates of the form-factor parts: FP64 power series (a few
// roundings; their own cancellation is that of the reference) and FP32
// closed forms / quadratures (a few FP32 roundings).
#define EPS_SERIES 1.0e-14
#define EPS_PQ 3.0e-7
#define EPS_PEAK 1.0e-12  // peak sums beyond their own estimate (pair sums, table rounding)

// decision guard: true when v is within `band` relative of threshold t
__device__ __forceinline__ bool near(double v, double t, double band) { return fabs(v - t) <= band * fabs(t); }

// Detector geometry. In beam geometry it is taken in FP64 without
// transcendentals: cos(phi)sin(theta) = xdet/L, sin(phi)sin(theta) = ydet/L,
// cos(theta) = det/L, L = |(xdet,ydet,det)|, which agrees with the reference's
// atan2/sin/cos form to a few ulp; the pixel-independent factors (QGeom) are
// formed once per thread, which leaves two FP64 divisions per pixel. The
// z-direction cylinder keys take the drop-in's own convert_idx2q instead (same
// rounding: this unit is compiled without contraction, as the drop-in is):
// their power series in (qx+qy)^2 can cancel by up to 1e15, where a few-ulp
// change of q moves the reference's own value by O(1), and the mixed path then
// reproduces the FP64 value exactly instead of a different rounding of it.
struct QGeom {
    double sy, sx, k;  // pixnoy/(2 zmax), pixnox/(2 zmax), 2 pi/lambda
};

__device__ __forceinline__ QGeom q_geom(const cs_prepared &P) {
    QGeom g;
    g.sy = P.pixnoy / (2.0 * P.zmax);
    g.sx = P.pixnox / (2.0 * P.zmax);
    g.k = 2 * M_PI / P.wave;
    return g;
}

template <int KEY>
__device__ __forceinline__ void q_of_pixel(const cs_prepared &P, const QGeom &g, int ihex, int i, double &qx,
                                           double &qy, double &qz) {
    if (KEY == CS_KEY_CYL_NONE_ZDIR || KEY == CS_KEY_CYL_GAUSS_BCT_ZDIR || P.use1d || !P.usebeamstop) {
        cs64::convert_idx2q(P, ihex, i, qx, qy, qz);
        return;
    }
    const double mdet = (ihex)*g.sy;
    const double ndet = (i)*g.sx;
    const double xdet = P.pixx_m * (ndet - P.beamx0);
    const double ydet = P.pixy_m * (mdet - P.beamy0);
    const double r2 = xdet * xdet + ydet * ydet;
    const double L = sqrt(r2 + P.det * P.det);
    const double kl = g.k / L;
    qx = kl * xdet;
    qy = kl * ydet;
    // 1 - cos(theta) = r^2 / (L (L + det)), free of cancellation
    qz = kl * r2 / (L + P.det);
}

// ---------------------------------------------------------------- asymptotes
// Every closed form below also returns `rel`, a first-order estimate of its
// relative error; the sum of the terms' absolute errors over the magnitude of
// the result accounts for cancellation between the terms (near zeros of the
// form factors). Its sines and cosines take arguments theta = c atan(x) with
// c up to ~400, and its powers (1+x^2)^e = exp2(e log2(1+x^2)) exponents of up
// to a few hundred. Two forms of those arguments (ClosedArgs):
//  * FP32: theta = c atanf(x) is off by ~|theta| 1.2e-7 (absolute: 1.8e-5 at
//    theta = 150), the power by ~|e log2(1+x^2)| 8e-8 + 1.2e-7 (relative);
//  * FP64: atan and log1p in FP64, theta reduced to [-pi, pi] before its FP32
//    rounding (error |r| 6e-8 + the FP32 sine's 1.2e-7), the exponent split
//    into an integer and a fraction in [-1/2, 1/2] (error 1.8e-7).
// A closed form is evaluated in FP32 first and again with the FP64 arguments
// when its estimate exceeds acc_switch<LAT>(); that costs one FP64 atan and
// log1p. Lattice pixels amplify the form factors' errors where the structure
// factor cancels (see lattice_combine) and switch early; the others only
// need the estimate below the 5e-6 guard.
#define TRIG_ERR(theta) (fabsf(theta) * 1.2e-7f + 6e-8f)
template <bool LAT> __device__ __forceinline__ float acc_switch() { return LAT ? 4e-7f : 2e-6f; }

template <bool ACC> struct ClosedArgs;

template <> struct ClosedArgs<false> {
    float t, l2;  // atan(x), log2(1 + x2)
    __device__ __forceinline__ ClosedArgs(double x, double x2)
        : t(atanf((float)x)), l2(log1pf((float)x2) * LOG2E_F) {}
    __device__ __forceinline__ float angle(double c, float &err) const {
        const float th = (float)c * t;
        err = TRIG_ERR(th);
        return th;
    }
    __device__ __forceinline__ float power(double e, float &err) const {
        const float y = (float)e * l2;
        err = fabsf(y) * 8e-8f + 1.2e-7f;
        return exp2f(y);
    }
};

template <> struct ClosedArgs<true> {
    double t, l2;
    __device__ __forceinline__ ClosedArgs(double x, double x2) : t(atan(x)), l2(log1p(x2) * 1.4426950408889634) {}
    __device__ __forceinline__ float angle(double c, float &err) const {
        const double th = c * t;
        const double k = rint(th * (0.5 / M_PI));
        const float r = (float)(th - k * (2.0 * M_PI));
        err = fabsf(r) * 6e-8f + 1.2e-7f;
        return r;
    }
    __device__ __forceinline__ float power(double e, float &err) const {
        const double y = e * l2;
        const double n = fmin(fmax(rint(y), -300.0), 300.0);
        err = 1.8e-7f;
        return ldexpf(exp2f((float)(y - n)), (int)n);
    }
};

// sphere P(q), q >= 0.4 limq4 (Source/sc_lib_formpq_partSphere.h:263-269)
template <bool ACC>
__device__ float sphere_pq_asym(double argq_d, double zr_d, float &rel) {
    const ClosedArgs<ACC> A(2.0 * argq_d, 4.0 * argq_d * argq_d);
    const float argq = (float)argq_d, zr = (float)zr_d;
    const float pqr = (1.0f / (2.0f * zr * (zr - 1) * (zr - 2) * (zr - 3))) / (argq * argq * argq * argq);
    float e1, e2, e3, g1, g2, g3;
    const float th1 = A.angle(zr_d - 3, g1), th2 = A.angle(zr_d - 4, g2), th3 = A.angle(zr_d - 5, g3);
    const float P1 = A.power((zr_d - 3) / 2.0, e1), P2 = A.power((zr_d - 4) / 2.0, e2), P3 = A.power(zr_d - 5, e3);
    const float C1 = cosf(th1), S2 = sinf(th2), C3 = cosf(th3);
    const float pq1 = pqr * (1 + C1 / P1);
    const float b2 = pqr / ((zr - 4) * argq);
    const float pq2 = b2 * S2 / P2;
    const float b3 = pqr / ((zr - 4) * (zr - 5) * argq * argq);
    // the reference divides by 2 outside the pow (reproduced)
    const float pq3 = b3 * (1 - C3 / P3 / 2.0f);
    const float v = 9.0f * (pq1 - 2.0f * pq2 + pq3);
    const float E = fabsf(pqr) * ((g1 + fabsf(C1) * e1) / P1 + 3e-7f * fabsf(1 + C1 / P1)) +
                    2.0f * fabsf(b2) * ((g2 + fabsf(S2) * e2) / P2 + 3e-7f * fabsf(S2 / P2)) +
                    fabsf(b3) * ((g3 + fabsf(C3) * e3) / (2.0f * P3) + 3e-7f * fabsf(1 - C3 / P3 / 2.0f));
    rel = 9.0f * E / fabsf(v) + 3e-7f;
    return v;
}

// sphere F(q), q >= 0.4 limq4f (Source/sc_lib_formfq_partSphere.h:443-448)
template <bool ACC>
__device__ float sphere_fq_asym(double argq_d, double zr_d, float &rel) {
    const ClosedArgs<ACC> A(argq_d, argq_d * argq_d);
    const float argq = (float)argq_d, zr = (float)zr_d;
    const float pqr = 1.0f / (zr * (zr - 1)) / (argq * argq);
    float e1, e2, g1, g2;
    const float th1 = A.angle(zr_d - 1, g1), th2 = A.angle(zr_d - 2, g2);
    const float P1 = A.power((zr_d - 1) / 2.0, e1), P2 = A.power((zr_d - 2) / 2.0, e2);
    const float C1 = cosf(th1), S2 = sinf(th2);
    const float pq1 = pqr * C1 / P1;
    const float b2 = pqr / ((zr - 2) * argq);
    const float pq2 = b2 * S2 / P2;
    const float pq3 = 3 * (pq2 - pq1);
    const float E = 3.0f * (fabsf(pqr) * (g1 + fabsf(C1) * e1) / P1 + 3e-7f * fabsf(pq1) +
                            fabsf(b2) * (g2 + fabsf(S2) * e2) / P2 + 3e-7f * fabsf(pq2));
    rel = 2.0f * E / fabsf(pq3) + 3e-7f;
    return pq3 * pq3;
}

// cylinder cross-section P(q), q >= 0.65 limq4 (Source/sc_lib_formpq_partCylinder.h:271-275)
template <bool ACC>
__device__ float cyl_pqr_asym(double argpq_d, double zr_d, float &rel) {
    const ClosedArgs<ACC> A(2.0 * argpq_d, 4.0 * argpq_d * argpq_d);
    const float argpq = (float)argpq_d, zr = (float)zr_d;
    const float a3 = argpq * argpq * argpq;
    const float pqr1 = (1.0f / (zr * (zr - 1) * (zr - 2))) / a3;
    float e2, e3, g2, g3;
    const float th2 = A.angle(zr_d - 2, g2), th3 = A.angle(zr_d - 3, g3);
    const float P2 = A.power((zr_d - 2) / 2.0, e2), P3 = A.power((zr_d - 3) / 2.0, e3);
    const float S2 = sinf(th2), C3 = cosf(th3);
    const float pqr2 = pqr1 * S2 / P2;
    const float b3 = (1.0f / (zr * (zr - 1) * (zr - 2) * (zr - 3))) / (a3 * argpq);
    const float pqr3 = b3 * C3 / P3;
    const float v = (4.0f / (float)M_PI) * (pqr1 - pqr2 - (9.0f / 8.0f) * pqr3);
    const float E = 3e-7f * fabsf(pqr1) + fabsf(pqr1) * (g2 + fabsf(S2) * e2) / P2 + 3e-7f * fabsf(pqr2) +
                    1.125f * (fabsf(b3) * (g3 + fabsf(C3) * e3) / P3 + 3e-7f * fabsf(pqr3));
    rel = (4.0f / (float)M_PI) * E / fabsf(v) + 3e-7f;
    return v;
}

// FP64 amplitude of the cylinder cross-section F(q) asymptote (the drop-in's
// expression with the prepared Gamma ratios), for lattice pixels (whose F(q)
// radial factor is almost always its FP64 series: q below limqf4)
__device__ double cyl_fqr_asym_d(double a, double zr, double g0, double g1, float &rel) {
    const double t = atan(a);
    const double p1 = g0 * pow(a, -3 / 2.0) * (sin((zr - 1 / 2.0) * t) - cos((zr - 1 / 2.0) * t)) /
                      pow(1.0 + a * a, (zr - 1 / 2.0) / 2.0);
    const double p2 = g1 * pow(a, -5 / 2.0) * (sin((zr - 3 / 2.0) * t) + cos((zr - 3 / 2.0) * t)) /
                      pow(1.0 + a * a, (zr - 3 / 2.0) / 2.0);
    const double v = (2 / sqrt(M_PI)) * (p1 + (9 / 16.0) * p2);
    rel = (float)(2.0 * (fabs(p1) + fabs(p2)) * 1e-13 / fabs(v) + 1e-15);
    return v;
}

// cylinder cross-section F(q), q >= limq4f (Source/sc_lib_formfq_partCylinder.h)
// amplitude squared; gamma ratios from the preparation
template <bool ACC>
__device__ float cyl_fqr_asym(double a_d, double z_d, double g0, double g1, float &rel) {
    const ClosedArgs<ACC> A(a_d, a_d * a_d);
    const float a = (float)a_d;
    const float a2 = a * a;
    float e1, e2, h1, h2;
    const float s1 = A.angle(z_d - 0.5, h1), s2 = A.angle(z_d - 1.5, h2);
    const float P1 = A.power((z_d - 0.5) / 2.0, e1), P2 = A.power((z_d - 1.5) / 2.0, e2);
    const float b1 = (float)g0 * rsqrtf(a2 * a), b2 = (float)g1 * rsqrtf(a2 * a2 * a);
    const float T1 = sinf(s1) - cosf(s1), T2 = sinf(s2) + cosf(s2);
    const float pqr1 = b1 * T1 / P1;
    const float pqr2 = b2 * T2 / P2;
    const float pqr3 = (2.0f / sqrtf((float)M_PI)) * (pqr1 + (9.0f / 16.0f) * pqr2);
    // amplitude error (two trig terms each), doubled for the square
    const float E = fabsf(b1) * (2.0f * h1 + fabsf(T1) * e1) / P1 + 3e-7f * fabsf(pqr1) +
                    0.5625f * (fabsf(b2) * (2.0f * h2 + fabsf(T2) * e2) / P2 + 3e-7f * fabsf(pqr2));
    rel = 2.0f * (2.0f / sqrtf((float)M_PI)) * E / fabsf(pqr3) + 3e-7f;
    return pqr3;
}

// Length factor of the Schulz cylinder P(q) along its axis,
//   (1/(2z(z-1) a^2)) (1 - cos((z-1) atan 2a) / (1+4a^2)^((z-1)/2)),
// which tends to 1 for a -> 0 with cancellation in the bracket. With m = z-1
// the bracket is 1 - Re (1+2ia)^(-m) = -sum_{j>=1} C(m+2j-1, 2j) (-4a^2)^j, so
// the function is the series 1 + sum_{j>=1} T_j with
//   T_j / T_(j-1) = -4a^2 (m+2j)(m+2j+1)/((2j+1)(2j+2)),
// whose ratios lie between the first one, 4a^2 (m+2)(m+3)/12, and their limit
// 4a^2. Where both are below 0.12, ten terms leave a remainder below 1e-9 and
// S = sum T_j (|S| < 0.14, largest terms first) then 1 + S round to < 1.2e-7;
// elsewhere the closed form is used.
__device__ __forceinline__ bool len_series_ok(float a, float m) {
    const float x = 4.0f * a * a;
    return x < 0.12f && x * (m + 2.0f) * (m + 3.0f) < 1.44f;
}

__device__ __forceinline__ float len_series(float a, float m) {
    const float x = -4.0f * a * a;
    float term = 1.0f, sum = 0.0f;
#pragma unroll
    for (int j = 1; j <= 10; j++) {
        term *= x * (m + 2 * j) * (m + 2 * j + 1) * (1.0f / ((2 * j + 1) * (2 * j + 2)));
        sum += term;
    }
    return 1.0f + sum;
}

// The orientation integrand's form (per quadrature node): 4 a1 = 2/(z(z-1)) is
// a per-pixel constant, and the power enters as (1+4a^2)^(-m/2), so one
// division remains.
__device__ __forceinline__ float cyl_len_factor(float a, float z, float a4) {
    const float m = z - 1.0f;
    if (len_series_ok(a, m)) return len_series(a, m);
    const float x = 4.0f * a * a;
    const float c = cosf(m * atanf(2.0f * a));
    const float ipw = exp2f((-0.5f * m) * (log1pf(x) * LOG2E_F));
    return a4 * fmaf(-c, ipw, 1.0f) / x;
}

// the same with a relative error estimate (see the asymptotes above)
template <bool ACC>
__device__ float cyl_len_factor_e(double a_d, double z_d, float &rel) {
    const float a = (float)a_d, z = (float)z_d;
    const float m = z - 1.0f;
    if (len_series_ok(a, m)) {
        rel = 1.5e-7f;
        return len_series(a, m);
    }
    const ClosedArgs<ACC> A(2.0 * a_d, 4.0 * a_d * a_d);
    const float a1 = 1.0f / (2.0f * z * m);
    float ep, g;
    const float th = A.angle(z_d - 1.0, g);
    const float P = A.power((z_d - 1.0) / 2.0, ep);
    const float C = cosf(th);
    const float br = 1.0f - C / P;
    rel = ((g + fabsf(C) * ep) / P) / fabsf(br) + 3e-7f;
    return (a1 / (a * a)) * br;
}

// ------------------------------------------------------- FP32 Romberg (chi)
struct ChiArgsF {
    float qx, qy, lz;  // lz = l/(z+1)
    float z;
    float b;           // upper chi limit
    float a4;          // 2/(z(z-1)) of the length factor
    double qxs, qys;   // the FP64 arguments, for the FP64 fallback of one integral
    float p11, p12, p13, p21, p22, p23;
    int i1;
};

// Where m*a is small (m = z-1) the closed form of the length factor cancels;
// both paths take its power series there (cs64::len_factor_small and
// len_series_ok above), so the FP32 node value agrees with the FP64 one to
// FP32 accuracy everywhere.
__device__ __forceinline__ float chi_integrand_f(const ChiArgsF &A, float cx, float sx, float cd, float sd,
                                                 bool &guard) {
    const float eps = 1e-10f;
    float s;
    switch (A.i1) {
    case 1: {
        const float mlx1 = fmaf(fmaf(A.p11, cx, A.p12 * sx), sd, A.p13 * cd);
        const float mlx2 = fmaf(fmaf(A.p21, sx, A.p22 * cx), sd, A.p23 * cd);
        s = fmaf(A.qx, mlx1, fmaf(A.qy, mlx2, eps));
        break;
    }
    case 2: s = fmaf(A.qx, cd, fmaf(-A.qy * sx, sd, eps)); break;
    case 3: s = fmaf(A.qx * sx, sd, fmaf(A.qy, cd, eps)); break;
    case 4: s = fmaf(fmaf(A.qx, sx, -A.qy * cx), sd, eps); break;
    default: return 0.0f;
    }
    const float a = s * A.lz;
    return cyl_len_factor(a, A.z, A.a4);
}

// Neville extrapolation to 0 of the last five trapezoid estimates, whose
// abscissae are always 1, 1/4, 1/16, 1/64, 1/256 (times a common power of 2):
// its value is the Lagrange combination sum_i W_i y_i and its error estimate
// (the last correction, Neville's d column) is the 5-point value minus the
// 4-point value through the last four estimates, sum_i U_i y_i with
// sum_i U_i = 0. Written on the differences y_i - y_4 (no cancellation of the
// common part) it agrees with the reference's Neville tableau to ~1e-15 in the
// value and ~1e-11 in the error estimate, far inside the decision guard band,
// with 12 FP64 operations instead of ~60 and 10 divisions.
__device__ __forceinline__ void richardson5(const double y[5], double &pq, double &dss) {
    const double W0 = 1.0 / 722925.0, W1 = -4.0 / 8505.0, W2 = 64.0 / 2025.0, W3 = -4096.0 / 8505.0;
    const double U0 = 1.0 / 722925.0, U1 = -1.0 / 8505.0, U2 = 4.0 / 2025.0, U3 = -64.0 / 8505.0;
    const double d0 = y[0] - y[4], d1 = y[1] - y[4], d2 = y[2] - y[4], d3 = y[3] - y[4];
    pq = y[4] + (W0 * d0 + W1 * d1 + W2 * d2 + W3 * d3);
    dss = U0 * d0 + U1 * d1 + U2 * d2 + U3 * d3;
}

// Romberg convergence test of the reference in FP64 on the FP32-accurate
// estimates; `guard` flags a decision inside the band where FP32 rounding of
// the estimates could change it.
__device__ __forceinline__ bool romb_stop(const double win[5], double &pq, double tiny, bool &guard) {
    double dss;
    richardson5(win, pq, dss);
    const double lhs = fabs(dss), rhs = 1.0e-4 * fabs(pq);
    if (fabs(lhs - rhs) <= 3e-3 * rhs + 1e-300) guard = true;
    if (lhs < rhs) return true;
    if (fabs(pq) < tiny) return true;
    return false;
}

// The same extrapolation and test in FP32 for the inner (chi) integrals, whose
// estimates are FP32-accurate in any case. The differences y_i - y_4 carry the
// estimates' rounding (~6e-8 |y|), which moves dss by ~1e-9 |y|: about 1e-5 of
// the threshold 1e-4 |pq|, far inside the decision band. A result below
// 1e-30 (the reference stops below 1e-300, which FP32 cannot hold) is decided
// in FP64 by the redo, and so is a non-finite one.
__device__ __forceinline__ bool romb_stop_f(const float y[5], float &pq, bool &guard) {
    const float W0 = 1.0f / 722925.0f, W1 = -4.0f / 8505.0f, W2 = 64.0f / 2025.0f, W3 = -4096.0f / 8505.0f;
    const float U0 = 1.0f / 722925.0f, U1 = -1.0f / 8505.0f, U2 = 4.0f / 2025.0f, U3 = -64.0f / 8505.0f;
    const float d0 = y[0] - y[4], d1 = y[1] - y[4], d2 = y[2] - y[4], d3 = y[3] - y[4];
    pq = y[4] + fmaf(W0, d0, fmaf(W1, d1, fmaf(W2, d2, W3 * d3)));
    const float dss = fmaf(U0, d0, fmaf(U1, d1, fmaf(U2, d2, U3 * d3)));
    const float lhs = fabsf(dss), rhs = 1.0e-4f * fabsf(pq);
    if (!(fabsf(pq) >= 1e-30f) || !(fabsf(pq) < INFINITY)) {
        guard = true;
        return true;
    }
    if (fabsf(lhs - rhs) <= 3e-3f * rhs) guard = true;
    return lhs < rhs;
}

struct KahanF {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float v) {
        const float y = v - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ float value() const { return s - c; }
};

// qrombchid over chi in [0, b] in FP32: nodes from the FP32 copy of the node
// table, compensated trapezoid sums, extrapolation and stop test in FP32.
__device__ float qromb_chi_f(const Ctx &C, const ChiArgsF &A, float cd, float sd, bool &guard) {
    const float b = A.b;
    const cs_chi_node_f *__restrict__ nf = reinterpret_cast<const cs_chi_node_f *>(C.chi + CS_NODE_COUNT);
    float win[5];
    float cur;
    int cnt;
    float pq = 0.0f;
    {
        const cs_chi_node_f n0 = nf[0], n1 = nf[1];
        const float pa = chi_integrand_f(A, n0.c, n0.s, cd, sd, guard);
        const float pb = chi_integrand_f(A, n1.c, n1.s, cd, sd, guard);
        cur = 0.5f * b * (pa + pb);
        cnt = 1;
    }
    float rcnt = 1.0f;
    win[4] = cur;
    for (int j = 2; j <= 20; j++) {
        KahanF sum;
        if (j <= CS_NODE_LEVELS) {
            const cs_chi_node_f *nd = nf + CS_NODE_OFFSET(j);
            if ((A.i1 == 2 || A.i1 == 3) && cnt >= 4) {
                // the axis-along-x/y integrands depend on sin(chi) alone, and
                // the nodes of a level come in pairs chi, pi - chi (3 pi - chi
                // in the upper half) up to the rounding of the limit 2 pi to
                // FP32 (their sines differ by < 1e-7): one evaluation at the
                // pair's mean sine stands for both (second-order error ~1e-14)
                const int qn = cnt >> 2;
                for (int h = 0; h < 2; h++) {
                    const cs_chi_node_f *hn = nd + h * 2 * qn;
                    for (int k = 0; k < qn; k++) {
                        const float sm = 0.5f * (hn[k].s + hn[2 * qn - 1 - k].s);
                        sum.add(2.0f * chi_integrand_f(A, 0.0f, sm, cd, sd, guard));
                    }
                }
            } else if (A.i1 == 4 && cnt >= 2) {
                // axis along z: the integrand is even in its argument, which
                // changes sign from chi to chi + pi (node k to k + cnt/2)
                const int hn = cnt >> 1;
                for (int k = 0; k < hn; k++) {
                    const cs_chi_node_f u = nd[k], v = nd[k + hn];
                    sum.add(2.0f * chi_integrand_f(A, 0.5f * (u.c - v.c), 0.5f * (u.s - v.s), cd, sd, guard));
                }
            } else {
                for (int k = 0; k < cnt; k++) {
                    const cs_chi_node_f n = nd[k];
                    sum.add(chi_integrand_f(A, n.c, n.s, cd, sd, guard));
                }
            }
        } else {
            const double del = (double)b / cnt;
            double x = 0.5 * del;
            for (int k = 0; k < cnt; k++) {
                float s, c;
                sincosf((float)x, &s, &c);
                sum.add(chi_integrand_f(A, c, s, cd, sd, guard));
                x += del;
            }
        }
        cur = 0.5f * (cur + b * sum.value() * rcnt);  // rcnt = 1/cnt exactly (cnt is a power of 2)
        cnt *= 2;
        rcnt *= 0.5f;
        win[0] = win[1];
        win[1] = win[2];
        win[2] = win[3];
        win[3] = win[4];
        win[4] = cur;
        if (j >= 5 && romb_stop_f(win, pq, guard)) break;
    }
    return pq;
}

__device__ double qromb_delta_f(const Ctx &C, const ChiArgsF &A, bool &guard) {
    // the integral of the identically-zero integrand is exactly +0 (as in the
    // FP64 form, cs64::qromb_delta_cyl)
    if (A.i1 < 1 || A.i1 > 4) return 0.0;
    const cs_prepared &P = *C.P;
    const double b = P.romb_delta_b;
    const double dbeta = P.romb_dbeta;
    double win[5];
    double cur;
    int cnt;
    double pq = 0.0;
    const double inv2pi = 1.0 / (2.0 * M_PI);
    {
        const cs_delta_node n0 = C.dnode[0], n1 = C.dnode[1];
        // the delta = 0 endpoint has weight sin(0) = 0: its chi integral only
        // matters when it is not finite, so its nodes raise no guard
        bool g0 = false;
        const double c0 = qromb_chi_f(C, A, (float)n0.c, (float)n0.s, g0);
        if (n0.w != 0.0 || !isfinite(c0)) guard = guard || g0 || !isfinite(c0);
        const double pa = n0.w * c0 * inv2pi;
        const double pb = n1.w * qromb_chi_f(C, A, (float)n1.c, (float)n1.s, guard) * inv2pi;
        cur = 0.5 * b * (pa + pb);
        cnt = 1;
    }
    double rcnt = 1.0;
    win[4] = cur;
    for (int j = 2; j <= 20; j++) {
        double sump = 0.0;
        if (j <= CS_NODE_LEVELS) {
            const cs_delta_node *nd = C.dnode + CS_NODE_OFFSET(j);
            for (int k = 0; k < cnt; k++) {
                const cs_delta_node n = nd[k];
                sump += n.w * qromb_chi_f(C, A, (float)n.c, (float)n.s, guard) * inv2pi;
            }
        } else {
            const double del = b / cnt;
            double x = 0.5 * del;
            for (int k = 0; k < cnt; k++) {
                double s, c;
                sincos(x, &s, &c);
                sump += s * exp(-x * x / (dbeta * dbeta)) * qromb_chi_f(C, A, (float)c, (float)s, guard) * inv2pi;
                x += del;
            }
        }
        cur = 0.5 * (cur + b * sump * rcnt);
        cnt *= 2;
        rcnt *= 0.5;
        win[0] = win[1];
        win[1] = win[2];
        win[2] = win[3];
        win[3] = win[4];
        win[4] = cur;
        if (j >= 5 && romb_stop(win, pq, 1.0e-100, guard)) break;
    }
    return pq;
}

// qrombchid by the whole warp (chi nodes over the lanes, FP64 sums and
// extrapolation, the FP64 path's arguments) with the integrand's closed form
// in float pairs (csff::cyl_len_closed, ~1e-13) instead of FP64: the value
// agrees with cs64::qromb_chi_warp to ~1e-12, and its stop decisions are the
// FP64 path's except within 1e-8 of the threshold, which sets `band` (the
// caller then takes the FP64 form).
__device__ double qromb_chi_warp_pair(const Ctx &C, const cs64::ChiArgs &A, double cd, double sd, bool &band) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const double b = C.P->romb_chi_b;
    auto f = [&](double cx, double sx) -> double {
        double argx;
        if (!cs64::chi_argument(A, cx, sx, cd, sd, argx)) return 0.0;
        if (cs64::len_factor_small(argx, A.zm1)) return cs64::len_factor_series(argx, A.zm1);
        float rel;
        return csff::cyl_len_closed(argx, A.z, rel);
    };
    double win[5];
    double cur, pq = 0.0, dss = 0.0;
    int cnt;
    {
        double v = 0.0;
        if (lane < 2) {
            const cs_chi_node n = C.chi[lane];
            v = f(n.c, n.s);
        }
        cur = 0.5 * b * (__shfl_sync(full, v, 0) + __shfl_sync(full, v, 1));
        cnt = 1;
    }
    win[4] = cur;
    for (int j = 2; j <= CS_NODE_LEVELS; j++) {
        const cs_chi_node *nd = C.chi + CS_NODE_OFFSET(j);
        double sump = 0.0;
        for (int base = 0; base < cnt; base += 32) {
            double v = 0.0;
            if (base + lane < cnt) {
                const cs_chi_node n = nd[base + lane];
                v = f(n.c, n.s);
            }
            const int m = (cnt - base) < 32 ? (cnt - base) : 32;
            for (int u = 0; u < m; u++) sump += __shfl_sync(full, v, u);
        }
        cur = 0.5 * (cur + b * sump / (double)cnt);
        cnt = 2 * cnt;
        win[0] = win[1];
        win[1] = win[2];
        win[2] = win[3];
        win[3] = win[4];
        win[4] = cur;
        if (j >= 5) {
            cs64::polint5(win, pq, dss);
            const double lhs = fabs(dss), rhs = 1.0e-4 * fabs(pq);
            if (fabs(lhs - rhs) <= 1e-8 * rhs || !isfinite(pq)) band = true;
            if (lhs < rhs) return pq;
            if (fabs(pq) < 1.0e-300) return pq;
        }
    }
    band = true;  // beyond the node table: the FP64 form's own loop
    return pq;
}

// The outer (delta) quadrature for the warp-level redo of one guarded pixel:
// the delta nodes of a level spread over the lanes, each lane's inner
// integral in FP32; an inner integral whose FP32 form is in its guard band is
// recomputed by the whole warp with the float-pair integrand
// (qromb_chi_warp_pair), and in FP64 (cs64::qromb_chi_warp on the FP64
// arguments: the FP64 path's value) where that one's decision is in its band. Every lane returns the same value and
// guard; what stays guarded (the outer decision, a non-finite value) is left
// to the exact FP64 pixel.
__device__ double qromb_delta_warp_f(const Ctx &C, const ChiArgsF &A, bool &guard) {
    if (A.i1 < 1 || A.i1 > 4) return 0.0;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const cs_prepared &P = *C.P;
    const double b = P.romb_delta_b;
    const double inv2pi = 1.0 / (2.0 * M_PI);
    const cs64::ChiArgs A64 = cs64::chi_args(P, A.qxs, A.qys, P.sigmal, A.i1);
    bool bad = false;
    // inner integral of this lane's node (c, s) when active; guarded ones in FP64 by the warp
    auto node_value = [&](bool active, double c, double s) -> double {
        bool g = false;
        double v = 0.0;
        if (active) v = qromb_chi_f(C, A, (float)c, (float)s, g);
        unsigned m = __ballot_sync(full, g);
        while (m) {
            const int l = __ffs(m) - 1;
            m &= m - 1;
            const double cl = __shfl_sync(full, c, l), sl = __shfl_sync(full, s, l);
            bool band = false;
            double w = qromb_chi_warp_pair(C, A64, cl, sl, band);
            if (band) w = cs64::qromb_chi_warp(C, A64, cl, sl);
            if (lane == l) v = w;
        }
        if (active && !isfinite(v)) bad = true;
        return v;
    };
    double cur;
    {
        const bool act = lane < 2;
        const cs_delta_node n = C.dnode[act ? lane : 0];
        const double v = node_value(act, n.c, n.s);
        const double c0 = __shfl_sync(full, v, 0), c1 = __shfl_sync(full, v, 1);
        cur = 0.5 * b * (C.dnode[0].w * c0 * inv2pi + C.dnode[1].w * c1 * inv2pi);
    }
    double win[5];
    win[4] = cur;
    int cnt = 1;
    double rcnt = 1.0, pq = 0.0;
    for (int j = 2; j <= 20; j++) {
        double sump = 0.0;
        if (j <= CS_NODE_LEVELS) {
            const cs_delta_node *nd = C.dnode + CS_NODE_OFFSET(j);
            for (int base = 0; base < cnt; base += 32) {
                const bool act = base + lane < cnt;
                const cs_delta_node n = nd[act ? base + lane : 0];
                const double v = node_value(act, n.c, n.s);
                const double px = act ? n.w * v * inv2pi : 0.0;
                const int m = (cnt - base) < 32 ? (cnt - base) : 32;
                for (int u = 0; u < m; u++) sump += __shfl_sync(full, px, u);
            }
        } else {
            // beyond the node table (not reached in practice): node by node
            const double dbeta = P.romb_dbeta;
            const double del = b / cnt;
            double x = 0.5 * del;
            for (int k = 0; k < cnt; k++) {
                double sn, cs;
                sincos(x, &sn, &cs);
                const double v = __shfl_sync(full, node_value(lane == 0, cs, sn), 0);
                sump += sn * exp(-x * x / (dbeta * dbeta)) * v * inv2pi;
                x += del;
            }
        }
        cur = 0.5 * (cur + b * sump * rcnt);
        cnt *= 2;
        rcnt *= 0.5;
        win[0] = win[1];
        win[1] = win[2];
        win[2] = win[3];
        win[3] = win[4];
        win[4] = cur;
        if (j >= 5 && romb_stop(win, pq, 1.0e-100, guard)) break;
    }
    if (__any_sync(full, bad)) guard = true;
    return pq;
}

// ----------------------------------------------------------- peak sums FP32
// Lattice peak sums of the FCC/BCT pixel functions over sorted, compacted
// reflection tables. The radial Gaussian of every reflection underflows FP32
// for |q - q_hkl| beyond ~9.3 widths; those reflections are skipped (a binary
// search bounds the window). q is carried as a float pair (qf + ql) so that
// q - q_hkl is formed exactly (Sterbenz) before squaring.
__device__ __forceinline__ int lower_bound_f(const float *__restrict__ a, int n, float v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(a + mid) < v)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Float-pair helpers of the peak sums (this unit is compiled without
// contraction, so the error terms below are exact where stated).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// k d^2 as a float pair (xh + xl) from k = kh + kl and d = dh + dl
__device__ __forceinline__ void scaled_square(float kh, float kl, float dh, float dl, float &xh, float &xl) {
    const float p = dh * dh;
    const float pe = fmaf(dh, dh, -p) + 2.0f * dh * dl;
    xh = kh * p;
    xl = fmaf(kh, p, -xh) + fmaf(kh, pe, kl * p);
}


// s + e = a + b exactly, for |a| >= |b| (or a = 0)
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    e = b - (s - a);
}

// 2^-(xh + xl) as a float pair (eh + el), 0 <= xh < 2^14 (xl a low part),
// with the table of 2^(-j/64) of cs_ff.cuh (Tang's table-driven
// exponential): xh = k/64 + r with r exact (both sides are multiples of xh's
// ulp, |r| <= 1/128), a = -(r + xl) ln 2 as a pair, and 2^-(r + xl) = 1 + p,
// p = a + a^2/2 + a^3 (1/6 + a/24 + a^2/120) (remainder < 3e-17; the cubic
// tail, below 3e-8, in FP32). The pair is within ~3e-14 (relative) of
// 2^-(xh + xl).
__device__ __forceinline__ void exp2m_pair(float xh, float xl, float &eh, float &el) {
    const float k = rintf(xh * 64.0f);
    const float r = fmaf(k, -0.015625f, xh);  // exact
    const int ki = (int)k;
    const csff::ff t = csff::from_pair(&csff::kExp2m64[ki & 63]);
    csff::ff rr;
    csff::two_sum(r, xl, rr.hi, rr.lo);
    const csff::ff a = csff::neg(csff::mul(rr, csff::ff{0x1.62e43p-1f, -0x1.05c61p-29f}));  // -(r + xl) ln 2
    const float ah = a.hi;
    const float tail = ah * ah * ah * fmaf(ah, fmaf(ah, 1.0f / 120.0f, 1.0f / 24.0f), 1.0f / 6.0f);
    const csff::ff p = csff::add_f(csff::add(a, csff::mul_f(csff::sqr(a), 0.5f)), tail);
    const csff::ff e = csff::add(t, csff::mul(t, p));
    eh = ldexpf(e.hi, -(ki >> 6));
    el = ldexpf(e.lo, -(ki >> 6));
}

// float-pair accumulator (sum of float pairs, error ~1e-13 of the sum of
// magnitudes)
struct SumFF {
    float h = 0.0f, l = 0.0f;
    __device__ __forceinline__ void add(float bh, float bl) {
        float s, e;
        two_sum(h, bh, s, e);
        e += l + bl;
        fast_two_sum(s, e, h, l);
    }
    __device__ __forceinline__ double value() const { return (double)h + (double)l; }
};

// yphi = acos(1 - s) = 2 asin(sqrt(s/2)) and yphi^2 = 2 s (1 + r(s)) with
// r(s) = sum_{n>=2} 2^n s^(n-1) / (n^2 C(2n, n)) (the series of asin^2); through
// n = 17 the remainder is below 1e-12 for s < 1/2 (yphi < 60 degrees).
// r(s) for s = sh + sl as a pair (rh + rl): r = s (1/6 + s (2/45 + s Q(s)))
// with 1/6 and 2/45 as float pairs and the product s (2/45 + s Q) exact, so
// that the FP32 rounding of Q's Horner sum enters r only through terms of
// ~s^2/70 of it: r within ~1e-8 (relative) instead of ~1e-7
__device__ __forceinline__ void asin2_rest_pair(float sh, float sl, float &rh, float &rl) {
    const float c[14] = {1.428571429e-02f, 5.079365079e-03f, 1.924001924e-03f, 7.611436183e-04f,
                         3.108003108e-04f, 1.300079731e-04f, 5.542445171e-05f, 2.399326914e-05f,
                         1.051878828e-05f, 4.660632346e-06f, 2.083721869e-06f, 9.388723824e-07f,
                         4.258997702e-07f, 1.943499843e-07f};
    const float c0h = (float)(1.0 / 6.0), c0l = (float)(1.0 / 6.0 - (double)(float)(1.0 / 6.0));
    const float c1h = (float)(2.0 / 45.0), c1l = (float)(2.0 / 45.0 - (double)(float)(2.0 / 45.0));
    float q = c[13];
#pragma unroll
    for (int n = 12; n >= 0; n--) q = fmaf(q, sh, c[n]);
    const float inner = fmaf(q, sh, c1h) + c1l;  // 2/45 + s Q
    const float ph = sh * inner;
    const float pe = fmaf(sh, inner, -ph);
    float bh, be;
    two_sum(c0h, ph, bh, be);
    be += c0l + fmaf(sl, inner, pe);  // 1/6 + s inner = bh + be
    rh = sh * bh;
    rl = fmaf(sh, bh, -rh) + fmaf(sh, be, sl * bh);
}


// Error estimates of the sums: the terms are float pairs (exp2m_pair times the
// reflection's factor as a float pair) summed as float pairs; a term carries
// the pair exponential's error (c0) and the error of its angular argument
// (ephi); the radial argument k (q - q_hkl)^2 is a float pair, exact to ~1e-12
// of its size. The sums' relative errors are the term-weighted means (eps_rad,
// eps_int).
__device__ void peak_sums_f(const cs_prepared &P, const PeakTab &T, double qx, double qy, double qz, double q,
                            double &radint, double &intens, double &eps_rad, double &eps_int, bool &guard) {
    // per term: the pair exponential (3e-14) and the argument pair's own
    // rounding (~4e-15 of the exponent, added per term below)
    const float c0 = 5e-14f;
    // per-set factors from the table (the anisotropic width depends on q when
    // para is set: then it and its factors are formed here)
    double kd_an = T.kd_an, inv_an = T.inv_an;
    float dmax_an = T.dmax_an;
    if (P.para) {
        double width = 1;
        if (P.debyescherrer) width = 4.0 / P.domainsize;
        if (P.para) width = (4.0 / P.domainsize) + cs64::sqr(P.reldis) * P.dist * cs64::sqr(q);
        width *= P.width_zuf;
        kd_an = 4.0 / M_PI / (width * width) * 1.4426950408889634;
        inv_an = 1.0 / (M_PI * width / 2.0);
        dmax_an = (float)(9.4 * width);
    }
    const float qf = (float)q;
    const float ql = (float)(q - (double)qf);
    // isotropic peaks: exp(-4 x2/pi) / (pi widthiso/2), x2 = (q-qhkl)^2/widthiso^2
    {
        const double kd = T.kd_iso;
        const float kh = (float)kd, kl = (float)(kd - (double)kh);
        const float dmax = T.dmax_iso;
        int i = lower_bound_f(T.iq, T.n_iso, qf - dmax);
        SumFF s;
        float w = 0.0f;
        for (; i < T.n_iso; i++) {
            const float qh = __ldg(T.iq + i);
            float dh, de;
            two_sum(qf, -qh, dh, de);
            const float dl = de + ql;
            if (dh + dl < -dmax) break;
            float xh, xl, eh, el;
            scaled_square(kh, kl, dh, dl, xh, xl);
            exp2m_pair(xh, xl, eh, el);
            const float m = __ldg(T.imf + i);  // an integer, exact
            const float th = eh * m;
            s.add(th, fmaf(eh, m, -th) + el * m);
            w = fmaf(fabsf(th), fmaf(4e-15f, xh, c0), w);
        }
        // the normalisation is a product (the pair sum is far more accurate
        // than the bound needs) and the estimate's quotient FP32
        radint = s.value() * T.inv_iso;
        eps_rad = s.h != 0.0f ? (double)(w / fabsf(s.h)) : 0.0;
    }
    // anisotropic peaks
    {
        const double kd = kd_an;
        const float kh = (float)kd, kl = (float)(kd - (double)kh);
        const float dmax = dmax_an;
        const double kphid = q * q * T.kphi;
        const float kph = (float)kphid, kpl = (float)(kphid - (double)kph);
        // unit q as a float pair; eps = 1 - |q|/q of the reference's cosine
        // (its q carries CS_EPS9)
        const double rn = 1.0 / (q - CS_EPS9);
        const double uxd = qx * rn, uyd = qy * rn, uzd = qz * rn;
        const float fx = (float)uxd, fy = (float)uyd, fz = (float)uzd;
        const float lx = (float)(uxd - fx), ly = (float)(uyd - fy), lz = (float)(uzd - fz);
        const float epsq = (float)CS_EPS9 / qf;
        int i = lower_bound_f(T.aq, T.n_aniso, qf - dmax);
        SumFF s;
        float w = 0.0f;
        for (; i < T.n_aniso; i++) {
            const float qh = __ldg(T.aq + i);
            float dh, de;
            two_sum(qf, -qh, dh, de);
            const float dl = de + ql;
            if (dh + dl < -dmax) break;
            const float4 v = __ldg(T.av + 2 * i);       // unit q_hkl (x, y, z), mult * g3/peaknorm1
            const float4 vl = __ldg(T.av + 2 * i + 1);  // low parts, 1 - |h|/q_hkl
            const float c = fmaf(fx, v.x, fmaf(fy, v.y, fz * v.z));
            // myacos: the reference maps c < -1 to 0 and c > 1 to pi. For q
            // (anti)parallel to q_hkl the FP64 rounding of the reference's
            // cosine decides between those and acos(c) ~ 0, a jump of the
            // Gaussian; there the cosine is taken as the reference computes it.
            // Up to 90 degrees the angle comes from 1 - c_ref = eh + (1 - eh)
            // |u - h|^2/2 (eh: the reference's norms), free of acos's
            // cancellation near 1; below 1 - c_ref = 0.05 (18 degrees) yphi^2
            // itself comes from the series of 4 asin^2(sqrt(s/2)) with |u - h|^2
            // as a float pair. Beyond 90 degrees acos(c) is used, off by
            // ~2e-7/sin(yphi).
            float xph, xpl = 0.0f, ephi;  // angular argument kphi yphi^2 (pair) and its error
            if (fabsf(c) > 1.0f - 1e-5f) {
                const int ii = __ldg(T.aidx + i);
                const double cd = (qx * (double)P.latpar3[ii][2] + qy * (double)P.latpar3[ii][3] +
                                   qz * (double)P.latpar3[ii][4]) /
                                  (q * (double)P.latpar3[ii][5]);
                const float yphi = (float)((cd < -1) ? 0.0 : ((cd > 1) ? M_PI : acos(cd)));
                xph = kph * yphi * yphi;
                ephi = 2e-7f * xph;
            } else if (c > 0.0f) {
                // u - h as float pairs (the high differences are not always
                // exact: components near zero may differ in sign)
                float dxh, dxe, dyh, dye, dzh, dze;
                two_sum(fx, -v.x, dxh, dxe);
                two_sum(fy, -v.y, dyh, dye);
                two_sum(fz, -v.z, dzh, dze);
                const float dxl = dxe + (lx - vl.x), dyl = dye + (ly - vl.y), dzl = dze + (lz - vl.z);
                const float px = dxh * dxh, py = dyh * dyh, pz = dzh * dzh;
                const float pe = fmaf(dxh, dxh, -px) + fmaf(dyh, dyh, -py) + fmaf(dzh, dzh, -pz) +
                                 2.0f * fmaf(dxh, dxl, fmaf(dyh, dyl, dzh * dzl));
                float s1, e1, ddh, e2;
                two_sum(px, py, s1, e1);
                two_sum(s1, pz, ddh, e2);
                const float ddl = e1 + e2 + pe;
                const float eh = epsq + vl.w;
                const float shh = 0.5f * ddh;  // exact
                const float shl = fmaf(0.5f, ddl, eh * (1.0f - shh));
                const float sh = shh + shl;
                if (sh < 0.5f) {
                    // kphi yphi^2 = 2 kphi s (1 + r): 2 kphi s as a pair, r small
                    const float ah = (2.0f * kph) * shh;
                    const float al = fmaf(2.0f * kph, shh, -ah) + 2.0f * fmaf(kph, shl, kpl * shh);
                    // r as a pair from the pair s: ~2e-8 of r; s itself: ~4e-15
                    // of kphi absolute
                    float rh, rl;
                    asin2_rest_pair(shh, shl, rh, rl);
                    // (ah + al)(1 + rh + rl): the low parts take their shares too
                    two_sum(ah, fmaf(ah, rh, fmaf(al, rh, fmaf(ah, rl, al))), xph, xpl);
                    ephi = fmaf(xph, fmaf(3e-8f, rh, 1e-13f), 4e-15f * kph);
                } else {
                    const float yphi = 2.0f * asinf(sqrtf(0.5f * sh));
                    xph = kph * yphi * yphi;
                    ephi = 6e-7f * xph;
                }
            } else {
                const float yphi = acosf(c);
                xph = kph * yphi * yphi;
                ephi = 2.1e-7f * kph * yphi / sqrtf(fmaxf(1.0f - c * c, 1e-10f));
            }
            float xh, xl, sx, ex, eh, el;
            scaled_square(kh, kl, dh, dl, xh, xl);
            two_sum(xh, xph, sx, ex);
            exp2m_pair(sx, ex + xl + xpl, eh, el);
            // times mult g3/peaknorm1 as a float pair (v.w + awl)
            const float wl = __ldg(T.awl + i);
            const float th = eh * v.w;
            s.add(th, fmaf(eh, v.w, -th) + fmaf(eh, wl, el * v.w));
            w = fmaf(fabsf(th), fmaf(4e-15f, sx, c0) + ephi, w);
        }
        intens = s.value() * inv_an;
        eps_int = s.h != 0.0f ? (double)(w / fabsf(s.h)) : 0.0;
        if (!isfinite(intens)) guard = true;  // the reference stops at an infinite sum
    }
}

// ---------------------------------------------------------------- pixels
__device__ __forceinline__ double zr_asym(const cs_prepared &P) {
    double zr = (1 - cs64::sqr(P.sigma)) / cs64::sqr(P.sigma);
    if (zr * (zr - 1) * (zr - 2) * (zr - 3) * (zr - 4) * (zr - 5) == 0) zr += CS_EPS3;
    return zr;
}

template <bool LAT>
__device__ double sphere_pq_mixed(const cs_prepared &P, double q, bool &guard, double &err) {
    if (P.cs != 0) {
        guard = true;
        return 0.0;
    }
    const double thr = 0.4 * P.limq[4];
    if (near(q, thr, 1e-12)) guard = true;
    if (q < thr) {
        err = EPS_SERIES;
        return cs64::series_q(P.carrp[3], q, 100);
    }
    const double zr = zr_asym(P);
    float rel;
    const double argq = q * P.radius / (zr + 1);
    float v = sphere_pq_asym<false>(argq, zr, rel);
    if (!(rel <= acc_switch<LAT>())) v = sphere_pq_asym<true>(argq, zr, rel);
    err = rel;
    return v;
}

template <bool LAT>
__device__ double sphere_fq_mixed(const cs_prepared &P, double q, bool &guard, double &err) {
    const double thr = 0.4 * P.limqf[4];
    if (near(q, thr, 1e-12)) guard = true;
    if (q < thr) {
        err = EPS_SERIES;
        return cs64::series_q(P.carrf[3], q, 100);
    }
    const double zr = (1 - cs64::sqr(P.sigma)) / cs64::sqr(P.sigma);
    float rel;
    const double argq = q * P.radius / (zr + 1);
    float v = sphere_fq_asym<false>(argq, zr, rel);
    if (!(rel <= acc_switch<LAT>())) v = sphere_fq_asym<true>(argq, zr, rel);
    err = rel;
    return v;
}

// formpq_partCylinder, ordis 0 and 6, cs 0 (mixed)
// PAIR: the closed forms in float pairs (csff::cyl_len_closed,
// csff::cyl_cross_asym: ~1e-13), for lattice pixels, whose structure factor
// can amplify the form factors' errors by orders of magnitude.
template <bool LAT, bool WARP = false, bool PAIR = false>
__device__ double cyl_pq_mixed(const Ctx &C, double qxs, double qys, double q, bool &guard, double &err) {
    const cs_prepared &P = *C.P;
    if (P.cs != 0) {
        guard = true;
        return 0.0;
    }
    // Schulz exponents of length and radius, formed on the branches that use
    // them (two FP64 divisions the other pixels do not pay)
    auto z_of = [](double sg) { return sg == 1.0 ? CS_EPS9 : (1 - cs64::sqr(sg)) / cs64::sqr(sg); };
    double pql = 0, pqr = 0;
    double el = EPS_SERIES, er = EPS_SERIES;
    if (P.ordis == 6) {
        const double thr = 0.6 * P.limq[1];
        if (near(q, thr, 1e-12)) guard = true;
        if (q < thr) {
            pql = cs64::series_zdir(P.carrp[0], qxs, qys);
        } else {
            const double zl = z_of(P.sigmal);
            const double arglq = (qxs + qys + CS_EPS9) * P.length / (zl + 1);
            // FP32 closed form (its small-argument series where it cancels),
            // refined with FP64 arguments when its own estimate exceeds the
            // switch; lattice pixels take the float-pair form (PAIR)
            if (PAIR) {
                if (cs64::len_factor_small(arglq, zl - 1)) {
                    pql = cs64::len_factor_series(arglq, zl - 1);
                } else {
                    float rel;
                    pql = csff::cyl_len_closed(arglq, zl, rel);
                    el = rel;
                }
            } else {
                float rel;
                pql = cyl_len_factor_e<false>(arglq, zl, rel);
                if (!LAT && !(rel <= acc_switch<LAT>())) pql = cyl_len_factor_e<true>(arglq, zl, rel);
                el = rel;
            }
        }
    } else if (P.ordis == 0) {
        const double thr = 0.4 * P.limq[1];
        if (near(q, thr, 1e-12)) guard = true;
        if (q < thr) {
            pql = 1.0;
            if (P.orcase == 1 || P.orcase == 2)
                pql = cs64::cyl_double_series(P, qxs, qys, P.carrp[0], 0);
            else if (P.orcase == 3)
                pql = cs64::cyl_double_series(P, qxs, qys, P.carrp[0], 1);
        } else if (P.orcase < 1 || P.orcase > 4) {
            // the integrand is identically zero (trapzdchid has no case for
            // the general orientation): the quadrature gives +0, and +0 / norm
            // is +0 for a positive norm
            pql = P.norm > 0 ? 0.0 : 0.0 / P.norm;
        } else {
            ChiArgsF A;
            const double s = P.sigmal;
            const double z = (1 - s * s) / (s * s);
            A.qx = (float)qxs;
            A.qy = (float)qys;
            A.lz = (float)(P.length / (z + 1));
            A.a4 = (float)(2.0 / (z * (z - 1)));
            A.z = (float)z;
            A.p11 = (float)P.romb_p[0];
            A.p12 = (float)P.romb_p[1];
            A.p13 = (float)P.romb_p[2];
            A.p21 = (float)P.romb_p[3];
            A.p22 = (float)P.romb_p[4];
            A.p23 = (float)P.romb_p[5];
            A.i1 = P.orcase;
            A.b = (float)P.romb_chi_b;
            A.qxs = qxs;
            A.qys = qys;
            pql = (WARP ? qromb_delta_warp_f(C, A, guard) : qromb_delta_f(C, A, guard)) / P.norm;
            el = EPS_PQ;
        }
    } else {
        guard = true;
        return 0.0;
    }
    // A length factor of exactly zero (the general orientation's identically
    // zero integrand, or an exact zero of the series) makes the product zero
    // wherever the radial factor is finite. On the series side of its switch
    // it is (a converged sum of finite terms): the FP64 series is skipped
    // there, and the switch needs no guard (a zero either way, the closed form
    // being finite at the switch). On the closed-form side it is skipped where
    // it is provably finite; elsewhere it is still evaluated so that a
    // non-finite value reaches the product as in the drop-in. The sign of a
    // zero product does not change the pixel's value.
    const bool zero_len = !LAT && pql == 0.0;
    if ((P.length / P.radius) < 2)
        pqr = 1;
    else {
        const double thr = 0.65 * P.limq[4];
        if (!zero_len && near(q, thr, 1e-12)) guard = true;
        if (q < thr) {
            if (zero_len) {
                err = el;
                return 0.0;
            }
            pqr = cs64::series_q(P.carrp[3], q, 120);
        } else {
            // the closed form is finite for zr > 3.16 (sigma < 0.49) and an
            // argument q R sigma^2 that is not tiny: a zero product then
            if (zero_len && P.sigma > 0 && P.sigma < 0.49 && q * P.radius * P.sigma * P.sigma > 1e-28) {
                err = el;
                return 0.0;
            }
            float rel;
            const double zr = z_of(P.sigma);
            const double argpq = q * P.radius / (zr + 1);
            if (PAIR) {
                pqr = csff::cyl_cross_asym(argpq, zr, rel);
            } else {
                pqr = cyl_pqr_asym<false>(argpq, zr, rel);
                // (a zero length factor makes the product zero: no need to refine)
                if (!LAT && !(rel <= acc_switch<LAT>()) && !zero_len) pqr = cyl_pqr_asym<true>(argpq, zr, rel);
            }
            // a finite factor of a zero product carries no error into it
            er = (zero_len && isfinite(pqr)) ? 0.0f : rel;
        }
    }
    err = el + er;
    return pql * pqr;
}


// formfq_partCylinder, ordis 0 and 6, cs 0 (mixed)
template <bool LAT, bool PAIR = false>
__device__ double cyl_fq_mixed(const Ctx &C, double limql, double qxs, double qys, double q, bool &guard,
                             double &err) {
    const cs_prepared &P = *C.P;
    if (P.cs != 0) {
        guard = true;
        return 0.0;
    }
    const double zl = (1 - cs64::sqr(P.sigmal)) / cs64::sqr(P.sigmal);
    const double zr = (1 - cs64::sqr(P.sigma)) / cs64::sqr(P.sigma);
    double pql = 0, pqr = 0;
    double el = EPS_SERIES, er = EPS_SERIES;
    if (P.ordis == 6) {
        const double thr = 0.6 * P.limqf[1];
        if (near(limql, thr, 1e-12)) guard = true;
        if (limql < thr) {
            pql = cs64::series_zdir(P.carrf[0], qxs, qys);
        } else {
            const double arglq = (qxs + qys + CS_EPS9) * P.length / (zl + 1);
            // FP32 closed form (its small-argument series where it cancels),
            // refined with FP64 arguments when its own estimate exceeds the
            // switch; lattice pixels take the float-pair form (PAIR)
            if (PAIR) {
                if (cs64::len_factor_small(arglq, zl - 1)) {
                    pql = cs64::len_factor_series(arglq, zl - 1);
                } else {
                    float rel;
                    pql = csff::cyl_len_closed(arglq, zl, rel);
                    el = rel;
                }
            } else {
                float rel;
                pql = cyl_len_factor_e<false>(arglq, zl, rel);
                if (!LAT && !(rel <= acc_switch<LAT>())) pql = cyl_len_factor_e<true>(arglq, zl, rel);
                el = rel;
            }
        }
    } else if (P.ordis == 0) {
        const double thr = 0.2 * P.limqf[1];
        if (near(limql, thr, 1e-12)) guard = true;
        if (limql < thr) {
            double pqsum = 1.0;
            if (P.orcase == 1) pqsum = cs64::cyl_double_series(P, qxs, qys, P.carrf[0], 2);
            if (P.orcase == 2) pqsum = cs64::cyl_double_series(P, qxs, qys, P.carrf[0], 0);
            if (P.orcase == 3) pqsum = cs64::cyl_double_series(P, qxs, qys, P.carrf[0], 3);
            pql = pqsum;
        } else {
            ChiArgsF A;
            const double s = P.sigmal;
            const double z = (1 - s * s) / (s * s);
            A.qx = (float)qxs;
            A.qy = (float)qys;
            A.lz = (float)(P.length / (z + 1));
            A.a4 = (float)(2.0 / (z * (z - 1)));
            A.z = (float)z;
            A.p11 = (float)P.romb_p[0];
            A.p12 = (float)P.romb_p[1];
            A.p13 = (float)P.romb_p[2];
            A.p21 = (float)P.romb_p[3];
            A.p22 = (float)P.romb_p[4];
            A.p23 = (float)P.romb_p[5];
            A.i1 = P.orcase;
            A.b = (float)P.romb_chi_b;
            A.qxs = qxs;
            A.qys = qys;
            pql = qromb_delta_f(C, A, guard) / P.norm;
            el = EPS_PQ;
        }
    } else {
        guard = true;
        return 0.0;
    }
    const double thr = 1.0 * P.limqf[4];
    if (near(q, thr, 1e-12)) guard = true;
    if (q < thr) {
        pqr = cs64::series_q(P.carrf[3], q, 120);
    } else {
        const double a = q * P.radius / (zr + 1);
        float rel;
        double amp;
        if (PAIR) {
            amp = cyl_fqr_asym_d(a, zr, P.gamma_ratio[0], P.gamma_ratio[1], rel);
        } else {
            amp = cyl_fqr_asym<false>(a, zr, P.gamma_ratio[0], P.gamma_ratio[1], rel);
            if (!LAT && !(rel <= acc_switch<LAT>())) amp = cyl_fqr_asym<true>(a, zr, P.gamma_ratio[0], P.gamma_ratio[1], rel);
        }
        pqr = amp * amp;
        er = rel;
    }
    err = el + er;
    return pql * pqr;
}

// Final combination of the lattice pixel functions,
//   I = base + I0 (szq pq + iso szqiso pqi) + tail,
//   szq = 1 + (fq/pq)(2 pi I_aniso/V - 1) e^(-dw q^2),
//   szqiso = 1 + (8 pi^3 I_iso/(4 pi V) - 1) e^(-ucb q^2),
// in FP64 from inputs with the relative error estimates errp/errf/errpi
// (EPS_SERIES or EPS_PQ per part) and EPS_PEAK (peak sums). Where the terms cancel
// (szq -> 0 between peaks, I0 szq pq against base) the input errors are
// amplified; a first-order estimate of the result's error is propagated
// alongside, and a pixel whose estimate exceeds 5e-6 of |I| (half the 1e-5 bar)
// is recomputed in FP64. The Debye-Waller factors are FP64 exponentials (in
// FP32 the rounding of the argument alone moved them by |arg| 6e-8, which
// dominated the estimate where szq cancels; the iso factor szqiso cancels
// too), the ratio F/P a float-pair quotient, and the lattice volume's factors
// 2 pi/V and 2 pi^2/V per set.
__device__ __forceinline__ double lattice_combine(const cs_prepared &P, const PeakTab &T, double q, double pq,
                                                  double errp, double fq, double errf, double pqi, double errpi,
                                                  double radint, double intens, double eps_rad, double eps_int,
                                                  double tailv, bool &guard, bool fq_exact = false) {
    const double r2 = radint * T.c_r2;
    const double e2 = exp(-P.ucb * q * q), e1 = exp(-P.dwfactor * q * q);  // the drop-in's operations
    const double ee2 = 4e-16, ee1 = 4e-16;
    const double szqiso = 1 + (r2 - 1) * e2;
    const double r1 = intens * T.c_r1;
    if (fq_exact && !isfinite(fq) && isfinite(pq)) {
        // F(q) from the FP64 series, bit for bit the drop-in's, is not finite:
        // so is the drop-in's result, its class (NaN, +-inf) set by the signs
        // of the finite factors, which are the drop-in's unless r1 - 1 is
        // within its error of 0
        const double res = P.base + P.izero * ((1 + (fq / pq) * (r1 - 1) * e1) * pq + P.iso * szqiso * pqi) + tailv;
        if (!(fabs(r1 - 1) > 1e-9 * fabs(r1)) && !isnan(fq)) guard = true;
        return res;
    }
    const double ratio = csff::to_double(csff::div(csff::from_double(fq), csff::from_double(pq)));
    const double t = ratio * (r1 - 1) * e1;
    const double szq = 1 + t;
    const double res = P.base + P.izero * (szq * pq + P.iso * szqiso * pqi) + tailv;
    // first-order error bound (the quotient's own 1e-14 included)
    const double dt = fabs(t) * (errf + errp + ee1 + 1e-14) + fabs(ratio * e1 * r1) * (eps_int + EPS_PEAK);
    const double d1 = fabs(pq) * dt + fabs(szq * pq) * errp;
    const double d2 = fabs(P.iso) * (fabs(pqi) * (fabs(r2 * e2) * (eps_rad + EPS_PEAK) + fabs((r2 - 1) * e2) * ee2) +
                                     fabs(szqiso * pqi) * errpi);
    const double bound = fabs(P.izero) * (d1 + d2);
    if (!(bound <= 5e-6 * fabs(res))) guard = true;
    return res;
}

template <int KEY, bool WARP = false>
__device__ double calc_mixed(const Ctx &C, const PeakTab &T, double qx, double qy, double qz, bool &guard) {
    const cs_prepared &P = *C.P;
    const double q = sqrt(qx * qx + qy * qy + qz * qz) + CS_EPS9;
    // the fluctuation term (its FP64 division skipped when it is zero)
    const double tailv = P.ifluc == 0.0 ? 0.0 : P.ifluc / (1 + q * q * P.rfluc * P.rfluc);
    double ep = 0, ef = 0;  // relative error estimates of pq and fq
    if (KEY == CS_KEY_SPHERE_NONE_ISO) {
        const double pq = sphere_pq_mixed<false>(P, q, guard, ep);
        if (!(ep <= 5e-6)) guard = true;
        return P.base + P.izero * (pq + P.iso * pq) + tailv;
    }
    // lattice keys: near q = 0 the structure factor's exact value is formed
    // from series differences by the FP64 function (cs64::lattice_factors_small_q)
    if ((KEY == CS_KEY_SPHERE_GAUSS_FCC_GAUSS || KEY == CS_KEY_CYL_GAUSS_BCT_ZDIR) && q < CS_SMALL_Q) guard = true;
    if (KEY == CS_KEY_SPHERE_GAUSS_FCC_GAUSS) {
        const double pq = sphere_pq_mixed<true>(P, q, guard, ep);
        const double fq = sphere_fq_mixed<true>(P, q, guard, ef);
        double radint, intens, erad, eint;
        peak_sums_f(P, T, qx, qy, qz, q, radint, intens, erad, eint, guard);
        return lattice_combine(P, T, q, pq, ep, fq, ef, pq, ep, radint, intens, erad, eint, tailv, guard);
    }
    if (KEY == CS_KEY_CYL_NONE_GAUSS) {
        double pq;
        if (P.orcase == CS_ORC_GENERAL)
            pq = cyl_pq_mixed<false, WARP>(C, qx * P.cosphic - qy * P.sinphic, qx * P.sinphic + qy * P.cosphic, q, guard, ep);
        else
            pq = cyl_pq_mixed<false, WARP>(C, qx, qy, q, guard, ep);
        if (!(ep <= 5e-6)) guard = true;
        return P.base + P.izero * (pq + P.iso) + tailv;
    }
    if (KEY == CS_KEY_CYL_NONE_ZDIR) {
        double pq;
        switch (P.orcase) {
        case CS_ORC_GENERAL: pq = cyl_pq_mixed<false>(C, qx * P.cosphi * P.sintheta, qy * P.sinphi * P.sintheta, q, guard, ep); break;
        case CS_ORC_XAXIS: pq = cyl_pq_mixed<false>(C, qx, 0, q, guard, ep); break;
        case CS_ORC_YAXIS: pq = cyl_pq_mixed<false>(C, 0, qy, q, guard, ep); break;
        default: pq = cyl_pq_mixed<false>(C, qx, qy, q, guard, ep); break;
        }
        if (!(ep <= 5e-6)) guard = true;
        return P.base + P.izero * (pq + P.iso) + tailv;
    }
    if (KEY == CS_KEY_CYL_GAUSS_BCT_ZDIR) {
        // form factors of the orientation case, closed forms in float pairs:
        // the structure factor's cancellation (lattice_combine) amplifies
        // their error by orders of magnitude. (An FP32 first pass with a
        // second pass where the bound fails was slower: 30 % of the pixels
        // failed, and a warp runs both passes when one lane fails.)
        auto forms = [&](double &pq, double &fq) {
            constexpr bool F = true;
            switch (P.orcase) {
            case CS_ORC_GENERAL:
                pq = cyl_pq_mixed<true, false, F>(C, qx * P.cosphi * P.sintheta, qy * P.sinphi * P.sintheta, q, guard, ep);
                fq = cyl_fq_mixed<true, F>(C, sqrt(P.cosphi * qx * qx + P.sinphi * qy * qy + CS_EPS9),
                                           qx * P.cosphi * P.sintheta, qy * P.sinphi * P.sintheta, q, guard, ef);
                break;
            case CS_ORC_XAXIS:
                pq = cyl_pq_mixed<true, false, F>(C, qx, 0, q, guard, ep);
                fq = cyl_fq_mixed<true, F>(C, fabs(qx), qx, 0, q, guard, ef);
                break;
            case CS_ORC_YAXIS:
                pq = cyl_pq_mixed<true, false, F>(C, 0, qy, q, guard, ep);
                fq = cyl_fq_mixed<true, F>(C, fabs(qy), 0, qy, q, guard, ef);
                break;
            default:
                pq = cyl_pq_mixed<true, false, F>(C, qx, qy, q, guard, ep);
                fq = cyl_fq_mixed<true, F>(C, q, qx, qy, q, guard, ef);
                break;
            }
        };
        double pq = 0, fq = 0;
        forms(pq, fq);
        double radint, intens, erad, eint;
        peak_sums_f(P, T, qx, qy, qz, q, radint, intens, erad, eint, guard);
        // F(q) of the z-direction cylinder from its two FP64 series (length
        // factor below 0.6 limqf1 of its argument, radial below limqf4): the
        // drop-in's value bit for bit
        double limql = q;
        switch (P.orcase) {
        case CS_ORC_GENERAL: limql = sqrt(P.cosphi * qx * qx + P.sinphi * qy * qy + CS_EPS9); break;
        case CS_ORC_XAXIS: limql = fabs(qx); break;
        case CS_ORC_YAXIS: limql = fabs(qy); break;
        default: break;
        }
        const bool fq_exact = P.ordis == 6 && P.cs == 0 && limql < 0.6 * P.limqf[1] && q < P.limqf[4];
        // the reference's BCT function multiplies szqiso by 1 instead of pq
        return lattice_combine(P, T, q, pq, ep, fq, ef, 1.0, 0.0, radint, intens, erad, eint, tailv, guard, fq_exact);
    }
    guard = true;
    return 0.0;
}

// Mixed image kernel: writes every pixel; pixels with a guarded decision are
// appended to the redo list (device counter) and rewritten by k_redo.
template <int KEY>
__global__ void __launch_bounds__(256) k_image_mixed(Ctx C, PeakTab T, double *__restrict__ out, int nx, long npix,
                                                      int *__restrict__ redo_count, int *__restrict__ redo_list,
                                                      int redo_cap) {
    const cs_prepared &P = *C.P;
    const int xstride = P.xmax - P.xmin;
    const QGeom g = q_geom(P);
    // persistent warps take 32-pixel chunks from redo_count[1] (zeroed with
    // the redo counter): balanced however unevenly the pixel cost varies
    int *next = redo_count + 1;
    for (;;) {
        int base = 0;
        if ((threadIdx.x & 31) == 0) base = atomicAdd(next, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if ((long)base >= npix) break;
        // images are below 2^30 pixels (checked on the host): 32-bit indices
        const int t = base + (int)(threadIdx.x & 31);
        if ((long)t >= npix) continue;
        const int ihex = P.zzmin + t % nx;
        const int i = P.iimin + t / nx;
        double qx, qy, qz;
        q_of_pixel<KEY>(P, g, ihex, i, qx, qy, qz);
        bool guard = false;
        const double v = calc_mixed<KEY>(C, T, qx, qy, qz, guard);
        out[(long)(ihex - P.xmin) + (long)xstride * (long)(i - P.ymin)] = v;
        if (guard) {
            const int pos = atomicAdd(redo_count, 1);
            if (pos < redo_cap) redo_list[pos] = t;
        }
    }
}


// Persistent mixed-precision kernel over one group of a batch, pixel
// arithmetic as k_image_mixed, guarded pixels appended to the group's redo
// list as (set, pixel). Work comes from the group's counter either as whole
// block tiles (chunk = 0: CS_BATCH_TILE pixels per block, thread 0 takes the
// tile, two barriers per tile) or as warp chunks (chunk = 32..CS_BATCH_TILE
// pixels per warp, no barrier); `limit` > 0 stops after that many chunks
// (the autotuner's timed samples).
template <int KEY>
__device__ __forceinline__ void batch_mixed_pixel(const cs::BatchSetDev *__restrict__ sets, int k, long t,
                                                  const cs_chi_node *__restrict__ chi, double *__restrict__ out,
                                                  int *__restrict__ redo_count, int2 *__restrict__ redo_list,
                                                  long redo_cap) {
    const cs::BatchSetDev &S = sets[k];
    if (t >= S.npix) return;
    const cs_prepared &P = *S.prep;
    const Ctx C{S.prep, chi, S.delta};
    const int ihex = P.zzmin + (int)(t % S.nx);
    const int i = P.iimin + (int)(t / S.nx);
    double qx, qy, qz;
    if (!cs::batch_q_from_table(S, ihex, i, qx, qy, qz)) q_of_pixel<KEY>(P, q_geom(P), ihex, i, qx, qy, qz);
    bool guard = false;
    const double v = calc_mixed<KEY>(C, S.peaks, qx, qy, qz, guard);
    out[S.out_offset + (long)(ihex - P.xmin) + (long)(P.xmax - P.xmin) * (long)(i - P.ymin)] = v;
    if (guard) {
        const int pos = atomicAdd(redo_count, 1);
        if (pos < redo_cap) redo_list[pos] = make_int2(k, (int)t);
    }
}

template <int KEY>
__global__ void __launch_bounds__(CS_BATCH_TILE) k_batch_mixed(const cs::BatchSetDev *__restrict__ sets,
                                                               int set_begin, int set_end, long tiles, int chunk,
                                                               long limit, unsigned long long *__restrict__ counter,
                                                               const cs_chi_node *__restrict__ chi,
                                                               double *__restrict__ out, int *__restrict__ redo_count,
                                                               int2 *__restrict__ redo_list, long redo_cap) {
    int cur = set_begin;
    int k;
    if (chunk == 0) {
        long tile;
        const long lim = limit > 0 && limit < tiles ? limit : tiles;
        while (cs::batch_next_tile(sets, set_begin, set_end, lim, counter, cur, tile, k))
            batch_mixed_pixel<KEY>(sets, k, (tile - sets[k].tile_begin) * CS_BATCH_TILE + threadIdx.x, chi, out,
                                   redo_count, redo_list, redo_cap);
        return;
    }
    const int lane = threadIdx.x & 31;
    long pix0;
    while (cs::batch_next_chunk(sets, set_begin, set_end, tiles, chunk, limit, counter, cur, pix0, k))
        for (int o = 0; o < chunk; o += 32)
            batch_mixed_pixel<KEY>(sets, k, pix0 + o + lane, chi, out, redo_count, redo_list, redo_cap);
}

// Redo of the guarded pixels of the orientation-averaged cylinder, one pixel
// per warp (qromb_delta_warp_f): most of them only had an inner integral in its
// guard band, which the warp recomputes in FP64; the rest run the exact FP64
// pixel with the warp over the delta nodes (cs64::calc_cyl_none_gauss<true>).
// Where the geometry or thresholds matter, q is the FP64 path's own.
__global__ void __launch_bounds__(128) k_redo_cyl_warp(Ctx C, double *__restrict__ out, int nx,
                                                        const int *__restrict__ redo_count,
                                                        const int *__restrict__ redo_list, int redo_cap) {
    const cs_prepared &P = *C.P;
    const int xstride = P.xmax - P.xmin;
    int n = *redo_count;
    if (n > redo_cap) n = redo_cap;
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const PeakTab T{};
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += nw) {
        const long t = redo_list[r];
        const int ihex = P.zzmin + (int)(t % nx);
        const int i = P.iimin + (int)(t / nx);
        double qx, qy, qz;
        cs64::convert_idx2q(P, ihex, i, qx, qy, qz);
        bool guard = false;
        double v = calc_mixed<CS_KEY_CYL_NONE_GAUSS, true>(C, T, qx, qy, qz, guard);
        if (__any_sync(0xffffffffu, guard)) v = cs64::calc_cyl_none_gauss<true>(C, qx, qy, qz);
        if (lane == 0) out[(long)(ihex - P.xmin) + (long)xstride * (long)(i - P.ymin)] = v;
    }
}

// the same for the (set, pixel) redo list of a batch group
__global__ void __launch_bounds__(128) k_batch_redo_cyl_warp(const cs::BatchSetDev *__restrict__ sets,
                                                              const cs_chi_node *__restrict__ chi,
                                                              double *__restrict__ out,
                                                              const int *__restrict__ redo_count,
                                                              const int2 *__restrict__ redo_list, long redo_cap) {
    long n = *redo_count;
    if (n > redo_cap) n = redo_cap;
    const int lane = threadIdx.x & 31;
    const long nw = ((long)gridDim.x * blockDim.x) >> 5;
    const PeakTab T{};
    for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += nw) {
        const int2 e = redo_list[r];
        const cs::BatchSetDev &S = sets[e.x];
        const cs_prepared &P = *S.prep;
        const Ctx C{S.prep, chi, S.delta};
        const long t = e.y;
        const int ihex = P.zzmin + (int)(t % S.nx);
        const int i = P.iimin + (int)(t / S.nx);
        double qx, qy, qz;
        cs64::convert_idx2q(P, ihex, i, qx, qy, qz);
        bool guard = false;
        double v = calc_mixed<CS_KEY_CYL_NONE_GAUSS, true>(C, T, qx, qy, qz, guard);
        if (__any_sync(0xffffffffu, guard)) v = cs64::calc_cyl_none_gauss<true>(C, qx, qy, qz);
        if (lane == 0) out[S.out_offset + (long)(ihex - P.xmin) + (long)(P.xmax - P.xmin) * (long)(i - P.ymin)] = v;
    }
}

}  // namespace csm

namespace cs {

void peak_constants(const cs_prepared &P, csm::PeakTab &T) {
    const double widthiso = 1.0 / P.uca;
    T.kd_iso = 4.0 / M_PI / (widthiso * widthiso) * 1.4426950408889634;
    T.inv_iso = 1.0 / (M_PI * widthiso / 2.0);
    T.dmax_iso = (float)(9.4 * widthiso);
    double width = 1;
    if (P.debyescherrer) width = 4.0 / P.domainsize;
    width *= P.width_zuf;
    T.kd_an = 4.0 / M_PI / (width * width) * 1.4426950408889634;
    T.inv_an = 1.0 / (M_PI * width / 2.0);
    T.dmax_an = (float)(9.4 * width);
    T.kphi = 4.0 / (M_PI * P.phiwidth * P.phiwidth) * 1.4426950408889634;
    const double v = P.latpar[1] * P.latpar[2];
    T.c_r1 = 2 * M_PI / v;
    T.c_r2 = 8 * M_PI * M_PI * M_PI / (4 * M_PI * v);
}

// Compact, sorted reflection tables from the prepared block (see PeakTab).
void build_peak_tables(const cs_prepared &P, HostPeaks &H) {
    H.aq.clear(); H.awl.clear(); H.av.clear(); H.iq.clear(); H.imf.clear(); H.aidx.clear();
    struct A { float q; float4 v, vl; float wl; int idx; };
    std::vector<A> an;
    for (int ii = 1; ii <= P.peakmax2 && ii < CS_LATPARLEN; ii++) {
        const float qh = P.latpar3[ii][5];
        const int mf = P.latpar2[ii][4] * P.latpar2[ii][5];
        if (!(qh > 0) || mf == 0) continue;
        const double q = qh;
        A a;
        a.q = qh;
        // unit vector of q_hkl as a float pair, and 1 - |h|/q_hkl (the stored
        // components and magnitude are rounded separately)
        const double hx = P.latpar3[ii][2], hy = P.latpar3[ii][3], hz = P.latpar3[ii][4];
        const double hn = std::sqrt(hx * hx + hy * hy + hz * hz);
        const double ux = hx / hn, uy = hy / hn, uz = hz / hn;
        const double wd = (double)P.latpar3[ii][10] / (double)P.latpar3[ii][11] * (double)mf;
        a.v = make_float4((float)ux, (float)uy, (float)uz, (float)wd);
        a.wl = (float)(wd - (double)(float)wd);
        a.vl = make_float4((float)(ux - (double)(float)ux), (float)(uy - (double)(float)uy), (float)(uz - (double)(float)uz),
                           (float)(1.0 - hn / q));
        a.idx = ii;
        an.push_back(a);
    }
    std::stable_sort(an.begin(), an.end(), [](const A &x, const A &y) { return x.q < y.q; });
    for (auto &a : an) {
        H.aq.push_back(a.q);
        H.av.push_back(a.v);
        H.av.push_back(a.vl);
        H.awl.push_back(a.wl);
        H.aidx.push_back(a.idx);
    }
    struct I { float q; float mf; };
    std::vector<I> is;
    for (int ii = 1; ii <= P.peakmax1 && ii < CS_LATPARLEN; ii++) {
        const int mhkl = P.latpar1[ii][4], fhkl = P.latpar1[ii][5];
        if (mhkl == 0 || fhkl == 0) continue;
        is.push_back({P.latpar3[ii][5], (float)mhkl * (float)fhkl});
    }
    std::stable_sort(is.begin(), is.end(), [](const I &x, const I &y) { return x.q < y.q; });
    for (auto &i : is) {
        H.iq.push_back(i.q);
        H.imf.push_back(i.mf);
    }
}

static int sm_count_m() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

template <int KEY>
static void launch_mixed_key(const DevSet &D, const csm::PeakTab &T, const cs_prepared &P, double *d_out,
                             MixedScratch &S, cudaStream_t s) {
    const int nx = P.zzmax - P.zzmin;
    const long npix = (long)nx * (long)(P.iimax - P.iimin);
    cs64::Ctx C{D.d_prep, D.d_chi, D.d_delta};
    // persistent grid: the resident blocks of every SM (warps take work from
    // a counter), fewer when the image is small
    static int per_sm = 0;
    if (per_sm == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, csm::k_image_mixed<KEY>, 256, 0);
        if (per_sm < 1) per_sm = 1;
    }
    const long need = (npix + 255) / 256;
    const long cap = (long)sm_count_m() * per_sm;
    const int grid = (int)(need < cap ? (need < 1 ? 1 : need) : cap);
    cudaMemsetAsync(S.d_count, 0, 2 * sizeof(int), s);  // redo counter and pixel queue
    csm::k_image_mixed<KEY><<<grid, 256, 0, s>>>(C, T, d_out, nx, npix, S.d_count, S.d_list, S.cap);
    if (KEY == CS_KEY_CYL_NONE_GAUSS)
        csm::k_redo_cyl_warp<<<sm_count_m() * 4, 128, 0, s>>>(C, d_out, nx, S.d_count, S.d_list, S.cap);
    else
        launch_redo(D, P, d_out, S, s);
}

int launch_image_mixed(const DevSet &D, const csm::PeakTab &T0, const cs_prepared &P, double *d_out, MixedScratch &S,
                       cudaStream_t s) {
    csm::PeakTab T = T0;
    if (P.lattice) peak_constants(P, T);
    const int nx = P.zzmax - P.zzmin, ny = P.iimax - P.iimin;
    if (nx <= 0 || ny <= 0) return CS_OK;
    if (P.twin) return CS_ERR_UNSUPPORTED;
    if ((long)nx * (long)ny > (1L << 30)) return CS_ERR_SIZE;  // the pixel queue counts in int
    switch (P.key) {
    case CS_KEY_SPHERE_NONE_ISO: launch_mixed_key<CS_KEY_SPHERE_NONE_ISO>(D, T, P, d_out, S, s); break;
    case CS_KEY_SPHERE_GAUSS_FCC_GAUSS: launch_mixed_key<CS_KEY_SPHERE_GAUSS_FCC_GAUSS>(D, T, P, d_out, S, s); break;
    case CS_KEY_CYL_NONE_GAUSS: launch_mixed_key<CS_KEY_CYL_NONE_GAUSS>(D, T, P, d_out, S, s); break;
    case CS_KEY_CYL_NONE_ZDIR: launch_mixed_key<CS_KEY_CYL_NONE_ZDIR>(D, T, P, d_out, S, s); break;
    case CS_KEY_CYL_GAUSS_BCT_ZDIR: launch_mixed_key<CS_KEY_CYL_GAUSS_BCT_ZDIR>(D, T, P, d_out, S, s); break;
    default: return CS_ERR_UNSUPPORTED;
    }
    if (P.expand && P.calc_quadrants != CS_RADQ4 && P.calc_quadrants != CS_RAD1D) launch_mirror(P, d_out, s);
    return launch_status();
}


// ---- batch launchers -------------------------------------------------------

// Pixel geometry table (cs_batch.h): the drop-in's convert_idx2q of every
// pixel of [-half, half]^2; this unit rounds as the FP64 units do (no
// contraction), so the values are the ones each set would compute.
__global__ void k_qtable(const cs_prepared *__restrict__ P, int half, double *__restrict__ q) {
    const int w = 2 * half + 1;
    const long n = (long)w * w;
    for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < n; j += (long)gridDim.x * blockDim.x) {
        const int ihex = (int)(j % w) - half;
        const int i = (int)(j / w) - half;
        double qx, qy, qz;
        cs64::convert_idx2q(*P, ihex, i, qx, qy, qz);
        q[j] = qx;
        q[j + n] = qy;
        q[j + 2 * n] = qz;
    }
}

int launch_qtable(const QTable &t, cudaStream_t s) {
    const long n = (long)(2 * t.half + 1) * (2 * t.half + 1);
    const int grid = (int)std::min<long>((n + 255) / 256, (long)sm_count_m() * 8);
    k_qtable<<<grid, 256, 0, s>>>(t.prep, t.half, t.d);
    return launch_status();
}

int launch_batch_mixed(const BatchSetDev *d_sets, const BatchGroup &g, int group_index, unsigned long long *d_counter,
                       const cs_chi_node *d_chi, double *d_out, const BatchRedo &R, int grid, cudaStream_t s,
                       cudaEvent_t mid, int chunk, long limit, bool redo) {
    if (g.tiles <= 0) return CS_OK;
    int *cnt = R.d_count + group_index;
    int2 *list = R.d_list + (size_t)group_index * (size_t)R.cap;
    switch (g.key) {
#define CS_CASE(K)                                                                                                \
    case K:                                                                                                       \
        csm::k_batch_mixed<K><<<grid, CS_BATCH_TILE, 0, s>>>(d_sets, g.set_begin, g.set_end, g.tiles, chunk,       \
                                                              limit, d_counter, d_chi, d_out, cnt, list, R.cap);  \
        break;
        CS_FOR_EACH_KEY(CS_CASE)
#undef CS_CASE
    default: return CS_ERR_UNSUPPORTED;
    }
    if (launch_status() != CS_OK) return CS_ERR_CUDA;
    if (mid) cudaEventRecord(mid, s);
    if (!redo) return CS_OK;
    if (g.key == CS_KEY_CYL_NONE_GAUSS) {
        csm::k_batch_redo_cyl_warp<<<sm_count_m() * 4, 128, 0, s>>>(d_sets, d_chi, d_out, cnt, list, R.cap);
        return launch_status();
    }
    return launch_batch_redo(d_sets, g.key, d_chi, d_out, cnt, list, R.cap, s);
}

int batch_blocks_per_sm_mixed(int key) {
    int n = 0;
    switch (key) {
#define CS_CASE(K) \
    case K: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, csm::k_batch_mixed<K>, CS_BATCH_TILE, 0); break;
        CS_FOR_EACH_KEY(CS_CASE)
#undef CS_CASE
    default: return 0;
    }
    return n;
}

}  // namespace cs
