// cs_fp64.cuh — FP64 per-pixel functions (the plain GPU drop-in).
//
// Device restatement of the reference's pixel path with the reference's
// operation order, so that results agree with its FP64 CPU path to ~1e-12:
//   convert_idx2q              Source/sc_calc_generic_gpu.cu:249-287
//   formpq_partSphere          Source/sc_lib_formpq_partSphere.h:11-196 (cs 0, 1)
//   formfq_partSphere          Source/sc_lib_formfq_partSphere.h:8-52 (cs 0)
//   formpq_partCylinder        Source/sc_lib_formpq_partCylinder.h:8-391 (ordis 0, 6; cs 0)
//   formfq_partCylinder        Source/sc_lib_formfq_partCylinder.h:8-216 (ordis 0, 6; cs 0)
//   qrombdeltac/trapzddeltac   Source/sc_calc_generic_gpu.cu:1370-1488, 956-1272 (i0 = 4)
//   qrombchid/trapzdchid       Source/sc_calc_generic_gpu.cu:1495-1583, 1590-2965 (i1 = 1..4)
//   polint                     Source/sc_calc_generic_gpu.cu:1280-1335
//   calc_partSphere_lattNone_ordisIsotropic      Source/sc_gpu_pSph_lNon_oIso.h:15-51
//   calc_partSphere_peakGauss_lattFCC_ordisGauss Source/sc_gpu_pSph_pGau_lFCC_oGau.h:15-171
//   calc_partCylinder_lattNone_ordisGauss        Source/sc_gpu_pCyl_lNon_oGau.h:15-100
//   calc_partCylinder_lattNone_ordisZDir         Source/sc_gpu_pCyl_lNon_oZDi.h:17-88
//   calc_partCylinder_peakGauss_lattBCT_ordisZDir Source/sc_gpu_pCyl_pGau_lBCT_oZDi.h:16-245
// Quirks of the reference (0-based orcase compared with 1-based integers,
// the inverted acos clamp, latpar3 read with the isotropic peak index, the
// misplaced parenthesis in the sphere asymptote) are reproduced on purpose.
#ifndef CS_FP64_CUH
#define CS_FP64_CUH

#include "cs_prepared.h"
#include "cs_tables.h"
#include "cs_series_stop.h"

namespace cs64 {

#define CS_EPS9 0.000000001
#define CS_EPS3 0.001

__device__ __forceinline__ double sqr(double x) { return x * x; }

// myacos of the reference (Source/sc_calc_generic_gpu.cu:30): the clamp maps
// x < -1 to 0 and x > 1 to pi.
__device__ __forceinline__ double myacos(double x) { return (x < -1) ? 0.0 : ((x > +1) ? M_PI : acos(x)); }

struct Ctx {
    const cs_prepared *__restrict__ P;
    const cs_chi_node *__restrict__ chi;     // chi node table (global, levels 1..CS_NODE_LEVELS)
    const cs_delta_node *__restrict__ dnode; // delta node table of this parameter set (may be null)
};

__device__ __forceinline__ void convert_idx2q(const cs_prepared &P, int ihex, int i, double &qx, double &qy,
                                              double &qz) {
    if (P.use1d) {
        qx = (P.qmax - P.qmin) / (double)(P.zmax) * (double)ihex;
        qy = 1e-20;
        qz = 1e-20;
    } else if (P.usebeamstop) {
        double mdet = (ihex)*P.pixnoy / (2.0 * P.zmax);
        double ndet = (i)*P.pixnox / (2.0 * P.zmax);
        double xdet = P.pixx_m * (ndet - P.beamx0);
        double ydet = P.pixy_m * (mdet - P.beamy0);
        double rdet = sqrt(xdet * xdet + ydet * ydet);
        double phidet = atan2(ydet, xdet);
        double thetadet = atan2(rdet, P.det);
        qx = 2 * M_PI * cos(phidet) * sin(thetadet) / P.wave;
        qy = 2 * M_PI * sin(phidet) * sin(thetadet) / P.wave;
        qz = 2 * M_PI * (1 - cos(thetadet)) / P.wave;
    } else {
        qx = P.qmax * i / (double)(P.zmax);
        qy = P.qmax * ihex / (double)(P.zmax);
        qz = 1e-20;
    }
}

// power series 1 + sum_n c[n] (q^2)^n with the reference's qq = qq*q*q
// and its stop at relative increment < 1e-4 (the loops of the formpq/formfq
// libraries)
// The power series below stop at the first term whose relative increment is
// below 1e-4, a discrete decision on a sum that can cancel by many orders of
// magnitude; a different rounding of one partial sum can move the stop by one
// term (a jump of ~1e-4 relative). Their products and sums are therefore
// written with __dmul_rn/__dadd_rn, which are never fused into a
// multiply-add, so they round as the reference's separate operations in every
// translation unit, also in those compiled with contraction.
// The reference's stop test fabs((s - old) / s) < 0.0001 with its decision in
// every case, almost always without the FP64 division (cs_series_stop.h).
using cs_series::series_converged;

__device__ __forceinline__ double series_q(const double *__restrict__ c, double q, int nmax) {
    double pqsum = 1.0;
    double oldpqsum = 0.0;
    double qq = 1.0;
    for (int nser = 1; nser <= nmax; nser++) {
        qq = __dmul_rn(__dmul_rn(qq, q), q);
        pqsum = __dadd_rn(pqsum, __dmul_rn(c[nser], qq));
        if (series_converged(pqsum, oldpqsum)) break;
        oldpqsum = pqsum;
    }
    return pqsum;
}

// 1D series in (qxs+qys)^2 of the z-direction cylinder (formpq_partCylinder
// ordis 6, Source/sc_lib_formpq_partCylinder.h:93-124; formfq_partCylinder
// ordis 6, Source/sc_lib_formfq_partCylinder.h:55-87).
__device__ __forceinline__ double series_zdir(const double *__restrict__ c, double qxs, double qys) {
    double pql = 1.0;
    double oldpqsum = 0.0;
    double qqnn = 1.0;
    const double s = qxs + qys;
    for (int nser = 1; nser <= 120; nser++) {
        qqnn = __dmul_rn(__dmul_rn(qqnn, s), s);
        pql = __dadd_rn(pql, __dmul_rn(c[nser], qqnn));
        if (series_converged(pql, oldpqsum)) break;
        oldpqsum = pql;
    }
    return pql;
}

// ------------------------------------------------------------------ spheres
__device__ inline double formpq_sphere(const cs_prepared &P, double q) {
    double zr = (1 - sqr(P.sigma)) / (sqr(P.sigma));
    const double radiusm = P.radius / P.p1;
    const double zz = zr;
    if (P.cs == 0) {
        if (q < 0.4 * P.limq[4]) {
            return series_q(P.carrp[3], q, 100);
        }
        const double argq = q * P.radius / (zr + 1);
        if (zr * (zr - 1) * (zr - 2) * (zr - 3) * (zr - 4) * (zr - 5) == 0) zr += CS_EPS3;
        double pqr = (1 / (2.0 * zr * (zr - 1) * (zr - 2) * (zr - 3))) * pow(argq, -4);
        const double pq1 = pqr * (1 + cos((zr - 3) * atan(2.0 * argq)) / pow(1.0 + 4 * argq * argq, (zr - 3) / 2.0));
        const double pq2 = (pqr / ((zr - 4) * argq)) * sin((zr - 4) * atan(2.0 * argq)) / pow(1.0 + 4 * argq * argq, (zr - 4) / 2.0);
        const double pq3 = (pqr / ((zr - 4) * (zr - 5) * argq * argq)) *
                           (1 - cos((zr - 5) * atan(2.0 * argq)) / pow(1.0 + 4 * argq * argq, zr - 5) / 2.0);
        return 9.0 * (pq1 - 2.0 * pq2 + pq3);
    }
    if (P.cs == 1) {
        const double cc1 = sqr(P.rho);
        const double cc2 = 2 * P.p1 * P.rho * (1 - P.rho);
        const double cc3 = sqr(1 - P.rho) * sqr(P.p1);
        const double cc4 = -2 * sqr(P.rho);
        const double cc5 = -2 * P.p1 * P.rho * (1 - P.rho);
        const double cc6 = sqr(P.rho);
        const double cc7 = -2 * P.rho * (1 - P.rho);
        const double cc8 = -sqr(1 - P.rho) * 2 * P.p1;
        const double cc9 = 2 * P.rho * (1 - P.rho);
        const double cc10 = sqr(1 - P.rho);
        const double ccc1 = sqr(1 - P.rho) * pow(P.p1, 6);
        const double ccc2 = 2 * P.rho * (1 - P.rho) * pow(P.p1, 3);
        const double ccc3 = P.rho * P.rho;
        const double vv3 = sqr((1 - P.rho) * pow(P.p1, 3) + P.rho);
        const double argq = q * radiusm / (zz + 1);
        const double argpq = q * P.radius / (zz + 1);
        const double pqr = (1 / (2.0 * zr * (zr - 1) * (zr - 2) * (zr - 3))) * pow(argq, -4);
        double F121, F122, F123;
        if (q < (0.5 * P.limq[4])) {
            F121 = ccc1 * series_q(P.carrp[3], q, 120) / vv3;
        } else {
            const double ac3 = pqr * (1 + cos((zr - 3) * atan(2.0 * argpq)) / pow(1.0 + 4 * argpq * argpq, (zr - 3) / 2.0));
            const double ac8 = (pqr / ((zr - 4) * argq)) * sin((zr - 4) * atan(2.0 * argpq)) / pow(1.0 + 4 * argpq * argpq, (zr - 4) / 2.0);
            const double ac10 = (pqr / ((zr - 4) * (zr - 5) * argq * argq)) *
                                (1 - cos((zr - 5) * atan(2.0 * argpq)) / pow(1.0 + 4 * argpq * argpq, (zr - 5) / 2.0));
            F121 = 9 * (cc3 * ac3 + cc8 * ac8 + cc10 * ac10) / vv3;
        }
        if (q < (0.5 * P.limq[5])) {
            F122 = ccc2 * series_q(P.carrp[4], q, 120) / vv3;
        } else {
            const double argbm = (zr - 3) * atan(argpq - argq);
            const double nenbm = pow(1.0 + sqr(argpq - argq), (zr - 3) / 2.0);
            const double argbp = (zr - 3) * atan(argpq + argq);
            const double nenbp = pow(1.0 + sqr(argpq + argq), (zr - 3) / 2.0);
            const double ac2 = pqr * (cos(argbm) / nenbm + cos(argbp) / nenbp);
            const double argep = (zr - 4) * atan(argpq + argq);
            const double nenep = pow(1.0 + sqr(argpq + argq), (zr - 4) / 2.0);
            const double argem = (zr - 4) * atan(argpq - argq);
            const double nenem = pow(1.0 + sqr(argpq - argq), (zr - 4) / 2.0);
            const double ac5 = (pqr / ((zr - 4) * argq)) * (sin(argep) / nenep - sin(argem) / nenem);
            const double arggp = (zr - 4) * atan(argpq + argq);
            const double nengp = pow(1.0 + sqr(argpq + argq), (zr - 4) / 2.0);
            const double arggm = (zr - 4) * atan(argq - argpq);
            const double nengm = pow(1.0 + sqr(argq - argpq), (zr - 4) / 2.0);
            const double ac7 = (pqr / ((zr - 4) * argq)) * (sin(arggp) / nengp - sin(arggm) / nengm);
            const double ac9 = (pqr / ((zr - 4) * (zr - 5) * argq * argq)) * (cos(argbm) / nenbm - cos(argbp) / nenbp);
            F122 = 9 * (cc2 * ac2 + cc5 * ac5 + cc7 * ac7 + cc9 * ac9) / vv3;
        }
        if (q < (0.5 * P.limq[6])) {
            F123 = ccc3 * series_q(P.carrp[5], q, 120) / vv3;
        } else {
            const double ac1 = pqr * (1 + cos((zr - 3) * atan(2.0 * argq)) / pow(1.0 + 4 * argq * argq, (zr - 3) / 2.0));
            const double ac4 = (pqr / ((zr - 4) * argq)) * sin((zr - 4) * atan(2.0 * argq)) / pow(1.0 + 4 * argq * argq, (zr - 4) / 2.0);
            const double ac6 = (pqr / ((zr - 4) * (zr - 5) * argq * argq)) *
                               (1 - cos((zr - 5) * atan(2.0 * argq)) / pow(1.0 + 4 * argq * argq, (zr - 5) / 2.0));
            F123 = 9 * (cc1 * ac1 + cc4 * ac4 + cc6 * ac6) / vv3;
        }
        return F121 + F122 + F123;
    }
    return 0.0;
}

__device__ inline double formfq_sphere(const cs_prepared &P, double q) {
    const double zr = (1 - sqr(P.sigma)) / sqr(P.sigma);
    if (P.cs == 0) {
        if (q < (0.4 * P.limqf[4])) {
            return series_q(P.carrf[3], q, 100);
        }
        const double argq = q * P.radius / (zr + 1);
        const double pqr = (1 / (zr * (zr - 1)) * pow(argq, -2));
        const double pq1 = pqr * cos((zr - 1) * atan(argq)) / pow(1.0 + argq * argq, (zr - 1) / 2.0);
        const double pq2 = (pqr / ((zr - 2) * argq)) * sin((zr - 2) * atan(argq)) / pow(1.0 + argq * argq, (zr - 2) / 2.0);
        const double pq3 = 3 * (pq2 - pq1);
        return pq3 * pq3;
    }
    return 0.0;
}

// ------------------------------------------------- Romberg orientation average
// Neville extrapolation to 0 over the last five trapezoid estimates; the
// abscissae are 1, 1/4, ..., 1/256 times a power of two for every window, which
// leaves each rounding equal to the reference's.
__device__ __forceinline__ void polint5(const double ya[5], double &y, double &dy) {
    const double xa[5] = {1.0, 0.25, 0.0625, 0.015625, 0.00390625};
    double c[5], d[5];
#pragma unroll
    for (int i = 0; i < 5; i++) {
        c[i] = ya[i];
        d[i] = ya[i];
    }
    int ns = 4;  // smallest |xa| is the last one (0-based)
    y = ya[4];
    ns = ns - 1;
#pragma unroll
    for (int m = 1; m <= 4; m++) {
#pragma unroll
        for (int i = 0; i < 5 - m; i++) {
            double ho = xa[i];
            double hp = xa[i + m];
            double w = c[i + 1] - d[i];
            double den = ho - hp;
            if (den != 0) den = w / den;
            d[i] = hp * den;
            c[i] = ho * den;
        }
        // reference (1-based ns1 = ns+1): if 2*ns1 < 5-m then dy=c[ns1+1] else dy=d[ns1], ns1--
        if (2 * (ns + 1) < 5 - m)
            dy = c[ns + 1];
        else {
            dy = d[ns];
            ns = ns - 1;
        }
        y = y + dy;
    }
}

// Length factor of the Schulz-averaged cylinder along its axis,
//   L(a) = (1/(2z(z-1)a^2)) (1 - cos(m atan 2a) / (1+4a^2)^(m/2)),  m = z-1,
// in the reference's closed form (formpq/formfq_partCylinder ordis 6,
// Source/sc_lib_formpq_partCylinder.h:115-119; the integrand of trapzdchid
// i1 = 1..4, Source/sc_calc_generic_gpu.cu:1590-2965). For small |m a| the
// bracket cancels: it is ~2 m(m+1) a^2 while its terms carry FP64 rounding of
// ~1e-16, so the reference's FP64 value is off by up to ~1e-16/(m a)^2
// relative (O(1) on pixels on the cylinder axis, where a is eps-sized) and
// moves by as much under one-ulp changes of cos/pow. Below |m a| = 0.05 the
// closed form's exact value is taken from its power series instead: the
// bracket is 1 - Re (1+2ia)^(-m) = -sum_{j>=1} C(m+2j-1, 2j) (-4a^2)^j, so
//   L = 1 + sum_{j>=1} T_j,  T_j/T_(j-1) = -4a^2 (m+2j)(m+2j+1)/((2j+1)(2j+2)),
// whose ratios there are below ~1e-3: a few terms reach the FP64 rounding of
// the sum. Elsewhere the reference's own expression is evaluated (same
// operations, same rounding).
__device__ __forceinline__ bool len_factor_small(double a, double m) { return fabs(m * a) < 0.05 && fabs(a) < 0.05; }

__device__ __forceinline__ double len_factor_series(double a, double m) {
    const double x = -4.0 * a * a;
    double term = 1.0, sum = 0.0;
    for (int j = 1; j <= 40; j++) {
        term = term * (x * ((m + 2 * j) * (m + 2 * j + 1)) / ((2 * j + 1) * (2 * j + 2)));
        sum = sum + term;
        if (fabs(term) <= 1e-18 * fabs(sum) || term == 0.0) break;
    }
    return 1.0 + sum;
}

// chi integrand of trapzdchid for the cylinder cases i1 = 1..4; any other i1
// leaves the integrand 0 (the reference has no branch for orcGeneral = 0).
struct ChiArgs {
    double qx, qy, l, z, zp1, a1, zm1, zm1h;
    double p11, p12, p13, p21, p22, p23;
    int i1;
};

// the integrand's argument; false for the cases without one (integrand 0)
__device__ __forceinline__ bool chi_argument(const ChiArgs &A, double cx, double sx, double cd, double sd,
                                             double &argx) {
    const double eps = 0.0000000001;
    switch (A.i1) {
    case 1: {
        const double mlx1 = A.p11 * cx * sd + A.p12 * sx * sd + A.p13 * cd;
        const double mlx2 = A.p21 * sx * sd + A.p22 * cx * sd + A.p23 * cd;
        argx = (A.qx * mlx1 + A.qy * mlx2 + eps) * A.l / A.zp1;
        return true;
    }
    case 2: argx = (A.qx * cd - A.qy * sx * sd + eps) * A.l / A.zp1; return true;
    case 3: argx = (A.qx * sx * sd + A.qy * cd + eps) * A.l / A.zp1; return true;
    case 4: argx = (A.qx * sx * sd - A.qy * cx * sd + eps) * A.l / A.zp1; return true;
    default: return false;
    }
}

__device__ __forceinline__ double chi_integrand(const ChiArgs &A, double cx, double sx, double cd, double sd) {
    double argx;
    if (!chi_argument(A, cx, sx, cd, sd, argx)) return 0.0;
    if (len_factor_small(argx, A.zm1)) return len_factor_series(argx, A.zm1);
    return (A.a1 / (argx * argx)) * (1 - cos(A.zm1 * atan(2.0 * argx)) / pow(1.0 + 4 * argx * argx, A.zm1h));
}

// The integrand at the interval's ends (level 1 of trapzdchid): for the
// cylinder cases both ends take their own angle.
__device__ __forceinline__ void chi_ends(const ChiArgs &A, const cs_chi_node &n0, const cs_chi_node &n1, double cd,
                                         double sd, double &pa, double &pb) {
    pa = chi_integrand(A, n0.c, n0.s, cd, sd);
    pb = chi_integrand(A, n1.c, n1.s, cd, sd);
}

// chi integrand of trapzdchid for the disk P(q) cases i1 = 8..11 (i3 = 0),
// Source/sc_calc_generic_gpu.cu:1849-2260 (interval ends) and 2604-2840
// (interior nodes), with sigma = sigmal and l = the disk radius (length). The
// unit vector of the pixel's q (qxl, qyl) meets the disk normal at qnn; the
// Schulz-averaged disk factor at x = sqrt(1 - qnn^2) l qn/(z+1) is, for
// sigmal < 0.15, its series in x^2/4 (carr2p) below x = 0.015 and its
// asymptote above, otherwise the Ornstein-Zernike-like form.
struct DiskChiArgs {
    double qxl, qyl, qn, l, z, sigma;
    double p11, p12, p13, p21, p22, p23;
    const double *carr;
    int i1;
};

__device__ __forceinline__ DiskChiArgs disk_chi_args(const cs_prepared &P, double qx, double qy, int i1,
                                                     const double *carr) {
    const double eps = 0.0000000001;
    DiskChiArgs A;
    A.sigma = P.sigmal;
    A.z = (1 - A.sigma * A.sigma) / (A.sigma * A.sigma);
    A.qn = sqrt(qx * qx + qy * qy + eps);
    A.qxl = qx / A.qn;
    A.qyl = qy / A.qn;
    A.l = P.length;
    A.p11 = P.romb_p[0];
    A.p12 = P.romb_p[1];
    A.p13 = P.romb_p[2];
    A.p21 = P.romb_p[3];
    A.p22 = P.romb_p[4];
    A.p23 = P.romb_p[5];
    A.carr = carr;
    A.i1 = i1;
    return A;
}

// qnn from the angle chi: (c1, s1) enter the first direction component and
// (s2, c2) the second; every interior node passes (cos, sin, sin, cos) of its
// own chi. The reference's general-case end a takes cos(a) with sin(b) and
// sin(a) with cos(b) (:1856-1857); disk_chi_ends passes them so.
__device__ __forceinline__ double disk_chi_value(const DiskChiArgs &A, double c1, double s1, double s2, double c2,
                                                 double cd, double sd) {
    const double eps = 0.0000000001;
    double qnn;
    switch (A.i1) {
    case 8: {
        const double ml1 = A.p11 * c1 * sd + A.p12 * s1 * sd + A.p13 * cd;
        const double ml2 = A.p21 * s2 * sd + A.p22 * c2 * sd + A.p23 * cd;
        qnn = A.qxl * ml1 + A.qyl * ml2;
        break;
    }
    case 9: qnn = A.qxl * cd - A.qyl * s1 * sd; break;
    case 10: qnn = A.qxl * s1 * sd + A.qyl * cd; break;
    case 11: qnn = A.qxl * s1 * sd - A.qyl * c1 * sd; break;
    default: return 0.0;
    }
    const double z = A.z;
    const double x = sqrt(1.0 - qnn * qnn + eps) * A.l * A.qn / (z + 1);
    if (A.sigma < 0.15) {
        if (x < 0.015) {
            double px = 1, oldpx = 0, argser = 1;
            for (int i = 1; i <= 50; i++) {
                argser = argser * x * x / 4.0;
                px = px + A.carr[i] * argser;
                if (series_converged(px, oldpx)) break;
                oldpx = px;
            }
            return px;
        }
        const double px1 = (1 / (z * (z - 1) * (z - 2))) * pow(x, -3);
        const double px2 = (1 / (z * (z - 1) * (z - 2))) * pow(x, -3) * sin((z - 2) * atan(2.0 * x)) /
                           pow(1.0 + 4 * x * x, (z - 2) / 2.0);
        const double px3 = (1 / (z * (z - 1) * (z - 2) * (z - 3))) * pow(x, -4) * cos((z - 3) * atan(2.0 * x)) /
                           pow(1.0 + 4 * x * x, (z - 3) / 2.0);
        return (4 / M_PI) * (px1 - px2 - (9 / 8.0) * px3);
    }
    const double px1 = (1 / (z * (z - 1) * (z - 2))) * pow(x, -3);
    return 1 / (1.0 + M_PI / (4.0 * px1));
}

__device__ __forceinline__ double chi_integrand(const DiskChiArgs &A, double cx, double sx, double cd, double sd) {
    return disk_chi_value(A, cx, sx, sx, cx, cd, sd);
}

__device__ __forceinline__ void chi_ends(const DiskChiArgs &A, const cs_chi_node &n0, const cs_chi_node &n1, double cd,
                                         double sd, double &pa, double &pb) {
    if (A.i1 == 8)
        pa = disk_chi_value(A, n0.c, n1.s, n0.s, n1.c, cd, sd);
    else
        pa = disk_chi_value(A, n0.c, n0.s, n0.s, n0.c, cd, sd);
    pb = disk_chi_value(A, n1.c, n1.s, n1.s, n1.c, cd, sd);
}

// qrombchid over chi in [0, chi_b] for one delta node (cd = cos(delta), sd = sin(delta)).
template <class Args>
__device__ inline double qromb_chi(const Ctx &C, const Args &A, double cd, double sd) {
    const double a = 0.0, b = C.P->romb_chi_b;
    double win[5];
    double cur;
    int cnt;
    double pq = 0.0, dss = 0.0;
    {
        const cs_chi_node n0 = C.chi[0], n1 = C.chi[1];
        double pa, pb;
        chi_ends(A, n0, n1, cd, sd, pa, pb);
        cur = 0.5 * (b - a) * (pa + pb);
        cnt = 1;
    }
    win[4] = cur;
    for (int j = 2; j <= 20; j++) {
        const double tnm = cnt;
        const double del = (b - a) / tnm;
        double sump = 0.0;
        if (j <= CS_NODE_LEVELS) {
            const cs_chi_node *nd = C.chi + CS_NODE_OFFSET(j);
            for (int k = 0; k < cnt; k++) {
                const cs_chi_node n = nd[k];
                sump += chi_integrand(A, n.c, n.s, cd, sd);
            }
        } else {
            double x = a + 0.5 * del;
            for (int k = 0; k < cnt; k++) {
                double s, c;
                sincos(x, &s, &c);
                sump += chi_integrand(A, c, s, cd, sd);
                x += del;
            }
        }
        cur = 0.5 * (cur + (b - a) * sump / tnm);
        cnt = 2 * cnt;
        win[0] = win[1];
        win[1] = win[2];
        win[2] = win[3];
        win[3] = win[4];
        win[4] = cur;
        if (j >= 5) {
            polint5(win, pq, dss);
            if (fabs(dss) < (1.0e-4 * fabs(pq))) break;
            if (fabs(pq) < 1.0e-300) break;
        }
    }
    return pq;
}

// qromb_chi with the chi nodes of a level spread over the lanes of a warp:
// lane k evaluates node base + k, every lane adds the level's values in node
// order, so each lane returns qromb_chi's value bit for bit. Levels beyond the
// node table run on every lane in turn. All lanes call it with the same
// arguments.
__device__ inline double qromb_chi_warp(const Ctx &C, const ChiArgs &A, double cd, double sd) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const double a = 0.0, b = C.P->romb_chi_b;
    double win[5];
    double cur;
    int cnt;
    double pq = 0.0, dss = 0.0;
    {
        double v = 0.0;
        if (lane < 2) {
            const cs_chi_node n = C.chi[lane];
            v = chi_integrand(A, n.c, n.s, cd, sd);
        }
        const double pa = __shfl_sync(full, v, 0), pb = __shfl_sync(full, v, 1);
        cur = 0.5 * (b - a) * (pa + pb);
        cnt = 1;
    }
    win[4] = cur;
    for (int j = 2; j <= 20; j++) {
        const double tnm = cnt;
        const double del = (b - a) / tnm;
        double sump = 0.0;
        if (j <= CS_NODE_LEVELS) {
            const cs_chi_node *nd = C.chi + CS_NODE_OFFSET(j);
            for (int base = 0; base < cnt; base += 32) {
                double v = 0.0;
                if (base + lane < cnt) {
                    const cs_chi_node n = nd[base + lane];
                    v = chi_integrand(A, n.c, n.s, cd, sd);
                }
                const int m = (cnt - base) < 32 ? (cnt - base) : 32;
                for (int u = 0; u < m; u++) sump += __shfl_sync(full, v, u);
            }
        } else {
            double x = a + 0.5 * del;
            for (int k = 0; k < cnt; k++) {
                double s, c;
                sincos(x, &s, &c);
                sump += chi_integrand(A, c, s, cd, sd);
                x += del;
            }
        }
        cur = 0.5 * (cur + (b - a) * sump / tnm);
        cnt = 2 * cnt;
        win[0] = win[1];
        win[1] = win[2];
        win[2] = win[3];
        win[3] = win[4];
        win[4] = cur;
        if (j >= 5) {
            polint5(win, pq, dss);
            if (fabs(dss) < (1.0e-4 * fabs(pq))) break;
            if (fabs(pq) < 1.0e-300) break;
        }
    }
    return pq;
}

// qrombdeltac(i0 = 4 cylinder, 6 disk form factor): Gaussian-weighted delta
// integral of qrombchid (both cases weigh alike, :1051-1070, 1104-1120).
template <class Args>
__device__ inline double qromb_delta(const Ctx &C, const Args &A) {
    const cs_prepared &P = *C.P;
    const double a = 0.0, b = P.romb_delta_b;
    const double dbeta = P.romb_dbeta;
    double win[5];
    double cur;
    int cnt;
    double pq = 0.0, dss = 0.0;
    {
        const cs_delta_node n0 = C.dnode[0], n1 = C.dnode[1];
        double pa = qromb_chi(C, A, n0.c, n0.s);
        double pb = qromb_chi(C, A, n1.c, n1.s);
        pa = n0.w * pa / (2.0 * M_PI);
        pb = n1.w * pb / (2.0 * M_PI);
        cur = 0.5 * (b - a) * (pa + pb);
        cnt = 1;
    }
    win[4] = cur;
    for (int j = 2; j <= 20; j++) {
        const double tnm = cnt;
        const double del = (b - a) / tnm;
        double sump = 0.0;
        if (j <= CS_NODE_LEVELS) {
            const cs_delta_node *nd = C.dnode + CS_NODE_OFFSET(j);
            for (int k = 0; k < cnt; k++) {
                const cs_delta_node n = nd[k];
                double px = qromb_chi(C, A, n.c, n.s);
                px = n.w * px / (2.0 * M_PI);
                sump = sump + px;
            }
        } else {
            double x = a + 0.5 * del;
            for (int k = 0; k < cnt; k++) {
                double s, c;
                sincos(x, &s, &c);
                double px = qromb_chi(C, A, c, s);
                px = s * exp(-x * x / (dbeta * dbeta)) * px / (2.0 * M_PI);
                sump = sump + px;
                x = x + del;
            }
        }
        cur = 0.5 * (cur + (b - a) * sump / tnm);
        cnt = 2 * cnt;
        win[0] = win[1];
        win[1] = win[2];
        win[2] = win[3];
        win[3] = win[4];
        win[4] = cur;
        if (j >= 5) {
            polint5(win, pq, dss);
            if (fabs(dss) < (1.0e-4 * fabs(pq))) break;
            if (fabs(pq) < 1.0e-100) break;
        }
    }
    return pq;
}

// i0 = 4. Orientation cases outside 1..4 (the 0-based general case) reach no
// branch of the chi integrand, which is then 0 at every node: every trapezoid
// estimate is +0, the Neville extrapolation gives +0, and the reference's loop
// stops at j = 5 on |I| < 1e-100 with +0. That value is returned directly.
__device__ inline double qromb_delta_cyl(const Ctx &C, const ChiArgs &A) {
    if (A.i1 < 1 || A.i1 > 4) return 0.0;
    return qromb_delta(C, A);
}

// The same integral with the delta nodes of a level spread over the lanes of a
// warp: lane k computes node base + k (its chi integral and weighting exactly
// as above), and every lane then adds the level's values in node order, so
// each lane returns qromb_delta_cyl's value bit for bit. A pixel's latency
// falls from one chi integral per node to about one per level. Levels beyond
// the node table (never reached in practice) run on every lane in turn. All
// lanes of the warp call it with the same arguments.
__device__ inline double qromb_delta_cyl_warp(const Ctx &C, const ChiArgs &A) {
    if (A.i1 < 1 || A.i1 > 4) return 0.0;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const cs_prepared &P = *C.P;
    const double a = 0.0, b = P.romb_delta_b;
    const double dbeta = P.romb_dbeta;
    double win[5];
    double cur;
    int cnt;
    double pq = 0.0, dss = 0.0;
    {
        double v = 0.0;
        if (lane < 2) {
            const cs_delta_node n = C.dnode[lane];
            v = qromb_chi(C, A, n.c, n.s);
            v = n.w * v / (2.0 * M_PI);
        }
        const double pa = __shfl_sync(full, v, 0), pb = __shfl_sync(full, v, 1);
        cur = 0.5 * (b - a) * (pa + pb);
        cnt = 1;
    }
    win[4] = cur;
    for (int j = 2; j <= 20; j++) {
        const double tnm = cnt;
        const double del = (b - a) / tnm;
        double sump = 0.0;
        if (j <= CS_NODE_LEVELS) {
            const cs_delta_node *nd = C.dnode + CS_NODE_OFFSET(j);
            for (int base = 0; base < cnt; base += 32) {
                double px = 0.0;
                if (base + lane < cnt) {
                    const cs_delta_node n = nd[base + lane];
                    px = qromb_chi(C, A, n.c, n.s);
                    px = n.w * px / (2.0 * M_PI);
                }
                const int m = (cnt - base) < 32 ? (cnt - base) : 32;
                for (int u = 0; u < m; u++) sump = sump + __shfl_sync(full, px, u);
            }
        } else {
            double x = a + 0.5 * del;
            for (int k = 0; k < cnt; k++) {
                double s, c;
                sincos(x, &s, &c);
                double px = qromb_chi(C, A, c, s);
                px = s * exp(-x * x / (dbeta * dbeta)) * px / (2.0 * M_PI);
                sump = sump + px;
                x = x + del;
            }
        }
        cur = 0.5 * (cur + (b - a) * sump / tnm);
        cnt = 2 * cnt;
        win[0] = win[1];
        win[1] = win[2];
        win[2] = win[3];
        win[3] = win[4];
        win[4] = cur;
        if (j >= 5) {
            polint5(win, pq, dss);
            if (fabs(dss) < (1.0e-4 * fabs(pq))) break;
            if (fabs(pq) < 1.0e-100) break;
        }
    }
    return pq;
}

__device__ __forceinline__ ChiArgs chi_args(const cs_prepared &P, double qxs, double qys, double sigma, int i1) {
    ChiArgs A;
    A.qx = qxs;
    A.qy = qys;
    A.l = P.length;
    A.z = (1 - sigma * sigma) / (sigma * sigma);
    A.zp1 = A.z + 1;
    A.a1 = 1 / (2.0 * A.z * (A.z - 1));
    A.zm1 = A.z - 1;
    A.zm1h = (A.z - 1) / 2.0;
    A.p11 = P.romb_p[0];
    A.p12 = P.romb_p[1];
    A.p13 = P.romb_p[2];
    A.p21 = P.romb_p[3];
    A.p22 = P.romb_p[4];
    A.p23 = P.romb_p[5];
    A.i1 = i1;
    return A;
}

// ---------------------------------------------------------------- cylinders
// double series of the general orientation (ordis 0, q < 0.4 limq1); the
// power tables qxn/qyn live in local memory as in the reference.
__device__ inline double cyl_double_series(const cs_prepared &P, double qxs, double qys, const double *__restrict__ carr1,
                                    int variant) {
    double pql = 1.0;
    double oldpqsum = 0.0;
    double qxn[121], qyn[121];
    qxn[0] = 1.0;
    qyn[0] = 1.0;
    for (int nser = 1; nser <= 120; nser++) {
        qxn[nser] = __dmul_rn(__dmul_rn(qxn[nser - 1], qxs), qxs);
        qyn[nser] = __dmul_rn(__dmul_rn(qyn[nser - 1], qys), qys);
        double binsum = 0.0;
        // binsum += c * a * b, rounded as ((c*a)*b) then the sum
        if (variant == 0) {
            for (int mser = 0; mser <= nser; mser++)
                binsum = __dadd_rn(binsum, __dmul_rn(__dmul_rn(P.carr11pm[nser - mser][mser], qxn[mser]), qyn[nser - mser]));
        } else if (variant == 1) {
            for (int mser = 0; mser <= nser; mser++)
                binsum = __dadd_rn(binsum, __dmul_rn(__dmul_rn(P.carr11pm[nser - mser][mser], qyn[mser]), qxn[nser - mser]));
        } else if (variant == 2) {
            for (int mser = 0; mser <= nser; mser++)
                binsum = __dadd_rn(binsum, __dmul_rn(__dmul_rn(P.carr11pm[mser][nser - mser], qyn[mser]), qxn[nser - mser]));
        } else {
            for (int mser = 0; mser <= nser; mser++)
                binsum = __dadd_rn(binsum, __dmul_rn(__dmul_rn(P.carr11pm[mser][nser - mser], qxn[mser]), qyn[nser - mser]));
        }
        pql = __dadd_rn(pql, __dmul_rn(carr1[nser], binsum));
        if (series_converged(pql, oldpqsum)) break;
        oldpqsum = pql;
    }
    return pql;
}

// Length factor of the z-direction cylinder in the reference's closed form
// (formpq/formfq_partCylinder ordis 6, Source/sc_lib_formpq_partCylinder.h:115-119).
__device__ __forceinline__ double len_factor_ref(double arglq, double zl) {
    return (1 / (2.0 * zl * (zl - 1))) * (1 / (arglq * arglq)) *
           (1 - cos((zl - 1) * atan(2.0 * arglq)) / pow(1.0 + 4 * arglq * arglq, (zl - 1) / 2.0));
}

// The same with its small-argument series where the closed form cancels
// (see len_factor_small above): the closed form's exact value everywhere.
__device__ __forceinline__ double len_factor(double arglq, double zl) {
    if (len_factor_small(arglq, zl - 1)) return len_factor_series(arglq, zl - 1);
    return len_factor_ref(arglq, zl);
}

// Isotropic orientation average of the cylinder's length factor
// (formpq_partCylinder ordis 7, Source/sc_lib_formpq_partCylinder.h:29-90):
// short cylinders (L/R < 2) take the exact average as a double series in q^2
// (carr11pm, carr2p) or the Porod tail; longer ones its factorised form, a
// series in q^2 (carr1p) or the closed form
//   (pi/(2z)) / a - cos((z-1) atan 2a) / (2z(z-1) a^2 (1+4a^2)^((z-1)/2)).
__device__ inline double cyl_len_iso(const cs_prepared &P, double q, double zl) {
    if ((P.length / P.radius) < 2) {
        if (q < (5 * P.limq[2])) {
            double qqn[101];
            qqn[0] = 1.0;
            for (int nser = 1; nser <= 100; nser++) qqn[nser] = qqn[nser - 1] * q * q;
            double pql = 0.0, oldpqsum = -10.0;
            for (int nser = 0; nser <= 100; nser++) {
                double binsum = 0.0;
                for (int mser = 0; mser <= 100; mser++) binsum += P.carr11pm[nser][mser] * qqn[mser];
                pql += P.carrp[1][nser] * qqn[nser] * binsum;
                const double delser = fabs((pql - oldpqsum) / pql);
                if (delser < 0.0001) break;
                oldpqsum = pql;
            }
            return pql;
        }
        return P.por / pow(q, 4);
    }
    if (q < (0.6 * P.limq[1])) return series_q(P.carrp[0], q, 120);
    const double arglq = q * P.length / (zl + 1);
    double pql = (M_PI / (2.0 * zl)) * (1 / arglq);
    pql = pql - (1 / (2.0 * zl * (zl - 1) * arglq * arglq)) * cos((zl - 1) * atan(2.0 * arglq)) /
                    pow(1.0 + 4 * arglq * arglq, (zl - 1) / 2.0);
    return pql;
}

// The Schulz cylinder cross-section's closed form shared by the terms below:
// (4/pi)(T1 - T2 - (9/8) T3) at argument x (Source/sc_lib_formpq_partCylinder.h:272-275)
__device__ __forceinline__ double cyl_cross_closed(double x, double zr) {
    const double pqr1 = (1 / (zr * (zr - 1) * (zr - 2))) * pow(x, -3);
    const double pqr2 = (1 / (zr * (zr - 1) * (zr - 2))) * pow(x, -3) * sin((zr - 2) * atan(2.0 * x)) /
                        pow(1.0 + 4 * x * x, (zr - 2) / 2.0);
    const double pqr3 = (1 / (zr * (zr - 1) * (zr - 2) * (zr - 3))) * pow(x, -4) * cos((zr - 3) * atan(2.0 * x)) /
                        pow(1.0 + 4 * x * x, (zr - 3) / 2.0);
    return (4 / M_PI) * (pqr1 - pqr2 - (9 / 8.0) * pqr3);
}

// Cross-section of the homogeneous core/shell cylinder, F121 + F122 + F123
// (Source/sc_lib_formpq_partCylinder.h:284-393): core, cross and shell
// terms, each a series (carr4p/5p/6p) below its switch point or its closed form.
__device__ inline double cyl_cross_coreshell(const cs_prepared &P, double q, double zr) {
    const double radiusm = P.radius / P.p1;
    const double zz = zr;
    const double ccc1 = sqr(1 - P.rho) * pow(P.p1, 4);
    const double ccc2 = 2 * P.rho * (1 - P.rho) * pow(P.p1, 2);
    const double ccc3 = P.rho * P.rho;
    const double vv3 = sqr((1 - P.rho) * pow(P.p1, 2) + P.rho);
    const double argq = q * radiusm / (zz + 1);
    const double argpq = q * P.radius / (zz + 1);
    double F121, F122, F123;
    if (q < (0.7 * P.limq[4]))
        F121 = ccc1 * series_q(P.carrp[3], q, 120) / vv3;
    else
        F121 = ccc1 * cyl_cross_closed(argpq, zr) / vv3;
    if (q < (1.5 * P.limq[5])) {
        F122 = ccc2 * series_q(P.carrp[4], q, 120) / vv3;
    } else {
        const double argbm = (zr - 2) * atan(argpq - argq);
        const double nenbm = pow(1.0 + sqr(argpq - argq), (zr - 2) / 2.0);
        const double argbp = (zr - 2) * atan(argpq + argq);
        const double nenbp = pow(1.0 + sqr(argpq + argq), (zr - 2) / 2.0);
        const double argem = (zr - 3) * atan(argpq - argq);
        const double nenem = pow(1.0 + sqr(argpq - argq), (zr - 3) / 2.0);
        const double argep = (zr - 3) * atan(argpq + argq);
        const double nenep = pow(1.0 + sqr(argpq + argq), (zr - 3) / 2.0);
        const double arggm = (zr - 4) * atan(argpq - argq);
        const double nengm = pow(1.0 + sqr(argpq - argq), (zr - 4) / 2.0);
        const double arggp = (zr - 4) * atan(argpq + argq);
        const double nengp = pow(1.0 + sqr(argpq + argq), (zr - 4) / 2.0);
        const double pqr1 = (1 / (zr * (zr - 1) * (zr - 2))) * pow(argq, -3) * (cos(argbm) / nenbm - sin(argbp) / nenbp);
        const double pqr2 = (1 / (zr * (zr - 1) * (zr - 2) * (zr - 3))) * pow(argq, -4) *
                            ((1 - 1 / P.p1) * sin(argem) / nenem - (1 + 1 / P.p1) * cos(argep) / nenep);
        const double pqr3 = (1 / (zr * (zr - 1) * (zr - 2) * (zr - 3) * (zr - 4))) * pow(argq, -5) * (1 / P.p1) *
                            (cos(arggm) / nengm - sin(arggp) / nengp);
        const double pqr = (4 / M_PI) * pow(P.p1, -3 / 2.0) * (pqr1 + (9 / 16.0) * pqr2 + (9 / 16.0) * (9 / 16.0) * pqr3);
        F122 = ccc2 * pqr / vv3;
    }
    if (q < (0.6 * P.limq[6]))
        F123 = ccc3 * series_q(P.carrp[5], q, 120) / vv3;
    else
        F123 = ccc3 * cyl_cross_closed(argq, zr) / vv3;
    return F121 + F122 + F123;
}

template <bool WARP = false>
__device__ inline double formpq_cylinder(const Ctx &C, double qxs, double qys, double q) {
    const cs_prepared &P = *C.P;
    double pqr = 0, pql = 0;
    // Schulz exponents, formed on the branches that use them
    auto zl_of = [&P]() { return P.sigmal == 1.0 ? CS_EPS9 : (1 - sqr(P.sigmal)) / sqr(P.sigmal); };
    auto zr_of = [&P]() { return P.sigma == 1.0 ? CS_EPS9 : (1 - sqr(P.sigma)) / (sqr(P.sigma)); };
    if (P.ordis == 7) pql = cyl_len_iso(P, q, zl_of());
    if (P.ordis == 6) {
        if (P.orcase == 4)
            pql = 1.0;
        else {
            if (q < (0.6 * P.limq[1])) {
                pql = series_zdir(P.carrp[0], qxs, qys);
            } else {
                const double zl = zl_of();
                const double arglq = (qxs + qys + CS_EPS9) * P.length / (zl + 1);
                pql = len_factor(arglq, zl);
            }
        }
    }
    if (P.ordis == 0) {
        if (P.orcase == 4)
            pql = 1.0;
        else {
            if (q < (0.4 * P.limq[1])) {
                pql = 1.0;
                // orcase 1 and 2 share one formula, orcase 3 swaps x and y, orcase 0 adds nothing
                if (P.orcase == 1 || P.orcase == 2)
                    pql = cyl_double_series(P, qxs, qys, P.carrp[0], 0);
                else if (P.orcase == 3)
                    pql = cyl_double_series(P, qxs, qys, P.carrp[0], 1);
            } else if (P.orcase < 1 || P.orcase > 4) {
                // the quadrature of trapzdchid's identically zero integrand
                // (no case for the general orientation) is +0, which
                // qromb_delta_cyl returns without evaluating it
                pql = 0.0 / P.norm;
            } else {
                const ChiArgs A = chi_args(P, qxs, qys, P.sigmal, P.orcase);
                pql = WARP ? qromb_delta_cyl_warp(C, A) : qromb_delta_cyl(C, A);
                pql = pql / P.norm;
            }
        }
    }
    if (P.cs == 0) {
        if ((P.length / P.radius) < 2)
            pqr = 1;
        else {
            // Without a lattice, a zero length factor times a finite radial
            // factor is a zero whose sign cannot change the pixel's value
            // (with a lattice it would decide the sign of F/P): the radial
            // factor is not formed where it is known to be finite, on the
            // series side of the switch (a converged sum of finite terms near
            // 1) and on the closed-form side when zr > 3 and the argument is
            // not tiny (finite Gamma-ratio prefactors, powers of 1 + 4x^2 >= 1
            // with positive exponents), both read off sigma without a division.
            const bool zero_len = (pql == 0.0) && !P.lattice;
            if (q < (0.65 * P.limq[4])) {
                if (zero_len) return 0.0;
                pqr = series_q(P.carrp[3], q, 120);
            } else {
                // zr > 3.16 for sigma < 0.49; argpq = q R sigma^2 to rounding
                if (zero_len && P.sigma > 0 && P.sigma < 0.49 && q * P.radius * P.sigma * P.sigma > 1e-28) return 0.0;
                const double zr = zr_of();
                const double argpq = q * P.radius / (zr + 1);
                const double pqr1 = (1 / (zr * (zr - 1) * (zr - 2))) * pow(argpq, -3);
                const double pqr2 = (1 / (zr * (zr - 1) * (zr - 2))) * pow(argpq, -3) * sin((zr - 2) * atan(2.0 * argpq)) /
                                    pow(1.0 + 4 * argpq * argpq, (zr - 2) / 2.0);
                const double pqr3 = (1 / (zr * (zr - 1) * (zr - 2) * (zr - 3))) * pow(argpq, -4) *
                                    cos((zr - 3) * atan(2.0 * argpq)) / pow(1.0 + 4 * argpq * argpq, (zr - 3) / 2.0);
                pqr = (4. / M_PI) * (pqr1 - pqr2 - (9. / 8.0) * pqr3);
            }
        }
        return pql * pqr;
    }
    if (P.cs == 1) return pql * cyl_cross_coreshell(P, q, zr_of());
    return 0.0;
}

__device__ inline double formfq_cylinder(const Ctx &C, double limql, double qxs, double qys, double q) {
    const cs_prepared &P = *C.P;
    const double zl = (1 - sqr(P.sigmal)) / sqr(P.sigmal);
    const double zr = (1 - sqr(P.sigma)) / sqr(P.sigma);
    double pql = 0, pqr = 0;
    if (P.ordis == 7) {
        // isotropic (Source/sc_lib_formfq_partCylinder.h:27-48)
        if (q < (0.6 * P.limqf[1])) {
            pql = series_q(P.carrf[0], q, 120);
        } else {
            const double arglq = q * P.length / (zl + 1);
            pql = (M_PI / (2.0 * zl)) * (1 / arglq);
            pql = pql - (1 / (2.0 * zl * (zl - 1) * arglq * arglq)) * cos((zl - 1) * atan(2.0 * arglq)) /
                            pow(1.0 + 4 * arglq * arglq, (zl - 1) / 2.0);
        }
    }
    if (P.ordis == 6) {
        if (P.orcase == 4)
            pql = 1.0;
        else {
            if (limql < (0.6 * P.limqf[1])) {
                pql = series_zdir(P.carrf[0], qxs, qys);
            } else {
                const double arglq = (qxs + qys + CS_EPS9) * P.length / (zl + 1);
                pql = len_factor(arglq, zl);
            }
        }
    }
    if (P.ordis == 0) {
        if (P.orcase == 4)
            pql = 1.0;
        else {
            if (limql < (0.2 * P.limqf[1])) {
                double pqsum = 1.0;
                if (P.orcase == 1)
                    pqsum = cyl_double_series(P, qxs, qys, P.carrf[0], 2);
                if (P.orcase == 2)
                    pqsum = cyl_double_series(P, qxs, qys, P.carrf[0], 0);
                if (P.orcase == 3)
                    pqsum = cyl_double_series(P, qxs, qys, P.carrf[0], 3);
                pql = pqsum;
            } else {
                const ChiArgs A = chi_args(P, qxs, qys, P.sigmal, P.orcase);
                pql = qromb_delta_cyl(C, A);
                pql = pql / P.norm;
            }
        }
    }
    if (P.cs == 0) {
        if (q < (1.0 * P.limqf[4])) {
            pqr = series_q(P.carrf[3], q, 120);
        } else {
            const double argpq = q * P.radius / (zr + 1);
            const double pqr1 = P.gamma_ratio[0] * pow(argpq, -3 / 2.0) *
                                (sin((zr - 1 / 2.0) * atan(argpq)) - cos((zr - 1 / 2.0) * atan(argpq))) /
                                pow(1.0 + argpq * argpq, (zr - 1 / 2.0) / 2.0);
            const double pqr2 = P.gamma_ratio[1] * pow(argpq, -5 / 2.0) *
                                (sin((zr - 3 / 2.0) * atan(argpq)) + cos((zr - 3 / 2.0) * atan(argpq))) /
                                pow(1.0 + argpq * argpq, (zr - 3 / 2.0) / 2.0);
            const double pqr3 = (2 / sqrt(M_PI)) * (pqr1 + (9 / 16.0) * pqr2);
            pqr = pqr3 * pqr3;
        }
        return pql * pqr;
    }
    if (P.cs == 1) {
        // homogeneous core/shell cylinder, Source/sc_lib_formfq_partCylinder.h:211-302;
        // the amplitude closed form A(x) = (2/sqrt pi)(T1 + (9/16) T2) with the
        // prepared Gamma ratios (as for cs 0)
        const double radiusm = P.radius / P.p1;
        const double ccc1 = sqr(1 - P.rho) * pow(P.p1, 4);
        const double ccc2 = 2 * P.rho * (1 - P.rho) * pow(P.p1, 2);
        const double ccc3 = sqr(P.rho);
        const double vv3 = sqr((1 - P.rho) * pow(P.p1, 2) + P.rho);
        const double zz = zr;
        const double argq = q * radiusm / (zz + 1);
        const double argpq = q * P.radius / (zz + 1);
        // T1, T2 of the amplitude at x, with the power's base 1 + x y (y = x
        // except where the reference multiplies argpq by argq, kept)
        auto t1 = [&](double x, double y) {
            return P.gamma_ratio[0] * pow(x, -3 / 2.0) * (sin((zr - 1 / 2.0) * atan(x)) - cos((zr - 1 / 2.0) * atan(x))) /
                   pow(1.0 + x * y, (zr - 1 / 2.0) / 2.0);
        };
        auto t2 = [&](double x, double y) {
            return P.gamma_ratio[1] * pow(x, -5 / 2.0) * (sin((zr - 3 / 2.0) * atan(x)) + cos((zr - 3 / 2.0) * atan(x))) /
                   pow(1.0 + x * y, (zr - 3 / 2.0) / 2.0);
        };
        double F121, F122, F123;
        if (q < (0.7 * P.limqf[4])) {
            F121 = ccc1 * series_q(P.carrf[3], q, 120) / vv3;
        } else {
            const double a = (2 / sqrt(M_PI)) * (t1(argpq, argpq) + (9 / 16.0) * t2(argpq, argpq));
            F121 = ccc1 * a * a / vv3;
        }
        if (q < (0.3 * P.limqf[5])) {
            F122 = ccc2 * series_q(P.carrf[4], q, 120) / vv3;
        } else {
            const double pqr = (4 / M_PI) * (t1(argpq, argq) + (9 / 16.0) * t2(argpq, argq)) *
                               (t1(argq, argq) + (9 / 16.0) * t2(argq, argq));
            F122 = ccc2 * pqr / vv3;
        }
        if (q < (0.6 * P.limqf[6])) {
            F123 = ccc3 * series_q(P.carrf[5], q, 120) / vv3;
        } else {
            const double a = (2 / sqrt(M_PI)) * (t1(argq, argq) + (9 / 16.0) * t2(argq, argq));
            F123 = ccc3 * a * a / vv3;
        }
        return pql * (F121 + F122 + F123);
    }
    return 0.0;
}

// calc_partSphere_lattNone_ordisIsotropic, Source/sc_gpu_pSph_lNon_oIso.h:15-51
__device__ inline double calc_sphere_none_iso(const Ctx &C, double qx, double qy, double qz) {
    const cs_prepared &P = *C.P;
    const double q = sqrt(qx * qx + qy * qy + qz * qz) + CS_EPS9;
    const double pq = formpq_sphere(P, q);
    return P.base + P.izero * (pq + P.iso * pq) + P.ifluc / (1 + q * q * P.rfluc * P.rfluc);
}

// Peak sums shared by the FCC and BCT kernels
// (Source/sc_gpu_pSph_pGau_lFCC_oGau.h:53-143, sc_gpu_pCyl_pGau_lBCT_oZDi.h:133-211).
// exp(-4 x2/pi) is exactly +0 for x2 above ~585 (its argument below the
// smallest subnormal's log, -744.4): such peak terms add exactly nothing
constexpr double kPeakZero = 600.0;

__device__ inline void peak_sums(const cs_prepared &P, double qx, double qy, double qz, double q, double &radintensity,
                          double &intensity) {
    double width = 1;
    if (P.debyescherrer) width = 4.0 / P.domainsize;
    if (P.para) width = (4.0 / P.domainsize) + sqr(P.reldis) * P.dist * sqr(q);
    width *= P.width_zuf;
    const double widthiso = 1.0 / P.uca;
    radintensity = 0.0;
    intensity = 0.0;
    // Far from a reflection its term is exactly +0 (x2 beyond kPeakZero).
    // That is settled first without the division: (q - qhkl)^2 above
    // kPeakZero width^2 (1 + 1e-12) puts x2 beyond kPeakZero whatever the
    // division's rounding; only the reflections nearer than that form x2 as
    // the reference does.
    const double far_iso = kPeakZero * sqr(widthiso) * (1 + 1e-12);
    const double far_aniso = kPeakZero * (width * width) * (1 + 1e-12);
    for (int ii = 1; ii <= P.peakmax1; ii++) {
        const int mhkl = P.latpar1[ii][4];
        const int fhkl = P.latpar1[ii][5];
        if (mhkl == 0 || fhkl == 0) continue;
        const double qhkl = P.latpar3[ii][5];
        if (sqr(q - qhkl) > far_iso) continue;  // the term is exactly +0
        const double x2 = sqr(q - qhkl) / sqr(widthiso);
        if (x2 > kPeakZero) continue;  // the term is exactly +0
        const double sq = exp(-4 * x2 / M_PI) / (M_PI * widthiso / 2.0);
        radintensity += sq * mhkl * fhkl;
    }
    const double x2phi = 4 * q * q / (M_PI * sqr(P.phiwidth));
    for (int ii = 1; ii <= P.peakmax2; ii++) {
        const double qhkl = P.latpar3[ii][5];
        const int mhkl_fhkl = P.latpar2[ii][4] * P.latpar2[ii][5];
        if (qhkl > 0 && mhkl_fhkl != 0) {
            if ((q - qhkl) * (q - qhkl) > far_aniso && !P.twin) {
                // radial Gaussian exactly +0: skipped when the angular factor
                // is finite (as below), without forming x2
                const double g3 = P.latpar3[ii][10], pn = P.latpar3[ii][11];
                if (isfinite(g3) && isfinite(pn) && pn != 0) continue;
            }
            const double qxhkl = P.latpar3[ii][2];
            const double qyhkl = P.latpar3[ii][3];
            const double qzhkl = P.latpar3[ii][4];
            const double g3 = P.latpar3[ii][10];
            const double peaknorm1 = P.latpar3[ii][11];
            const double x2 = (q - qhkl) * (q - qhkl) / (width * width);
            // a term whose radial Gaussian underflows is exactly +0 when its
            // angular factor is finite: skipped (same sum, bit for bit)
            if (x2 > kPeakZero && !P.twin && isfinite(g3) && isfinite(peaknorm1) && peaknorm1 != 0) continue;
            const double yphi = myacos((qx * qxhkl + qy * qyhkl + qz * qzhkl) / (q * qhkl));
            const double sq = exp(-4 * x2 / M_PI) / (M_PI * width / 2.0);
            double psiord = g3 * exp(-x2phi * yphi * yphi) / peaknorm1;
            if (P.twin) {
                const double qxhklt = P.latpar3[ii][7];
                const double qyhklt = P.latpar3[ii][8];
                const double qzhklt = P.latpar3[ii][9];
                const double qhklt = P.latpar3[ii][14];
                const double g3t = P.latpar3[ii][15];
                const double peaknorm1t = P.latpar3[ii][16];
                const double yphit = myacos((qx * qxhklt + qy * qyhklt + qz * qzhklt) / (q * qhklt));
                const double phiord = g3t * exp(-x2phi * yphit * yphit) / peaknorm1t;
                psiord = P.ceff * psiord + (1 - P.ceff) * phiord;
            }
            const double savintens = intensity;
            intensity += sq * mhkl_fhkl * psiord;
            if (isinf(intensity)) {
                intensity = savintens;
                break;
            }
        }
    }
}

// calc_partSphere_peakGauss_lattFCC_ordisGauss, Source/sc_gpu_pSph_pGau_lFCC_oGau.h:15-171
// Lattice factors near q = 0. The reference forms
//   szq    = 1 + (F/P) (r1 - 1) e1,   r1 = 2 pi I_aniso / V,  e1 = exp(-dw q^2),
//   szqiso = 1 + (r2 - 1) e2,         r2 = 8 pi^3 I_iso / (4 pi V), e2 = exp(-ucb q^2),
// which cancel as q -> 0 (F/P, e1, e2 -> 1, no reflection near): their exact
// values are O(q^2), while the FP64 forms round to 0 or to noise of ~1e-16
// (at the beam-centre pixel, q = 1e-9, the reference returns 0 where the
// exact value is ~1e-18). Below q = 1e-6 the form factors are their one-term
// series, P = 1 + cp q^2, F = 1 + cf q^2 (per factor; the stop rule ends each
// series after that term), so the factors are formed from the difference
//   1 - (F/P) e1 = ((P - F) + F (1 - e1)) / P,  1 - e1 = -expm1(-dw q^2),
// with P - F from the series coefficients: the exact values to rounding.
#define CS_SMALL_Q 1e-6

__device__ __forceinline__ void lattice_factors_small_q(const cs_prepared &P, double q, double pq, double fq,
                                                        double p_minus_f, double intensity, double radintensity,
                                                        double &szq, double &szqiso) {
    const double sphno_cubevol = P.latpar[1] * P.latpar[2];
    const double r1 = 2 * M_PI * intensity / sphno_cubevol;
    const double r2 = 8 * M_PI * M_PI * M_PI * radintensity / (4 * M_PI * sphno_cubevol);
    const double om1 = -expm1(-P.dwfactor * q * q), om2 = -expm1(-P.ucb * q * q);
    szq = (p_minus_f + fq * om1) / pq + (fq / pq) * r1 * (1 - om1);
    szqiso = om2 + r2 * (1 - om2);
}

__device__ inline double calc_sphere_fcc(const Ctx &C, double qx, double qy, double qz) {
    const cs_prepared &P = *C.P;
    const double q = sqrt(qx * qx + qy * qy + qz * qz) + CS_EPS9;
    const double pq = formpq_sphere(P, q);
    const double fq = formfq_sphere(P, q);
    const double pqiso = pq;
    double radintensity, intensity;
    peak_sums(P, qx, qy, qz, q, radintensity, intensity);
    const double sphno_cubevol = P.latpar[1] * P.latpar[2];
    const double szqiso = (1 + (1) * (8 * M_PI * M_PI * M_PI * radintensity / (4 * M_PI * sphno_cubevol) - 1) *
                                   exp(-P.ucb * q * q));
    double szq = (1 + (fq / pq) * (2 * M_PI * intensity / sphno_cubevol - 1) * exp(-P.dwfactor * q * q));
    if (q < CS_SMALL_Q && P.cs == 0) {
        // homogeneous spheres: P and F are series in q^2 (carr4p, carr4f)
        double szi;
        const double q2 = q * q;
        lattice_factors_small_q(P, q, pq, fq, (P.carrp[3][1] - P.carrf[3][1]) * q2 + (P.carrp[3][2] - P.carrf[3][2]) * q2 * q2,
                                intensity, radintensity, szq, szi);
        return P.base + P.izero * (szq * pq + P.iso * szi * pqiso) + P.ifluc / (1 + q * q * P.rfluc * P.rfluc);
    }
    return P.base + P.izero * (szq * pq + P.iso * szqiso * pqiso) + P.ifluc / (1 + q * q * P.rfluc * P.rfluc);
}

// calc_partCylinder_lattNone_ordisGauss, Source/sc_gpu_pCyl_lNon_oGau.h:15-100
// (the lattice branch for F(q) is not taken: lattice is "None").
// (WARP: the orientation average's delta nodes spread over a warp, for the
// FP64 redo of single pixels; same value)
template <bool WARP = false>
__device__ inline double calc_cyl_none_gauss(const Ctx &C, double qx, double qy, double qz) {
    const cs_prepared &P = *C.P;
    double pq = 0;
    const double q = sqrt(qx * qx + qy * qy + qz * qz) + CS_EPS9;
    switch (P.orcase) {
    case CS_ORC_GENERAL:
        pq = formpq_cylinder<WARP>(C, qx * P.cosphic - qy * P.sinphic, qx * P.sinphic + qy * P.cosphic, q);
        break;
    case CS_ORC_XAXIS:
    case CS_ORC_YAXIS:
    case CS_ORC_ZAXIS:
        pq = formpq_cylinder<WARP>(C, qx, qy, q);
        break;
    }
    return P.base + P.izero * (pq + P.iso) + P.ifluc / (1 + q * q * P.rfluc * P.rfluc);
}

// calc_partCylinder_lattNone_ordisZDir, Source/sc_gpu_pCyl_lNon_oZDi.h:17-88
__device__ inline double calc_cyl_none_zdir(const Ctx &C, double qx, double qy, double qz) {
    const cs_prepared &P = *C.P;
    double pq = 0;
    const double q = sqrt(qx * qx + qy * qy + qz * qz) + CS_EPS9;
    switch (P.orcase) {
    case CS_ORC_GENERAL: pq = formpq_cylinder(C, qx * P.cosphi * P.sintheta, qy * P.sinphi * P.sintheta, q); break;
    case CS_ORC_XAXIS: pq = formpq_cylinder(C, qx, 0, q); break;
    case CS_ORC_YAXIS: pq = formpq_cylinder(C, 0, qy, q); break;
    case CS_ORC_ZAXIS: pq = formpq_cylinder(C, qx, qy, q); break;
    }
    return P.base + P.izero * (pq + P.iso) + P.ifluc / (1 + q * q * P.rfluc * P.rfluc);
}

// calc_partCylinder_peakGauss_lattBCT_ordisZDir, Source/sc_gpu_pCyl_pGau_lBCT_oZDi.h:16-245
__device__ inline double calc_cyl_bct_zdir(const Ctx &C, double qx, double qy, double qz) {
    const cs_prepared &P = *C.P;
    double pq = 0, fq = 0;
    const double q = sqrt(qx * qx + qy * qy + qz * qz) + CS_EPS9;
    const double pqiso = 1;
    switch (P.orcase) {
    case CS_ORC_GENERAL:
        pq = formpq_cylinder(C, qx * P.cosphi * P.sintheta, qy * P.sinphi * P.sintheta, q);
        fq = formfq_cylinder(C, sqrt(P.cosphi * qx * qx + P.sinphi * qy * qy + CS_EPS9), qx * P.cosphi * P.sintheta,
                             qy * P.sinphi * P.sintheta, q);
        break;
    case CS_ORC_XAXIS:
        pq = formpq_cylinder(C, qx, 0, q);
        fq = formfq_cylinder(C, fabs(qx), qx, 0, q);
        break;
    case CS_ORC_YAXIS:
        pq = formpq_cylinder(C, 0, qy, q);
        fq = formfq_cylinder(C, fabs(qy), 0, qy, q);
        break;
    case CS_ORC_ZAXIS:
        pq = formpq_cylinder(C, qx, qy, q);
        fq = formfq_cylinder(C, q, qx, qy, q);
        break;
    }
    double radintensity, intensity;
    peak_sums(P, qx, qy, qz, q, radintensity, intensity);
    const double sphno_cubevol = P.latpar[1] * P.latpar[2];
    const double szqiso = (1 + (1) * (8 * M_PI * M_PI * M_PI * radintensity / (4 * M_PI * sphno_cubevol) - 1) *
                                   exp(-P.ucb * q * q));
    double szq = (1 + (fq / pq) * (2 * M_PI * intensity / (sphno_cubevol)-1) * exp(-P.dwfactor * q * q));
    if (q < CS_SMALL_Q && P.cs == 0 && P.ordis == 6 && P.orcase != 4 && (P.length / P.radius) >= 2) {
        // P = Pl Pr and F = Fl Fr, each factor its one-term series: the length
        // series in s^2 (s = qxs + qys, carr1p/carr1f), the radial in q^2
        // (carr4p/carr4f); P - F = (Pl - Fl) Pr + Fl (Pr - Fr)
        double qxs = 0, qys = 0;
        switch (P.orcase) {
        case CS_ORC_GENERAL: qxs = qx * P.cosphi * P.sintheta; qys = qy * P.sinphi * P.sintheta; break;
        case CS_ORC_XAXIS: qxs = qx; break;
        case CS_ORC_YAXIS: qys = qy; break;
        default: qxs = qx; qys = qy; break;
        }
        const double s2 = (qxs + qys) * (qxs + qys), q2 = q * q;
        const double pl = 1 + P.carrp[0][1] * s2, fl = 1 + P.carrf[0][1] * s2;
        const double pr = 1 + P.carrp[3][1] * q2;
        const double pmf = (P.carrp[0][1] - P.carrf[0][1]) * s2 * pr + fl * (P.carrp[3][1] - P.carrf[3][1]) * q2;
        double szi;
        lattice_factors_small_q(P, q, pl * pr, fq, pmf, intensity, radintensity, szq, szi);
        return P.base + P.izero * (szq * pq + P.iso * szi * pqiso) + P.ifluc / (1 + q * q * P.rfluc * P.rfluc);
    }
    return P.base + P.izero * (szq * pq + P.iso * szqiso * pqiso) + P.ifluc / (1 + q * q * P.rfluc * P.rfluc);
}

// formpq_partCube, homogeneous isotropic cube (ordis 7, cs 0; the only cube
// case the preparation supports), Source/sc_lib_formpq_partCube.h:21-62
__device__ inline double formpq_cube(const cs_prepared &P, double q) {
    if (q < 1.2 * P.limq[4]) return series_q(P.carrp[3], q, 120);
    return P.por / (q * q * q * q);
}

// One term of polyvesicle: the averaged sin²/sincos/cos² moment of a
// Schulz-distributed size, cos or sin of zm·atan(2y) over (1+4y²)^(zm/2),
// with the exponent zm = z - k + 1 formed by the caller.
__device__ inline double vesicle_moment(double zm, double y, bool use_sin) {
    const double a = zm * atan(2. * y);
    const double t = use_sin ? sin(a) : cos(a);
    return t / exp(zm * log(1. + 4. * y * y) / 2.);
}

// polyvesicle, Schulz-polydisperse hollow shell between radius (inner) and
// length (outer) with polydispersities sigma (radius) and sigmal (thickness),
// Source/sc_calc_generic_gpu.cu:698-727
__device__ inline double polyvesicle(const cs_prepared &P, double q) {
    const double r = (P.length + P.radius) / 2.;
    if (q * r < 0.001) return 1;
    const double d = (P.length - P.radius) / 2.;
    const double zr = (1. - sqr(P.sigma)) / sqr(P.sigma);
    const double zd = (1. - sqr(P.sigmal)) / sqr(P.sigmal);
    const double yr = q * r / (zr + 1.);
    const double yd = q * d / (zd + 1.);
    const double c = 1. + d * d / (12. * r * r);
    const double gr1 = 1. / (2. * zr * (zr - 1.) * yr * yr);
    const double gr2 = gr1 / ((zr - 2.) * yr);
    const double gr3 = gr2 / ((zr - 3.) * yr);
    const double gd1 = 1. / (2. * zd * (zd - 1.) * yd * yd);
    const double gd2 = 1. / (2. * zd * yd);
    const double gd3 = 1. / 2.;
    const double hr1 = gr1 * (1. - vesicle_moment(zr - 2. + 1., yr, false));
    const double hr2 = gr2 * vesicle_moment(zr - 3. + 1., yr, true);
    const double hr3 = gr3 * (1. + vesicle_moment(zr - 4. + 1., yr, false));
    const double hd1 = gd1 * (1. - vesicle_moment(zd - 2. + 1., yd, false));
    const double hd2 = gd2 * vesicle_moment(zd - 1. + 1., yd, true);
    const double hd3 = gd3 * (1. + vesicle_moment(zd + 0. + 1., yd, false));
    return (hr1 * hd1 - 2. * hr2 * hd2 + 2. * hr2 * hd1 + hr3 * hd3 - 2. * hr3 * hd2 + hr3 * hd1) / (c * c);
}

// Integrand of trapzdchid for the isotropic biaxial ellipsoid, i1 = 13
// (Source/sc_calc_generic_gpu.cu:2338-2350, :2878-2889): the Schulz-averaged
// sphere form factor at the ellipsoid's radius seen at angle x from its long
// axis, times sin(x). The pixel-independent factors are formed once, with the
// reference's operations.
struct EllArgs {
    double qn, r, e2m1, zp1, a1, a1z4, a1z45, zm3, zm4, zm5, zm3h, zm4h, zm5h;
};

__device__ inline EllArgs ellipsoid_args(const cs_prepared &P, double qx, double qy) {
    EllArgs A;
    const double z = (1 - P.sigma * P.sigma) / (P.sigma * P.sigma);
    const double epsi = P.length / P.radius;
    A.qn = sqrt(qx * qx + qy * qy + 0.0000000001);
    A.r = P.radius;
    A.e2m1 = epsi * epsi - 1;
    A.zp1 = z + 1;
    A.a1 = (1 / (2.0 * z * (z - 1) * (z - 2) * (z - 3)));
    A.a1z4 = A.a1 / (z - 4);
    A.a1z45 = A.a1 / ((z - 4) * (z - 5));
    A.zm3 = z - 3;
    A.zm4 = z - 4;
    A.zm5 = z - 5;
    A.zm3h = (z - 3) / 2.0;
    A.zm4h = (z - 4) / 2.0;
    A.zm5h = (z - 5) / 2.0;
    return A;
}

__device__ inline double ellipsoid_integrand(const EllArgs &A, double x) {
    double sx, cx;
    sincos(x, &sx, &cx);
    const double arg = A.qn * A.r * sqrt(1.0 + A.e2m1 * cx * cx) / A.zp1;
    const double at = atan(2.0 * arg);
    const double den = 1.0 + 4 * arg * arg;
    const double p1 = A.a1 * pow(arg, -4) * (1 + cos(A.zm3 * at) / pow(den, A.zm3h));
    const double p2 = A.a1z4 * pow(arg, -5) * sin(A.zm4 * at) / pow(den, A.zm4h);
    const double p3 = A.a1z45 * pow(arg, -6) * (1 - cos(A.zm5 * at) / pow(den, A.zm5h));
    return 9 * (p1 - 2 * p2 + p3) * sx;
}

// qrombchid over x in [0, pi/2] (limits stored as float, :1429-1431) with the
// ellipsoid integrand: trapezoid doubling, Neville extrapolation over the last
// five estimates, stop at |dss| < 1e-4 |I| or |I| < 1e-300 (:1449-1463).
__device__ inline double qromb_ellipsoid(const EllArgs &A) {
    const double a = (double)0.0f, b = (double)(float)(M_PI / 2.0);
    double win[5];
    double cur = 0.5 * (b - a) * (ellipsoid_integrand(A, a) + ellipsoid_integrand(A, b));
    int cnt = 1;
    double pq = 0.0, dss = 0.0;
    win[4] = cur;
    for (int j = 2; j <= 20; j++) {
        const double tnm = cnt;
        const double del = (b - a) / tnm;
        double x = a + 0.5 * del;
        double sump = 0.0;
        for (int k = 0; k < cnt; k++) {
            sump += ellipsoid_integrand(A, x);
            x += del;
        }
        cur = 0.5 * (cur + (b - a) * sump / tnm);
        cnt = 2 * cnt;
        win[0] = win[1];
        win[1] = win[2];
        win[2] = win[3];
        win[3] = win[4];
        win[4] = cur;
        if (j >= 5) {
            polint5(win, pq, dss);
            if (fabs(dss) < (1.0e-4 * fabs(pq))) break;
            if (fabs(pq) < 1.0e-300) break;
        }
    }
    return pq;
}

// formpq_partEllips, homogeneous isotropic ellipsoid (ordis 7, cs 0),
// Source/sc_lib_formpq_partEllips.h:46-86: series below 0.8 limq4, Porod
// asymptote from 1.5 limq4, the orientation integral in between.
__device__ inline double formpq_ellipsoid(const cs_prepared &P, double qx, double qy, double q) {
    if (q < 0.8 * P.limq[4]) return series_q(P.carrp[3], q, 120);
    if (q >= 1.5 * P.limq[4]) return P.por / (q * q * q * q);
    return qromb_ellipsoid(ellipsoid_args(P, qx, qy));
}

// calc_partCube_lattNone_ordisIsotropic, Source/sc_gpu_pCub_lNon_oIso.h:16-77
__device__ inline double calc_cube_none_iso(const Ctx &C, double qx, double qy, double qz) {
    const cs_prepared &P = *C.P;
    const double q = sqrt(qx * qx + qy * qy + qz * qz) + CS_EPS9;
    const double pq = (P.cs == 0) ? formpq_cube(P, q) : 1.0;
    return P.base + P.izero * (pq + P.iso) + P.ifluc / (1 + q * q * P.rfluc * P.rfluc);
}

// Transverse factor of the core/shell disk, F121 + F122 + F123
// (Source/sc_lib_formpq_partDisk.h:344-420): core, cross and shell terms,
// each its series (carr4p/5p/6p) below its switch point or its closed form.
__device__ inline double disk_cross_coreshell(const cs_prepared &P, double q) {
    const double zr = (1 - sqr(P.sigma)) / (sqr(P.sigma));
    const double radiusm = P.radius / P.p1;
    const double ccc1 = sqr(1 - P.rho) * pow(P.p1, 2);
    const double ccc2 = 2 * P.rho * (1 - P.rho) * pow(P.p1, 1);
    const double ccc3 = P.rho * P.rho;
    const double vv3 = sqr((1 - P.rho) * pow(P.p1, 1) + P.rho);
    const double argq = q * radiusm / (zr + 1);
    const double argpq = q * P.radius / (zr + 1);
    double F121, F122, F123;
    if (q < (0.8 * P.limq[4])) {
        F121 = ccc1 * series_q(P.carrp[3], q, 120) / vv3;
    } else {
        const double pqr = (1 / (2.0 * zr * (zr - 1))) * pow(argpq, -2) *
                           (1 - cos((zr - 1) * atan(2.0 * argpq)) / pow(1.0 + 4 * argpq * argpq, (zr - 1) / 2.0));
        F121 = ccc1 * pqr / vv3;
    }
    if (q < (2.0 * P.limq[5])) {
        F122 = ccc2 * series_q(P.carrp[4], q, 120) / vv3;
    } else {
        const double argbm = (zr + 1) * atan(argpq - argq);
        const double nenbm = pow(1.0 + 4 * sqr(argpq - argq), (zr + 1) / 2.0);
        const double argbp = (zr + 1) * atan(argpq + argq);
        const double nenbp = pow(1.0 + 4 * sqr(argpq + argq), (zr + 1) / 2.0);
        const double pqr = (1 / (2.0 * zr * (zr - 1) * (zr - 2) * argpq * argq)) * (cos(argbm) / nenbm - cos(argbp) / nenbp);
        F122 = ccc2 * pqr / vv3;
    }
    if (q < (0.3 * P.limq[6])) {
        F123 = ccc3 * series_q(P.carrp[5], q, 120) / vv3;
    } else {
        const double pqr = (1 / (2.0 * zr * (zr - 1))) * pow(argq, -2) *
                           (1 - cos((zr - 1) * atan(2.0 * argq)) / pow(1.0 + 4 * argq * argq, (zr - 1) / 2.0));
        F123 = ccc3 * pqr / vv3;
    }
    return F121 + F122 + F123;
}

// Transverse factor of the disk (thickness 2 radius): homogeneous,
// Source/sc_lib_formpq_partDisk.h:310-340, its series below 0.5 limq4, else
// the closed form; core/shell above.
__device__ inline double disk_cross(const cs_prepared &P, double q) {
    if (P.cs == 1) return disk_cross_coreshell(P, q);
    const double zr = (1 - sqr(P.sigma)) / (sqr(P.sigma));
    double pqr;
    if (q < (0.5 * P.limq[4])) {
        pqr = 1.0;
        double oldpqsum = 0.0, qqnn = 1.0;
        for (int nser = 1; nser <= 100; nser++) {
            qqnn = qqnn * q * q;
            pqr += P.carrp[3][nser] * qqnn;
            if (series_converged(pqr, oldpqsum)) break;
            oldpqsum = pqr;
        }
    } else {
        const double argpq = q * P.radius / (zr + 1);
        pqr = (1 / (2.0 * zr * (zr - 1))) * pow(argpq, -2) *
              (1 - cos((zr - 1) * atan(2.0 * argpq)) / pow(1.0 + 4 * argpq * argpq, (zr - 1) / 2.0));
    }
    return pqr;
}

// formpq_partDisk, homogeneous disk, ordis 7 and 6 with its transverse part,
// Source/sc_lib_formpq_partDisk.h:8-136 and :310-340. orcase is compared with
// 1..4 as the reference compares it, although its enum is 0-based (1 = x
// axis, 2 = y axis, 3 = z axis): the x axis takes the sum of qxs and qys, the
// y axis qxs (which is 0 there), the z axis qys (= qy, not divided by q). The
// general case (0) takes no series branch and reads an uninitialised argument
// in the closed form; the preparation does not offer it.
__device__ inline double formpq_disk(const cs_prepared &P, double limql, double qxs, double qys, double q, int ordis) {
    const double zl = (1 - sqr(P.sigmal)) / sqr(P.sigmal);
    const double *c1 = P.carrp[0];
    double pql = 0;
    if (ordis == 7) {
        if (q < (0.5 * P.limq[1])) {
            pql = 1.0;
            double oldpqsum = 0.0, qqnn = 1.0;
            for (int nser = 1; nser <= 80; nser++) {
                qqnn = qqnn * q * q;
                pql += c1[nser] * qqnn;
                if (series_converged(pql, oldpqsum)) break;
                oldpqsum = pql;
            }
        } else {
            const double arglq = q * P.length / (zl + 1);
            pql = (2 / (zl * (zl - 1))) * pow(arglq, -2);
        }
    }
    if (ordis == 6) {
        if ((limql * P.length) < 5.0) {
            pql = 1.0;
            double oldpqsum = 0.0, qqnn = 1.0;
            // the factor (1 - w^2)^n of orcase 1..3 (none for 4)
            const double w = P.orcase == 1 ? qxs + qys : (P.orcase == 2 ? qxs : qys);
            for (int nser = 1; nser <= 120; nser++) {
                qqnn = qqnn * q * q;
                if (P.orcase == 4)
                    pql += c1[nser] * qqnn;
                else if (P.orcase >= 1 && P.orcase <= 3)
                    pql += c1[nser] * qqnn * pow(1.0 - w * w, nser);
                else
                    break;  // orcase 0: no branch, pql stays 1
                if (series_converged(pql, oldpqsum)) break;
                oldpqsum = pql;
            }
        } else {
            double arglq = 0;
            if (P.orcase == 1) {
                const double qnarg = qxs + qys;
                arglq = sqrt(1.0 - qnarg * qnarg) * q * P.length / (zl + 1) + CS_EPS9;
            }
            if (P.orcase == 2) arglq = sqrt(1.0 - qxs * qxs) * q * P.length / (zl + 1) + CS_EPS9;
            if (P.orcase == 3) arglq = sqrt(1.0 - qys * qys) * q * P.length / (zl + 1) + CS_EPS9;
            if (P.orcase == 4) arglq = q * P.length / (zl + 1) + CS_EPS9;
            const double pqr1 = (1 / (zl * (zl - 1) * (zl - 2))) * pow(arglq, -3);
            const double pqr2 = (1 / (zl * (zl - 1) * (zl - 2))) * pow(arglq, -3) * sin((zl - 2) * atan(2.0 * arglq)) /
                                pow(1.0 + 4 * arglq * arglq, (zl - 2) / 2.0);
            const double pqr3 = (1 / (zl * (zl - 1) * (zl - 2) * (zl - 3))) * pow(arglq, -4) *
                                cos((zl - 3) * atan(2.0 * arglq)) / pow(1.0 + 4 * arglq * arglq, (zl - 3) / 2.0);
            pql = (4 / M_PI) * (pqr1 - pqr2 - (9 / 8.0) * pqr3);
        }
    }
    return pql * disk_cross(P, q);
}

// Length factor of the homogeneous disk with the Gaussian orientation
// distribution along an axis (formpq_partDisk ordis 0,
// Source/sc_lib_formpq_partDisk.h:137-236; formfq_partDisk ordis 0,
// Source/sc_lib_formfq_partDisk.h:136-324, with the F coefficients). Below
// the switch value lim it is the triple series
//   1 + sum_n c1[n] q^2n sum_m carr11pm[n][m] sum_l qxs^2l qys^2(m-l)
// (carr22pm, the reference's inner weight, is 1 throughout); the inner sum
// over l depends on m alone and is formed once per m, in the reference's
// order, which leaves every rounding as it is. Above it, the delta/chi
// quadrature of trapzdchid's disk case i1 = orcase + 7 (orcase compared with
// 1..3 as the reference compares it) with the series coefficients c2,
// divided by the distribution's norm.
__device__ inline double disk_len_gauss(const Ctx &C, double qx, double qy, double qxs, double qys, double q,
                                        const double *c1, const double *c2, double lim) {
    const cs_prepared &P = *C.P;
    if (q < lim) {
        double qxn[121], qyn[121], bm[121];
        double pql = 1.0, oldpqsum = 0.0, qqnn = 1.0;
        qxn[0] = 1.0;
        qyn[0] = 1.0;
        bm[0] = 1.0;  // 0.0 + 1*1*1
        for (int nser = 1; nser <= 120; nser++) {
            qqnn = qqnn * q * q;
            qxn[nser] = qxn[nser - 1] * qxs * qxs;
            qyn[nser] = qyn[nser - 1] * qys * qys;
            double b1 = 0.0;
            for (int lser = 0; lser <= nser; lser++) b1 += qxn[lser] * qyn[nser - lser];
            bm[nser] = b1;
            double binsum = 0.0;
            for (int mser = 0; mser <= nser; mser++) binsum += P.carr11pm[nser][mser] * bm[mser];
            pql += c1[nser] * qqnn * binsum;
            if (series_converged(pql, oldpqsum)) break;
            oldpqsum = pql;
        }
        return pql;
    }
    const DiskChiArgs A = disk_chi_args(P, qx, qy, P.orcase + 7, c2);
    return qromb_delta(C, A) / P.norm;
}

// P(q) of the Gaussian disk: x axis (1) switching at 6 limq1, y (2) and z (3)
// at 6000 limq1
__device__ inline double formpq_disk_gauss(const Ctx &C, double qx, double qy, double qxs, double qys, double q) {
    const cs_prepared &P = *C.P;
    const double lim = (P.orcase == 1 ? 6.0 : 6000.0) * P.limq[1];
    return disk_len_gauss(C, qx, qy, qxs, qys, q, P.carrp[0], P.carrp[1], lim) * disk_cross(P, q);
}

// formfq_partDisk, homogeneous and core/shell disks (cs 0/1),
// Source/sc_lib_formfq_partDisk.h:8-441: the longitudinal factor from the F
// coefficients (carr1f, and carr2f in the quadrature's series) and the switch
// point limq1f, times the square of the transverse amplitude (homogeneous:
// series carr4f below 0.5 limq4f, else its closed form) or the core/shell
// sum of products of amplitudes. The z-direction closed form is the P(q)
// one, as in the reference.
__device__ inline double formfq_disk(const Ctx &C, double qx, double qy, double qxs, double qys, double q) {
    const cs_prepared &P = *C.P;
    const double zl = (1 - sqr(P.sigmal)) / sqr(P.sigmal);
    const double zr = (1 - sqr(P.sigma)) / (sqr(P.sigma));
    const double *c1 = P.carrf[0];
    double pql = 0, pqr;
    if (P.ordis == 7) {
        if (q < (0.5 * P.limqf[1])) {
            pql = 1.0;
            double oldpqsum = 0.0, qqnn = 1.0;
            for (int nser = 1; nser <= 80; nser++) {
                qqnn = qqnn * q * q;
                pql += c1[nser] * qqnn;
                if (series_converged(pql, oldpqsum)) break;
                oldpqsum = pql;
            }
        } else {
            const double arglq = q * P.length / (zl + 1);
            pql = (2 / (zl * (zl - 1))) * pow(arglq, -2);
        }
    }
    if (P.ordis == 6) {
        if (q < (0.5 * P.limqf[1])) {
            pql = 1.0;
            double oldpqsum = 0.0, qqnn = 1.0;
            const double w = P.orcase == 1 ? qxs + qys : (P.orcase == 2 ? qxs : qys);
            for (int nser = 1; nser <= 120; nser++) {
                qqnn = qqnn * q * q;
                if (P.orcase == 4)
                    pql += c1[nser] * qqnn;
                else if (P.orcase >= 1 && P.orcase <= 3)
                    pql += c1[nser] * qqnn * pow(1.0 - w * w, nser);
                else
                    break;
                if (series_converged(pql, oldpqsum)) break;
                oldpqsum = pql;
            }
        } else {
            double arglq = 0;
            if (P.orcase == 1) {
                const double qnarg = qxs + qys;
                arglq = sqrt(1.0 - qnarg * qnarg) * q * P.length / (zl + 1) + CS_EPS9;
            }
            if (P.orcase == 2) arglq = sqrt(1.0 - qxs * qxs) * q * P.length / (zl + 1) + CS_EPS9;
            if (P.orcase == 3) arglq = sqrt(1.0 - qys * qys) * q * P.length / (zl + 1) + CS_EPS9;
            if (P.orcase == 4) arglq = q * P.length / (zl + 1) + CS_EPS9;
            const double pqr1 = (1 / (zl * (zl - 1) * (zl - 2))) * pow(arglq, -3);
            const double pqr2 = (1 / (zl * (zl - 1) * (zl - 2))) * pow(arglq, -3) * sin((zl - 2) * atan(2.0 * arglq)) /
                                pow(1.0 + 4 * arglq * arglq, (zl - 2) / 2.0);
            const double pqr3 = (1 / (zl * (zl - 1) * (zl - 2) * (zl - 3))) * pow(arglq, -4) *
                                cos((zl - 3) * atan(2.0 * arglq)) / pow(1.0 + 4 * arglq * arglq, (zl - 3) / 2.0);
            pql = (4 / M_PI) * (pqr1 - pqr2 - (9 / 8.0) * pqr3);
        }
    }
    if (P.ordis == 0) {
        // x axis (1) switching at 1.2 limq1f, y (2) and z (3) at 0.9 limq1f
        const double lim = (P.orcase == 1 ? 1.2 : 0.9) * P.limqf[1];
        pql = disk_len_gauss(C, qx, qy, qxs, qys, q, c1, P.carrf[1], lim);
    }
    if (P.cs == 1) {
        // core/shell, :355-441: core, cross and shell amplitudes
        const double radiusm = P.radius / P.p1;
        const double ccc1 = sqr(1 - P.rho) * pow(P.p1, 2);
        const double ccc2 = 2 * P.rho * (1 - P.rho) * pow(P.p1, 1);
        const double ccc3 = sqr(P.rho);
        const double vv3 = sqr((1 - P.rho) * pow(P.p1, 1) + P.rho);
        const double argq = q * radiusm / (zr + 1);
        const double argpq = q * P.radius / (zr + 1);
        double F121, F122, F123;
        if (q < (0.8 * P.limqf[4])) {
            F121 = ccc1 * series_q(P.carrf[3], q, 120) / vv3;
        } else {
            const double a = (1 / zr) * pow(argpq, -1) * sin(zr * atan(argpq)) / pow(1.0 + argpq * argpq, zr / 2.0);
            F121 = ccc1 * a * a / vv3;
        }
        if (q < (1.0 * P.limqf[5])) {
            F122 = ccc2 * series_q(P.carrf[4], q, 120) / vv3;
        } else {
            const double a = (1 / zr) * pow(argpq, -1) * sin(zr * atan(argpq)) / pow(1.0 + argpq * argpq, zr / 2.0);
            const double a1 = (1 / zr) * pow(argq, -1) * sin(zr * atan(argq)) / pow(1.0 + argq * argq, zr / 2.0);
            F122 = ccc2 * a * a1 / vv3;
        }
        if (q < (0.3 * P.limqf[6])) {
            F123 = ccc3 * series_q(P.carrf[5], q, 120) / vv3;
        } else {
            const double a = (1 / zr) * pow(argq, -1) * sin(zr * atan(argq)) / pow(1.0 + argq * argq, zr / 2.0);
            F123 = ccc3 * a * a / vv3;
        }
        return pql * (F121 + F122 + F123);
    }
    if (q < (0.5 * P.limqf[4])) {
        pqr = 1.0;
        double oldpqsum = 0.0, qqnn = 1.0;
        for (int nser = 1; nser <= 120; nser++) {
            qqnn = qqnn * q * q;
            pqr += P.carrf[3][nser] * qqnn;
            if (series_converged(pqr, oldpqsum)) break;
            oldpqsum = pqr;
        }
    } else {
        const double argpq = q * P.radius / (zr + 1);
        pqr = (1 / zr) * pow(argpq, -1) * sin(zr * atan(argpq)) / pow(1.0 + argpq * argpq, zr / 2.0);
    }
    return pql * pqr * pqr;
}

// calc_GENERIC, Source/sc_gpu_generic.h:27-881, for the particles the
// preparation supports (spheres, cylinders with z-direction or Gaussian
// orientation, z-direction disks along an axis without a lattice, vesicles,
// homogeneous isotropic cubes and ellipsoids), any supported lattice and the
// peak shapes 1-7 (the reference's shape 7 falls to its `default: return 0`).
// (not inlined: the five kernels of the generic key share one copy, which
// keeps that unit's compile time down)
static __device__ __noinline__ double calc_generic(const Ctx &C, double qx, double qy, double qz) {
    const cs_prepared &P = *C.P;
    double pq = 0, fq = 0, intensity, radintensity;
    const double q = sqrt(qx * qx + qy * qy + qz * qz) + CS_EPS9;  // :33
    double pqiso = 1;
    double szqiso = 1, szq = 1;
    if (P.particle == 0) {  // spheres, :44-58
        pq = formpq_sphere(P, q);
        if (P.lattice) fq = formfq_sphere(P, q);
        pqiso = pq;
    } else if (P.particle == 1) {  // cylinders, :64-165
        if (P.ordis == 7) {  // isotropic, :67-74
            pq = formpq_cylinder(C, qx, qy, q);
            if (P.lattice) fq = formfq_cylinder(C, q, qx, qy, q);
        } else if (P.ordis == 6) {
            switch (P.orcase) {
            case CS_ORC_GENERAL:
                pq = formpq_cylinder(C, qx * P.cosphi * P.sintheta, qy * P.sinphi * P.sintheta, q);
                if (P.lattice)
                    fq = formfq_cylinder(C, sqrt(P.cosphi * qx * qx + P.sinphi * qy * qy + CS_EPS9),
                                         qx * P.cosphi * P.sintheta, qy * P.sinphi * P.sintheta, q);
                break;
            case CS_ORC_XAXIS:
                pq = formpq_cylinder(C, qx, 0, q);
                if (P.lattice) fq = formfq_cylinder(C, fabs(qx), qx, 0, q);
                break;
            case CS_ORC_YAXIS:
                pq = formpq_cylinder(C, 0, qy, q);
                if (P.lattice) fq = formfq_cylinder(C, fabs(qy), 0, qy, q);
                break;
            case CS_ORC_ZAXIS:
                pq = formpq_cylinder(C, qx, qy, q);
                if (P.lattice) fq = formfq_cylinder(C, q, qx, qy, q);
                break;
            }
        } else if (P.ordis == 0) {
            switch (P.orcase) {
            case CS_ORC_GENERAL:
                pq = formpq_cylinder(C, qx * P.cosphic - qy * P.sinphic, qx * P.sinphic + qy * P.cosphic, q);
                if (P.lattice)
                    fq = formfq_cylinder(C, q, qx * P.cosphic - qy * P.sinphic, qx * P.sinphic + qy * P.cosphic, q);
                break;
            case CS_ORC_XAXIS:
                pq = formpq_cylinder(C, qx, qy, q);
                if (P.lattice) fq = formfq_cylinder(C, sqrt(qx * qx + (1 - P.order) * qy * qy), qx, qy, q);
                break;
            case CS_ORC_YAXIS:
                pq = formpq_cylinder(C, qx, qy, q);
                if (P.lattice) fq = formfq_cylinder(C, sqrt((1.0 - P.order) * qx * qx + qy * qy), qx, qy, q);
                break;
            case CS_ORC_ZAXIS:
                pq = formpq_cylinder(C, qx, qy, q);
                if (P.lattice) fq = formfq_cylinder(C, q, qx, qy, q);
                break;
            }
        }
    } else if (P.particle == 2) {  // disks, :173-265 (isotropic, z-direction or Gaussian along an axis)
        if (P.ordis == 7) {
            pq = formpq_disk(P, q, qx, qy, q, 7);
            if (P.lattice) fq = formfq_disk(C, qx, qy, qx, qy, q);
        }
        if (P.ordis == 6) {
            switch (P.orcase) {
            case CS_ORC_XAXIS:
                pq = formpq_disk(P, fabs(qy), qx / q, 0, q, 6);
                if (P.lattice) fq = formfq_disk(C, qx, qy, qx / q, 0, q);
                break;
            case CS_ORC_YAXIS:
                pq = formpq_disk(P, fabs(qx), 0, qy / q, q, 6);
                if (P.lattice) fq = formfq_disk(C, qx, qy, 0, qy / q, q);
                break;
            case CS_ORC_ZAXIS:
                pq = formpq_disk(P, q, qx, qy, q, 6);
                if (P.lattice) fq = formfq_disk(C, qx, qy, qx, qy, q);
                break;
            }
        }
        pqiso = (P.iso > 0) ? formpq_disk(P, q, qx, qy, q, 7) : 0.0;
        if (P.ordis == 0) {
            switch (P.orcase) {
            case CS_ORC_XAXIS:
            case CS_ORC_YAXIS:
                pq = formpq_disk_gauss(C, qx, qy, qx / q, qy / q, q);
                if (P.lattice) fq = formfq_disk(C, qx, qy, qx / q, qy / q, q);
                break;
            case CS_ORC_ZAXIS:
                pq = formpq_disk_gauss(C, qx, qy, qx, qy, q);
                if (P.lattice) fq = formfq_disk(C, qx, qy, qx, qy, q);
                break;
            }
        }
    } else if (P.particle == 3) {  // vesicles, :271-277
        pq = polyvesicle(P, q);
        fq = pq;
    } else if (P.particle == 5) {  // ellipsoids, isotropic and homogeneous, :322-342
        pq = formpq_ellipsoid(P, qx, qy, q);
        fq = pq;
    } else if (P.particle == 4) {  // cubes, :291-320
        pq = formpq_cube(P, q);
        fq = pq;
    }

    double width = 1;  // :511-524
    if (P.debyescherrer) width = 4.0 / P.domainsize;
    if (P.para) width = (4.0 / P.domainsize) + sqr(P.reldis) * P.dist * sqr(q);
    // the anisotropic Gaussian peak on isotropic particles: |sig|/3
    const double sig_len = sqrt(sqr(P.sig[0]) + sqr(P.sig[1]) + sqr(P.sig[2]));
    if (P.lattice && P.shp == 8 && P.ordis == 7) width = sig_len / 3.0;
    width *= P.width_zuf;
    const double widthiso = 1.0 / P.uca;
    radintensity = 0.0;
    intensity = 0.0;
    if (P.lattice) {  // :537-846
        const double sphno_cubevol = P.latpar[1] * P.latpar[2];
        for (int ii = 1; ii <= P.peakmax1; ii++) {
            const int mhkl = P.latpar1[ii][4];
            const int fhkl = P.latpar1[ii][5];
            const double qhkl = P.latpar3[ii][5];
            const double x2 = sqr(q - qhkl) / sqr(widthiso);
            const double sq = exp(-4 * x2 / M_PI) / (M_PI * widthiso / 2.0);
            const double savintens = radintensity;
            radintensity += sq * mhkl * fhkl;
            if (isinf(radintensity) || isnan(radintensity)) {
                radintensity = savintens;
                break;
            }
        }
        for (int ii = 1; ii <= P.peakmax2; ii++) {
            const double qhkl = P.latpar3[ii][5];
            if (qhkl <= 0 || isnan(qhkl)) continue;
            const int mhkl = P.latpar2[ii][4];
            const int fhkl = P.latpar2[ii][5];
            const double qxhkl = P.latpar3[ii][2], qyhkl = P.latpar3[ii][3], qzhkl = P.latpar3[ii][4];
            const double qxhklt = P.latpar3[ii][7], qyhklt = P.latpar3[ii][8], qzhklt = P.latpar3[ii][9];
            const double g3 = P.latpar3[ii][10];
            const double peaknorm1 = P.latpar3[ii][11];
            double sq = 1.0, psiord = 1.0;
            const double yphi = myacos((qx * qxhkl + qy * qyhkl + qz * qzhkl) / (q * qhkl));
            const double x2 = (q - qhkl) * (q - qhkl) / (width * width);
            double yphit = 0;
            if (P.twin) yphit = myacos((qx * qxhklt + qy * qyhklt + qz * qzhklt) / (q * qhkl));
            switch (P.shp) {
            case 1: {  // Lorentzian, :692-704
                sq = sqrt(P.pk_c1) / (M_PI * width * (1.0 + P.pk_c1 * x2));
                const double x2phi = 4 * q * q / sqr(P.phiwidth);
                psiord = g3 / (peaknorm1 * (1 + x2phi * yphi * yphi));
                if (P.twin) {
                    const double phiord = g3 / (peaknorm1 * (1 + x2phi * yphit * yphit));
                    psiord = P.ceff * psiord + (1 - P.ceff) * phiord;
                }
                break;
            }
            case 2: {  // Gaussian, :706-727
                sq = exp(-4 * x2 / M_PI) / (M_PI * width / 2.0);
                const double x2phi = 4 * q * q / (M_PI * sqr(P.phiwidth));
                psiord = g3 * exp(-x2phi * yphi * yphi) / peaknorm1;
                if (P.twin) {
                    const double phiord = g3 * exp(-x2phi * yphit * yphit) / peaknorm1;
                    psiord = P.ceff * psiord + (1 - P.ceff) * phiord;
                }
                break;
            }
            case 3: {  // modified Lorentzian 1, :739-752
                sq = 2 * sqrt(P.pk_c2) / (M_PI * width * (1 + P.pk_c1 * x2) * (1 + P.pk_c1 * x2));
                const double x2phi = 4 * q * q / sqr(P.phiwidth);
                psiord = g3 / (peaknorm1 * (1 + x2phi * yphi * yphi) * (1 + x2phi * yphi * yphi));
                if (P.twin) {
                    const double phiord = g3 / (peaknorm1 * (1 + x2phi * yphit * yphit) * (1 + x2phi * yphit * yphit));
                    psiord = P.ceff * psiord + (1 - P.ceff) * phiord;
                }
                break;
            }
            case 4: {  // modified Lorentzian 2, :754-767
                sq = sqrt(P.pk_c3) / (2 * width * exp(3 * log(1 + P.pk_c1 * x2) / 2.0));
                const double x2phi = 4 * q * q / sqr(P.phiwidth);
                psiord = g3 / (peaknorm1 * exp(3 * log(1 + x2phi * yphi * yphi) / 2.0));
                if (P.twin) {
                    const double phiord = g3 / (peaknorm1 * exp(3 * log(1 + x2phi * yphit * yphit) / 2.0));
                    psiord = P.ceff * psiord + (1 - P.ceff) * phiord;
                }
                break;
            }
            case 5: {  // pseudo-Voigt, :769-785
                const double peaknorm2 = P.latpar3[ii][12];
                const double eta = P.pk_eta;
                sq = eta * sqrt(P.pk_c1) / (M_PI * width * (1 + P.pk_c1 * x2)) +
                     (1 - eta) * sqrt(1.0) * exp(-1.0 * x2) / (sqrt(M_PI) * width);
                const double x2psi = 4 * q * q / (M_PI * sqr(P.phiwidth));
                const double x2phi = 4 * q * q / sqr(P.phiwidth);
                psiord = g3 * (eta * (1 / (1 + x2phi * yphi * yphi)) + (1 - eta) * exp(-x2psi * yphi * yphi)) /
                         (eta * peaknorm1 + (1 - eta) * peaknorm2);
                if (P.twin) {
                    const double phiord =
                        g3 * (eta * (1 / (1 + x2phi * yphit * yphit)) + (1 - eta) * exp(-x2psi * yphit * yphit)) /
                        (eta * peaknorm1 + (1 - eta) * peaknorm2);
                    psiord = P.ceff * psiord + (1 - P.ceff) * phiord;
                }
                break;
            }
            case 6: {  // Pearson VII, :787-800
                const double beta = P.pk_beta;
                sq = P.pk_gbeta * P.pk_c4 * 2 /
                     (P.pk_gbeta_h * M_PI * width * exp(beta * log(1 + 4 * P.pk_c4 * x2)));
                const double x2phi = 4 * q * q / sqr(P.phiwidth);
                psiord = g3 / (peaknorm1 * exp(beta * log(1 + x2phi * yphi * yphi)));
                if (P.twin) {
                    const double phiord = g3 / (peaknorm1 * exp(beta * log(1 + x2phi * yphit * yphit)));
                    psiord = P.ceff * psiord + (1 - P.ceff) * phiord;
                }
                break;
            }
            case 8: {  // anisotropic Gaussian, :599-691 (perfect orientation or isotropic)
                auto aniso = [&](double hx, double hy, double hz) {
                    if (P.ordis == 6 || fabs(P.dbeta) < CS_EPS9) {
                        // the Gaussian ellipsoid of the unit-cell axes around q_hkl
                        const double dqx = qx - hx, dqy = qy - hy, dqz = qz - hz;
                        const double a1n = sqrt(sqr(P.ax1[0]) + sqr(P.ax1[1]) + sqr(P.ax1[2])) * P.sig[0];
                        const double a2n = sqrt(sqr(P.ax2[0]) + sqr(P.ax2[1]) + sqr(P.ax2[2])) * P.sig[1];
                        const double a3n = sqrt(sqr(P.ax3[0]) + sqr(P.ax3[1]) + sqr(P.ax3[2])) * P.sig[2];
                        const double dqs1 = (dqx * P.ax1[0] + dqy * P.ax1[1] + dqz * P.ax1[2]) / a1n;
                        const double dqs2 = (dqx * P.ax2[0] + dqy * P.ax2[1] + dqz * P.ax2[2]) / a2n;
                        const double dqs3 = (dqx * P.ax3[0] + dqy * P.ax3[1] + dqz * P.ax3[2]) / a3n;
                        const double xa = dqs1 * dqs1 + dqs2 * dqs2 + dqs3 * dqs3;
                        return exp(-4 * xa / M_PI) / (sqrt(M_PI * M_PI * M_PI) * P.sig[0] * P.sig[1] * P.sig[2] / 8.0);
                    }
                    // isotropic orientation (the preparation offers no other case)
                    const double locwidth = sig_len / 3.0;
                    const double xa = (q - qhkl) * (q - qhkl) / (locwidth * locwidth);
                    return g3 * exp(-4 * xa / M_PI) / (M_PI * locwidth / 2.0);
                };
                // with twinning the reference forms only the twin's term and
                // mixes it with sq = 1
                if (!P.twin) sq = aniso(qxhkl, qyhkl, qzhkl);
                psiord = 1.0;
                if (P.twin) sq = P.ceff * sq + (1 - P.ceff) * aniso(qxhklt, qyhklt, qzhklt);
                break;
            }
            default:
                return 0.0;  // :833-834
            }
            const double savintens = intensity;
            intensity += sq * mhkl * fhkl * psiord;
            if (isinf(intensity) || isnan(intensity)) {
                intensity = savintens;
                break;
            }
        }
        szqiso = (1 + (1) * (8 * M_PI * M_PI * M_PI * radintensity / (4 * M_PI * sphno_cubevol) - 1) *
                          exp(-P.ucb * q * q));
        szq = (1 + (fq / pq) * (2 * M_PI * intensity / (sphno_cubevol)-1) * exp(-P.dwfactor * q * q));
    }
    return P.base + P.izero * (szq * pq + P.iso * szqiso * pqiso) + P.ifluc / (1 + q * q * P.rfluc * P.rfluc);
}

template <int KEY>
__device__ __forceinline__ double calc_pixel(const Ctx &C, double qx, double qy, double qz) {
    if (KEY == CS_KEY_SPHERE_NONE_ISO) return calc_sphere_none_iso(C, qx, qy, qz);
    if (KEY == CS_KEY_SPHERE_GAUSS_FCC_GAUSS) return calc_sphere_fcc(C, qx, qy, qz);
    if (KEY == CS_KEY_CYL_NONE_GAUSS) return calc_cyl_none_gauss(C, qx, qy, qz);
    if (KEY == CS_KEY_CYL_NONE_ZDIR) return calc_cyl_none_zdir(C, qx, qy, qz);
    if (KEY == CS_KEY_CYL_GAUSS_BCT_ZDIR) return calc_cyl_bct_zdir(C, qx, qy, qz);
    if (KEY == CS_KEY_CUBE_NONE_ISO) return calc_cube_none_iso(C, qx, qy, qz);
    if (KEY == CS_KEY_GENERIC) return calc_generic(C, qx, qy, qz);
    return 0.0;
}

}  // namespace cs64

#endif
