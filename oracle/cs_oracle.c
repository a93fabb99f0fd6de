/*
 * cs_oracle.c — CPU test oracle: plain-C restatement of the reference's FP64
 * per-pixel calculation.
 *
 * TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load this library, always as the checker or as the timed
 * CPU baseline, never as part of the product path. It is pinned against the
 * reference itself (oracle/_ref, golden fixtures in tests/golden).
 *
 * Input is the prepared constant block (crystalscatter_gb300/csrc/cs_prepared.h)
 * that the library's host preparation produces; that preparation is pinned
 * separately against the reference's own coefficient arrays. Everything
 * per pixel is recomputed here the way the reference does it, with no shared
 * code and no precomputed tables: trapezoid nodes by repeated addition, libm
 * sines/cosines at every node, the Gamma function at every cylinder F(q)
 * asymptote, the Romberg state in arrays.
 *
 * Functions follow (paths relative to the reference tree):
 *   convert_idx2q            Source/sc_calc_generic_gpu.cu:249-287
 *   calcCPU_selection        Source/sc_calc_generic_gpu.cu:168-242
 *   checkFitRanges           Source/sc_calc_generic_gpu.cu:293-347
 *   gamma                    Source/sc_calc_generic_gpu.cu:613-673
 *   trapzddeltac             Source/sc_calc_generic_gpu.cu:956-1272 (i0 = 4)
 *   polint                   Source/sc_calc_generic_gpu.cu:1280-1335
 *   qrombdeltac              Source/sc_calc_generic_gpu.cu:1370-1488
 *   qrombchid                Source/sc_calc_generic_gpu.cu:1495-1583
 *   trapzdchid               Source/sc_calc_generic_gpu.cu:1590-2965 (i1 = 1..4)
 *   formpq_partSphere        Source/sc_lib_formpq_partSphere.h:11-196
 *   formfq_partSphere        Source/sc_lib_formfq_partSphere.h:8-52
 *   formpq_partCylinder      Source/sc_lib_formpq_partCylinder.h:8-391
 *   formfq_partCylinder      Source/sc_lib_formfq_partCylinder.h:8-216
 *   calc_partSphere_lattNone_ordisIsotropic       Source/sc_gpu_pSph_lNon_oIso.h:15-51
 *   calc_partSphere_peakGauss_lattFCC_ordisGauss  Source/sc_gpu_pSph_pGau_lFCC_oGau.h:15-171
 *   calc_partCylinder_lattNone_ordisGauss         Source/sc_gpu_pCyl_lNon_oGau.h:15-100
 *   calc_partCylinder_lattNone_ordisZDir          Source/sc_gpu_pCyl_lNon_oZDi.h:17-88
 *   calc_partCylinder_peakGauss_lattBCT_ordisZDir Source/sc_gpu_pCyl_pGau_lBCT_oZDi.h:16-245
 *   calc_GENERIC (restated combinations)          Source/sc_gpu_generic.h:27-881
 *   doCalculation (loops, quadrant mirroring)     Source/sc_calc_generic_cpu.cpp:1151-1275
 *   doFitCalculation (sum)                        Source/sc_calc_generic_cpu.cpp:1334-1443
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "../crystalscatter_gb300/csrc/cs_prepared.h"

#ifdef CS_ORACLE_PROBE
/* Conditioning probe build (liboracle_cs_probe.so, test infrastructure): every
   math-library result is moved by one ulp, up or down per function as the
   probe mode selects. The spread of images over a few modes measures how much
   the reference's own result depends on last-bit differences of the math
   library; pixels with a large spread cannot be reproduced to 1e-10 by any
   other libm and are reported separately. Mode 0 disables the probe. */
static int g_probe_mode = 0;
static int g_probe_mask = 0x1FF; /* functions the probe moves (bit k = function k) */
void oracle_set_probe(int mode) { g_probe_mode = mode; }
void oracle_set_probe_mask(int mask) { g_probe_mask = mask; }
static double probe_(double r, int fn) {
    if (!g_probe_mode || !((g_probe_mask >> fn) & 1) || !isfinite(r)) return r;
    return nextafter(r, ((g_probe_mode >> fn) & 1) ? INFINITY : -INFINITY);
}
#define sin(x) probe_(sin(x), 0)
#define cos(x) probe_(cos(x), 1)
#define atan(x) probe_(atan(x), 2)
#define atan2(y, x) probe_(atan2(y, x), 3)
#define pow(x, y) probe_(pow(x, y), 4)
#define exp(x) probe_(exp(x), 5)
#define sqrt(x) probe_(sqrt(x), 6)
#define log(x) probe_(log(x), 7)
#define acos(x) probe_(acos(x), 8)
#endif

/* element type of the prepared block's arrays as seen by the functions below
   (the block's own double; the high-precision build evaluates in another
   type but reads the same block) */
#ifndef CS_PDOUBLE_T
#define CS_PDOUBLE_T double
#endif

/* sin, cos and exp of quadrature node positions (pixel-independent values;
   the operation-counting build evaluates them without counting, as the GPU
   paths read them from node tables) */
#ifndef NODE_SIN
#define NODE_SIN(x) sin(x)
#define NODE_COS(x) cos(x)
#define NODE_EXP(x) exp(x)
#endif

#define EPS9 0.000000001
#define EPS3 0.001

static double sqr(double x) { return x * x; }

/* myacos, Source/sc_calc_generic_gpu.cu:30 */
static double myacos(double x) { return (x < -1) ? (double)0.0 : ((x > +1) ? (double)M_PI : acos(x)); }

static double frac_part(double x) {
    double ip;
    return modf(x, &ip);
}

/* gamma, Source/sc_calc_generic_gpu.cu:613-673 */
static double ref_gamma(double z) {
    static const double bm[] = {0.0, -0.577191652, 0.988205891, -0.897056937, 0.918206857,
                                -0.756704078, 0.482199394, -0.193527818, 0.035868343};
    static const double cm[] = {0.0, 1.0000000000000000, 0.5772156649015329, -0.6558780715202538,
                                -0.0420026350340952, 0.1665386113822915, -0.0421977345555443,
                                -0.0096219715278770, 0.00721894322466630, -0.0011651675918591,
                                -0.0002152416741149, 0.0001280502823882, -0.0000201348547807,
                                -0.0000012504934821, 0.0000011330272320, -0.0000002056338417,
                                0.0000000061160950, 0.0000000050020075, -0.0000000011812746,
                                0.0000000001043427, 0.0000000000077823, -0.0000000000036968,
                                0.0000000000005100, -0.0000000000000206, -0.0000000000000054,
                                0.0000000000000014, 0.0000000000000001};
    int negative;
    if (fabs(z) < EPS9) z = z + EPS9;
    if (z > 0)
        negative = 0;
    else {
        negative = 1;
        if (fabs(frac_part(z)) < EPS9) z = z + EPS9;
    }
    const double absz = fabs(z);
    if (absz > 0.0 && absz <= 1) {
        double fct = 0;
        for (int i = 1; i <= 26; i++) fct += cm[i] * pow(absz, i);
        if (negative) return -M_PI * fct / (absz * sin(M_PI * absz));
        return 1. / fct;
    }
    if (absz > 1 && absz <= 1000) {
        if (fabs(frac_part(absz)) < EPS9) {
            double fct = 1;
            for (int i = 1; i <= trunc(absz) - 1; i++) fct = fct * i;
            if (negative) return -M_PI / (absz * fct * sin(M_PI * absz));
            return fct;
        }
        const double y = absz - 1;
        const double di = trunc(y);
        const double x = absz - trunc(absz);
        double fak = y;
        if (di == 0)
            fak = 1;
        else
            for (int i = 1; i < di; i++) fak = fak * (y - i);
        double f = 1;
        for (int i = 1; i <= 8; i++) f = f + bm[i] * pow(x, i);
        if (negative) return -M_PI / (absz * fak * f * sin(M_PI * absz));
        return fak * f;
    }
    double fct = exp(-absz) * exp((absz - 0.5) * log(absz)) * sqrt(2 * M_PI);
    if (negative) return -M_PI / (absz * fct * sin(M_PI * absz));
    return fct;
}

/* convert_idx2q, Source/sc_calc_generic_gpu.cu:249-287 */
static void convert_idx2q(const cs_prepared *P, int ihex, int i, double *qx, double *qy, double *qz) {
    if (P->use1d) {
        *qx = (P->qmax - P->qmin) / (double)(P->zmax) * (double)ihex;
        *qy = 1e-20;
        *qz = 1e-20;
    } else if (P->usebeamstop) {
        double mdet = (ihex)*P->pixnoy / (2.0 * P->zmax);
        double ndet = (i)*P->pixnox / (2.0 * P->zmax);
        double xdet = P->pixx_m * (ndet - P->beamx0);
        double ydet = P->pixy_m * (mdet - P->beamy0);
        double rdet = sqrt(xdet * xdet + ydet * ydet);
        double phidet = atan2(ydet, xdet);
        double thetadet = atan2(rdet, P->det);
        *qx = 2 * M_PI * cos(phidet) * sin(thetadet) / P->wave;
        *qy = 2 * M_PI * sin(phidet) * sin(thetadet) / P->wave;
        *qz = 2 * M_PI * (1 - cos(thetadet)) / P->wave;
    } else {
        *qx = P->qmax * i / (double)(P->zmax);
        *qy = P->qmax * ihex / (double)(P->zmax);
        *qz = 1e-20;
    }
}

/* ------------------------------------------------------------------ spheres */

static double series_q(const CS_PDOUBLE_T *c, double q, int nmax) {
    double pqsum = 1.0, oldpqsum = 0.0, qq = 1.0;
    for (int nser = 1; nser <= nmax; nser++) {
        qq = qq * q * q;
        pqsum = pqsum + c[nser] * qq;
        double delser = fabs((pqsum - oldpqsum) / pqsum);
        if (delser < 0.0001) break;
        oldpqsum = pqsum;
    }
    return pqsum;
}

/* formpq_partSphere, Source/sc_lib_formpq_partSphere.h:11-196 (cs 0 and 1) */
static double formpq_partSphere(const cs_prepared *P, double q) {
    double zr = (1 - sqr(P->sigma)) / (sqr(P->sigma));
    const double radiusm = P->radius / P->p1;
    const double zz = zr;
    if (P->cs == 0) {
        if (q < 0.4 * P->limq[4]) {
            double pqsum = 1.0, oldpqsum = 0.0, qq2 = 1.0;
            for (int nser = 1; nser <= 100; nser++) {
                qq2 = qq2 * q * q;
                pqsum = pqsum + P->carrp[3][nser] * qq2;
                double delser = fabs((pqsum - oldpqsum) / pqsum);
                if (delser < 0.0001) break;
                oldpqsum = pqsum;
            }
            return pqsum;
        } else {
            const double argq = q * P->radius / (zr + 1);
            double pqr;
            if (zr * (zr - 1) * (zr - 2) * (zr - 3) * (zr - 4) * (zr - 5) == 0) zr += EPS3;
            pqr = (1 / (2.0 * zr * (zr - 1) * (zr - 2) * (zr - 3))) * pow(argq, -4);
            const double pq1 = pqr * (1 + cos((zr - 3) * atan(2.0 * argq)) / pow(1.0 + 4 * argq * argq, (zr - 3) / 2.0));
            const double pq2 =
                (pqr / ((zr - 4) * argq)) * sin((zr - 4) * atan(2.0 * argq)) / pow(1.0 + 4 * argq * argq, (zr - 4) / 2.0);
            const double pq3 = (pqr / ((zr - 4) * (zr - 5) * argq * argq)) *
                               (1 - cos((zr - 5) * atan(2.0 * argq)) / pow(1.0 + 4 * argq * argq, zr - 5) / 2.0);
            return 9.0 * (pq1 - 2.0 * pq2 + pq3);
        }
    }
    if (P->cs == 1) {
        const double rho = P->rho, p1 = P->p1;
        const double cc1 = sqr(rho);
        const double cc2 = 2 * p1 * rho * (1 - rho);
        const double cc3 = sqr(1 - rho) * sqr(p1);
        const double cc4 = -2 * sqr(rho);
        const double cc5 = -2 * p1 * rho * (1 - rho);
        const double cc6 = sqr(rho);
        const double cc7 = -2 * rho * (1 - rho);
        const double cc8 = -sqr(1 - rho) * 2 * p1;
        const double cc9 = 2 * rho * (1 - rho);
        const double cc10 = sqr(1 - rho);
        const double ccc1 = sqr(1 - rho) * pow(p1, 6);
        const double ccc2 = 2 * rho * (1 - rho) * pow(p1, 3);
        const double ccc3 = rho * rho;
        const double vv3 = sqr((1 - rho) * pow(p1, 3) + rho);
        const double argq = q * radiusm / (zz + 1);
        const double argpq = q * P->radius / (zz + 1);
        const double pqr = (1 / (2.0 * zr * (zr - 1) * (zr - 2) * (zr - 3))) * pow(argq, -4);
        double F121, F122, F123;
        if (q < (0.5 * P->limq[4])) {
            F121 = ccc1 * series_q(P->carrp[3], q, 120) / vv3;
        } else {
            const double ac3 = pqr * (1 + cos((zr - 3) * atan(2.0 * argpq)) / pow(1.0 + 4 * argpq * argpq, (zr - 3) / 2.0));
            const double ac8 = (pqr / ((zr - 4) * argq)) * sin((zr - 4) * atan(2.0 * argpq)) /
                               pow(1.0 + 4 * argpq * argpq, (zr - 4) / 2.0);
            const double ac10 = (pqr / ((zr - 4) * (zr - 5) * argq * argq)) *
                                (1 - cos((zr - 5) * atan(2.0 * argpq)) / pow(1.0 + 4 * argpq * argpq, (zr - 5) / 2.0));
            F121 = 9 * (cc3 * ac3 + cc8 * ac8 + cc10 * ac10) / vv3;
        }
        if (q < (0.5 * P->limq[5])) {
            F122 = ccc2 * series_q(P->carrp[4], q, 120) / vv3;
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
        if (q < (0.5 * P->limq[6])) {
            F123 = ccc3 * series_q(P->carrp[5], q, 120) / vv3;
        } else {
            const double ac1 = pqr * (1 + cos((zr - 3) * atan(2.0 * argq)) / pow(1.0 + 4 * argq * argq, (zr - 3) / 2.0));
            const double ac4 =
                (pqr / ((zr - 4) * argq)) * sin((zr - 4) * atan(2.0 * argq)) / pow(1.0 + 4 * argq * argq, (zr - 4) / 2.0);
            const double ac6 = (pqr / ((zr - 4) * (zr - 5) * argq * argq)) *
                               (1 - cos((zr - 5) * atan(2.0 * argq)) / pow(1.0 + 4 * argq * argq, (zr - 5) / 2.0));
            F123 = 9 * (cc1 * ac1 + cc4 * ac4 + cc6 * ac6) / vv3;
        }
        return F121 + F122 + F123;
    }
    return 0.0;
}

/* formfq_partSphere, Source/sc_lib_formfq_partSphere.h:8-52 (cs 0) */
static double formfq_partSphere(const cs_prepared *P, double q) {
    const double zr = (1 - sqr(P->sigma)) / sqr(P->sigma);
    if (P->cs == 0) {
        if (q < (0.4 * P->limqf[4])) {
            double pqsum = 1.0, oldpqsum = 0.0, qqnn = 1.0;
            for (int nser = 1; nser <= 100; nser++) {
                qqnn = qqnn * q * q;
                pqsum = pqsum + P->carrf[3][nser] * qqnn;
                double delser = fabs((pqsum - oldpqsum) / pqsum);
                if (delser < 0.0001) break;
                oldpqsum = pqsum;
            }
            return pqsum;
        } else {
            const double argq = q * P->radius / (zr + 1);
            const double pqr = (1 / (zr * (zr - 1)) * pow(argq, -2));
            const double pq1 = pqr * cos((zr - 1) * atan(argq)) / pow(1.0 + argq * argq, (zr - 1) / 2.0);
            const double pq2 = (pqr / ((zr - 2) * argq)) * sin((zr - 2) * atan(argq)) / pow(1.0 + argq * argq, (zr - 2) / 2.0);
            const double pq3 = 3 * (pq2 - pq1);
            return pq3 * pq3;
        }
    }
    return 0.0;
}

/* ----------------------------------------------------------------- Romberg */

/* polint, Source/sc_calc_generic_gpu.cu:1280-1335 (1-based arrays, x = 0) */
static void polint(const double *xa, const double *ya, int n, double *y, double *dy) {
    int ns, m, i;
    double w, hp, ho, dift, dif, den;
    double c[8], d[8];
    ns = 1;
    dif = fabs(xa[1]);
    for (i = 1; i <= n; i++) {
        dift = fabs(xa[i]);
        if (dift < dif) {
            ns = i;
            dif = dift;
        }
        c[i] = ya[i];
        d[i] = ya[i];
    }
    *y = ya[ns];
    ns = ns - 1;
    for (m = 1; m <= n - 1; m++) {
        for (i = 1; i <= n - m; i++) {
            ho = xa[i];
            hp = xa[i + m];
            w = c[i + 1] - d[i];
            den = ho - hp;
            if (den != 0) den = w / den;
            d[i] = hp * den;
            c[i] = ho * den;
        }
        if (2 * ns < n - m)
            *dy = c[ns + 1];
        else {
            *dy = d[ns];
            ns = ns - 1;
        }
        *y = *y + *dy;
    }
}

typedef struct {
    double l, sigma, qx, qy;
    double p11, p12, p13, p21, p22, p23;
    const CS_PDOUBLE_T *carr1; /* carr2p for the disk cases */
    int i1;
} chid_args;

/* disk P(q) integrand of trapzdchid (i1 = 8..11, i3 = 0) for the cosines and
   sines of chi entering the two direction components: (c1, s1) the first,
   (s2, c2) the second. Source/sc_calc_generic_gpu.cu:1849-2260 (interval
   ends, where case 8 pairs cos(a) with sin(b) and sin(a) with cos(b)) and
   2604-2840 (interior nodes). */
static double disk_chid_value(const chid_args *A, double c1, double s1, double s2, double c2, double delta) {
    const double eps = 0.0000000001;
    const double sigma = A->sigma, qx = A->qx, qy = A->qy, l = A->l;
    const double z = (1 - sigma * sigma) / (sigma * sigma);
    const double qn = sqrt(qx * qx + qy * qy + eps);
    const double qxl = qx / qn;
    const double qyl = qy / qn;
    double qnn;
    if (A->i1 == 8) {
        const double ml1 = A->p11 * c1 * NODE_SIN(delta) + A->p12 * s1 * NODE_SIN(delta) + A->p13 * NODE_COS(delta);
        const double ml2 = A->p21 * s2 * NODE_SIN(delta) + A->p22 * c2 * NODE_SIN(delta) + A->p23 * NODE_COS(delta);
        qnn = qxl * ml1 + qyl * ml2;
    } else if (A->i1 == 9) {
        qnn = qxl * NODE_COS(delta) - qyl * s1 * NODE_SIN(delta);
    } else if (A->i1 == 10) {
        qnn = qxl * s1 * NODE_SIN(delta) + qyl * NODE_COS(delta);
    } else {
        qnn = qxl * s1 * NODE_SIN(delta) - qyl * c1 * NODE_SIN(delta);
    }
    const double x = sqrt(1.0 - qnn * qnn + eps) * l * qn / (z + 1);
    if (sigma < 0.15) {
        if (x < 0.015) {
            double px = 1, oldpx = 0, argser = 1;
            for (int i = 1; i <= 50; i++) {
                argser = argser * x * x / 4.0;
                px = px + A->carr1[i] * argser;
                const double delser = fabs((px - oldpx) / px);
                if (delser < 0.0001) break;
                oldpx = px;
            }
            return px;
        }
        const double px1 = (1 / (z * (z - 1) * (z - 2))) * pow(x, -3);
        const double px2 = (1 / (z * (z - 1) * (z - 2))) * pow(x, -3) * sin((z - 2) * atan(2.0 * x)) / pow(1.0 + 4 * x * x, (z - 2) / 2.0);
        const double px3 = (1 / (z * (z - 1) * (z - 2) * (z - 3))) * pow(x, -4) * cos((z - 3) * atan(2.0 * x)) / pow(1.0 + 4 * x * x, (z - 3) / 2.0);
        return (4 / M_PI) * (px1 - px2 - (9 / 8.0) * px3);
    }
    const double px1 = (1 / (z * (z - 1) * (z - 2))) * pow(x, -3);
    return 1 / (1.0 + M_PI / (4.0 * px1));
}

/* one trapzdchid integrand value, Source/sc_calc_generic_gpu.cu:1632-1734, 2455-2528 */
static double chid_value(const chid_args *A, double x, double delta) {
    const double eps = 0.0000000001;
    const double sigma = A->sigma, qx = A->qx, qy = A->qy, l = A->l;
    const double z = (1 - sigma * sigma) / (sigma * sigma);
    double argx;
    if (A->i1 == 1) {
        const double mlx1 = A->p11 * NODE_COS(x) * NODE_SIN(delta) + A->p12 * NODE_SIN(x) * NODE_SIN(delta) + A->p13 * NODE_COS(delta);
        const double mlx2 = A->p21 * NODE_SIN(x) * NODE_SIN(delta) + A->p22 * NODE_COS(x) * NODE_SIN(delta) + A->p23 * NODE_COS(delta);
        argx = (qx * mlx1 + qy * mlx2 + eps) * l / (z + 1);
    } else if (A->i1 == 2) {
        argx = (qx * NODE_COS(delta) - qy * NODE_SIN(x) * NODE_SIN(delta) + eps) * l / (z + 1);
    } else if (A->i1 == 3) {
        argx = (qx * NODE_SIN(x) * NODE_SIN(delta) + qy * NODE_COS(delta) + eps) * l / (z + 1);
    } else if (A->i1 == 4) {
        argx = (qx * NODE_SIN(x) * NODE_SIN(delta) - qy * NODE_COS(x) * NODE_SIN(delta) + eps) * l / (z + 1);
    } else if (A->i1 >= 8 && A->i1 <= 11) {
        return disk_chid_value(A, NODE_COS(x), NODE_SIN(x), NODE_SIN(x), NODE_COS(x), delta);
    } else {
        return 0.0; /* no branch of trapzdchid for this i1: the integrand stays 0 */
    }
    const double a1 = 1 / (2.0 * z * (z - 1));
    return (a1 / (argx * argx)) * (1 - cos((z - 1) * atan(2.0 * argx)) / pow(1.0 + 4 * argx * argx, (z - 1) / 2.0));
}

/* trapzdchid, Source/sc_calc_generic_gpu.cu:1590-2965 */
static void trapzdchid(double a, double b, const chid_args *A, double delta, double *pq, int n, int *cnt) {
    if (n == 1) {
        double pa = A->i1 == 8 ? disk_chid_value(A, NODE_COS(a), NODE_SIN(b), NODE_SIN(a), NODE_COS(b), delta)
                               : chid_value(A, a, delta);
        double pb = chid_value(A, b, delta);
        *pq = 0.5 * (b - a) * (pa + pb);
        *cnt = 1;
    } else {
        const double tnm = *cnt;
        const double del = (b - a) / tnm;
        double x = a + 0.5 * del;
        double sump = 0.0;
        for (int j = 1; j <= *cnt; j++) {
            double px = chid_value(A, x, delta);
            sump += px;
            x += del;
        }
        *pq = 0.5 * (*pq + (b - a) * sump / tnm);
        *cnt = 2 * *cnt;
    }
}

/* qrombchid, Source/sc_calc_generic_gpu.cu:1495-1583 (cylinder branches) */
static double qrombchid(const chid_args *A, double delta) {
    const double eps = 1.0e-4;
    const int jmax = 20, k = 5;
    double hp[24], sp[24], cp[8], dp[8];
    double pq = 0, dssp = 0;
    float alim = 0.0, blim = 2 * M_PI;
    int cnt = 0;
    hp[1] = 1.0;
    for (int j = 1; j <= jmax; j++) {
        trapzdchid(alim, blim, A, delta, &sp[j], j, &cnt);
        if (j >= k) {
            for (int i = 1; i <= k; i++) {
                cp[i] = hp[j - k + i];
                dp[i] = sp[j - k + i];
            }
            polint(cp, dp, k, &pq, &dssp);
            if (fabs(dssp) < (eps * fabs(pq))) break;
            if (fabs(pq) < 1.0e-300) break;
        }
        sp[j + 1] = sp[j];
        hp[j + 1] = 0.25 * hp[j];
    }
    return pq;
}

/* trapzddeltac with i0 = 4 (cylinder form factor), Source/sc_calc_generic_gpu.cu:1051-1070, 1167-1182 */
static void trapzddeltac4(double a, double b, double dbeta, const chid_args *A, double *pq, int n, int *cnt) {
    if (n == 1) {
        double pa = qrombchid(A, a);
        double pb = qrombchid(A, b);
        pa = NODE_SIN(a) * NODE_EXP(-a * a / (dbeta * dbeta)) * pa / (2.0 * M_PI);
        pb = NODE_SIN(b) * NODE_EXP(-b * b / (dbeta * dbeta)) * pb / (2.0 * M_PI);
        *pq = 0.5 * (b - a) * (pa + pb);
        *cnt = 1;
    } else {
        const double tnm = *cnt;
        const double del = (b - a) / tnm;
        double x = a + 0.5 * del;
        double sump = 0.0;
        for (int j = 1; j <= *cnt; j++) {
            double px = qrombchid(A, x);
            px = NODE_SIN(x) * NODE_EXP(-x * x / (dbeta * dbeta)) * px / (2.0 * M_PI);
            sump = sump + px;
            x = x + del;
        }
        *pq = 0.5 * (*pq + (b - a) * sump / tnm);
        *cnt = 2 * *cnt;
    }
}

/* qrombdeltac(p1, sigma, alfa, theta, phi, qx, qy, qz, 9,9,9,9, i0=4, i1, 0,0,0, ...),
   Source/sc_calc_generic_gpu.cu:1370-1488 */
static double qrombdeltac_carr(const cs_prepared *P, double sigma, double theta_deg, double phi_deg, double qx,
                               double qy, int i1, const CS_PDOUBLE_T *carr1);

static double qrombdeltac4(const cs_prepared *P, double sigma, double theta_deg, double phi_deg, double qx, double qy,
                           int i1) {
    return qrombdeltac_carr(P, sigma, theta_deg, phi_deg, qx, qy, i1, P->carrp[1]);
}

/* the same with i0 = 6 (disk form factor), whose delta weighting is that of
   i0 = 4 (:1104-1120) and whose chi integrand reads the series carr1 */
static double qrombdeltac_carr(const cs_prepared *P, double sigma, double theta_deg, double phi_deg, double qx,
                               double qy, int i1, const CS_PDOUBLE_T *carr1) {
#ifdef CS_ORACLE_SKIP_ZERO_INTEGRAL
    /* operation-counting build only: an orientation case outside 1..4 has an
       identically zero integrand whose Romberg result is exactly +0; its
       (result-free) work is left out of the algorithmic operation count */
    if ((i1 < 1 || i1 > 4) && (i1 < 8 || i1 > 11)) return 0.0;
#endif
    const double eps = 1.0e-4;
    const int jmax = 20, k = 5;
    const double prmin = 0.00001;
    double hp[24], sp[24], cp[8], dp[8];
    double pq = 0, dssp = 0, delmax;
    float alim, blim, p11, p12, p13, p21, p22, p23;
    int cnt = 0;
    double dbeta = P->dbeta * M_PI / 180.0;
    const double theta = theta_deg * M_PI / 180.0;
    const double phi = phi_deg * M_PI / 180.0;
    delmax = dbeta * sqrt(log(1.0 / prmin));
    if (delmax > M_PI / 2.0) delmax = M_PI / 2.0;
    alim = 0.0;
    blim = delmax;
    p11 = -cos(phi) * cos(theta);
    p12 = sin(phi);
    p13 = cos(phi) * sin(theta);
    p21 = -cos(phi);
    p22 = -sin(phi) * cos(theta);
    p23 = sin(phi) * sin(theta);
    chid_args A;
    A.l = P->length;
    A.sigma = sigma;
    A.qx = qx;
    A.qy = qy;
    A.p11 = p11;
    A.p12 = p12;
    A.p13 = p13;
    A.p21 = p21;
    A.p22 = p22;
    A.p23 = p23;
    A.carr1 = carr1;
    A.i1 = i1;
    hp[1] = 1.0;
    for (int j = 1; j <= jmax; j++) {
        trapzddeltac4(alim, blim, dbeta, &A, &sp[j], j, &cnt);
        if (j >= k) {
            for (int i = 1; i <= k; i++) {
                cp[i] = hp[j - k + i];
                dp[i] = sp[j - k + i];
            }
            polint(cp, dp, k, &pq, &dssp);
            if (fabs(dssp) < (eps * fabs(pq))) break;
            if (fabs(pq) < 1.0e-100) break;
        }
        sp[j + 1] = sp[j];
        hp[j + 1] = 0.25 * hp[j];
    }
    return pq;
}

/* ----------------------------------------------------------------- cylinders */

/* the ordis-0 double series; variant selects the carr11pm index/power order */
static double cyl_double_series(const cs_prepared *P, double qxs, double qys, const CS_PDOUBLE_T *carr1, int variant) {
    double pql = 1.0, oldpqsum = 0.0;
    double qxn[121], qyn[121];
    qxn[0] = 1.0;
    qyn[0] = 1.0;
    for (int nser = 1; nser <= 120; nser++) {
        qxn[nser] = qxn[nser - 1] * qxs * qxs;
        qyn[nser] = qyn[nser - 1] * qys * qys;
        double binsum = 0.0;
        for (int mser = 0; mser <= nser; mser++) {
            if (variant == 0)
                binsum += P->carr11pm[nser - mser][mser] * qxn[mser] * qyn[nser - mser];
            else if (variant == 1)
                binsum += P->carr11pm[nser - mser][mser] * qyn[mser] * qxn[nser - mser];
            else if (variant == 2)
                binsum += P->carr11pm[mser][nser - mser] * qyn[mser] * qxn[nser - mser];
            else
                binsum += P->carr11pm[mser][nser - mser] * qxn[mser] * qyn[nser - mser];
        }
        pql += carr1[nser] * binsum;
        double delser = fabs((pql - oldpqsum) / pql);
        if (delser < 0.0001) break;
        oldpqsum = pql;
    }
    return pql;
}

/* cross-section closed form (4/pi)(T1 - T2 - 9/8 T3), Source/sc_lib_formpq_partCylinder.h:272-275 */
static double cyl_cross_closed(double x, double zr) {
    const double pqr1 = (1 / (zr * (zr - 1) * (zr - 2))) * pow(x, -3);
    const double pqr2 = (1 / (zr * (zr - 1) * (zr - 2))) * pow(x, -3) * sin((zr - 2) * atan(2.0 * x)) /
                        pow(1.0 + 4 * x * x, (zr - 2) / 2.0);
    const double pqr3 = (1 / (zr * (zr - 1) * (zr - 2) * (zr - 3))) * pow(x, -4) * cos((zr - 3) * atan(2.0 * x)) /
                        pow(1.0 + 4 * x * x, (zr - 3) / 2.0);
    return (4 / M_PI) * (pqr1 - pqr2 - (9 / 8.0) * pqr3);
}

/* core/shell cross-section F121 + F122 + F123, Source/sc_lib_formpq_partCylinder.h:284-393 */
static double cyl_cross_coreshell(const cs_prepared *P, double q, double zr) {
    const double radiusm = P->radius / P->p1;
    const double ccc1 = sqr(1 - P->rho) * pow(P->p1, 4);
    const double ccc2 = 2 * P->rho * (1 - P->rho) * pow(P->p1, 2);
    const double ccc3 = P->rho * P->rho;
    const double vv3 = sqr((1 - P->rho) * pow(P->p1, 2) + P->rho);
    const double argq = q * radiusm / (zr + 1);
    const double argpq = q * P->radius / (zr + 1);
    double F121, F122, F123;
    if (q < (0.7 * P->limq[4]))
        F121 = ccc1 * series_q(P->carrp[3], q, 120) / vv3;
    else
        F121 = ccc1 * cyl_cross_closed(argpq, zr) / vv3;
    if (q < (1.5 * P->limq[5])) {
        F122 = ccc2 * series_q(P->carrp[4], q, 120) / vv3;
    } else {
        const double d = argpq - argq, u = argpq + argq;
        const double pqr1 = (1 / (zr * (zr - 1) * (zr - 2))) * pow(argq, -3) *
                            (cos((zr - 2) * atan(d)) / pow(1.0 + sqr(d), (zr - 2) / 2.0) -
                             sin((zr - 2) * atan(u)) / pow(1.0 + sqr(u), (zr - 2) / 2.0));
        const double pqr2 = (1 / (zr * (zr - 1) * (zr - 2) * (zr - 3))) * pow(argq, -4) *
                            ((1 - 1 / P->p1) * sin((zr - 3) * atan(d)) / pow(1.0 + sqr(d), (zr - 3) / 2.0) -
                             (1 + 1 / P->p1) * cos((zr - 3) * atan(u)) / pow(1.0 + sqr(u), (zr - 3) / 2.0));
        const double pqr3 = (1 / (zr * (zr - 1) * (zr - 2) * (zr - 3) * (zr - 4))) * pow(argq, -5) * (1 / P->p1) *
                            (cos((zr - 4) * atan(d)) / pow(1.0 + sqr(d), (zr - 4) / 2.0) -
                             sin((zr - 4) * atan(u)) / pow(1.0 + sqr(u), (zr - 4) / 2.0));
        const double pqr = (4 / M_PI) * pow(P->p1, -3 / 2.0) * (pqr1 + (9 / 16.0) * pqr2 + (9 / 16.0) * (9 / 16.0) * pqr3);
        F122 = ccc2 * pqr / vv3;
    }
    if (q < (0.6 * P->limq[6]))
        F123 = ccc3 * series_q(P->carrp[5], q, 120) / vv3;
    else
        F123 = ccc3 * cyl_cross_closed(argq, zr) / vv3;
    return F121 + F122 + F123;
}

/* isotropic length factor, Source/sc_lib_formpq_partCylinder.h:29-90 */
static double cyl_len_iso(const cs_prepared *P, double q, double zl) {
    if ((P->length / P->radius) < 2) {
        if (q < (5 * P->limq[2])) {
            double qqn[101];
            qqn[0] = 1.0;
            for (int nser = 1; nser <= 100; nser++) qqn[nser] = qqn[nser - 1] * q * q;
            double pql = 0.0, oldpqsum = -10.0;
            for (int nser = 0; nser <= 100; nser++) {
                double binsum = 0.0;
                for (int mser = 0; mser <= 100; mser++) binsum += P->carr11pm[nser][mser] * qqn[mser];
                pql += P->carrp[1][nser] * qqn[nser] * binsum;
                const double delser = fabs((pql - oldpqsum) / pql);
                if (delser < 0.0001) break;
                oldpqsum = pql;
            }
            return pql;
        }
        return P->por / pow(q, 4);
    }
    if (q < (0.6 * P->limq[1])) return series_q(P->carrp[0], q, 120);
    const double arglq = q * P->length / (zl + 1);
    double pql = (M_PI / (2.0 * zl)) * (1 / arglq);
    pql = pql - (1 / (2.0 * zl * (zl - 1) * arglq * arglq)) * cos((zl - 1) * atan(2.0 * arglq)) /
                    pow(1.0 + 4 * arglq * arglq, (zl - 1) / 2.0);
    return pql;
}

/* formpq_partCylinder, Source/sc_lib_formpq_partCylinder.h:8-393 (ordis 0/6/7, cs 0/1) */
static double formpq_partCylinder(const cs_prepared *P, double qxs, double qys, double q) {
    double pqr = 0, pql = 0;
    const double zl = P->sigmal == 1.0 ? (double)EPS9 : (1 - sqr(P->sigmal)) / sqr(P->sigmal);
    const double zr = P->sigma == 1.0 ? (double)EPS9 : (1 - sqr(P->sigma)) / (sqr(P->sigma));
    if (P->ordis == 7) pql = cyl_len_iso(P, q, zl);
    if (P->ordis == 6) {
        if (P->orcase == 4)
            pql = 1.0;
        else if (q < (0.6 * P->limq[1])) {
            pql = 1.0;
            double oldpqsum = 0.0, qqnn = 1.0;
            for (int nser = 1; nser <= 120; nser++) {
                qqnn = qqnn * (qxs + qys) * (qxs + qys);
                pql += P->carrp[0][nser] * qqnn;
                const double delser = fabs((pql - oldpqsum) / pql);
                if (delser < 0.0001) break;
                oldpqsum = pql;
            }
        } else {
            const double arglq = (qxs + qys + EPS9) * P->length / (zl + 1);
            pql = (1 / (2.0 * zl * (zl - 1))) * (1 / (arglq * arglq)) *
                  (1 - cos((zl - 1) * atan(2.0 * arglq)) / pow(1.0 + 4 * arglq * arglq, (zl - 1) / 2.0));
        }
    }
    if (P->ordis == 0) {
        if (P->orcase == 4)
            pql = 1.0;
        else if (q < (0.4 * P->limq[1])) {
            pql = 1.0;
            if (P->orcase == 1)
                pql = cyl_double_series(P, qxs, qys, P->carrp[0], 0);
            else if (P->orcase == 2)
                pql = cyl_double_series(P, qxs, qys, P->carrp[0], 0);
            else if (P->orcase == 3)
                pql = cyl_double_series(P, qxs, qys, P->carrp[0], 1);
        } else {
            pql = qrombdeltac4(P, P->sigmal, P->poltheta, 0, qxs, qys, P->orcase);
            pql = pql / P->norm;
        }
    }
    if (P->cs == 0) {
        if ((P->length / P->radius) < 2)
            pqr = 1;
        else if (q < (0.65 * P->limq[4])) {
            pqr = series_q(P->carrp[3], q, 120);
        } else {
            const double argpq = q * P->radius / (zr + 1);
            const double pqr1 = (1 / (zr * (zr - 1) * (zr - 2))) * pow(argpq, -3);
            const double pqr2 = (1 / (zr * (zr - 1) * (zr - 2))) * pow(argpq, -3) * sin((zr - 2) * atan(2.0 * argpq)) /
                                pow(1.0 + 4 * argpq * argpq, (zr - 2) / 2.0);
            const double pqr3 = (1 / (zr * (zr - 1) * (zr - 2) * (zr - 3))) * pow(argpq, -4) *
                                cos((zr - 3) * atan(2.0 * argpq)) / pow(1.0 + 4 * argpq * argpq, (zr - 3) / 2.0);
            pqr = (4. / M_PI) * (pqr1 - pqr2 - (9. / 8.0) * pqr3);
        }
        return pql * pqr;
    }
    if (P->cs == 1) return pql * cyl_cross_coreshell(P, q, zr);
    return 0.0;
}

/* formpq_partDisk, isotropic, homogeneous: Source/sc_lib_formpq_partDisk.h:17-36 (longitudinal)
   and :313-339 (cross-section) */
static double formpq_partDisk_iso(const cs_prepared *P, double q) {
    const double zl = (1 - sqr(P->sigmal)) / sqr(P->sigmal);
    const double zr = (1 - sqr(P->sigma)) / (sqr(P->sigma));
    double pql, pqr;
    if (q < (0.5 * P->limq[1])) {
        pql = 1.0;
        double oldpqsum = 0.0, qqnn = 1.0;
        for (int nser = 1; nser <= 80; nser++) {
            qqnn = qqnn * q * q;
            pql += P->carrp[0][nser] * qqnn;
            const double delser = fabs((pql - oldpqsum) / pql);
            if (delser < 0.0001) break;
            oldpqsum = pql;
        }
    } else {
        const double arglq = q * P->length / (zl + 1);
        pql = (2 / (zl * (zl - 1))) * pow(arglq, -2);
    }
    if (q < (0.5 * P->limq[4])) {
        pqr = series_q(P->carrp[3], q, 100);
    } else {
        const double argpq = q * P->radius / (zr + 1);
        pqr = (1 / (2.0 * zr * (zr - 1))) * pow(argpq, -2) *
              (1 - cos((zr - 1) * atan(2.0 * argpq)) / pow(1.0 + 4 * argpq * argpq, (zr - 1) / 2.0));
    }
    return pql * pqr;
}

/* formpq_partDisk, homogeneous disk with the Gaussian orientation
   distribution along an axis (ordis 0), Source/sc_lib_formpq_partDisk.h:137-236,
   times its transverse part (:310-340). orcase is compared with 1..3 as the
   reference compares it: the x axis switches to the quadrature at 6 limq1, the
   y and z axes at 6000 limq1. */
static double formpq_partDisk_gauss(const cs_prepared *P, double qx, double qy, double qxs, double qys, double q) {
    const double zr = (1 - sqr(P->sigma)) / (sqr(P->sigma));
    double pql, pqr;
    if (q < ((P->orcase == 1 ? 6.0 : 6000.0) * P->limq[1])) {
        double qxn[121], qyn[121];
        double oldpqsum = 0.0, qqnn = 1.0;
        pql = 1.0;
        qxn[0] = 1.0;
        qyn[0] = 1.0;
        for (int nser = 1; nser <= 120; nser++) {
            qqnn = qqnn * q * q;
            qxn[nser] = qxn[nser - 1] * qxs * qxs;
            qyn[nser] = qyn[nser - 1] * qys * qys;
            double binsum = 0.0;
            for (int mser = 0; mser <= nser; mser++) {
                double binsum1 = 0.0;
                for (int lser = 0; lser <= mser; lser++) binsum1 += 1.0 * qxn[lser] * qyn[mser - lser]; /* carr22pm = 1 */
                binsum += P->carr11pm[nser][mser] * binsum1;
            }
            pql += P->carrp[0][nser] * qqnn * binsum;
            const double delser = fabs((pql - oldpqsum) / pql);
            if (delser < 0.0001) break;
            oldpqsum = pql;
        }
    } else {
        pql = qrombdeltac_carr(P, P->sigmal, P->poltheta, P->polphi, qx, qy, P->orcase + 7, P->carrp[1]);
        pql = pql / P->norm;
    }
    if (q < (0.5 * P->limq[4])) {
        pqr = series_q(P->carrp[3], q, 100);
    } else {
        const double argpq = q * P->radius / (zr + 1);
        pqr = (1 / (2.0 * zr * (zr - 1))) * pow(argpq, -2) *
              (1 - cos((zr - 1) * atan(2.0 * argpq)) / pow(1.0 + 4 * argpq * argpq, (zr - 1) / 2.0));
    }
    return pql * pqr;
}

/* formfq_partCylinder, Source/sc_lib_formfq_partCylinder.h:8-216 (ordis 0/6, cs 0) */
static double formfq_partCylinder(const cs_prepared *P, double limql, double qxs, double qys, double q) {
    const double zl = (1 - sqr(P->sigmal)) / sqr(P->sigmal);
    const double zr = (1 - sqr(P->sigma)) / sqr(P->sigma);
    double pql = 0, pqr = 0;
    if (P->ordis == 6) {
        if (P->orcase == 4)
            pql = 1.0;
        else if (limql < (0.6 * P->limqf[1])) {
            double pqsum = 1.0, oldpqsum = 0.0, qqnn = 1.0;
            for (int nser = 1; nser <= 120; nser++) {
                qqnn = qqnn * (qxs + qys) * (qxs + qys);
                pqsum = pqsum + P->carrf[0][nser] * qqnn;
                const double delser = fabs((pqsum - oldpqsum) / pqsum);
                if (delser < 0.0001) break;
                oldpqsum = pqsum;
            }
            pql = pqsum;
        } else {
            const double arglq = (qxs + qys + EPS9) * P->length / (zl + 1);
            pql = (1 / (2.0 * zl * (zl - 1))) * (1 / (arglq * arglq)) *
                  (1 - cos((zl - 1) * atan(2.0 * arglq)) / pow(1.0 + 4 * arglq * arglq, (zl - 1) / 2.0));
        }
    }
    if (P->ordis == 0) {
        if (P->orcase == 4)
            pql = 1.0;
        else if (limql < (0.2 * P->limqf[1])) {
            double pqsum = 1.0;
            if (P->orcase == 1) pqsum = cyl_double_series(P, qxs, qys, P->carrf[0], 2);
            if (P->orcase == 2) pqsum = cyl_double_series(P, qxs, qys, P->carrf[0], 0);
            if (P->orcase == 3) pqsum = cyl_double_series(P, qxs, qys, P->carrf[0], 3);
            pql = pqsum;
        } else {
            pql = qrombdeltac4(P, P->sigmal, P->poltheta, 0, qxs, qys, P->orcase);
            pql = pql / P->norm;
        }
    }
    if (P->cs == 0) {
        if (q < (1.0 * P->limqf[4])) {
            pqr = series_q(P->carrf[3], q, 120);
        } else {
            const double argpq = q * P->radius / (zr + 1);
            const double pqr1 = (ref_gamma(zr - 1 / 2.0) / ref_gamma(zr + 1)) * pow(argpq, -3 / 2.0) *
                                (sin((zr - 1 / 2.0) * atan(argpq)) - cos((zr - 1 / 2.0) * atan(argpq))) /
                                pow(1.0 + argpq * argpq, (zr - 1 / 2.0) / 2.0);
            const double pqr2 = (ref_gamma(zr - 3 / 2.0) / ref_gamma(zr + 1)) * pow(argpq, -5 / 2.0) *
                                (sin((zr - 3 / 2.0) * atan(argpq)) + cos((zr - 3 / 2.0) * atan(argpq))) /
                                pow(1.0 + argpq * argpq, (zr - 3 / 2.0) / 2.0);
            const double pqr3 = (2 / sqrt(M_PI)) * (pqr1 + (9 / 16.0) * pqr2);
            pqr = pqr3 * pqr3;
        }
        return pql * pqr;
    }
    return 0.0;
}

/* ------------------------------------------------------------ peak lattices */

static void peak_sums(const cs_prepared *P, double qx, double qy, double qz, double q, double *radint, double *intens) {
    double width = 1;
    if (P->debyescherrer) width = 4.0 / P->domainsize;
    if (P->para) width = (4.0 / P->domainsize) + sqr(P->reldis) * P->dist * sqr(q);
    width *= P->width_zuf;
    const double widthiso = 1.0 / P->uca;
    double radintensity = 0.0, intensity = 0.0;
    for (int ii = 1; ii <= P->peakmax1; ii++) {
        const int mhkl = P->latpar1[ii][4];
        const int fhkl = P->latpar1[ii][5];
        if (mhkl == 0 || fhkl == 0) continue;
        const double qhkl = P->latpar3[ii][5];
        const double x2 = sqr(q - qhkl) / sqr(widthiso);
        const double sq = exp(-4 * x2 / M_PI) / (M_PI * widthiso / 2.0);
        radintensity += sq * mhkl * fhkl;
    }
    for (int ii = 1; ii <= P->peakmax2; ii++) {
        const double qhkl = P->latpar3[ii][5];
        const int mhkl_fhkl = P->latpar2[ii][4] * P->latpar2[ii][5];
        if (qhkl > 0 && mhkl_fhkl != 0) {
            const double qxhkl = P->latpar3[ii][2];
            const double qyhkl = P->latpar3[ii][3];
            const double qzhkl = P->latpar3[ii][4];
            const double g3 = P->latpar3[ii][10];
            const double peaknorm1 = P->latpar3[ii][11];
            const double yphi = myacos((qx * qxhkl + qy * qyhkl + qz * qzhkl) / (q * qhkl));
            const double x2 = (q - qhkl) * (q - qhkl) / (width * width);
            const double sq = exp(-4 * x2 / M_PI) / (M_PI * width / 2.0);
            const double x2phi = 4 * q * q / (M_PI * sqr(P->phiwidth));
            double psiord = g3 * exp(-x2phi * yphi * yphi) / peaknorm1;
            if (P->twin) {
                const double qxhklt = P->latpar3[ii][7];
                const double qyhklt = P->latpar3[ii][8];
                const double qzhklt = P->latpar3[ii][9];
                const double qhklt = P->latpar3[ii][14];
                const double g3t = P->latpar3[ii][15];
                const double peaknorm1t = P->latpar3[ii][16];
                const double yphit = myacos((qx * qxhklt + qy * qyhklt + qz * qzhklt) / (q * qhklt));
                const double phiord = g3t * exp(-x2phi * yphit * yphit) / peaknorm1t;
                psiord = P->ceff * psiord + (1 - P->ceff) * phiord;
            }
            const double savintens = intensity;
            intensity += sq * mhkl_fhkl * psiord;
            if (isinf(intensity)) {
                intensity = savintens;
                break;
            }
        }
    }
    *radint = radintensity;
    *intens = intensity;
}

/* calc_GENERIC's lattice factor, Source/sc_gpu_generic.h:511-846: the isotropic
   peak sum with the isotropic width 1/uca, then the oriented peaks with the
   selected peak shape (1 Lorentzian, 2 Gaussian, 3/4 modified Lorentzians,
   5 pseudo-Voigt, 6 Pearson VII, 8 anisotropic Gaussian for perfect or
   isotropic orientation; any other shape returns 0 for the pixel). Both sums
   keep their last finite value when a term makes them infinite or NaN. The
   twin's angle is normalised by q_hkl, not by the twin's own |q_hkl|.
   Returns 0 when the shape has no branch. */
static int peak_sums_generic(const cs_prepared *P, double qx, double qy, double qz, double q, double *radint,
                             double *intens) {
    const double c0 = 1.0; /* Source/sc_calc_generic_cpu.cpp:585 */
    const double siglen = sqrt(sqr(P->sig[0]) + sqr(P->sig[1]) + sqr(P->sig[2]));
    double width = 1;
    if (P->debyescherrer) width = 4.0 / P->domainsize;
    if (P->para) width = (4.0 / P->domainsize) + sqr(P->reldis) * P->dist * sqr(q);
    if (P->lattice && P->shp == 8 && P->ordis == 7) width = siglen / 3.0;
    width *= P->width_zuf;
    const double widthiso = 1.0 / P->uca;
    double radintensity = 0.0, intensity = 0.0;
    for (int ii = 1; ii <= P->peakmax1; ii++) {
        const double qhkl = P->latpar3[ii][5];
        const double x2 = sqr(q - qhkl) / sqr(widthiso);
        const double sq = exp(-4 * x2 / M_PI) / (M_PI * widthiso / 2.0);
        const double keep = radintensity;
        radintensity += sq * P->latpar1[ii][4] * P->latpar1[ii][5];
        if (isinf(radintensity) || isnan(radintensity)) {
            radintensity = keep;
            break;
        }
    }
    /* ax_k.length() * sig_k, Source/sc_calc_generic_cpu.cpp:396-398 */
    const double a1n = sqrt(sqr(P->ax1[0]) + sqr(P->ax1[1]) + sqr(P->ax1[2])) * P->sig[0];
    const double a2n = sqrt(sqr(P->ax2[0]) + sqr(P->ax2[1]) + sqr(P->ax2[2])) * P->sig[1];
    const double a3n = sqrt(sqr(P->ax3[0]) + sqr(P->ax3[1]) + sqr(P->ax3[2])) * P->sig[2];
    for (int ii = 1; ii <= P->peakmax2; ii++) {
        const double qhkl = P->latpar3[ii][5];
        if (qhkl <= 0 || isnan(qhkl)) continue;
        const int mhkl = P->latpar2[ii][4], fhkl = P->latpar2[ii][5];
        const double hx = P->latpar3[ii][2], hy = P->latpar3[ii][3], hz = P->latpar3[ii][4];
        const double tx = P->latpar3[ii][7], ty = P->latpar3[ii][8], tz = P->latpar3[ii][9];
        const double g3 = P->latpar3[ii][10];
        const double pn1 = P->latpar3[ii][11];
        double sq = 1.0, psiord = 1.0;
        if (P->shp == 8) {
            /* perfect orientation (ordis 6 or dbeta 0): a Gaussian ellipsoid
               along the cell axes around the peak; isotropic: a radial
               Gaussian of width |sig|/3 */
            double term[2];
            for (int t = 0; t < 2; t++) {
                const double px = t ? tx : hx, py = t ? ty : hy, pz = t ? tz : hz;
                if (P->ordis == 6 || fabs(P->dbeta) < EPS9) {
                    const double dx = qx - px, dy = qy - py, dz = qz - pz;
                    const double s1 = (dx * P->ax1[0] + dy * P->ax1[1] + dz * P->ax1[2]) / a1n;
                    const double s2 = (dx * P->ax2[0] + dy * P->ax2[1] + dz * P->ax2[2]) / a2n;
                    const double s3 = (dx * P->ax3[0] + dy * P->ax3[1] + dz * P->ax3[2]) / a3n;
                    const double x2 = s1 * s1 + s2 * s2 + s3 * s3;
                    term[t] = exp(-4 * x2 / M_PI) /
                              (sqrt(M_PI * M_PI * M_PI) * P->sig[0] * P->sig[1] * P->sig[2] / 8.0);
                } else {
                    const double lw = siglen / 3.0;
                    const double x2 = (q - qhkl) * (q - qhkl) / (lw * lw);
                    term[t] = g3 * exp(-4 * x2 / M_PI) / (M_PI * lw / 2.0);
                }
            }
            /* without a twin the peak's own term; with one, sq keeps 1 and is
               mixed with the twin's term (:600-661) */
            if (!P->twin) sq = term[0];
            else sq = P->ceff * sq + (1 - P->ceff) * term[1];
        } else {
            if (P->shp < 1 || P->shp > 6) return 0;
            const double x2 = (q - qhkl) * (q - qhkl) / (width * width);
            const double cphi[2] = {(qx * hx + qy * hy + qz * hz) / (q * qhkl), (qx * tx + qy * ty + qz * tz) / (q * qhkl)};
            double ord[2];
            for (int t = 0; t < (P->twin ? 2 : 1); t++) {
                const double y = myacos(cphi[t]);
                const double b = 4 * q * q / sqr(P->phiwidth); /* b/c factors */
                const double a = 4 * q * q / (M_PI * sqr(P->phiwidth)); /* a factor */
                switch (P->shp) {
                case 1: ord[t] = g3 / (pn1 * (1 + b * y * y)); break;
                case 2: ord[t] = g3 * exp(-a * y * y) / pn1; break;
                case 3: ord[t] = g3 / (pn1 * (1 + b * y * y) * (1 + b * y * y)); break;
                case 4: ord[t] = g3 / (pn1 * exp(3 * log(1 + b * y * y) / 2.0)); break;
                case 5: {
                    const double e = P->pk_eta;
                    ord[t] = g3 * (e * (1 / (1 + b * y * y)) + (1 - e) * exp(-a * y * y)) /
                             (e * pn1 + (1 - e) * P->latpar3[ii][12]);
                    break;
                }
                default: ord[t] = g3 / (pn1 * exp(P->pk_beta * log(1 + b * y * y))); break;
                }
            }
            switch (P->shp) {
            case 1: sq = sqrt(P->pk_c1) / (M_PI * width * (1.0 + P->pk_c1 * x2)); break;
            case 2: sq = exp(-4 * x2 / M_PI) / (M_PI * width / 2.0); break;
            case 3: sq = 2 * sqrt(P->pk_c2) / (M_PI * width * (1 + P->pk_c1 * x2) * (1 + P->pk_c1 * x2)); break;
            case 4: sq = sqrt(P->pk_c3) / (2 * width * exp(3 * log(1 + P->pk_c1 * x2) / 2.0)); break;
            case 5:
                sq = P->pk_eta * sqrt(P->pk_c1) / (M_PI * width * (1 + P->pk_c1 * x2)) +
                     (1 - P->pk_eta) * sqrt(c0) * exp(-c0 * x2) / (sqrt(M_PI) * width);
                break;
            default:
                sq = ref_gamma(P->pk_beta) * P->pk_c4 * 2 /
                     (ref_gamma(P->pk_beta - 0.5) * M_PI * width * exp(P->pk_beta * log(1 + 4 * P->pk_c4 * x2)));
                break;
            }
            psiord = ord[0];
            if (P->twin) psiord = P->ceff * psiord + (1 - P->ceff) * ord[1];
        }
        const double keep = intensity;
        intensity += sq * mhkl * fhkl * psiord;
        if (isinf(intensity) || isnan(intensity)) {
            intensity = keep;
            break;
        }
    }
    *radint = radintensity;
    *intens = intensity;
    return 1;
}

/* szq and szqiso of calc_GENERIC on a lattice, :848-851, from the peak sums */
static int lattice_factors_generic(const cs_prepared *P, double qx, double qy, double qz, double q, double pq, double fq,
                                   double *szq, double *szqiso) {
    double radintensity, intensity;
    if (!peak_sums_generic(P, qx, qy, qz, q, &radintensity, &intensity)) return 0;
    const double sphno_cubevol = P->latpar[1] * P->latpar[2];
    *szqiso = (1 + (1) * (8 * M_PI * M_PI * M_PI * radintensity / (4 * M_PI * sphno_cubevol) - 1) * exp(-P->ucb * q * q));
    *szq = (1 + (fq / pq) * (2 * M_PI * intensity / (sphno_cubevol)-1) * exp(-P->dwfactor * q * q));
    return 1;
}

/* ------------------------------------------------------- pixel functions */

double oracle_pixel_q(const cs_prepared *P, double qx, double qy, double qz) {
    const double q = sqrt(qx * qx + qy * qy + qz * qz) + EPS9;
    switch (P->key) {
    case CS_KEY_SPHERE_NONE_ISO: {
        const double pq = formpq_partSphere(P, q);
        return P->base + P->izero * (pq + P->iso * pq) + P->ifluc / (1 + q * q * P->rfluc * P->rfluc);
    }
    case CS_KEY_SPHERE_GAUSS_FCC_GAUSS: {
        const double pq = formpq_partSphere(P, q);
        const double fq = formfq_partSphere(P, q);
        const double pqiso = pq;
        double radintensity, intensity;
        peak_sums(P, qx, qy, qz, q, &radintensity, &intensity);
        const double sphno_cubevol = P->latpar[1] * P->latpar[2];
        const double szqiso =
            (1 + (1) * (8 * M_PI * M_PI * M_PI * radintensity / (4 * M_PI * sphno_cubevol) - 1) * exp(-P->ucb * q * q));
        const double szq = (1 + (fq / pq) * (2 * M_PI * intensity / sphno_cubevol - 1) * exp(-P->dwfactor * q * q));
        return P->base + P->izero * (szq * pq + P->iso * szqiso * pqiso) + P->ifluc / (1 + q * q * P->rfluc * P->rfluc);
    }
    case CS_KEY_CYL_NONE_GAUSS: {
        double pq = 0;
        switch (P->orcase) {
        case CS_ORC_GENERAL:
            pq = formpq_partCylinder(P, qx * P->cosphic - qy * P->sinphic, qx * P->sinphic + qy * P->cosphic, q);
            break;
        default: pq = formpq_partCylinder(P, qx, qy, q); break;
        }
        return P->base + P->izero * (pq + P->iso) + P->ifluc / (1 + q * q * P->rfluc * P->rfluc);
    }
    case CS_KEY_CYL_NONE_ZDIR: {
        double pq = 0;
        switch (P->orcase) {
        case CS_ORC_GENERAL: pq = formpq_partCylinder(P, qx * P->cosphi * P->sintheta, qy * P->sinphi * P->sintheta, q); break;
        case CS_ORC_XAXIS: pq = formpq_partCylinder(P, qx, 0, q); break;
        case CS_ORC_YAXIS: pq = formpq_partCylinder(P, 0, qy, q); break;
        default: pq = formpq_partCylinder(P, qx, qy, q); break;
        }
        return P->base + P->izero * (pq + P->iso) + P->ifluc / (1 + q * q * P->rfluc * P->rfluc);
    }
    case CS_KEY_CYL_GAUSS_BCT_ZDIR: {
        double pq = 0, fq = 0;
        const double pqiso = 1;
        switch (P->orcase) {
        case CS_ORC_GENERAL:
            pq = formpq_partCylinder(P, qx * P->cosphi * P->sintheta, qy * P->sinphi * P->sintheta, q);
            fq = formfq_partCylinder(P, sqrt(P->cosphi * qx * qx + P->sinphi * qy * qy + EPS9),
                                     qx * P->cosphi * P->sintheta, qy * P->sinphi * P->sintheta, q);
            break;
        case CS_ORC_XAXIS:
            pq = formpq_partCylinder(P, qx, 0, q);
            fq = formfq_partCylinder(P, fabs(qx), qx, 0, q);
            break;
        case CS_ORC_YAXIS:
            pq = formpq_partCylinder(P, 0, qy, q);
            fq = formfq_partCylinder(P, fabs(qy), 0, qy, q);
            break;
        default:
            pq = formpq_partCylinder(P, qx, qy, q);
            fq = formfq_partCylinder(P, q, qx, qy, q);
            break;
        }
        double radintensity, intensity;
        peak_sums(P, qx, qy, qz, q, &radintensity, &intensity);
        const double sphno_cubevol = P->latpar[1] * P->latpar[2];
        const double szqiso =
            (1 + (1) * (8 * M_PI * M_PI * M_PI * radintensity / (4 * M_PI * sphno_cubevol) - 1) * exp(-P->ucb * q * q));
        const double szq = (1 + (fq / pq) * (2 * M_PI * intensity / (sphno_cubevol)-1) * exp(-P->dwfactor * q * q));
        return P->base + P->izero * (szq * pq + P->iso * szqiso * pqiso) + P->ifluc / (1 + q * q * P->rfluc * P->rfluc);
    }
    case CS_KEY_CUBE_NONE_ISO: {
        /* calc_partCube_lattNone_ordisIsotropic, Source/sc_gpu_pCub_lNon_oIso.h:16-77, with
           formpq_partCube's homogeneous isotropic branch, Source/sc_lib_formpq_partCube.h:21-62 */
        double pq = 1.0;
        if (P->cs == 0) {
            if (q < 1.2 * P->limq[4])
                pq = series_q(P->carrp[3], q, 120);
            else
                pq = P->por / (q * q * q * q);
        }
        return P->base + P->izero * (pq + P->iso) + P->ifluc / (1 + q * q * P->rfluc * P->rfluc);
    }
    case CS_KEY_GENERIC:
        /* calc_GENERIC, Source/sc_gpu_generic.h:27-881, for the combinations
           restated here: homogeneous spheres and homogeneous z-direction
           cylinders on any lattice with the peak shapes 1-8; without a
           lattice (szq = szqiso = 1) isotropic cylinders (cs 0/1), isotropic
           homogeneous disks and homogeneous disks with the Gaussian
           orientation along an axis */
        if (P->particle == 0 && P->lattice) {
            /* spheres, :44-58, on a lattice */
            const double pq = formpq_partSphere(P, q);
            const double fq = formfq_partSphere(P, q);
            double szq, szqiso;
            if (!lattice_factors_generic(P, qx, qy, qz, q, pq, fq, &szq, &szqiso)) return 0.0;
            return P->base + P->izero * (szq * pq + P->iso * szqiso * pq) + P->ifluc / (1 + q * q * P->rfluc * P->rfluc);
        }
        if (P->particle == 1 && P->ordis == 6 && P->lattice) {
            /* z-direction cylinders, :318-353, on a lattice (pqiso stays 1) */
            double pq = 0, fq = 0;
            switch (P->orcase) {
            case CS_ORC_GENERAL:
                pq = formpq_partCylinder(P, qx * P->cosphi * P->sintheta, qy * P->sinphi * P->sintheta, q);
                fq = formfq_partCylinder(P, sqrt(P->cosphi * qx * qx + P->sinphi * qy * qy + EPS9),
                                         qx * P->cosphi * P->sintheta, qy * P->sinphi * P->sintheta, q);
                break;
            case CS_ORC_XAXIS:
                pq = formpq_partCylinder(P, qx, 0, q);
                fq = formfq_partCylinder(P, fabs(qx), qx, 0, q);
                break;
            case CS_ORC_YAXIS:
                pq = formpq_partCylinder(P, 0, qy, q);
                fq = formfq_partCylinder(P, fabs(qy), 0, qy, q);
                break;
            default:
                pq = formpq_partCylinder(P, qx, qy, q);
                fq = formfq_partCylinder(P, q, qx, qy, q);
                break;
            }
            double szq, szqiso;
            if (!lattice_factors_generic(P, qx, qy, qz, q, pq, fq, &szq, &szqiso)) return 0.0;
            return P->base + P->izero * (szq * pq + P->iso * szqiso * 1.0) + P->ifluc / (1 + q * q * P->rfluc * P->rfluc);
        }
        if (P->particle == 1 && P->ordis == 7) {
            const double pq = formpq_partCylinder(P, qx, qy, q);
            return P->base + P->izero * (pq + P->iso * 1.0) + P->ifluc / (1 + q * q * P->rfluc * P->rfluc);
        }
        if (P->particle == 2 && P->ordis == 7) {
            const double pq = formpq_partDisk_iso(P, q);
            const double pqiso = (P->iso > 0) ? formpq_partDisk_iso(P, q) : (double)0.0;
            return P->base + P->izero * (pq + P->iso * pqiso) + P->ifluc / (1 + q * q * P->rfluc * P->rfluc);
        }
        if (P->particle == 2 && P->ordis == 0) {
            /* :255-288, orcXaxis and orcYaxis pass qx/q, qy/q, orcZaxis qx, qy */
            const double pq = P->orcase == 3 ? formpq_partDisk_gauss(P, qx, qy, qx, qy, q)
                                             : formpq_partDisk_gauss(P, qx, qy, qx / q, qy / q, q);
            const double pqiso = (P->iso > 0) ? formpq_partDisk_iso(P, q) : (double)0.0;
            return P->base + P->izero * (pq + P->iso * pqiso) + P->ifluc / (1 + q * q * P->rfluc * P->rfluc);
        }
        return NAN;
    default:
        return NAN;
    }
}

int oracle_supported(const cs_prepared *P) {
    if (P->ign_switch) return 0;
    switch (P->key) {
    case CS_KEY_SPHERE_NONE_ISO:
    case CS_KEY_SPHERE_GAUSS_FCC_GAUSS:
    case CS_KEY_CYL_NONE_GAUSS:
    case CS_KEY_CYL_NONE_ZDIR:
    case CS_KEY_CYL_GAUSS_BCT_ZDIR:
    case CS_KEY_CUBE_NONE_ISO: return 1;
    case CS_KEY_GENERIC:
        if (P->lattice && P->cs == 0 && (P->particle == 0 || (P->particle == 1 && P->ordis == 6))) return 1;
        return !P->lattice &&((P->ordis == 7 && ((P->particle == 1 && (P->cs == 0 || P->cs == 1)) ||
                                                  (P->particle == 2 && P->cs == 0))) ||
                               (P->ordis == 0 && P->particle == 2 && P->cs == 0 && P->orcase >= 1 &&
                                P->orcase <= 3));
    default: return 0;
    }
}

/* Image extents, calculated region and dispatch key of a prepared block, for
   callers that hold the block as raw bytes:
   e = {xmin, xmax, ymin, ymax, zzmin, zzmax, iimin, iimax, key}. */
void oracle_extents(const cs_prepared *P, int *e) {
    e[0] = P->xmin;
    e[1] = P->xmax;
    e[2] = P->ymin;
    e[3] = P->ymax;
    e[4] = P->zzmin;
    e[5] = P->zzmax;
    e[6] = P->iimin;
    e[7] = P->iimax;
    e[8] = P->key;
}

/* hook on the pixel's q vector (the high-precision build uses it to move q by
   a few double ulps and measure how much the exact value depends on it) */
#ifndef CS_ORACLE_Q_HOOK
#define CS_ORACLE_Q_HOOK(qx, qy, qz)
#endif

double oracle_pixel(const cs_prepared *P, int ihex, int i) {
    double qx, qy, qz;
    convert_idx2q(P, ihex, i, &qx, &qy, &qz);
    CS_ORACLE_Q_HOOK(qx, qy, qz);
    return oracle_pixel_q(P, qx, qy, qz);
}

/* ------------------------------------------------------------ image loops */

typedef struct {
    const cs_prepared *P;
    double *out;
    int next_row, row_end;
    const int *list; /* when set: rows list[next_row], next_row < row_end */
    pthread_mutex_t lock;
} row_queue;

static void *row_worker(void *arg) {
    row_queue *Q = (row_queue *)arg;
    const cs_prepared *P = Q->P;
    const int xs = P->xmax - P->xmin;
    for (;;) {
        pthread_mutex_lock(&Q->lock);
        int pos = Q->next_row++;
        pthread_mutex_unlock(&Q->lock);
        if (pos >= Q->row_end) break;
        const int ihex = Q->list ? Q->list[pos] : pos;
        if (ihex < P->zzmin || ihex >= P->zzmax) continue;
        /* one image row per step as the reference's threads (doThreadCalculation) */
        for (int i = P->iimin; i < P->iimax; i++)
            Q->out[(long)(ihex - P->xmin) + (long)xs * (long)(i - P->ymin)] = oracle_pixel(P, ihex, i);
    }
    return NULL;
}

/* Computes the ihex rows listed in rows[0..nrows) (a sample of the image;
   rows outside the calculated region are skipped) with nthreads threads.
   Returns the pixel count. */
long oracle_image_rowlist(const cs_prepared *P, double *out, const int *rows, int nrows, int nthreads) {
    if (!oracle_supported(P)) return -1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 512) nthreads = 512;
    row_queue Q;
    Q.P = P;
    Q.out = out;
    Q.next_row = 0;
    Q.row_end = nrows;
    Q.list = rows;
    pthread_mutex_init(&Q.lock, NULL);
    pthread_t th[512];
    int started = 0;
    for (int t = 0; t < nthreads; t++)
        if (pthread_create(&th[t], NULL, row_worker, &Q) == 0) started++;
        else break;
    if (started == 0) row_worker(&Q);
    for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
    pthread_mutex_destroy(&Q.lock);
    long n = 0;
    for (int r = 0; r < nrows; r++)
        if (rows[r] >= P->zzmin && rows[r] < P->zzmax) n += P->iimax - P->iimin;
    return n;
}

/* Computes the ihex rows [row0,row1) of the calculated region (all rows when
   row1 <= row0) with nthreads threads, then mirrors quadrants like
   doCalculation when the whole region was computed. Returns the pixel count. */
long oracle_image_rows(const cs_prepared *P, double *out, int row0, int row1, int nthreads) {
    if (!oracle_supported(P)) return -1;
    if (row1 <= row0) {
        row0 = P->zzmin;
        row1 = P->zzmax;
    }
    if (row0 < P->zzmin) row0 = P->zzmin;
    if (row1 > P->zzmax) row1 = P->zzmax;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 512) nthreads = 512;
    row_queue Q;
    Q.P = P;
    Q.out = out;
    Q.next_row = row0;
    Q.row_end = row1;
    Q.list = NULL;
    pthread_mutex_init(&Q.lock, NULL);
    if (nthreads == 1)
        row_worker(&Q);
    else {
        pthread_t th[512];
        int started = 0;
        for (int t = 0; t < nthreads; t++)
            if (pthread_create(&th[t], NULL, row_worker, &Q) == 0) started++;
            else break;
        if (started == 0) row_worker(&Q);
        for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
    }
    pthread_mutex_destroy(&Q.lock);
    const int full = (row0 == P->zzmin && row1 == P->zzmax);
    if (full && P->expand && P->calc_quadrants != CS_RADQ4 && P->calc_quadrants != CS_RAD1D) {
        const int zmax = P->zmax, xs = P->xmax - P->xmin;
#define AT(x, y) out[(long)((x)-P->xmin) + (long)xs * (long)((y)-P->ymin)]
        if (P->calc_quadrants == CS_RADQ1) {
            for (int ihex = 0; ihex < zmax; ihex++)
                for (int i = 0; i < zmax; i++) {
                    AT(-ihex, i) = AT(ihex, i);
                    AT(-ihex, -i - 1) = AT(ihex, i);
                    AT(ihex, -i - 1) = AT(ihex, i);
                }
        } else {
            for (int ihex = 0; ihex < zmax; ihex++)
                for (int i = -zmax + 1; i < zmax; i++) AT(-ihex, -i) = AT(ihex, i);
        }
#undef AT
    }
    return (long)(row1 - row0) * (long)(P->iimax - P->iimin);
}

/* doFitCalculation on the CPU: FQS per pixel and the sequential sum. The
   prepared block must carry the fit geometry (fit_width ..., nofit_*). */
double oracle_fit(const cs_prepared *P, const double *data, double *fqs, long *cnt, long *nancnt) {
    const int w = P->fit_width, h = P->fit_height;
    const int xs = P->xmax - P->xmin;
    const long nbuf = (long)w * h;
    for (long t = 0; t < nbuf; t++) fqs[t] = 0.0;
    for (int x0 = 0; x0 < w; x0++)
        for (int y0 = 0; y0 < h; y0++) {
            int x = x0, y = y0, skip = 0;
            for (int i = 0; i < 4 && !skip; i++) {
                if (P->nofit_x0[i] < 0) continue;
                if (x < P->nofit_x0[i]) continue;
                if (P->nofit_x1[i] < x) continue;
                if (y < P->nofit_y0[i]) continue;
                if (P->nofit_y1[i] < y) continue;
                fqs[x + (long)w * y] = 0.0;
                skip = 1;
            }
            if (skip) continue;
            if (P->fit_border > 0 || P->fit_bstop > 0) {
                if (x < P->xmin + P->fit_border || x >= P->xmax - P->fit_border || y < P->ymin + P->fit_border ||
                    y >= P->ymax - P->fit_border) {
                    fqs[x + (long)w * y] = 0.0;
                    continue;
                }
                if (x >= P->beamx0 - P->fit_bstop && x < P->beamx0 + P->fit_bstop && y >= P->beamy0 - P->fit_bstop &&
                    y < P->beamy0 + P->fit_bstop) {
                    fqs[x + (long)w * y] = 0.0;
                    continue;
                }
            } else if (P->fit_bstop == -1) {
                const long idx = x + (long)w * y;
                if (data[idx] <= data[0]) {
                    fqs[idx] = 0.0;
                    continue;
                }
            }
            x += P->iimin;
            y += P->iimin;
            const double pixval = oracle_pixel(P, x, y);
            const long idx = (long)(x - P->xmin) + (long)xs * (long)(y - P->ymin);
            if (idx < 0 || idx >= nbuf) continue;
            if (pixval > 0 && data[idx] > 0)
                fqs[idx] = sqr(log(pixval) / log(10.) - log(data[idx]) / log(10.));
            else
                fqs[idx] = 0.0;
        }
    double erg = 0.0;
    long c = 0, nn = 0;
    for (long i = 0; i < nbuf; i++) {
        if (isnan(fqs[i]))
            nn++;
        else {
            if (fqs[i] != 0) c++;
            erg += fqs[i];
        }
    }
    if (cnt) *cnt = c;
    if (nancnt) *nancnt = nn;
    return erg;
}
