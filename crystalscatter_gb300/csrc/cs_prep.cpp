// cs_prep.cpp — host preparation of one parameter set.
//
// Restates the host side of the reference calculation class for the paths this
// library implements: parameter validation (checkAllParameters / isCbsValid,
// Source/sc_calc_generic_cpu.cpp:119-308), prepareCalculation
// (sc_calc_generic_cpu.cpp:319-988), the reached branches of coefficients()
// (sc_calc_generic_cpu.cpp:2099-8195), the reflection tables of ButtonHKLClick
// (:8246-10295), fhkl_c (:10299) and corotations (:1487-2098).
//
// The coefficient recurrences keep the reference's operand types (double,
// float and long double exactly where the reference declares them) and its
// operation order: the series coefficients feed 1e-10 parity tests, and the
// series/asymptote switch points limqN are data-dependent thresholds whose
// value decides branches per pixel. This translation unit must be compiled
// without floating-point contraction (-ffp-contract=off).

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "cs_prep.h"
#include "cs_launch.h"

namespace cs {

namespace {

constexpr int kNmax = 120;           // nnmax, sc_calc_generic_cpu.cpp:2102
constexpr double kMin = 1E-30;       // min, :2103
constexpr double kEps9 = 0.000000001; // eps9, Source/sc_math.h:45
constexpr double kEps3 = 0.001;       // eps3, Source/sc_math.h:39

inline double sqr(double x) { return x * x; }

// Threads for the per-n loops of coefficients(): the O(n^2) sums over
// long-double factorials (software-emulated quad precision on aarch64) are
// independent for different n once the recurrences are done. A thread that
// prepares many sets at once (a batch worker) keeps them serial.
thread_local int t_prep_threads = 0;  // 0: min(8, hardware threads)

}  // namespace

void set_prep_threads(int n) { t_prep_threads = n; }

namespace {

int prep_threads() {
    if (t_prep_threads > 0) return t_prep_threads;
    const unsigned hw = std::thread::hardware_concurrency();
    return (int)std::max(1u, std::min(8u, hw));
}

// Persistent workers for parallel_n (created on first use). Tasks n are taken
// from an atomic counter; the calling thread works too. One loop at a time: a
// caller that finds the pool busy (another thread preparing) runs serially.
class PrepPool {
public:
    static PrepPool &get() {
        // never destroyed: its detached workers wait on its condition
        // variable until the process ends
        static PrepPool *pool = new PrepPool;
        return *pool;
    }
    bool try_run(int lo, int hi, int threads, const std::function<void(int)> &f) {
        std::unique_lock<std::mutex> busy(run_mu_, std::try_to_lock);
        if (!busy.owns_lock()) return false;
        ensure(threads - 1);
        {
            std::lock_guard<std::mutex> lk(mu_);
            job_ = &f;
            hi_ = hi;
            next_.store(lo);
            active_ = (int)workers_.size();
            gen_++;
        }
        cv_.notify_all();
        work();
        std::unique_lock<std::mutex> lk(mu_);
        done_cv_.wait(lk, [&] { return active_ == 0; });
        job_ = nullptr;
        return true;
    }

private:
    std::vector<std::thread> workers_;
    std::mutex run_mu_, mu_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(int)> *job_ = nullptr;
    std::atomic<int> next_{0};
    int hi_ = 0, active_ = 0;
    unsigned long gen_ = 0;

    void work() {
        for (;;) {
            const int n = next_.fetch_add(1);
            if (n > hi_) break;
            (*job_)(n);
        }
    }
    void ensure(int n) {
        while ((int)workers_.size() < n) {
            // the worker starts from the generation current now, before the
            // caller publishes the next job (a worker that read gen_ only
            // once running could miss that job and wait forever)
            unsigned long start;
            {
                std::lock_guard<std::mutex> lk(mu_);
                start = gen_;
            }
            workers_.emplace_back([this, start] {
                unsigned long seen = start;
                for (;;) {
                    {
                        std::unique_lock<std::mutex> lk(mu_);
                        cv_.wait(lk, [&] { return gen_ != seen; });
                        seen = gen_;
                    }
                    work();
                    {
                        std::lock_guard<std::mutex> lk(mu_);
                        active_--;
                    }
                    done_cv_.notify_one();
                }
            });
            workers_.back().detach();
        }
    }
};

// f(n) for n in [lo, hi] on the pool; every value is computed by the same
// operations as in a serial loop, only the order of independent n differs
template <class F>
void parallel_n(int lo, int hi, const F &f) {
    const int T = prep_threads();
    if (T > 1 && hi - lo >= 32) {
        const std::function<void(int)> fn = [&f](int n) { f(n); };
        if (PrepPool::get().try_run(lo, hi, T, fn)) return;
    }
    for (int n = lo; n <= hi; n++) f(n);
}

// log2 of a positive double, good to ~1e-15 absolute: the exponent from frexp
// (exact), the mantissa in [0.5, 1) through log2.
inline double lg2(double v) {
    int e;
    const double m = std::frexp(v, &e);
    return e + std::log2(m);
}

// log2 of the largest term that `acc += term` (term computed in long double,
// sum rounded to double) provably leaves unchanged, with a factor 16 to spare:
// a term below 1/8 ulp of a non-zero acc keeps the long-double sum strictly
// inside acc's rounding interval (also below a power of two, where the
// interval is ulp/4 wide on the lower side); a non-negative term below 2^-1075
// added to +0 rounds back to +0.
inline double negligible_lg2(double acc) {
    if (acc == 0.0) return -1076.0 - 4.0;
    int e;
    std::frexp(acc, &e);
    const int ulp = std::max(e - 53, -1074);
    return ulp - 3 - 4.0;
}

// cospi(v) of Source/sc_math.h:52 (1-2*(v&1)).
inline int cospi_i(int v) { return 1 - 2 * (v & 1); }

// ---------------------------------------------------------------------------
// One-dimensional Romberg integration over the orientation angle delta, the
// i0 = 1, 2, 3 integrands of qrombdeltac/trapzddeltac
// (Source/sc_calc_generic_gpu.cu:1370-1488, 956-1272) with i2 = 0 (Gaussian).
// polint (Neville extrapolation to 0, :1280-1335) is reproduced with its
// operation order; its abscissae are always 1, 1/4, 1/16, 1/64, 1/256 times a
// power of two, which leaves every rounding identical to the first window.
// ---------------------------------------------------------------------------
void polint5(const double *ya /*1..5*/, double &y, double &dy) {
    const double xa[6] = {0.0, 1.0, 0.25, 0.0625, 0.015625, 0.00390625};
    double c[7], d[7];
    int ns = 1;
    double dif = std::fabs(xa[1]);
    for (int i = 1; i <= 5; i++) {
        double dift = std::fabs(xa[i]);
        if (dift < dif) {
            ns = i;
            dif = dift;
        }
        c[i] = ya[i];
        d[i] = ya[i];
    }
    y = ya[ns];
    ns = ns - 1;
    for (int m = 1; m <= 4; m++) {
        for (int i = 1; i <= 5 - m; i++) {
            double ho = xa[i];
            double hp = xa[i + m];
            double w = c[i + 1] - d[i];
            double den = ho - hp;
            if (den != 0) den = w / den;
            d[i] = hp * den;
            c[i] = ho * den;
        }
        if (2 * ns < 5 - m)
            dy = c[ns + 1];
        else {
            dy = d[ns];
            ns = ns - 1;
        }
        y = y + dy;
    }
}

double delta_integrand(int i0, double x, double dbeta) {
    if (i0 == 3) return std::sin(x) * std::exp(-x * x / (dbeta * dbeta)) * (3 * std::cos(x) * std::cos(x) - 1) / 2.0;
    return std::sin(x) * std::exp(-x * x / (dbeta * dbeta));  // i0 = 1 and 2
}

// qrombdeltac(..., i0, i1, i2=0, ...) for i0 in {1,2,3}. dbeta_deg in degrees.
double qromb_delta_1d(int i0, int i1, double dbeta_deg) {
    const double eps = 1.0e-4;
    const int jmax = 20;
    const int k = 5;
    const double prmin = 0.00001;
    double dbeta = dbeta_deg * M_PI / 180.0;
    double delmax = dbeta * std::sqrt(std::log(1.0 / prmin));
    if (delmax > M_PI / 2.0) delmax = M_PI / 2.0;
    float alim = 0.0;
    float blim = delmax;
    if (i1 == 12) {
        alim = eps;
        blim = M_PI / 2.0 - eps;
    }
    if (i1 == 17) {
        alim = 0.0001;
        blim = M_PI / 2.0 - 0.0001;
    }
    const double a = alim, b = blim;
    double sp[jmax + 3];
    double pq = 0.0, dssp = 0.0;
    int cnt = 0;
    for (int j = 1; j <= jmax; j++) {
        // trapzddeltac(n=j)
        if (j == 1) {
            double pa = delta_integrand(i0, a, dbeta);
            double pb = delta_integrand(i0, b, dbeta);
            sp[j] = 0.5 * (b - a) * (pa + pb);
            cnt = 1;
        } else {
            double tnm = cnt;
            double del = (b - a) / tnm;
            double x = a + 0.5 * del;
            double sump = 0.0;
            for (int jj = 1; jj <= cnt; jj++) {
                sump = sump + delta_integrand(i0, x, dbeta);
                x = x + del;
            }
            sp[j] = 0.5 * (sp[j] + (b - a) * sump / tnm);
            cnt = 2 * cnt;
        }
        if (j >= k) {
            double dp[6];
            for (int i = 1; i <= k; i++) dp[i] = sp[j - k + i];
            polint5(dp, pq, dssp);
            if (std::fabs(dssp) < (eps * std::fabs(pq))) break;
            if (std::fabs(pq) < 1.0e-100) break;
        }
        sp[j + 1] = sp[j];
    }
    return pq;
}

// ---------------------------------------------------------------------------
// Peak normalisation integrals (Source/sc_calc_generic_gpu.cu:809-943).
// ---------------------------------------------------------------------------
double lorentznorm3(double a) {
    if (a > 0.01) {
        const double b0 = std::log(1 + a * M_PI * M_PI) / 2.;
        const double b1 = (a * M_PI * M_PI - std::log(1 + a * M_PI * M_PI)) / 12.;
        const double b2 = (-2 * a * M_PI * M_PI + a * a * M_PI * M_PI * M_PI * M_PI + 2 * std::log(1 + a * M_PI * M_PI)) / 480.;
        const double b3 = (a * M_PI * M_PI * (6 - 3 * a * M_PI * M_PI + 2 * a * a * M_PI * M_PI * M_PI * M_PI) -
                           6 * std::log(1 + a * M_PI * M_PI)) / 60480.;
        return b0 / a - b1 / (a * a) + b2 / (a * a * a) - b3 / (a * a * a * a);
    }
    const double a0 = 2;
    const double a1 = (M_PI * M_PI - 4);
    const double a2 = (18 - 12 * M_PI * M_PI + M_PI * M_PI * M_PI * M_PI) / 2.;
    const double a3 = (-1440 + 360 * M_PI * M_PI - 30 * M_PI * M_PI * M_PI * M_PI + M_PI * M_PI * M_PI * M_PI * M_PI * M_PI) / 6.;
    return a0 - a1 * a + a2 * a * a - a3 * a * a * a;
}

double gaussnorm3(double a) {
    if (a > 0.01) {
        const double b0 = (1 - std::exp(-a * M_PI * M_PI)) / 2.;
        const double b1 = (1 - std::exp(-a * M_PI * M_PI) * (1 + a * M_PI * M_PI)) / 12.;
        const double b2 = (2 - std::exp(-a * M_PI * M_PI) * (2 + 2 * a * M_PI * M_PI + a * a * M_PI * M_PI * M_PI * M_PI)) / 240.;
        const double b3 = (6 - std::exp(-a * M_PI * M_PI) *
                                   (6 + 6 * a * M_PI * M_PI + 3 * a * a * M_PI * M_PI * M_PI * M_PI +
                                    a * a * a * M_PI * M_PI * M_PI * M_PI * M_PI * M_PI)) / 10080.;
        return b0 / a - b1 / (a * a) + b2 / (a * a * a) - b3 / (a * a * a * a);
    }
    const double a0 = 2;
    const double a1 = (M_PI * M_PI - 4);
    const double a2 = (18 - 12 * M_PI * M_PI + M_PI * M_PI * M_PI * M_PI) / 2.;
    const double a3 = (-1440 + 360 * M_PI * M_PI - 30 * M_PI * M_PI * M_PI * M_PI + M_PI * M_PI * M_PI * M_PI * M_PI * M_PI) / 6.;
    return a0 - a1 * a + a2 * a * a - a3 * a * a * a;
}

void pearsonintegral3(double at, double bt, double a, double b, double &sx, int nx, int &trapzditx) {
    if (nx == 1) {
        const double fa = std::sin(at) / std::exp(b * std::log(1 + a * at * at));
        const double fb = std::sin(bt) / std::exp(b * std::log(1 + a * bt * bt));
        sx = 0.5 * (bt - at) * (fa + fb);
        trapzditx = 1;
    } else {
        const double tnmx = trapzditx;
        const double delx = (bt - at) / tnmx;
        double xt = at + 0.5 * delx;
        double sumx = 0.0;
        for (int jx = 1; jx <= trapzditx; jx++) {
            sumx += std::sin(xt) / std::exp(b * std::log(1 + a * xt * xt));
            xt = xt + delx;
        }
        sx = 0.5 * (sx + (bt - at) * sumx / tnmx);
        trapzditx = 2 * trapzditx;
    }
}

double pearsonnorm3(double a, double b) {
    b += 0.000001;
    if (a > 20.) {
        const double b0 = (1 - std::exp((1 - b) * std::log(1 + a * M_PI * M_PI))) / (2 * (b - 1));
        return b0 / a;
    }
    if (a <= 0.01) {
        const double a0 = 2.;
        const double a1 = (M_PI * M_PI - 4) * b;
        const double a2 = (18 - 12 * M_PI * M_PI + M_PI * M_PI * M_PI * M_PI) * b * (b + 1) / 2.;
        const double a3 = (-1440 + 360 * M_PI * M_PI - 30 * M_PI * M_PI * M_PI * M_PI + M_PI * M_PI * M_PI * M_PI * M_PI * M_PI) *
                          b * (b + 1) * (b + 2) / 6.;
        return a0 - a1 * a + a2 * a * a - a3 * a * a * a;
    }
    const int maxit = 10;
    int trapzditx = 0;
    double inttf = 0;
    pearsonintegral3(0, M_PI, a, b, inttf, 1, trapzditx);
    double oldinttf = inttf;
    for (int itf = 2; itf <= maxit; itf++) {
        pearsonintegral3(0, M_PI, a, b, inttf, itf, trapzditx);
        if (std::fabs(1 - inttf / oldinttf) < kEps3) break;
        oldinttf = inttf;
    }
    return inttf;
}

// ---------------------------------------------------------------------------
// Working state of one preparation: the reference class members that
// prepareCalculation() and coefficients() read and write.
// ---------------------------------------------------------------------------
struct Prep {
    cs_params in;
    cs_prepared *out;
    std::string err;

    // flags (prepareCalculation, sc_calc_generic_cpu.cpp:321-357)
    bool lat1d = false, lat2d = false, lat3d = true;
    int cdim = 0, partdim = 0;
    double phiwidth = 0, dist = 0, reldis = 0, ucvol = 0, dwfactor = 0;

    // long double scratch of coefficients() (_coeffMem, :2126-2131)
    long double gam3[2 * kNmax + 2], fkv[2 * kNmax + 2], fk2v[kNmax + 1], pn[kNmax + 1], z12vl[kNmax + 1];
    double fsum[kNmax + 1], u1ell[kNmax + 1], v1ell[3 * kNmax + 2];

    bool coefficients();
    bool coeff_sphere(double z, double xr2z, double xrm2z, double p, int &n4, int &n5, int &n6, int &n4f, int &n5f,
                      int &n6f);
    std::string hkl_tables(int ltype);
    void fhkl_c(int lat, int h, int k, int l, double &sphno, double &fhkl, double &qhkl, double &qhkl0);
    void corotations(double a, double b, double c, double alpha, double beta, double gamma, double u, double v,
                     double w, double ephi, bool lat1d, bool lat2d, double &m11, double &m12, double &m13,
                     double &m21, double &m22, double &m23, double &m31, double &m32, double &m33, double &mtw11,
                     double &mtw12, double &mtw13, double &mtw21, double &mtw22, double &mtw23, double &mtw31,
                     double &mtw32, double &mtw33, double &vvol);
};

// ---------------------------------------------------------------------------
// coefficients(), sc_calc_generic_cpu.cpp:2099-8195, reached branches only.
// ---------------------------------------------------------------------------
bool Prep::coefficients() {
    cs_prepared &P = *out;
    const int nmax = kNmax;
    double(*carrp)[CS_COEFF_LEN] = P.carrp;
    double(*carrf)[CS_COEFF_LEN] = P.carrf;
#define carr1p carrp[0]
#define carr2p carrp[1]
#define carr3p carrp[2]
#define carr4p carrp[3]
#define carr5p carrp[4]
#define carr6p carrp[5]
#define carr1f carrf[0]
#define carr2f carrf[1]
#define carr4f carrf[3]
#define carr5f carrf[4]
#define carr6f carrf[5]

    const double z = (1.0 - sqr(P.sigma)) / sqr(P.sigma);    // :2152
    const double zl = (1.0 - sqr(P.sigmal)) / sqr(P.sigmal); // :2153
    const double zz = z;
    const double zzl = zl;
    const double p = P.radius / P.radiusi; // :2159
    const double xlz = P.length / (2.0 * (zzl + 1)); // :2162
    const double xl2z = sqr(xlz);
    const double xrz = P.radius / (2.0 * (zz + 1));
    const double xr2z = sqr(xrz);
    const double xrmz = P.radiusi / (2.0 * (zz + 1));
    const double xrm2z = sqr(xrmz);
    double intl = 0.0;

    pn[0] = 1;
    z12vl[0] = 1;
    fsum[0] = 1;
    fkv[0] = 1;
    fk2v[0] = 1;
    gam3[0] = std::sqrt(M_PI) / 2.0;

    for (int n = 0; n < CS_COEFF_LEN; n++)
        for (int k = 0; k < 9; k++) {
            carrp[k][n] = 1;
            carrf[k][n] = 1;
        }
    for (int n = 0; n < CS_IMAX2D; n++)
        for (int m = 0; m < CS_IMAX2D; m++) P.carr11pm[n][m] = 1;

    bool search1 = true, search3 = true, search4 = true;
    int n1 = nmax, n2 = nmax, n3 = nmax, n4 = nmax, n5 = nmax, n6 = nmax, n7 = nmax, n8 = nmax, n9 = nmax;
    int n1f = nmax, n2f = nmax, n3f = nmax, n4f = nmax, n5f = nmax, n6f = nmax, n7f = nmax, n8f = nmax, n9f = nmax;

    // orientation case, :2493-2497 (0-based enum as in the reference)
    P.orcase = CS_ORC_GENERAL;
    if ((P.polphi == 0) && (P.poltheta == 90)) P.orcase = CS_ORC_XAXIS;
    if ((P.polphi == 90) && (P.poltheta == 90)) P.orcase = CS_ORC_YAXIS;
    if ((P.polphi == 0) && (P.poltheta == 0)) P.orcase = CS_ORC_ZAXIS;
    if ((P.polphi == 90) && (P.poltheta == 0)) P.orcase = CS_ORC_ZAXIS;

    bool done = false;
    bool supported = true;
    // The F(q) coefficients (carr*f, limq*f) are read only by the lattice
    // pixel functions (the structure factor's F/P); in the orientation-averaged
    // cylinder block, whose F sums cost as much as the rest of it, they are
    // formed only for lattices.
    const bool need_f = P.lattice != 0;

    if (cdim == 3) {
        // isotropic case for spheres, :2509-2754
        P.norm = 1;
        P.order = 0;
        if (P.cs == 0 || P.cs == 1) {
            done = coeff_sphere(z, xr2z, xrm2z, p, n4, n5, n6, n4f, n5f, n6f);
        } else {
            supported = false;
        }
    } else if ((P.ordis == 7) && (cdim == 4)) {
        // isotropic case for cubes, :2758-2877
        P.norm = 1;
        P.order = 0;
        if (P.cs == 0) {
            const double area = 6.0 * 4.0 * sqr(P.radius);
            const double vol = 8.0 * P.radius * sqr(P.radius);
            P.por = 2 * M_PI * std::pow(z + 1, 4) * area / (z * (z - 1) * (z - 2) * (z - 3) * vol * vol);
            long double z12v[kNmax + 1];
            z12v[0] = 1.0;
            long double xrn_n = 1.0;
            u1ell[0] = 2;
            for (int n = 1; n <= nmax; n++) {
                z12v[n] = z12v[n - 1] * ((z + 1) - 2 + 2 * n) * ((z + 1) - 1 + 2 * n);
                fkv[n] = fkv[n - 1] * n;
                gam3[n] = gam3[n - 1] * (2 * n + 1) / 2.0;
                u1ell[n] = 1 / ((n + 1 / 2.0) * (n + 1) * fkv[n]);
            }
            for (int n = 0; n <= nmax; n++) {
                double sump1 = 0.0;
                for (int m = 0; m <= n; m++) sump1 += u1ell[n - m] * u1ell[m];
                v1ell[n] = sump1;
            }
            for (int n = 1; n <= nmax; n++) {
                xrn_n = -xrn_n * xr2z;
                long double sumf = 0.0;
                for (int m = 0; m <= n; m++)
                    sumf += z12v[n - m] * z12v[m] / (gam3[n - m] * gam3[m] * fkv[n - m] * fkv[m]);
                fsum[n] = sumf;
                double sump = 0.0;
                for (int m = 0; m <= n; m++) sump += u1ell[n - m] * v1ell[m];
                carr4p[n] = std::sqrt(M_PI) * std::pow(4.0, n) * z12v[n] * xrn_n * sump / (16.0 * gam3[n]);
                sump = 0.0;
                for (int m = 0; m <= n; m++) {
                    double sump1 = 0.0;
                    for (int k = 0; k <= m; k++)
                        sump1 += fsum[m - k] * fsum[k] * gam3[m - k] * gam3[k] / ((k + 1 / 2.0) * (m - k + 1 / 2.0));
                    sump += sump1 * fsum[n - m] * gam3[n - m] / (n - m + 1 / 2.0);
                }
                carr4f[n] = M_PI * M_PI * xrn_n * sump / (128.0 * gam3[n]);
                if (std::fabs(carr4p[n]) < kMin) {
                    if (n < n4) n4 = n;
                }
                if (std::fabs(carr4f[n]) < kMin) {
                    if (n < n4f) n4f = n;
                }
            }
            done = true;
        } else {
            supported = false;
        }
    } else if ((P.ordis == 7) && (cdim == 5)) {
        // isotropic case for ellipsoids, :2966-3021 (semi-axes radius, radius
        // and length; eps = length/radius, :2166)
        P.norm = 1;
        P.order = 0;
        const double eps = P.length / P.radius;
        double area;
        if (eps > 1)
            area = 2 * M_PI * P.radius *
                   (P.radius + (sqr(P.length) / std::sqrt(sqr(P.length) - sqr(P.radius))) *
                                   std::asin(std::sqrt(sqr(P.length) - sqr(P.radius)) / P.length));
        else if (eps < 1)
            area = 2 * M_PI * P.radius *
                   (P.radius + (sqr(P.length) / std::sqrt(sqr(P.radius) - sqr(P.length))) *
                                   std::asinh(std::sqrt(sqr(P.radius) - sqr(P.length)) / P.length));
        else
            area = 4 * M_PI * P.radius * P.radius;
        const double vol = (4 * M_PI / 3.0) * sqr(P.radius) * P.length;
        P.por = 2 * M_PI * std::pow(z + 1, 4) * area / (z * (z - 1) * (z - 2) * (z - 3) * vol * vol);
        if (P.cs == 0) {
            // Only the P(q) coefficients: the reference's F(q) coefficients
            // of this case read fsum[1..n] that nothing has written, and the
            // ellipsoid pixel function takes F(q) = P(q).
            double e1[kNmax + 1];
            e1[0] = 1;
            double z12v_n = 1.0;
            double xrn_n = 1.0;
            for (int n = 1; n <= nmax; n++) {
                z12v_n = z12v_n * ((z + 1) - 2 + 2 * n) * ((z + 1) - 1 + 2 * n);
                fkv[n] = fkv[n - 1] * n;
                gam3[n] = gam3[n - 1] * (2 * n + 1) / 2.0;
                e1[n] = e1[n - 1] * (eps * eps - 1);
                xrn_n = -xrn_n * xr2z;
                double sump = 0.0;
                for (int m = 0; m <= n; m++) sump += e1[n - m] / (fkv[n - m] * fkv[m] * (2 * (n - m) + 1));
                carr4p[n] = (9 * std::sqrt(M_PI) / 2.0) * std::pow(4.0, n) * z12v_n * xrn_n * sump /
                            ((n + 3) * (n + 2) * (n + 3 / 2.0) * gam3[n]);
                if (std::fabs(carr4p[n]) < kMin) {
                    if (n < n4) n4 = n;
                }
            }
            done = true;
        } else {
            supported = false;
        }
    } else if ((P.ordis == 7) && (cdim != 3)) {
        // isotropic case for cylinders and disks, :3578-4122 (homogeneous and
        // core/shell; operand types as the reference declares them: the
        // local z12v and the recurrence factors in long double)
        P.norm = 1;
        P.order = 0;
        if (P.cs == 0 && (cdim == 1 || cdim == 2)) {
            long double z12v[kNmax + 1];
            z12v[0] = 1.0;
            double xrn[kNmax + 1];
            xrn[0] = 1;
            const double xrn_n0 = 1.0;
            long double xln_n = 1.0;
            if ((P.length / P.radius) < 2.0) {
                // small axial ratios (the double sum of the exact average), :3592-3626
                const double area = 2 * M_PI * sqr(P.radius) + 2 * M_PI * P.radius * (2. * P.length);
                const double vol = M_PI * sqr(P.radius) * (2. * P.length);
                P.por = 2 * M_PI * std::pow(z + 1, 4) * area / (z * (z - 1) * (z - 2) * (z - 3) * vol * vol);
                for (int n = 1; n <= nmax; n++) {
                    z12v[n] = z12v[n - 1] * ((z + 1) - 2 + 2 * n) * ((z + 1) - 1 + 2 * n);
                    z12vl[n] = z12vl[n - 1] * ((zl + 1) - 2 + 2 * n) * ((zl + 1) - 1 + 2 * n);
                    fkv[n] = fkv[n - 1] * n;
                    gam3[n] = gam3[n - 1] * (2 * n + 1) / 2.0;
                    xln_n = -xln_n * xl2z;
                    // the reference's running xrn_n is never advanced here:
                    // every xrn[n] is -xr2z (reproduced)
                    xrn[n] = -xrn_n0 * xr2z;
                }
                // xln_n keeps its n = nmax value in this loop (reproduced)
                for (int n = 0; n <= nmax; n++) {
                    const double binsum = 0.0;
                    P.carr11pm[n][0] = std::sqrt(M_PI) / gam3[n];
                    double a1 = std::sqrt(M_PI) / (2.0 * gam3[n]);
                    for (int m = 1; m <= nmax; m++) {
                        a1 = a1 * (m + 1 / 2.0) / (n + m + 1 / 2.0);
                        P.carr11pm[n][m] =
                            std::pow(4.0, m + 1) * a1 * z12v[m] * xrn[m] / ((m + 2) * (m + 1) * fkv[m] * (m + 1) * fkv[m]);
                    }
                    carrp[1][n] = std::pow(4.0, n - 1) * z12vl[n] * xln_n / ((n + 1 / 2.0) * (n + 1) * fkv[n]);
                    carrp[2][n] = std::pow(4.0, n) * binsum / gam3[n];
                }
            } else {
                // large axial ratios (factorisation), :3628-3706
                double xrn_n = 1.0;
                for (int n = 1; n <= nmax; n++) {
                    z12v[n] = z12v[n - 1] * ((z + 1) - 2 + 2 * n) * ((z + 1) - 1 + 2 * n);
                    z12vl[n] = z12vl[n - 1] * ((zl + 1) - 2 + 2 * n) * ((zl + 1) - 1 + 2 * n);
                    fkv[n] = fkv[n - 1] * n;
                    fk2v[n] = fk2v[n - 1] * (2 * n - 1) * (2 * n);
                    gam3[n] = gam3[n - 1] * (2 * n + 1) / 2.0;
                    xln_n = -xln_n * xl2z;
                    xrn_n = -xrn_n * xr2z;
                    if (cdim == 1) {
                        carr1p[n] = std::sqrt(M_PI) * std::pow(4.0, n) * z12vl[n] * xln_n /
                                    (2.0 * (2 * n + 1) * (n + 1) * gam3[n] * fkv[n]);
                        carr4p[n] = 4 * (n + 1 / 2.0) * fk2v[n] * z12v[n] * xrn_n /
                                    ((n + 2) * (n + 1) * fkv[n] * fkv[n] * (n + 1) * fkv[n] * fkv[n]);
                        double binsum = 0.0;
                        for (int m = 0; m <= n; m++)
                            binsum += z12vl[m] * z12vl[n - m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                        carr1f[n] = M_PI * xln_n * binsum / (4.0 * (2 * n + 1));
                        binsum = 0.0;
                        for (int m = 0; m <= n; m++)
                            binsum += z12v[m] * z12v[n - m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m] * fkv[m] * fkv[n - m]);
                        carr4f[n] = xrn_n * binsum;
                    }
                    if (cdim == 2) {
                        carr1p[n] = 2 * std::pow(4.0, n) * z12vl[n] * xln_n / ((n + 2) * (n + 1) * (n + 1) * fkv[n] * fkv[n]);
                        carr4p[n] = std::pow(4.0, n) * std::sqrt(M_PI) * z12v[n] * xrn_n / (2.0 * (n + 1) * gam3[n] * fkv[n]);
                        double binsum = 0.0;
                        for (int m = 0; m <= n; m++)
                            binsum += z12vl[m] * z12vl[n - m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m]);
                        carr1f[n] = std::sqrt(M_PI) * fkv[n] * xln_n * binsum / (2.0 * gam3[n]);
                        binsum = 0.0;
                        for (int m = 0; m <= n; m++)
                            binsum += z12v[m] * z12v[n - m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                        carr4f[n] = M_PI * xrn_n * binsum / 4.0;
                    }
                    if (std::fabs(carr1p[n]) < kMin) {
                        if (n < n1) n1 = n;
                    }
                    if (std::fabs(carrp[1][n]) < kMin) {
                        if (n < n2) n2 = n;
                    }
                    if (std::fabs(carrp[2][n]) < kMin) {
                        if (n < n3) n3 = n;
                    }
                    if (std::fabs(carr1f[n]) < kMin) {
                        if (n < n1f) n1f = n;
                    }
                    if (std::fabs(carr4p[n]) < kMin) {
                        if (n < n4) n4 = n;
                    }
                    if (std::fabs(carr4f[n]) < kMin) {
                        if (n < n4f) n4f = n;
                    }
                }
            }
            done = true;
        } else if (P.cs == 1 && (cdim == 1 || cdim == 2)) {
            // core/shell, :3709-3828
            long double xrmn_n = 1.0, xrn_n = 1.0, xln_n = 1.0;
            long double z12v[kNmax + 1];
            z12v[0] = 1.0;
            for (int n = 1; n <= nmax; n++) {
                z12v[n] = z12v[n - 1] * ((z + 1) - 2 + 2 * n) * ((z + 1) - 1 + 2 * n);
                z12vl[n] = z12vl[n - 1] * ((zl + 1) - 2 + 2 * n) * ((zl + 1) - 1 + 2 * n);
                fkv[n] = fkv[n - 1] * n;
                fk2v[n] = fk2v[n - 1] * (2 * n - 1) * (2 * n);
                gam3[n] = gam3[n - 1] * (2 * n + 1) / 2.0;
                xln_n = -xln_n * xl2z;
                xrn_n = -xrn_n * xr2z;
                xrmn_n = -xrmn_n * xrm2z;
                pn[n] = pn[n - 1] * p * p;
                if (cdim == 1) {
                    carr1p[n] = std::sqrt(M_PI) * std::pow(4.0, n) * z12vl[n] * xln_n /
                                (2.0 * (2 * n + 1) * (n + 1) * gam3[n] * fkv[n]);
                    carr4p[n] = 4 * (n + 1 / 2.0) * fk2v[n] * z12v[n] * xrn_n /
                                ((n + 2) * (n + 1) * fkv[n] * fkv[n] * (n + 1) * fkv[n] * fkv[n]);
                    double sump = 0.0;
                    for (int m = 0; m <= n; m++) sump += pn[m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m] * fkv[m] * fkv[n - m]);
                    carr5p[n] = z12v[n] * xrmn_n * sump;
                    carr6p[n] = carr4p[n] / pn[n];
                    double binsum = 0.0;
                    for (int m = 0; m <= n; m++)
                        binsum += z12vl[m] * z12vl[n - m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                    carr1f[n] = M_PI * xln_n * binsum / (4.0 * (2 * n + 1));
                    sump = 0.0;
                    for (int m = 0; m <= n; m++)
                        sump += z12v[m] * z12v[n - m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m] * fkv[m] * fkv[n - m]);
                    carr4f[n] = xrn_n * sump;
                    sump = 0.0;
                    for (int m = 0; m <= n; m++)
                        sump += z12v[m] * z12v[n - m] * pn[m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m] * fkv[m] * fkv[n - m]);
                    carr5f[n] = xrmn_n * sump;
                    carr6f[n] = carr4f[n] / pn[n];
                } else {
                    carr1p[n] = 2 * std::pow(4.0, n) * z12vl[n] * xln_n / ((n + 2) * (n + 1) * (n + 1) * fkv[n] * fkv[n]);
                    carr4p[n] = std::pow(4.0, n) * std::sqrt(M_PI) * z12v[n] * xrn_n / (2.0 * (n + 1) * gam3[n] * fkv[n]);
                    double sump = 0.0;
                    for (int m = 0; m <= n; m++) sump += pn[m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                    carr5p[n] = M_PI * z12v[n] * xrmn_n * sump / 4.0;
                    carr6p[n] = carr4p[n] / pn[n];
                    double binsum = 0.0;
                    for (int m = 0; m <= n; m++)
                        binsum += z12vl[m] * z12vl[n - m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m]);
                    carr1f[n] = std::sqrt(M_PI) * fkv[n] * xln_n * binsum / (2.0 * gam3[n]);
                    sump = 0.0;
                    for (int m = 0; m <= n; m++) sump += z12v[m] * z12v[n - m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                    carr4f[n] = M_PI * xrn_n * sump / 4.0;
                    sump = 0.0;
                    for (int m = 0; m <= n; m++)
                        sump += pn[m] * z12v[m] * z12v[n - m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                    carr5f[n] = M_PI * xrmn_n * sump / 4.0;
                    carr6f[n] = carr4f[n] / pn[n];
                }
                if (std::fabs(carr1p[n]) < kMin) {
                    if (n < n1) n1 = n;
                }
                if (std::fabs(carrp[2][n]) < kMin) {
                    if (n < n3) n3 = n;
                }
                if (std::fabs(carr4p[n]) < kMin) {
                    if (n < n4) n4 = n;
                }
                if (std::fabs(carr5p[n]) < kMin) {
                    if (n < n5) n5 = n;
                }
                if (std::fabs(carr6p[n]) < kMin) {
                    if (n < n6) n6 = n;
                }
                if (std::fabs(carr1f[n]) < kMin) {
                    if (n < n1f) n1f = n;
                }
                if (std::fabs(carr4f[n]) < kMin) {
                    if (n < n4f) n4f = n;
                }
                if (std::fabs(carr5f[n]) < kMin) {
                    if (n < n5f) n5f = n;
                }
                if (std::fabs(carr6f[n]) < kMin) {
                    if (n < n6f) n6f = n;
                }
            }
            done = true;
        } else {
            supported = false;
        }
    } else if ((P.ordis == 6) && (cdim != 3)) {
        // perfect orientation for cylinders and disks, :4124-4644
        P.norm = 1;
        P.order = 1;
        double z12v[kNmax + 1];
        z12v[0] = 1.0;
        long double xln_n = 1.0;
        if (P.cs == 0 && (cdim == 1 || cdim == 2)) {
            double xrn_n = 1.0;
            for (int n = 1; n <= nmax; n++) {
                z12v[n] = z12v[n - 1] * ((z + 1) - 2 + 2 * n) * ((z + 1) - 1 + 2 * n);
                z12vl[n] = z12vl[n - 1] * ((zl + 1) - 2 + 2 * n) * ((zl + 1) - 1 + 2 * n);
                fkv[n] = fkv[n - 1] * n;
                fk2v[n] = fk2v[n - 1] * (2 * n - 1) * (2 * n);
                gam3[n] = gam3[n - 1] * (2 * n + 1) / 2.0;
                xln_n = -xln_n * xl2z;
                xrn_n = -xrn_n * xr2z;
                if (cdim == 1) {
                    carr1p[n] = std::sqrt(M_PI) * std::pow(4.0, n) * z12vl[n] * xln_n / (2.0 * (n + 1) * gam3[n] * fkv[n]);
                    carr4p[n] = 4 * (n + 1 / 2.0) * fk2v[n] * z12v[n] * xrn_n /
                                ((n + 2) * (n + 1) * fkv[n] * fkv[n] * (n + 1) * fkv[n]);
                    double sump = 0.0;
                    for (int m = 0; m <= n; m++)
                        sump += z12vl[m] * z12vl[n - m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m] * fkv[m] * fkv[n - m]);
                    carr1f[n] = M_PI * xln_n * sump / 4.0;
                    sump = 0.0;
                    for (int m = 0; m <= n; m++)
                        sump += z12v[m] * z12v[n - m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m] * fkv[m] * fkv[n - m]);
                    carr4f[n] = xrn_n * sump;
                }
                if (cdim == 2) {
                    carr1p[n] = std::pow(4.0, n + 1) * gam3[n] * z12vl[n] * xln_n /
                                (std::sqrt(M_PI) * (n + 2) * (n + 1) * (n + 1) * fkv[n] * fkv[n] * fkv[n]);
                    carr4p[n] = std::pow(4.0, n) * std::sqrt(M_PI) * z12v[n] * xrn_n / (2.0 * (n + 1) * gam3[n] * fkv[n]);
                    double sump = 0.0;
                    for (int m = 0; m <= n; m++)
                        sump += z12vl[m] * z12vl[n - m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m] * fkv[m] * fkv[n - m]);
                    carr1f[n] = std::sqrt(M_PI) * fkv[n] * xln_n * sump / (2.0 * gam3[n]);
                    sump = 0.0;
                    for (int m = 0; m <= n; m++)
                        sump += z12v[m] * z12v[n - m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m] * fkv[m] * fkv[n - m]);
                    carr4f[n] = M_PI * xln_n * sump / 4.0;
                }
                if (search1) {
                    if (carr1p[n] < 1e-50) {
                        n1 = n;
                        search1 = false;
                    }
                }
                if (search4) {
                    if (carr4p[n] < 1e-50) {
                        n4 = n;
                        search4 = false;
                    }
                }
                if (std::fabs(carr1f[n]) < kMin) {
                    if (n < n1f) n1f = n;
                }
                if (std::fabs(carr4f[n]) < kMin) {
                    if (n < n4f) n4f = n;
                }
            }
            done = true;
        } else if (P.cs == 1 && (cdim == 1 || cdim == 2)) {
            // core/shell, :4213-4361: core (carr4), cross (carr5) and shell
            // (carr6) terms of the cross-section
            double xrmn_n = 1.0;
            double xrn_n = 1.0;
            for (int n = 1; n <= nmax; n++) {
                z12v[n] = z12v[n - 1] * ((z + 1) - 2 + 2 * n) * ((z + 1) - 1 + 2 * n);
                z12vl[n] = z12vl[n - 1] * ((zl + 1) - 2 + 2 * n) * ((zl + 1) - 1 + 2 * n);
                fkv[n] = fkv[n - 1] * n;
                fk2v[n] = fk2v[n - 1] * (2 * n - 1) * (2 * n);
                gam3[n] = gam3[n - 1] * (2 * n + 1) / 2.0;
                xln_n = -xln_n * xl2z;
                xrn_n = -xrn_n * xr2z;
                xrmn_n = -xrmn_n * xrm2z;
                pn[n] = pn[n - 1] * p * p;
                double sump;
                if (cdim == 1) {
                    carr1p[n] = std::sqrt(M_PI) * std::pow(4.0, n) * z12vl[n] * xln_n / (2.0 * (n + 1) * gam3[n] * fkv[n]);
                    carr4p[n] = 4 * (n + 1 / 2.0) * fk2v[n] * z12v[n] * xrn_n /
                                ((n + 2) * (n + 1) * fkv[n] * fkv[n] * (n + 1) * fkv[n] * fkv[n]);
                    sump = 0.0;
                    for (int m = 0; m <= n; m++) sump += pn[m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m]);
                    carr5p[n] = z12v[n] * xrmn_n * sump;
                    carr6p[n] = carr4p[n] / pn[n];
                    sump = 0.0;
                    for (int m = 0; m <= n; m++)
                        sump += z12vl[m] * z12vl[n - m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                    carr1f[n] = M_PI * xln_n * sump / 4.0;
                    sump = 0.0;
                    for (int m = 0; m <= n; m++)
                        sump += z12v[m] * z12v[n - m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m] * fkv[m] * fkv[n - m]);
                    carr4f[n] = xrn_n * sump;
                    sump = 0.0;
                    for (int m = 0; m <= n; m++)
                        sump += pn[m] * z12v[m] * z12v[n - m] /
                                ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m] * fkv[m] * fkv[n - m]);
                    carr5f[n] = xrmn_n * sump;
                    carr6f[n] = carr4f[n] / pn[n];
                } else {
                    carr1p[n] = std::pow(4.0, n + 1) * gam3[n] * z12vl[n] * xln_n /
                                (std::sqrt(M_PI) * (n + 2) * (n + 1) * (n + 1) * fkv[n] * fkv[n] * fkv[n]);
                    carr4p[n] = std::pow(4.0, n) * std::sqrt(M_PI) * z12v[n] * xrn_n / (2.0 * (n + 1) * gam3[n] * fkv[n]);
                    sump = 0.0;
                    for (int m = 0; m <= n; m++) sump += pn[m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                    carr5p[n] = M_PI * z12v[n] * xrmn_n * sump / 4.0;
                    carr6p[n] = carr4p[n] / pn[n];
                    sump = 0.0;
                    for (int m = 0; m <= n; m++)
                        sump += z12vl[m] * z12vl[n - m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m] * fkv[m] * fkv[n - m]);
                    carr1f[n] = std::sqrt(M_PI) * fkv[n] * xln_n * sump / (2.0 * gam3[n]);
                    sump = 0.0;
                    for (int m = 0; m <= n; m++) sump += z12v[m] * z12v[n - m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                    carr4f[n] = M_PI * xrn_n * sump / 4.0;
                    sump = 0.0;
                    for (int m = 0; m <= n; m++)
                        sump += pn[m] * z12v[m] * z12v[n - m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                    carr5f[n] = M_PI * xrmn_n * sump / 4.0;
                    carr6f[n] = carr4f[n] / pn[n];
                }
                if (std::fabs(carr1p[n]) < kMin) {
                    if (n < n1) n1 = n;
                }
                if (std::fabs(carr4p[n]) < kMin) {
                    if (n < n4) n4 = n;
                }
                if (std::fabs(carr5p[n]) < kMin) {
                    if (n < n5) n5 = n;
                }
                if (std::fabs(carr6p[n]) < kMin) {
                    if (n < n6) n6 = n;
                }
                if (std::fabs(carr1f[n]) < kMin) {
                    if (n < n1f) n1f = n;
                }
                if (std::fabs(carr4f[n]) < kMin) {
                    if (n < n4f) n4f = n;
                }
                if (std::fabs(carr5f[n]) < kMin) {
                    if (n < n5f) n5f = n;
                }
                if (std::fabs(carr6f[n]) < kMin) {
                    if (n < n6f) n6f = n;
                }
            }
            done = true;
        } else {
            supported = false;
        }
    } else if ((P.ordis == 0) && (cdim != 3)) {
        // orientational distribution for cylinders and disks, :4648-8035.
        // norm and order parameter, :4650-4652
        P.norm = qromb_delta_1d(2, 0, P.dbeta);
        P.order = qromb_delta_1d(3, 0, P.dbeta);
        P.order = P.order / P.norm;
        // Every intl of this block comes from qrombdeltac with i0 = 1, whose
        // integrand sin(x)exp(-x^2/dbeta^2) ignores i3/i4 (the moment powers
        // sit in code the reference compiles out), so all of them equal the
        // i0 = 2 norm integral bit for bit. It is computed once.
        const double intl_const = qromb_delta_1d(1, 0, P.dbeta);
        if (cdim == 2) {
            // disks along an axis, homogeneous: x :6045-6130, y :6875-6960,
            // z :7644-7730; core/shell: x :6137-6273, y :6966-7100, z
            // :7730-7860. The x and y blocks differ only in carr11pm (whose
            // moment-based first assignment the reference overwrites at once);
            // the z block leaves carr11pm at 1 and folds the delta moments into
            // carr1p. Core/shell adds the cross (carr5) and shell (carr6)
            // terms and forms carr4f with xrn (xln when homogeneous). The
            // general orientation is not offered: the reference's disk P(q) has
            // no branch for it and returns an uninitialised value.
            if ((P.cs != 0 && P.cs != 1) || P.orcase == CS_ORC_GENERAL) {
                supported = false;
            } else {
                const bool cs1 = P.cs == 1;
                bool search5 = true, search6 = true;
                double xrmn_n = 1.0;
                double z12v[kNmax + 1];
                z12v[0] = 1.0;
                double xrn_n = 1.0;
                long double xln_n = 1.0;
                const int orc = P.orcase;
                double carr2i[kNmax + 1];
                if (orc == CS_ORC_ZAXIS) {
                    carr2i[0] = 1;
                    for (int n = 1; n <= nmax; n++) {
                        fkv[n] = fkv[n - 1] * n;
                        fk2v[n] = fk2v[n - 1] * (2 * n - 1) * (2 * n);
                        carr2i[n] = std::pow(-1, n) * fk2v[n] * intl_const /
                                    (std::pow(4.0, n) * fkv[n] * fkv[n] * fkv[n] * P.norm);
                    }
                }
                for (int n = 1; n <= nmax; n++) {
                    z12v[n] = z12v[n - 1] * ((z + 1) - 2 + 2 * n) * ((z + 1) - 1 + 2 * n);
                    z12vl[n] = z12vl[n - 1] * ((zl + 1) - 2 + 2 * n) * ((zl + 1) - 1 + 2 * n);
                    if (orc != CS_ORC_ZAXIS) {
                        fkv[n] = fkv[n - 1] * n;
                        fk2v[n] = fk2v[n - 1] * (2 * n - 1) * (2 * n);
                    }
                    gam3[n] = gam3[n - 1] * (2 * n + 1) / 2.0;
                    xln_n = -xln_n * xl2z;
                    xrn_n = -xrn_n * xr2z;
                    if (cs1) {
                        xrmn_n = -xrmn_n * xrm2z;
                        pn[n] = pn[n - 1] * p * p;
                    }
                    double sump;
                    if (orc == CS_ORC_ZAXIS) {
                        sump = 0.0;
                        for (int m = 0; m <= n; m++) sump += carr2i[m] / fkv[n - m];
                        carr1p[n] = std::pow(4.0, n + 1) * gam3[n] * z12vl[n] * xln_n * sump /
                                    (std::sqrt(M_PI) * (n + 2) * (n + 1) * (n + 1) * fkv[n] * fkv[n]);
                        double sump1 = 0.0;
                        for (int m = 0; m <= n; m++)
                            sump1 += z12vl[m] * z12vl[n - m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m]);
                        carr1f[n] = xln_n * fkv[n] * sump1 * sump;
                    } else {
                        for (int m = 0; m <= n; m++) {
                            if (orc == CS_ORC_XAXIS)
                                P.carr11pm[n][m] = std::pow(-1, m) * fk2v[m] / (std::pow(4.0, m) * fkv[m] * fkv[n - m]);
                            else
                                P.carr11pm[n][m] = std::pow(-1, m) * fk2v[m] / (fkv[m] * fkv[n - m]);
                        }
                        carr1p[n] = std::pow(4.0, n + 1) * gam3[n] * z12vl[n] * xln_n /
                                    (std::sqrt(M_PI) * (n + 2) * (n + 1) * (n + 1) * fkv[n] * fkv[n]);
                        sump = 0.0;
                        for (int m = 0; m <= n; m++)
                            sump += z12vl[m] * z12vl[n - m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m]);
                        carr1f[n] = xln_n * fkv[n] * sump;
                    }
                    // cross-section
                    carr4p[n] = std::pow(4.0, n) * std::sqrt(M_PI) * z12v[n] * xrn_n / (2.0 * (n + 1) * gam3[n] * fkv[n]);
                    sump = 0.0;
                    for (int m = 0; m <= n; m++)
                        sump += z12v[m] * z12v[n - m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                    if (!cs1) {
                        carr4f[n] = M_PI * xln_n * sump / 4.0;
                    } else {
                        carr4f[n] = M_PI * xrn_n * sump / 4.0;
                        sump = 0.0;
                        for (int m = 0; m <= n; m++) sump += pn[m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                        carr5p[n] = M_PI * z12v[n] * xrmn_n * sump / 4.0;
                        carr6p[n] = carr4p[n] / pn[n];
                        sump = 0.0;
                        for (int m = 0; m <= n; m++)
                            sump += pn[m] * z12v[m] * z12v[n - m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                        carr5f[n] = M_PI * xrmn_n * sump / 4.0;
                        carr6f[n] = carr4f[n] / pn[n];
                    }
                    // the series of the orientation integral's Bessel approximation
                    carr2p[n] = std::pow(4.0, n + 1) * gam3[n] * z12vl[n] * xln_n /
                                (std::sqrt(M_PI) * (n + 2) * (n + 1) * (n + 1) * fkv[n] * fkv[n] * fkv[n]);
                    sump = 0.0;
                    for (int m = 0; m <= n; m++)
                        sump += z12vl[m] * z12vl[n - m] /
                                ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m] * fkv[m] * fkv[n - m]);
                    carr2f[n] = std::sqrt(M_PI) * fkv[n] * xln_n * sump / (2.0 * gam3[n]);
                    if (search1) {
                        if (carr1p[n] < 1e-50) {
                            n1 = n;
                            search1 = false;
                        }
                    }
                    if (search4) {
                        if (carr4p[n] < 1e-50) {
                            n4 = n;
                            search4 = false;
                        }
                    }
                    if (cs1 && search5) {
                        if (carr5p[n] < 1e-50) {
                            n5 = n;
                            search5 = false;
                        }
                    }
                    if (cs1 && search6) {
                        if (carr6p[n] < 1e-50) {
                            n6 = n;
                            search6 = false;
                        }
                    }
                    if (std::fabs(carr1f[n]) < kMin) {
                        if (n < n1f) n1f = n;
                    }
                    if (std::fabs(carr4f[n]) < kMin) {
                        if (n < n4f) n4f = n;
                    }
                    if (cs1 && std::fabs(carr5f[n]) < kMin) {
                        if (n < n5f) n5f = n;
                    }
                    if (cs1 && std::fabs(carr6f[n]) < kMin) {
                        if (n < n6f) n6f = n;
                    }
                }
                intl = intl_const;
                done = true;
            }
        } else if (cdim != 1) {
            supported = false;
        }

        if (supported && cdim == 1 && P.orcase == CS_ORC_GENERAL) {
            // :4655-4760 (cylinder, homogeneous) and :4763-4889 (core/shell:
            // the same carr11pm and length coefficients, its own cross-section)
            P.polphi = 0;
            const double p11 = -std::cos(P.polphi * M_PI / 180.0) * std::cos(P.poltheta * M_PI / 180.0);
            const double p13 = std::cos(P.polphi * M_PI / 180.0) * std::sin(P.poltheta * M_PI / 180.0);
            const double p21 = -std::cos(P.polphi * M_PI / 180.0);
            // The powers below are the same pow() calls as in the reference's
            // innermost loop (:4705-4719), evaluated once per exponent.
            double pw11[kNmax + 1], pw13[kNmax + 1], pw4[kNmax + 1], pw21[kNmax + 1];
            for (int e = 0; e <= nmax; e++) {
                pw11[e] = std::pow(p11 * p11, e);
                pw13[e] = std::pow(p13 * p13, e);
                pw4[e] = std::pow(4.0, e);
                pw21[e] = std::pow(sqr(p21), e);
            }
            if (P.cs == 0 || P.cs == 1) {
                const bool cs1 = P.cs == 1;
                bool search5 = true, search6 = true;
                double z12v[kNmax + 1];
                z12v[0] = 1.0;
                double xrn_n = 1.0;
                long double xln_n = 1.0;
                // log2 of the denominator factors, for the negligible-term test
                // (sums of log2 k: the long-double factorials overflow double)
                double lgfkv[kNmax + 1], lgfk2v[kNmax + 1];
                lgfkv[0] = 0.0;   // fkv[0] = 1
                lgfk2v[0] = 0.0;  // fk2v[0] = 1
                const double lgnorm = P.norm > 0 ? lg2(P.norm) : 0.0;
                const double lgintl = intl_const > 0 ? lg2(intl_const) : 0.0;
                const double lim0 = negligible_lg2(0.0);
                double lgpw11[kNmax + 1], lgpw13[kNmax + 1];
                for (int e = 0; e <= nmax; e++) {
                    lgpw11[e] = pw11[e] > 0 ? lg2(pw11[e]) : 0.0;  // unused where the product is 0
                    lgpw13[e] = pw13[e] > 0 ? lg2(pw13[e]) : 0.0;
                }
                // recurrences (serial), then the rows of every n (parallel),
                // then the searches over n (serial)
                long double xln[kNmax + 1];
                double xrn[kNmax + 1], xrmn[kNmax + 1];
                double xrmn_n = 1.0;
                for (int n = 1; n <= nmax; n++) {
                    z12v[n] = z12v[n - 1] * ((z + 1) - 2 + 2 * n) * ((z + 1) - 1 + 2 * n);
                    z12vl[n] = z12vl[n - 1] * ((zl + 1) - 2 + 2 * n) * ((zl + 1) - 1 + 2 * n);
                    fkv[n] = fkv[n - 1] * n;
                    fk2v[n] = fk2v[n - 1] * (2 * n - 1) * (2 * n);
                    lgfkv[n] = lgfkv[n - 1] + std::log2((double)n);
                    lgfk2v[n] = lgfk2v[n - 1] + std::log2((double)(2 * n - 1)) + std::log2((double)(2 * n));
                    gam3[n] = gam3[n - 1] * (2 * n + 1) / 2.0;
                    xln_n = -xln_n * xl2z;
                    xrn_n = -xrn_n * xr2z;
                    xln[n] = xln_n;
                    xrn[n] = xrn_n;
                    if (cs1) {
                        xrmn_n = -xrmn_n * xrm2z;
                        xrmn[n] = xrmn_n;
                        pn[n] = pn[n - 1] * p * p;
                    }
                }
                // pw11/pw13 are powers of numbers <= 1: once a power underflows
                // to 0 all higher ones are 0, and so is every numerator that
                // uses them (skipped below in any case): the ll loop runs over
                // the window where both powers are non-zero
                int e11 = nmax, e13 = nmax;
                while (e11 > 0 && pw11[e11] == 0.0) e11--;
                while (e13 > 0 && pw13[e13] == 0.0) e13--;
                parallel_n(1, nmax, [&](int n) {
                    const long double xln_n = xln[n];
                    const double xrn_n = xrn[n];
                    for (int m = 0; m <= n; m++) {
                        double sump = 0.0;
                        double lim = lim0;  // negligible_lg2(sump)
                        const int ll_lo = m - e13 > 0 ? m - e13 : 0;
                        const int ll_hi = m < e11 ? m : e11;
                        for (int ll = ll_lo; ll <= ll_hi; ll++) {
                            const double num = pw11[ll] * pw13[m - ll] * intl_const;
                            // a zero numerator adds exactly 0 (the long-double
                            // denominator is finite and non-zero): skipped
                            if (num == 0.0) continue;
                            // A positive term too small to change the double sum
                            // is skipped as well (the result is the same bits).
                            // With the polar axis in the detector plane the terms
                            // ll >= 1 carry pw11 = (cos 90deg)^(2ll) ~ 1e-33^ll.
                            if (num > 0.0 && P.norm > 0) {
                                // log2 of the two-rounding product from its factors
                                // (directly where subnormal rounding could matter)
                                const double lgnum = num < 1e-290 ? lg2(num) : lgpw11[ll] + lgpw13[m - ll] + lgintl;
                                if (lgnum - (2.0 * ll + lgfk2v[m - ll] + lgfkv[n - m + ll] + lgfkv[ll] + lgnorm) < lim)
                                    continue;
                            }
                            sump += num / (pw4[ll] * fk2v[m - ll] * fkv[n - m + ll] * fkv[ll] * P.norm);
                            lim = negligible_lg2(sump);
                        }
                        P.carr11pm[n][m] = pw4[m] * pw21[n - m] * sump / (fkv[n - m]);
                    }
                    carr1p[n] = std::pow(4.0, n) * z12vl[n] * xln_n / ((2.0 * n + 1) * (n + 1));
                    carr2p[n] = std::pow(4.0, n + 1) * gam3[n] * z12vl[n] * xln_n /
                                (std::sqrt(M_PI) * (n + 2) * (n + 1) * (n + 1) * fkv[n] * fkv[n] * fkv[n]);
                    if (need_f) {
                        double sump = 0.0;
                        for (int m = 0; m <= n; m++)
                            sump = sump + z12vl[m] * z12vl[n - m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                        carr1f[n] = fk2v[n] * xln_n * sump / (std::pow(4.0, n));
                    }
                    carr2f[n] = carr2p[n];
                    if (!cs1) {
                        carr4p[n] = 4 * (n + 1 / 2.0) * fk2v[n] * z12v[n] * xrn_n /
                                    ((n + 2) * (n + 1) * fkv[n] * fkv[n] * (n + 1) * fkv[n]);
                        if (need_f) {
                            double sump = 0.0;
                            for (int m = 0; m <= n; m++)
                                sump = sump + z12v[m] * z12v[n - m] /
                                                  ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m] * fkv[m] * fkv[n - m]);
                            carr4f[n] = xrn_n * sump;
                        }
                    } else {
                        // core (carr4), cross (carr5) and shell (carr6) terms
                        const double xrmn_n = xrmn[n];
                        carr4p[n] = 4 * (n + 1 / 2.0) * fk2v[n] * z12v[n] * xrn_n /
                                    ((n + 2) * (n + 1) * fkv[n] * fkv[n] * (n + 1) * fkv[n] * fkv[n]);
                        double sump = 0.0;
                        for (int m = 0; m <= n; m++) sump += pn[m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m]);
                        carr5p[n] = z12v[n] * xrmn_n * sump;
                        carr6p[n] = carr4p[n] / pn[n];
                        if (need_f) {
                            sump = 0.0;
                            for (int m = 0; m <= n; m++)
                                sump += z12v[m] * z12v[n - m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m]);
                            carr4f[n] = xrn_n * sump;
                            sump = 0.0;
                            for (int m = 0; m <= n; m++)
                                sump += pn[m] * z12v[m] * z12v[n - m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m]);
                            carr5f[n] = xrmn_n * sump;
                            carr6f[n] = carr4f[n] / pn[n];
                        }
                    }
                });
                for (int n = 1; n <= nmax; n++) {
                    if (search1) {
                        if (carr1p[n] < 1e-50) {
                            n1 = n;
                            search1 = false;
                        }
                    }
                    if (search4) {
                        if (carr4p[n] < 1e-50) {
                            n4 = n;
                            search4 = false;
                        }
                    }
                    if (cs1 && search5) {
                        if (carr5p[n] < 1e-50) {
                            n5 = n;
                            search5 = false;
                        }
                    }
                    if (cs1 && search6) {
                        if (carr6p[n] < 1e-50) {
                            n6 = n;
                            search6 = false;
                        }
                    }
                    if (std::fabs(carr1f[n]) < kMin) {
                        if (n < n1f) n1f = n;
                    }
                    if (std::fabs(carr4f[n]) < kMin) {
                        if (n < n4f) n4f = n;
                    }
                    if (cs1 && std::fabs(carr5f[n]) < kMin) {
                        if (n < n5f) n5f = n;
                    }
                    if (cs1 && std::fabs(carr6f[n]) < kMin) {
                        if (n < n6f) n6f = n;
                    }
                }
                done = true;
            } else {
                supported = false;
            }
        }
        if (supported && cdim == 1 && P.orcase == CS_ORC_GENERAL) {
            // second general-orientation block, :5549-5617. Its qrombdeltac
            // loop (:5562-5569) discards every result and is not repeated.
            for (int n = 1; n <= 2 * nmax; n++) fkv[n] = fkv[n - 1] * n;
            double b1sv_n = 1.0;
            double z12v_n = 1.0;
            double xrn_n = 1.0;
            long double xln_n = 1.0;
            double b1s = 2;  // cdim == 1: cylinder, cross-section is disk
            for (int n = 1; n <= nmax; n++) {
                z12v_n = z12v_n * ((z + 1) - 2 + 2 * n) * ((z + 1) - 1 + 2 * n);
                b1sv_n = b1sv_n * (b1s - 1 + n);
                xln_n = -xln_n * xl2z;
                xrn_n = -xrn_n * xr2z;
                carr1p[n] = std::pow(4.0, 2 * n) * z12v_n * xln_n / ((2.0 * n + 1) * (n + 1));
                carr3p[n] = 4 * (n + 1 / 2.0) * fk2v[n] * z12v_n * xrn_n / ((n + 2) * (n + 1) * fkv[n] * fkv[n] * b1sv_n * fkv[n]);
                if (search1) {
                    if (carr1p[n] < 1e-50) {
                        n1 = n;
                        search1 = false;
                    }
                }
                if (search3) {
                    if (carr3p[n] < 1e-50) {
                        n3 = n;
                        search3 = false;
                    }
                }
            }
            done = true;
        }
        if (supported && cdim == 1 && (P.orcase == CS_ORC_XAXIS || P.orcase == CS_ORC_YAXIS || P.orcase == CS_ORC_ZAXIS)) {
            // x-axis :5619-5692, y-axis :6453-6526, z-axis :7265-7331 (cylinder,
            // homogeneous); core/shell :5696-5817, :6530-6649, :7335-7447 (the
            // same length coefficients but for the x axis's z12vl, which uses
            // zl there, and the z axis's carr1f, divided by 4^(n+1); its own
            // cross-section)
            if (P.cs != 0 && P.cs != 1) {
                supported = false;
            } else {
                const bool cs1 = P.cs == 1;
                bool search5 = true, search6 = true;
                double z12v[kNmax + 1];
                z12v[0] = 1.0;
                double xrn_n = 1.0;
                long double xln_n = 1.0;
                const int orc = P.orcase;
                // recurrences (serial), rows of every n (parallel), searches (serial)
                long double xln[kNmax + 1];
                double xrn[kNmax + 1], xrmn[kNmax + 1];
                double xrmn_n = 1.0;
                for (int n = 1; n <= nmax; n++) {
                    z12v[n] = z12v[n - 1] * ((z + 1) - 2 + 2 * n) * ((z + 1) - 1 + 2 * n);
                    if (orc == CS_ORC_XAXIS && !cs1)
                        z12vl[n] = z12vl[n - 1] * ((z + 1) - 2 + 2 * n) * ((z + 1) - 1 + 2 * n);  // uses z, :5636
                    else
                        z12vl[n] = z12vl[n - 1] * ((zl + 1) - 2 + 2 * n) * ((zl + 1) - 1 + 2 * n);
                    fkv[n] = fkv[n - 1] * n;
                    fk2v[n] = fk2v[n - 1] * (2 * n - 1) * (2 * n);
                    gam3[n] = gam3[n - 1] * (2 * n + 1) / 2.0;
                    xln_n = -xln_n * xl2z;
                    xrn_n = -xrn_n * xr2z;
                    xln[n] = xln_n;
                    xrn[n] = xrn_n;
                    if (cs1) {
                        xrmn_n = -xrmn_n * xrm2z;
                        xrmn[n] = xrmn_n;
                        pn[n] = pn[n - 1] * p * p;
                    }
                }
                const double intl_v = intl_const;  // every qrombdeltac moment of these blocks
                parallel_n(1, nmax, [&](int n) {
                    const long double xln_n = xln[n];
                    const double xrn_n = xrn[n];
                    double sump;
                    if (orc == CS_ORC_XAXIS) {
                        for (int m = 0; m <= n; m++)
                            P.carr11pm[n][m] = std::pow(4.0, m) * intl_v / (fk2v[m] * fkv[n - m] * fkv[n - m] * P.norm);
                        carr1p[n] = std::pow(4.0, n) * z12vl[n] * xln_n / ((2.0 * n + 1) * (n + 1));
                        sump = 0.0;
                        for (int m = 0; m <= n; m++)
                            sump = sump + z12vl[m] * z12vl[n - m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                        carr1f[n] = fk2v[n] * xln_n * sump / (std::pow(4.0, n));
                    } else if (orc == CS_ORC_YAXIS) {
                        for (int m = 0; m <= n; m++)
                            P.carr11pm[n][m] = intl_v / (std::pow(4.0, m) * fk2v[n - m] * fkv[m] * fkv[m] * P.norm);
                        carr1p[n] = std::pow(4.0, 2 * n) * z12vl[n] * xln_n / ((2.0 * n + 1) * (n + 1));
                        sump = 0.0;
                        for (int m = 0; m <= n; m++)
                            sump += z12vl[m] * z12vl[n - m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                        carr1f[n] = fk2v[n] * xln_n * sump;
                    } else {
                        carr1p[n] = std::pow(4.0, n) * z12vl[n] * xln_n * intl_v / ((2.0 * n + 1) * (n + 1) * fkv[n] * fkv[n] * P.norm);
                        sump = 0.0;
                        for (int m = 0; m <= n; m++)
                            sump += z12vl[m] * z12vl[n - m] / (gam3[m] * gam3[n - m] * fkv[m] * fkv[n - m]);
                        carr1f[n] = fk2v[n] * xln_n * sump * intl_v /
                                    (std::pow(4.0, cs1 ? n + 1 : n) * fkv[n] * fkv[n] * P.norm);
                    }
                    if (!cs1) {
                        carr4p[n] = 4 * (n + 1 / 2.0) * fk2v[n] * z12v[n] * xrn_n /
                                    ((n + 2) * (n + 1) * fkv[n] * fkv[n] * (n + 1) * fkv[n]);
                        sump = 0.0;
                        for (int m = 0; m <= n; m++)
                            sump = sump + z12v[m] * z12v[n - m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m] * fkv[m] * fkv[n - m]);
                        carr4f[n] = xrn_n * sump;
                    } else {
                        // core (carr4), cross (carr5) and shell (carr6) terms
                        const double xrmn_n = xrmn[n];
                        carr4p[n] = 4 * (n + 1 / 2.0) * fk2v[n] * z12v[n] * xrn_n /
                                    ((n + 2) * (n + 1) * fkv[n] * fkv[n] * (n + 1) * fkv[n] * fkv[n]);
                        sump = 0.0;
                        for (int m = 0; m <= n; m++) sump = sump + pn[m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m]);
                        carr5p[n] = z12v[n] * xrmn_n * sump;
                        carr6p[n] = carr4p[n] / pn[n];
                        sump = 0.0;
                        for (int m = 0; m <= n; m++)
                            sump = sump + z12v[m] * z12v[n - m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m]);
                        carr4f[n] = xrn_n * sump;
                        sump = 0.0;
                        for (int m = 0; m <= n; m++)
                            sump = sump + pn[m] * z12v[m] * z12v[n - m] / ((m + 1) * fkv[m] * (n - m + 1) * fkv[n - m]);
                        carr5f[n] = xrmn_n * sump;
                        carr6f[n] = carr4f[n] / pn[n];
                    }
                });
                intl = intl_v;
                for (int n = 1; n <= nmax; n++) {
                    if (search1) {
                        if (carr1p[n] < 1e-50) {
                            n1 = n;
                            search1 = false;
                        }
                    }
                    if (search4) {
                        if (carr4p[n] < 1e-50) {
                            n4 = n;
                            search4 = false;
                        }
                    }
                    if (cs1 && search5) {
                        if (carr5p[n] < 1e-50) {
                            n5 = n;
                            search5 = false;
                        }
                    }
                    if (cs1 && search6) {
                        if (carr6p[n] < 1e-50) {
                            n6 = n;
                            search6 = false;
                        }
                    }
                    if (std::fabs(carr1f[n]) < kMin) {
                        if (n < n1f) n1f = n;
                    }
                    if (std::fabs(carr4f[n]) < kMin) {
                        if (n < n4f) n4f = n;
                    }
                    if (cs1 && std::fabs(carr5f[n]) < kMin) {
                        if (n < n5f) n5f = n;
                    }
                    if (cs1 && std::fabs(carr6f[n]) < kMin) {
                        if (n < n6f) n6f = n;
                    }
                }
                done = true;
            }
        }
    } else {
        supported = false;
    }
    (void)intl;

    if (!supported) {
        err = "coefficients: combination not implemented (cs=" + std::to_string(P.cs) + " cdim=" +
              std::to_string(cdim) + " ordis=" + std::to_string(P.ordis) + " orcase=" + std::to_string(P.orcase) + ")";
        return false;
    }

    // Label99, :8051-8090
    auto bad = [](double v) { return std::isinf(v) || std::isnan(v) || std::fabs(v) < 1e-99; };
    int np_[9] = {n1, n2, n3, n4, n5, n6, n7, n8, n9};
    int nf_[9] = {n1f, n2f, n3f, n4f, n5f, n6f, n7f, n8f, n9f};
    for (int k = 0; k < 9; k++)
        while (np_[k] > 1 && bad(carrp[k][np_[k]])) np_[k]--;
    for (int k = 0; k < 9; k++)
        while (nf_[k] > 1 && bad(carrf[k][nf_[k]])) nf_[k]--;
    for (int k = 0; k < 9; k++) {
        P.limq[k + 1] = std::pow(std::fabs(carrp[k][np_[k]]), -1 / (2.0 * np_[k]));
        P.limqf[k + 1] = std::pow(std::fabs(carrf[k][nf_[k]]), -1 / (2.0 * nf_[k]));
    }
#undef carr1p
#undef carr2p
#undef carr3p
#undef carr4p
#undef carr5p
#undef carr6p
#undef carr1f
#undef carr2f
#undef carr4f
#undef carr5f
#undef carr6f
    return done;
}

// Sphere branches cs = 0 (:2514-2544) and cs = 1 (:2546-2610).
bool Prep::coeff_sphere(double z, double xr2z, double xrm2z, double p, int &n4, int &n5, int &n6, int &n4f,
                        int &n5f, int &n6f) {
    cs_prepared &P = *out;
    const int nmax = kNmax;
    double *carr4p = P.carrp[3], *carr5p = P.carrp[4], *carr6p = P.carrp[5];
    double *carr4f = P.carrf[3], *carr5f = P.carrf[4], *carr6f = P.carrf[5];
    if (P.cs == 0) {
        long double xrn_n = 1.0;
        long double z12v[kNmax + 1], xrn[kNmax + 1];
        z12v[0] = 1.0;
        // recurrences (serial), values of every n (parallel), searches (serial)
        for (int n = 1; n <= nmax; n++) {
            z12v[n] = z12v[n - 1] * ((z + 1) - 2 + 2 * n) * ((z + 1) - 1 + 2 * n);
            fkv[n] = fkv[n - 1] * n;
            gam3[n] = gam3[n - 1] * (2 * n + 1) / 2.0;
            xrn_n = -xrn_n * xr2z;
            xrn[n] = xrn_n;
        }
        parallel_n(1, nmax, [&](int n) {
            carr4p[n] = 9 * std::sqrt(M_PI) * std::pow(4.0, n) * z12v[n] * xrn[n] /
                        (2.0 * (n + 3) * (n + 2) * (n + 3 / 2.0) * gam3[n] * fkv[n]);
            double binsum = 0.0;
            for (int m = 0; m <= n; m++)
                binsum += z12v[m] * z12v[n - m] / ((m + 3 / 2.0) * gam3[m] * (n - m + 3 / 2.0) * gam3[n - m] * fkv[m] * fkv[n - m]);
            carr4f[n] = 9 * M_PI * xrn[n] * binsum / 16.0;
        });
        for (int n = 1; n <= nmax; n++) {
            if (std::fabs(carr4p[n]) < kMin) {
                if (n < n4) n4 = n;
            }
            if (std::fabs(carr4f[n]) < kMin) {
                if (n < n4f) n4f = n;
            }
        }
        return true;
    }
    // cs == 1, core/shell
    long double xrn_n = 1.0;
    long double xrmn_n = 1.0;
    long double z12v[kNmax + 1];
    z12v[0] = 1.0;
    for (int n = 1; n <= nmax; n++) {
        z12v[n] = z12v[n - 1] * ((z + 1) - 2 + 2 * n) * ((z + 1) - 1 + 2 * n);
        fkv[n] = fkv[n - 1] * n;
        gam3[n] = gam3[n - 1] * (2 * n + 1) / 2.0;
        xrn_n = -xrn_n * xr2z;
        xrmn_n = -xrmn_n * xrm2z;
        pn[n] = pn[n - 1] * p * p;
        long double sump = 0.0;
        for (int m = 0; m <= n; m++)
            sump += pn[m] / ((m + 3 / 2.0) * gam3[m] * (n - m + 3 / 2.0) * gam3[n - m] * fkv[m] * fkv[n - m]);
        carr4p[n] = 9 * std::sqrt(M_PI) * std::pow(4.0, n) * z12v[n] * xrn_n /
                    (2.0 * (n + 3) * (n + 2) * (n + 3 / 2.0) * gam3[n] * fkv[n]);
        carr5p[n] = (9 * M_PI / 16.0) * z12v[n] * xrmn_n * sump;
        carr6p[n] = carr4p[n] / pn[n];
        sump = 0.0;
        for (int m = 0; m <= n; m++)
            sump += z12v[m] * z12v[n - m] / ((m + 3 / 2.0) * gam3[m] * (n - m + 3 / 2.0) * gam3[n - m] * fkv[m] * fkv[n - m]);
        carr4f[n] = (9 * M_PI / 16.0) * xrn_n * sump;
        sump = 0.0;
        for (int m = 0; m <= n; m++)
            sump += pn[m] * z12v[m] * z12v[n - m] / ((m + 3 / 2.0) * gam3[m] * (n - m + 3 / 2.0) * gam3[n - m] * fkv[m] * fkv[n - m]);
        carr5f[n] = (9 * M_PI / 16.0) * xrmn_n * sump;
        carr6f[n] = carr4f[n] / pn[n];
        if (std::fabs(carr4p[n]) < kMin) {
            if (n < n4) n4 = n;
        }
        if (std::fabs(carr5p[n]) < kMin) {
            if (n < n5) n5 = n;
        }
        if (std::fabs(carr6p[n]) < kMin) {
            if (n < n6) n6 = n;
        }
        if (std::fabs(carr4f[n]) < kMin) {
            if (n < n4f) n4f = n;
        }
        if (std::fabs(carr5f[n]) < kMin) {
            if (n < n5f) n5f = n;
        }
        if (std::fabs(carr6f[n]) < kMin) {
            if (n < n6f) n6f = n;
        }
    }
    return true;
}

// ---------------------------------------------------------------------------
// Reflection list (ButtonHKLClick, sc_calc_generic_cpu.cpp:8246-10295) for the
// cubic and tetragonal lattices.
// ---------------------------------------------------------------------------
std::string Prep::hkl_tables(int ltype) {
    cs_prepared &P = *out;
    bool cubic = false, tetragonal = false;
    int c1 = -1, c2 = -1, c4 = -1, c6 = -1, c7 = -1, c8 = -1, c10 = -1;
    // SETCX(a..n): c1=a c2=b c4=d c6=f c7=g c8=h c10=j (the other letters are unused)
    auto setcx = [&](int a, int b, int d, int f, int g, int h, int j) {
        c1 = a; c2 = b; c4 = d; c6 = f; c7 = g; c8 = h; c10 = j;
    };
    switch (ltype) {
    case 4:   // BCC: cubic 7 "I---", :8641
    case 11:  // Im3m: cubic 7
        cubic = true;
        setcx(0, 0, -1, -1, 0, -1, 0);
        break;
    case 5:   // FCC: cubic 12 "F---", :8657
        cubic = true;
        setcx(6, 4, -1, -1, 0, -1, 2);
        break;
    case 7:   // SC: cubic 0 "P---"
        cubic = true;
        setcx(-1, -1, -1, -1, -1, -1, -1);
        break;
    case 10:  // Pn3m: cubic 5 "Pn--"
        cubic = true;
        setcx(-1, 0, -1, -1, 0, -1, -1);
        break;
    case 9:   // Ia3d: cubic 11 "Ia-d"
        cubic = true;
        setcx(0, 4, -1, -1, 1, -1, 4);
        break;
    case 17:  // Fd3m: cubic 15 "Fd--"
        cubic = true;
        setcx(6, 3, -1, -1, 1, -1, 2);
        break;
    case 8:   // BCT: tetragonal 23 "I---"
        tetragonal = true;
        setcx(0, 0, 0, 0, 0, -1, 0);
        break;
    default:
        return "unsupported lattice";
    }
    const int hm = in.hklmax;
    int hmin = 0, kmin = 0, lmin = 0;
    const int kmax = hm, lmax = hm;
    P.latpar1[1][0] = 0;
    P.latpar2[1][0] = 0;
    for (int ii = 1; ii <= 2; ii++) {
        int ct1 = 1;
        if (ii == 2) {
            hmin = -hm;
            kmin = -hm;
            lmin = -hm;
        }
        for (int h = hmin; h <= hm; h++)
            for (int k = kmin; k <= kmax; k++)
                for (int l = lmin; l <= lmax; l++) {
                    enum { _000, _0kl, _h0l, _hk0, _h00, _0k0, _00l, _hhl, _hlh, _lhh, _hh0, _h0h, _0hh, _hhh, _hkl };
                    int hklcase = _hkl;
                    if ((h == 0) && (k == 0) && (l == 0)) hklcase = _000;
                    if ((h == 0) && (k != 0) && (l != 0) && (k != l)) hklcase = _0kl;
                    if ((k == 0) && (h != 0) && (l != 0) && (h != l)) hklcase = _h0l;
                    if ((l == 0) && (h != 0) && (k != 0) && (h != k)) hklcase = _hk0;
                    if ((h != 0) && (k == 0) && (l == 0)) hklcase = _h00;
                    if ((k != 0) && (h == 0) && (l == 0)) hklcase = _0k0;
                    if ((l != 0) && (h == 0) && (k == 0)) hklcase = _00l;
                    if ((h != 0) && (h == k) && (l != 0) && (l != h)) hklcase = _hhl;
                    if ((h != 0) && (h == l) && (k != 0) && (k != h)) hklcase = _hlh;
                    if ((k != 0) && (k == l) && (h != 0) && (h != k)) hklcase = _lhh;
                    if ((h != 0) && (h == k) && (l == 0)) hklcase = _hh0;
                    if ((h != 0) && (h == l) && (k == 0)) hklcase = _h0h;
                    if ((k != 0) && (k == l) && (h == 0)) hklcase = _0hh;
                    if ((h != 0) && (h == k) && (h == l)) hklcase = _hhh;
                    int mult = 0;
                    if (cubic) {
                        switch (hklcase) {
                        case _hkl: mult = 48; break;
                        case _hhl: case _hlh: case _hk0: case _h0l: case _0kl: case _lhh: mult = 24; break;
                        case _hh0: case _h0h: case _0hh: mult = 12; break;
                        case _hhh: mult = 8; break;
                        case _h00: case _0k0: case _00l: mult = 6; break;
                        default: mult = 0; break;
                        }
                    } else if (tetragonal) {
                        switch (hklcase) {
                        case _hkl: mult = 16; break;
                        case _hhl: case _hlh: case _lhh: case _h0h: case _0hh: case _hhh: case _hk0: case _h0l:
                        case _0kl: mult = 8; break;
                        case _hh0: case _h00: case _0k0: mult = 4; break;
                        case _00l: mult = 2; break;
                        default: mult = 0; break;
                        }
                    }
                    int ccase = 0;
                    if (cubic) {
                        int c1case = 0, c2case = 1, c7case = 1, c10case = 1;
                        if (c1 == -1) c1case = 1;
                        if (c1 == 0)
                            if (((h + k + l) % 2) == 0) c1case = 1;
                        if (c1 == 6)
                            if ((((h + k) % 2) == 0) && (((h + l) % 2) == 0) && (((k + l) % 2) == 0)) c1case = 1;
                        if ((c2 == 0) && (h == 0) && !(((k + l) % 2) == 0)) c2case = 0;
                        if ((c2 == 0) && (k == 0) && !(((h + l) % 2) == 0)) c2case = 0;
                        if ((c2 == 0) && (l == 0) && !(((h + k) % 2) == 0)) c2case = 0;
                        if ((c2 == 3) && (h == 0) && !((((k + l) % 4) == 0) && ((k % 2) == 0) && ((l % 2) == 0))) c2case = 0;
                        if ((c2 == 3) && (k == 0) && !((((h + l) % 4) == 0) && ((h % 2) == 0) && ((l % 2) == 0))) c2case = 0;
                        if ((c2 == 3) && (l == 0) && !((((h + k) % 4) == 0) && ((h % 2) == 0) && ((k % 2) == 0))) c2case = 0;
                        if ((c2 == 4) && (h == 0) && !(((k % 2) == 0) && ((l % 2) == 0))) c2case = 0;
                        if ((c2 == 4) && (k == 0) && !(((h % 2) == 0) && ((l % 2) == 0))) c2case = 0;
                        if ((c2 == 4) && (l == 0) && !(((h % 2) == 0) && ((k % 2) == 0))) c2case = 0;
                        if ((c2 == 5) && (h == 0) && !((k % 2) == 0)) c2case = 0;
                        if ((c2 == 5) && (k == 0) && !((l % 2) == 0)) c2case = 0;
                        if ((c2 == 5) && (l == 0) && !((h % 2) == 0)) c2case = 0;
                        if ((c10 == 0) && (h == k) && (l != 0) && !((l % 2) == 0)) c10case = 0;
                        if ((c10 == 0) && (h == l) && (k != 0) && !((k % 2) == 0)) c10case = 0;
                        if ((c10 == 0) && (k == l) && (h != 0) && !((h % 2) == 0)) c10case = 0;
                        if ((c10 == 2) && (h == k) && (l != 0) && !(((h + l) % 2) == 0)) c10case = 0;
                        if ((c10 == 2) && (h == l) && (k != 0) && !(((h + k) % 2) == 0)) c10case = 0;
                        if ((c10 == 2) && (k == l) && (h != 0) && !(((h + k) % 2) == 0)) c10case = 0;
                        if ((c10 == 4) && (h == k) && (l != 0) && !((((2 * h + l) % 4) == 0) && ((l % 2) == 0))) c10case = 0;
                        if ((c10 == 4) && (h == l) && (k != 0) && !((((2 * h + k) % 4) == 0) && ((k % 2) == 0))) c10case = 0;
                        if ((c10 == 4) && (k == l) && (h != 0) && !((((2 * k + h) % 4) == 0) && ((h % 2) == 0))) c10case = 0;
                        if ((c10 == 5) && (h == k) && (l != 0) && !(((h % 2) == 0) && ((l % 2) == 0))) c10case = 0;
                        if ((c10 == 5) && (h == l) && (k != 0) && !(((h % 2) == 0) && ((k % 2) == 0))) c10case = 0;
                        if ((c10 == 5) && (k == l) && (h != 0) && !(((k % 2) == 0) && ((h % 2) == 0))) c10case = 0;
                        if ((c7 == 0) && (h == 0) && (k == 0) && !((l % 2) == 0)) c7case = 0;
                        if ((c7 == 0) && (h == 0) && (l == 0) && !((k % 2) == 0)) c7case = 0;
                        if ((c7 == 0) && (k == 0) && (l == 0) && !((h % 2) == 0)) c7case = 0;
                        if ((c7 == 1) && (h == 0) && (k == 0) && !((l % 4) == 0)) c7case = 0;
                        if ((c7 == 1) && (h == 0) && (l == 0) && !((k % 4) == 0)) c7case = 0;
                        if ((c7 == 1) && (k == 0) && (l == 0) && !((h % 4) == 0)) c7case = 0;
                        ccase = c1case * c2case * c7case * c10case;
                    }
                    if (tetragonal) {
                        int c1case = 0, c2case = 1, c4case = 1, c6case = 1, c7case = 1, c8case = 1, c10case = 1;
                        if (c1 == -1) c1case = 1;
                        if (c1 == 0)
                            if ((h + k + l) % 2 == 0) c1case = 1;
                        if ((c2 == 0) && (h == 0) && !((k + l) % 2 == 0)) c2case = 0;
                        if ((c2 == 0) && (k == 0) && !((h + l) % 2 == 0)) c2case = 0;
                        if ((c2 == 1) && (h == 0) && !(k % 2 == 0)) c2case = 0;
                        if ((c2 == 1) && (k == 0) && !(h % 2 == 0)) c2case = 0;
                        if ((c2 == 2) && (h == 0) && !(l % 2 == 0)) c2case = 0;
                        if ((c2 == 2) && (k == 0) && !(l % 2 == 0)) c2case = 0;
                        if ((c2 == 4) && (h == 0) && !((k % 2 == 0) && (l % 2 == 0))) c2case = 0;
                        if ((c2 == 4) && (k == 0) && !((h % 2 == 0) && (l % 2 == 0))) c2case = 0;
                        if ((c4 == 0) && (l == 0) && !((h + k) % 2 == 0)) c4case = 0;
                        if ((c4 == 4) && (l == 0) && !((h % 2 == 0) && (k % 2 == 0))) c4case = 0;
                        if ((c10 == 0) && (h == k) && (l != 0) && !(l % 2 == 0)) c10case = 0;
                        if ((c10 == 4) && (h == k) && (l != 0) && !(((2 * h + l) % 4 == 0) && (l % 2 == 0))) c10case = 0;
                        if ((c6 == 0) && (h == 0) && (l == 0) && !(k % 2 == 0)) c6case = 0;
                        if ((c6 == 0) && (k == 0) && (l == 0) && !(h % 2 == 0)) c6case = 0;
                        if ((c7 == 0) && (h == 0) && (k == 0) && !(l % 2 == 0)) c7case = 0;
                        if ((c7 == 1) && (h == 0) && (k == 0) && !(l % 4 == 0)) c7case = 0;
                        if ((c8 == 0) && (h == k) && (l == 0) && !(h % 2 == 0)) c8case = 1;
                        ccase = c1case * c2case * c4case * c6case * c7case * c8case * c10case;
                    }
                    if ((h == 0) && (k == 0) && (l == 0)) ccase = 0;
                    if (ccase == 1) {
                        if (ct1 >= CS_LATPARLEN) return "reflection table overflow";
                        int(*lp)[6] = (ii == 1) ? P.latpar1 : P.latpar2;
                        lp[1][0] = ct1;
                        lp[ct1][1] = h;
                        lp[ct1][2] = k;
                        lp[ct1][3] = l;
                        lp[ct1][4] = mult;
                        ct1++;
                    }
                }
    }
    return "";
}

// fhkl_c, sc_calc_generic_cpu.cpp:10299-10578 (lattices 4, 5, 7, 8, 9, 10, 11, 17).
void Prep::fhkl_c(int lat, int h, int k, int l, double &sphno, double &fhkl, double &qhkl, double &qhkl0) {
    const double a = out->uca;
    double sumc, sums, arg, invd;
    float r[13][4];
    int nn;
    auto sum_r = [&](int count) {
        sumc = 0.0;
        sums = 0.0;
        for (int i = 1; i <= count; i++) {
            arg = 2 * M_PI * (h * r[i][1] + k * r[i][2] + l * r[i][3]);
            sumc = sumc + std::cos(arg);
            sums = sums + std::sin(arg);
        }
        fhkl = std::round(sumc * sumc + sums * sums);
    };
    switch (lat) {
    case 4:
    case 8:
    case 9:
    case 11:
        sphno = 2;
        nn = 2;
        r[1][1] = 0; r[1][2] = 0; r[1][3] = 0;
        r[2][1] = 1 / 2.; r[2][2] = 1 / 2.; r[2][3] = 1 / 2.;
        sum_r(nn);
        invd = (h * h + k * k + l * l) / (a * a);
        qhkl = 2 * M_PI * std::sqrt(invd);
        qhkl0 = (lat == 11) ? 2 * M_PI * std::sqrt(2.) / 2. : 2 * M_PI * std::sqrt(2.) / a;
        break;
    case 5:
        sphno = 4;
        nn = 4;
        r[1][1] = 0; r[1][2] = 0; r[1][3] = 0;
        r[2][1] = 1 / 2.; r[2][2] = 1 / 2.; r[2][3] = 0;
        r[3][1] = 0; r[3][2] = 1 / 2.; r[3][3] = 1 / 2.;
        r[4][1] = 1 / 2.; r[4][2] = 0; r[4][3] = 1 / 2.;
        sum_r(nn);
        invd = (h * h + k * k + l * l) / (a * a);
        qhkl = 2 * M_PI * std::sqrt(invd);
        qhkl0 = 2 * M_PI * std::sqrt(3.) / a;
        break;
    case 7:
    case 10:
        sphno = 1;
        fhkl = 1;
        invd = (h * h + k * k + l * l) / (a * a);
        qhkl = 2 * M_PI * std::sqrt(invd);
        qhkl0 = 2 * M_PI / a;
        break;
    case 17:
        sphno = 8;
        nn = 8;
        r[1][1] = 0; r[1][2] = 0; r[1][3] = 0;
        r[2][1] = 1 / 2.; r[2][2] = 1 / 2.; r[2][3] = 0;
        r[3][1] = 0; r[3][2] = 1 / 2.; r[3][3] = 1 / 2.;
        r[4][1] = 1 / 2.; r[4][2] = 0; r[4][3] = 1 / 2.;
        r[5][1] = 1 / 4.; r[5][2] = 1 / 4.; r[5][3] = 1 / 4.;
        r[6][1] = 3 / 4.; r[6][2] = 3 / 4.; r[6][3] = 1 / 4.;
        r[7][1] = 1 / 4.; r[7][2] = 3 / 4.; r[7][3] = 3 / 4.;
        r[8][1] = 3 / 4.; r[8][2] = 1 / 4.; r[8][3] = 3 / 4.;
        sum_r(nn);
        invd = (h * h + k * k + l * l) / (a * a);
        qhkl = 2 * M_PI * std::sqrt(invd);
        qhkl0 = 2 * M_PI * std::sqrt(3.) / a;
        break;
    default:
        sphno = 1;
        fhkl = 1;
        qhkl = 0;
        qhkl0 = 0;
        break;
    }
}

// corotations, sc_calc_generic_cpu.cpp:1487-2098. Variable types follow the
// reference (a mix of float and double); only the outputs used later are kept.
void Prep::corotations(double a, double b, double c, double alpha, double beta, double gamma, double u, double v,
                       double w, double ephi, bool lat1d_, bool lat2d_, double &m11, double &m12, double &m13,
                       double &m21, double &m22, double &m23, double &m31, double &m32, double &m33, double &mtw11,
                       double &mtw12, double &mtw13, double &mtw21, double &mtw22, double &mtw23, double &mtw31,
                       double &mtw32, double &mtw33, double &vvol) {
    double ca, cb, cg, sb, sg, n1, n2, n3, l1, l2, l3, mm1, mm2, mm3;
    double msi11, msi12, msi13, msi21, msi22, msi23, msi31, msi32, msi33, detmsi;
    double ms11, ms12, ms13, ms21, ms22, ms23, ms31, ms32, ms33;
    double mst11, mst12, mst13, mst21, mst22, mst23, mst31, mst32, mst33, detmst;
    double mt11, mt12, mt13, mt21, mt22, mt23, mt31, mt32, mt33;
    float g11, g12, g13, g21, g22, g23, g31, g32, g33, gi11, gi12, gi13, gi21, gi22, gi23, gi31, gi32, gi33, detg;
    double ri11, ri12, ri13, ri21, ri22, ri23, ri31, ri32, ri33, detr;
    float aax, aay, aaz, bax, bay, baz, cax, cay, caz;
    float aaxt, aayt, aazt, baxt, bayt, bazt, caxt, cayt, cazt;
    float aex, aey, aez, bex, bey, bez, cex, cey, cez;
    float asxn, asyn, aszn, bsxn, bsyn, bszn, csxn, csyn, cszn;
    float aext, aeyt, aezt, bext, beyt, bezt, cext, ceyt, cezt;
    float epsi, etheta, len, r11, r12, r13, r21, r22, r23, r31, r32, r33;
    float aedx, aedy, aedz, bedx, bedy, bedz, cedx, cedy, cedz;
    float nxyzx, nxyzy, nxyzz, nxyznx, nxyznz;
    double asedx, asedy, asedz, bsedx, bsedy, bsedz, csedx, csedy, csedz;
    double asedxt, asedyt, asedzt, bsedxt, bsedyt, bsedzt, csedxt, csedyt, csedzt;
    double aedxt, aedyt, aedzt, bedxt, bedyt, bedzt, cedxt, cedyt, cedzt;
    double m11DD, m12DD, m13DD, m21DD, m22DD, m23DD;
    double aexDD, aeyDD, bexDD, beyDD;
    double asxDD, asyDD, aszDD, bsxDD, bsyDD, bszDD, csxDD, csyDD, cszDD, area;
    double asedxDD, asedyDD, asedzDD, bsedxDD, bsedyDD, bsedzDD, csedxDD, csedyDD, csedzDD;
    double asxDL, asyDL, aszDL, bsxDL, bsyDL, bszDL, csxDL, csyDL, cszDL, area1;
    double asedxDL, asedyDL, asedzDL, bsedxDL, bsedyDL, bsedzDL, csedxDL, csedyDL, csedzDL;

    alpha = alpha * M_PI / 180.0;
    beta = beta * M_PI / 180.0;
    gamma = gamma * M_PI / 180.0;
    ephi = ephi * M_PI / 180.0;
    ca = std::cos(alpha);
    cb = std::cos(beta);
    cg = std::cos(gamma);
    sb = std::sin(beta);
    sg = std::sin(gamma);
    n1 = 0;
    n2 = 0;
    n3 = 1;
    l1 = sb;
    l2 = 0;
    l3 = cb;
    mm1 = (cg - cb * ca) / sb;
    mm2 = std::sqrt(1.0 - mm1 * mm1 - ca * ca);
    mm3 = ca;

    msi11 = a * l1; msi12 = a * l2; msi13 = a * l3;
    msi21 = b * mm1; msi22 = b * mm2; msi23 = b * mm3;
    msi31 = c * n1; msi32 = c * n2; msi33 = c * n3;
    detmsi = msi11 * msi22 * msi33 + msi12 * msi23 * msi31 + msi13 * msi21 * msi32 - msi31 * msi22 * msi13 -
             msi32 * msi23 * msi11 - msi33 * msi21 * msi12;
    ms11 = (msi22 * msi33 - msi23 * msi32) / detmsi;
    ms12 = (msi13 * msi32 - msi12 * msi33) / detmsi;
    ms13 = (msi12 * msi23 - msi13 * msi22) / detmsi;
    ms21 = (msi23 * msi31 - msi21 * msi33) / detmsi;
    ms22 = (msi11 * msi33 - msi13 * msi31) / detmsi;
    ms23 = (msi13 * msi21 - msi11 * msi23) / detmsi;
    ms31 = (msi21 * msi32 - msi22 * msi31) / detmsi;
    ms32 = (msi12 * msi31 - msi11 * msi32) / detmsi;
    ms33 = (msi11 * msi22 - msi12 * msi21) / detmsi;
    mst11 = ms11; mst12 = ms21; mst13 = ms31;
    mst21 = ms12; mst22 = ms22; mst23 = ms32;
    mst31 = ms13; mst32 = ms23; mst33 = ms33;
    detmst = mst11 * mst22 * mst33 + mst12 * mst23 * mst31 + mst13 * mst21 * mst32 - mst31 * mst22 * mst13 -
             mst32 * mst23 * mst11 - mst33 * mst21 * mst12;
    mt11 = (mst22 * mst33 - mst23 * mst32) / detmst;
    mt12 = (mst13 * mst32 - mst12 * mst33) / detmst;
    mt13 = (mst12 * mst23 - mst13 * mst22) / detmst;
    mt21 = (mst23 * mst31 - mst21 * mst33) / detmst;
    mt22 = (mst11 * mst33 - mst13 * mst31) / detmst;
    mt23 = (mst13 * mst21 - mst11 * mst23) / detmst;
    mt31 = (mst21 * mst32 - mst22 * mst31) / detmst;
    mt32 = (mst12 * mst31 - mst11 * mst32) / detmst;
    mt33 = (mst11 * mst22 - mst12 * mst21) / detmst;
    m11 = mt11; m12 = mt21; m13 = mt31;
    m21 = mt12; m22 = mt22; m23 = mt32;
    m31 = mt13; m32 = mt23; m33 = mt33;
    m11DD = a; m12DD = b * cg; m13DD = 0;
    m21DD = 0; m22DD = b * sg; m23DD = 0;

    float mi11, mi12, mi13, mi21, mi22, mi23, mi31, mi32, mi33, detm;
    detm = m11 * m22 * m33 + m12 * m23 * m31 + m13 * m21 * m32 - m31 * m22 * m13 - m32 * m23 * m11 - m33 * m21 * m12;
    mi11 = (m22 * m33 - m23 * m32) / detm;
    mi12 = (m13 * m32 - m12 * m33) / detm;
    mi13 = (m12 * m23 - m13 * m22) / detm;
    mi21 = (m23 * m31 - m21 * m33) / detm;
    mi22 = (m11 * m33 - m13 * m31) / detm;
    mi23 = (m13 * m21 - m11 * m23) / detm;
    mi31 = (m21 * m32 - m22 * m31) / detm;
    mi32 = (m12 * m31 - m11 * m32) / detm;
    mi33 = (m11 * m22 - m12 * m21) / detm;
    (void)mi11; (void)mi12; (void)mi13; (void)mi21; (void)mi22; (void)mi23; (void)mi31; (void)mi32; (void)mi33;

    aax = 1; aay = 0; aaz = 0;
    bax = 0; bay = 1; baz = 0;
    cax = 0; cay = 0; caz = 1;
    aaxt = 2 / 3.0; aayt = 2 / 3.0; aazt = -1 / 3.0;
    baxt = -1 / 3.0; bayt = 2 / 3.0; bazt = 2 / 3.0;
    caxt = 2 / 3.0; cayt = -1 / 3.0; cazt = 2 / 3.0;

    aex = m11 * aax + m12 * aay + m13 * aaz;
    aey = m21 * aax + m22 * aay + m23 * aaz;
    aez = m31 * aax + m32 * aay + m33 * aaz;
    bex = m11 * bax + m12 * bay + m13 * baz;
    bey = m21 * bax + m22 * bay + m23 * baz;
    bez = m31 * bax + m32 * bay + m33 * baz;
    cex = m11 * cax + m12 * cay + m13 * caz;
    cey = m21 * cax + m22 * cay + m23 * caz;
    cez = m31 * cax + m32 * cay + m33 * caz;
    aexDD = m11DD * aax + m12DD * aay + m13DD * aaz;
    aeyDD = m21DD * aax + m22DD * aay + m23DD * aaz;
    bexDD = m11DD * bax + m12DD * bay + m13DD * baz;
    beyDD = m21DD * bax + m22DD * bay + m23DD * baz;
    aext = m11 * aaxt + m12 * aayt + m13 * aazt;
    aeyt = m21 * aaxt + m22 * aayt + m23 * aazt;
    aezt = m31 * aaxt + m32 * aayt + m33 * aazt;
    bext = m11 * baxt + m12 * bayt + m13 * bazt;
    beyt = m21 * baxt + m22 * bayt + m23 * bazt;
    bezt = m31 * baxt + m32 * bayt + m33 * bazt;
    cext = m11 * caxt + m12 * cayt + m13 * cazt;
    ceyt = m21 * caxt + m22 * cayt + m23 * cazt;
    cezt = m31 * caxt + m32 * cayt + m33 * cazt;

    vvol = aex * (bey * cez - bez * cey) + aey * (bez * cex - bex * cez) + aez * (bex * cey - bey * cex);
    area = a * b * sg;
    asxDD = beyDD / area;
    asyDD = -bexDD / area;
    aszDD = 0;
    bsxDD = -aeyDD / area;
    bsyDD = aexDD / area;
    bszDD = 0;
    csxDD = 0;
    csyDD = 0;
    cszDD = 1;
    area1 = a;
    asxDL = 1 / area1;
    asyDL = 0;
    aszDL = 0;
    bsxDL = 0;
    bsyDL = 1;
    bszDL = 0;
    csxDL = 0;
    csyDL = 0;
    cszDL = 1;

    g11 = aex; g12 = bex; g13 = cex;
    g21 = aey; g22 = bey; g23 = cey;
    g31 = aez; g32 = bez; g33 = cez;
    detg = g11 * g22 * g33 + g12 * g23 * g31 + g13 * g21 * g32 - g31 * g22 * g13 - g32 * g23 * g11 - g33 * g21 * g12;
    gi11 = (g22 * g33 - g23 * g32) / detg;
    gi12 = (g13 * g32 - g12 * g33) / detg;
    gi13 = (g12 * g23 - g13 * g22) / detg;
    gi21 = (g23 * g31 - g21 * g33) / detg;
    gi22 = (g11 * g33 - g13 * g31) / detg;
    gi23 = (g13 * g21 - g11 * g23) / detg;
    gi31 = (g21 * g32 - g22 * g31) / detg;
    gi32 = (g12 * g31 - g11 * g32) / detg;
    gi33 = (g11 * g22 - g12 * g21) / detg;
    asxn = gi11; asyn = gi12; aszn = gi13;
    bsxn = gi21; bsyn = gi22; bszn = gi23;
    csxn = gi31; csyn = gi32; cszn = gi33;
    (void)asxn; (void)asyn; (void)aszn; (void)bsxn; (void)bsyn; (void)bszn; (void)csxn; (void)csyn; (void)cszn;

    nxyzx = m11 * u + m12 * v + m13 * w;
    nxyzy = m21 * u + m22 * v + m23 * w;
    nxyzz = m31 * u + m32 * v + m33 * w;
    len = std::sqrt(nxyzx * nxyzx + nxyzy * nxyzy + nxyzz * nxyzz);
    nxyznx = nxyzx / len;
    nxyznz = nxyzz / len;
    etheta = std::acos(-nxyznz);
    epsi = std::asin(nxyznx / std::sin(etheta));
    r11 = std::cos(epsi) * std::cos(ephi) - std::sin(epsi) * std::cos(etheta) * std::sin(ephi);
    r12 = -std::cos(epsi) * std::sin(ephi) - std::sin(epsi) * std::cos(etheta) * std::cos(ephi);
    r13 = std::sin(epsi) * std::sin(etheta);
    r21 = std::sin(epsi) * std::cos(ephi) + std::cos(epsi) * std::cos(etheta) * std::sin(ephi);
    r22 = -std::sin(epsi) * std::sin(ephi) + std::cos(epsi) * std::cos(etheta) * std::cos(ephi);
    r23 = -std::cos(epsi) * std::sin(etheta);
    r31 = std::sin(etheta) * std::sin(ephi);
    r32 = std::sin(etheta) * std::cos(ephi);
    r33 = std::cos(etheta);

    detr = r11 * r22 * r33 + r12 * r23 * r31 + r13 * r21 * r32 - r31 * r22 * r13 - r32 * r23 * r11 - r33 * r21 * r12;
    ri11 = (r22 * r33 - r23 * r32) / detr;
    ri12 = (r13 * r32 - r12 * r33) / detr;
    ri13 = (r12 * r23 - r13 * r22) / detr;
    ri21 = (r23 * r31 - r21 * r33) / detr;
    ri22 = (r11 * r33 - r13 * r31) / detr;
    ri23 = (r13 * r21 - r11 * r23) / detr;
    ri31 = (r21 * r32 - r22 * r31) / detr;
    ri32 = (r12 * r31 - r11 * r32) / detr;
    ri33 = (r11 * r22 - r12 * r21) / detr;

    aedx = ri11 * aex + ri12 * aey + ri13 * aez;
    aedy = ri21 * aex + ri22 * aey + ri23 * aez;
    aedz = ri31 * aex + ri32 * aey + ri33 * aez;
    bedx = ri11 * bex + ri12 * bey + ri13 * bez;
    bedy = ri21 * bex + ri22 * bey + ri23 * bez;
    bedz = ri31 * bex + ri32 * bey + ri33 * bez;
    cedx = ri11 * cex + ri12 * cey + ri13 * cez;
    cedy = ri21 * cex + ri22 * cey + ri23 * cez;
    cedz = ri31 * cex + ri32 * cey + ri33 * cez;
    aedxt = ri11 * aext + ri12 * aeyt + ri13 * aezt;
    aedyt = ri21 * aext + ri22 * aeyt + ri23 * aezt;
    aedzt = ri31 * aext + ri32 * aeyt + ri33 * aezt;
    bedxt = ri11 * bext + ri12 * beyt + ri13 * bezt;
    bedyt = ri21 * bext + ri22 * beyt + ri23 * bezt;
    bedzt = ri31 * bext + ri32 * beyt + ri33 * bezt;
    cedxt = ri11 * cext + ri12 * ceyt + ri13 * cezt;
    cedyt = ri21 * cext + ri22 * ceyt + ri23 * cezt;
    cedzt = ri31 * cext + ri32 * ceyt + ri33 * cezt;

    asedx = (bedy * cedz - bedz * cedy) / vvol;
    asedy = (bedz * cedx - bedx * cedz) / vvol;
    asedz = (bedx * cedy - bedy * cedx) / vvol;
    bsedx = (aedz * cedy - aedy * cedz) / vvol;
    bsedy = (aedx * cedz - aedz * cedx) / vvol;
    bsedz = (aedy * cedx - aedx * cedy) / vvol;
    csedx = (aedy * bedz - aedz * bedy) / vvol;
    csedy = (aedz * bedx - aedx * bedz) / vvol;
    csedz = (aedx * bedy - aedy * bedx) / vvol;

    asedxDD = ri11 * asxDD + ri12 * asyDD + ri13 * aszDD;
    asedyDD = ri21 * asxDD + ri22 * asyDD + ri23 * aszDD;
    asedzDD = ri31 * asxDD + ri32 * asyDD + ri33 * aszDD;
    bsedxDD = ri11 * bsxDD + ri12 * bsyDD + ri13 * bszDD;
    bsedyDD = ri21 * bsxDD + ri22 * bsyDD + ri23 * bszDD;
    bsedzDD = ri31 * bsxDD + ri32 * bsyDD + ri33 * bszDD;
    csedxDD = ri11 * csxDD + ri12 * csyDD + ri13 * cszDD;
    csedyDD = ri21 * csxDD + ri22 * csyDD + ri23 * cszDD;
    csedzDD = ri31 * csxDD + ri32 * csyDD + ri33 * cszDD;
    asedxDL = ri11 * asxDL + ri12 * asyDL + ri13 * aszDL;
    asedyDL = ri21 * asxDL + ri22 * asyDL + ri23 * aszDL;
    asedzDL = ri31 * asxDL + ri32 * asyDL + ri33 * aszDL;
    bsedxDL = ri11 * bsxDL + ri12 * bsyDL + ri13 * bszDL;
    bsedyDL = ri21 * bsxDL + ri22 * bsyDL + ri23 * bszDL;
    bsedzDL = ri31 * bsxDL + ri32 * bsyDL + ri33 * bszDL;
    csedxDL = ri11 * csxDL + ri12 * csyDL + ri13 * cszDL;
    csedyDL = ri21 * csxDL + ri22 * csyDL + ri23 * cszDL;
    csedzDL = ri31 * csxDL + ri32 * csyDL + ri33 * cszDL;

    asedxt = (bedyt * cedzt - bedzt * cedyt) / vvol;
    asedyt = (bedzt * cedxt - bedxt * cedzt) / vvol;
    asedzt = (bedxt * cedyt - bedyt * cedxt) / vvol;
    bsedxt = (aedzt * cedyt - aedyt * cedzt) / vvol;
    bsedyt = (aedxt * cedzt - aedzt * cedxt) / vvol;
    bsedzt = (aedyt * cedxt - aedxt * cedyt) / vvol;
    csedxt = (aedyt * bedzt - aedzt * bedyt) / vvol;
    csedyt = (aedzt * bedxt - aedxt * bedzt) / vvol;
    csedzt = (aedxt * bedyt - aedyt * bedxt) / vvol;

    m11 = asedx; m21 = bsedx; m31 = csedx;
    m12 = asedy; m22 = bsedy; m32 = csedy;
    m13 = asedz; m23 = bsedz; m33 = csedz;
    if (lat2d_) {
        m11 = asedxDD; m21 = bsedxDD; m31 = csedxDD;
        m12 = asedyDD; m22 = bsedyDD; m32 = csedyDD;
        m13 = asedzDD; m23 = bsedzDD; m33 = csedzDD;
        vvol = area;
    }
    if (lat1d_) {
        m11 = asedxDL; m21 = bsedxDL; m31 = csedxDL;
        m12 = asedyDL; m22 = bsedyDL; m32 = csedyDL;
        m13 = asedzDL; m23 = bsedzDL; m33 = csedzDL;
        vvol = area1;
    }
    mtw11 = asedxt; mtw21 = bsedxt; mtw31 = csedxt;
    mtw12 = asedyt; mtw22 = bsedyt; mtw32 = csedyt;
    mtw13 = asedzt; mtw23 = bsedzt; mtw33 = csedzt;
}

}  // namespace

// ---------------------------------------------------------------------------
// Gamma function exactly as the reference evaluates it
// (Source/sc_calc_generic_gpu.cu:613-673): polynomial of Abramowitz-Stegun
// 6.1.34 on (0,1], the 8-term fit 6.1.35 times a rising product on (1,1000],
// Stirling above. The coefficient tables must equal the reference's.
// ---------------------------------------------------------------------------
double ref_gamma(double z) {
    static const double bm[] = {0.0,         -0.577191652, 0.988205891,  -0.897056937, 0.918206857,
                                -0.756704078, 0.482199394, -0.193527818, 0.035868343};
    static const double cm[] = {0.0,
                                1.0000000000000000,  0.5772156649015329,  -0.6558780715202538, -0.0420026350340952,
                                0.1665386113822915,  -0.0421977345555443, -0.0096219715278770, 0.00721894322466630,
                                -0.0011651675918591, -0.0002152416741149, 0.0001280502823882,  -0.0000201348547807,
                                -0.0000012504934821, 0.0000011330272320,  -0.0000002056338417, 0.0000000061160950,
                                0.0000000050020075,  -0.0000000011812746, 0.0000000001043427,  0.0000000000077823,
                                -0.0000000000036968, 0.0000000000005100,  -0.0000000000000206, -0.0000000000000054,
                                0.0000000000000014,  0.0000000000000001};
    auto frac = [](double x) {
        double ip;
        return std::modf(x, &ip);
    };
    bool negative;
    if (std::fabs(z) < kEps9) z = z + kEps9;
    if (z > 0)
        negative = false;
    else {
        negative = true;
        if (std::fabs(frac(z)) < kEps9) z = z + kEps9;
    }
    const double absz = std::fabs(z);
    if (absz > 0.0 && absz <= 1) {
        double fct = 0;
        for (int i = 1; i <= 26; i++) fct += cm[i] * std::pow(absz, i);
        if (negative) return -M_PI * fct / (absz * std::sin(M_PI * absz));
        return 1. / fct;
    }
    if (absz > 1 && absz <= 1000) {
        if (std::fabs(frac(absz)) < kEps9) {
            double fct = 1;
            for (int i = 1; i <= std::trunc(absz) - 1; i++) fct = fct * i;
            if (negative) return -M_PI / (absz * fct * std::sin(M_PI * absz));
            return fct;
        }
        const double y = absz - 1;
        const double di = std::trunc(y);
        const double x = absz - std::trunc(absz);
        double fak = y;
        if (di == 0)
            fak = 1;
        else
            for (int i = 1; i < di; i++) fak = fak * (y - i);
        double f = 1;
        for (int i = 1; i <= 8; i++) f = f + bm[i] * std::pow(x, i);
        if (negative) return -M_PI / (absz * fak * f * std::sin(M_PI * absz));
        return fak * f;
    }
    double fct = std::exp(-absz) * std::exp((absz - 0.5) * std::log(absz)) * std::sqrt(2 * M_PI);
    if (negative) return -M_PI / (absz * fct * std::sin(M_PI * absz));
    return fct;
}

// ---------------------------------------------------------------------------
// Validation: isCbsValid / checkAllParameters, sc_calc_generic_cpu.cpp:119-308.
// ---------------------------------------------------------------------------
std::string check_all_parameters(const cs_params &in, int shp, int ign_cbs) {
    if (in.uca <= 0.01) return "uca<=0.01";
    if (in.ucb <= 0.01) return "ucb<=0.01";
    if (in.ucc <= 0.01) return "ucb<=0.01";  // the reference reports ucc with this text
    if (!ign_cbs) {
        const int lt = in.ltype, pa = in.particle, od = in.ordis, inn = in.interior, pk = shp;
        if ((lt < 0) || (lt > 19)) return "INVALID ltype value";
        if ((pa < 0) || (pa > 10)) return "INVALID Particle value";
        if ((od < 0) || (od > 13)) return "INVALID Ordis value";
        if ((inn < 0) || (inn > 4)) return "INVALID Interior value";
        if ((pk < 1) || (pk > 8)) return "INVALID Peak value";
        int fixed_part = -1, fixed_peak = -1;
        switch (lt) {
        case 0: fixed_part = 2; break;
        case 1: case 2: case 3: fixed_part = 1; break;
        case 4: case 5: case 6: case 7: case 8: case 17: fixed_part = 0; break;
        case 9: case 10: case 11: fixed_part = 3; break;
        case 12: break;
        case 13: fixed_part = 0; fixed_peak = 7; break;
        case 14: case 15: fixed_part = 0; break;
        case 16: fixed_part = 2; break;
        case 18: fixed_part = 0; break;
        case 19: fixed_part = 0; fixed_peak = 7; break;
        }
        if (fixed_part != -1 && in.particle != fixed_part) return "INVALID CBParticle due to LatticeType";
        if (lt != 12) {
            if (fixed_peak != -1 && shp != fixed_peak) return "INVALID CBPeak due to LatticeType";
        }
    }
    if (in.ltype == 0 && in.particle == 2 && in.ordis == 0 && in.interior == 0 && shp == 7) return "INVALID";
    if (in.ltype == 0 && in.particle == 2 && in.ordis == 0 && in.interior == 3 && (shp == 1 || shp == 2 || shp == 8) &&
        in.radiusi >= 0.5)
        return "EditRadiusi>=0.5";
    return "";
}

// ---------------------------------------------------------------------------
// prepareCalculation, sc_calc_generic_cpu.cpp:319-988.
// ---------------------------------------------------------------------------
int prepare(const cs_params &in, int calc_quadrants, int expand, int ign_new_switch, int ign_cbs, int check,
            cs_prepared *out, std::string &err) {
    const int shp = in.peak + 1;  // setComboBoxPeak: shp = v+1
    if (check) {
        err = check_all_parameters(in, shp, ign_cbs);
        if (!err.empty()) return CS_ERR_PARAM;
    }

    Prep S;
    S.in = in;
    S.out = out;
    cs_prepared &P = *out;
    std::memset(&P, 0, sizeof(P));

    P.particle = in.particle;
    P.shp = shp;
    P.ltype = in.ltype;
    P.ordis = in.ordis;
    P.ign_switch = ign_new_switch ? 1 : 0;

    if (in.ltype == 0) {
        S.lat1d = true;
        S.lat3d = false;
    }
    if ((in.ltype == 1) || (in.ltype == 2) || (in.ltype == 3)) {
        S.lat2d = true;
        S.lat3d = false;
    }
    P.use1d = in.use1d ? 1 : 0;
    P.zmax = in.gridpoints;
    if (in.use1d) {
        P.zzmin = 0;
        P.zzmax = P.zmax;
        P.iimin = 0;
        P.iimax = 1;
        calc_quadrants = CS_RAD1D;
        expand = 0;
    } else {
        if (in.ltype == 14 || in.ltype == 15) calc_quadrants = CS_RADQ4;
        P.zzmin = calc_quadrants == CS_RADQ4 ? -P.zmax : 0;
        P.zzmax = P.zmax;
        P.iimin = calc_quadrants == CS_RADQ1 ? 0 : -P.zmax;
        P.iimax = P.zmax;
    }
    P.calc_quadrants = calc_quadrants;
    P.expand = expand;

    // copy parameters into the prepared block (params.* and members)
    P.radius = in.radius;
    P.radiusi = in.radiusi;
    P.sigma = in.sigma;
    P.sigmal = in.sigmal;
    P.length = in.length;
    P.rho = in.rho;
    P.alphash1 = in.alphash;
    P.alpha = in.alpha;
    P.poltheta = in.theta;
    P.polphi = in.phi;
    P.dbeta = in.dbeta;
    P.uca = in.uca;
    P.ucb = in.ucb;
    P.domainsize = in.domainsize;
    // domain-size width factor: 1, or its training-data randomisation
    // 1 * (1 + dev) (tpvPerformRandom, :1076, :1112-1113)
    P.width_zuf = 1 + in.tpv_domain_dev;
    P.ceff = in.ceff;
    P.qmax = in.qmax;
    P.qmin = in.qmin;
    P.pixnox = in.pixnox;
    P.pixnoy = in.pixnoy;
    P.pixx_m = in.pixx_mm / 1000.;
    P.pixy_m = in.pixy_mm / 1000.;
    P.det = in.det;
    P.wave = in.wavelength;
    P.beamx0 = in.beamx;
    P.beamy0 = in.beamy;
    P.usebeamstop = in.usebeamstop ? 1 : 0;
    P.base = in.base;
    P.izero = in.izero;
    P.iso = in.iso;
    P.ifluc = in.ifluc;
    P.rfluc = in.rfluc;
    for (int i = 0; i < 3; i++) {
        P.ax1[i] = in.ax1[i];
        P.ax2[i] = in.ax2[i];
        P.ax3[i] = in.ax3[i];
        P.sig[i] = 4.0 / in.sigxyz[i];
    }
    S.dwfactor = in.debyewaller * in.debyewaller / 3.0;  // setDisplacement
    // training-data randomisation of dwfactor (tpvPerformRandom, :1126-1129)
    if (in.tpv_dw_dev != 0) S.dwfactor = S.dwfactor * (1 + in.tpv_dw_dev);
    P.dwfactor = S.dwfactor;

    S.phiwidth = 4. / in.azi;
    P.phiwidth = S.phiwidth;
    P.p1 = P.radius / P.radiusi;

    P.cosphi = std::cos(P.polphi * M_PI / 180.0);
    P.sinphi = std::sin(P.polphi * M_PI / 180.0);
    P.costheta = std::cos(P.poltheta * M_PI / 180.0);
    P.sintheta = std::sin(P.poltheta * M_PI / 180.0);

    const double cosa = std::cos(in.ucalpha * M_PI / 180.0);
    const double cosb = std::cos(in.ucbeta * M_PI / 180.0);
    const double cosg = std::cos(in.ucgamma * M_PI / 180.0);
    S.ucvol = in.uca * in.ucb * in.ucc * std::sqrt(1.0 - sqr(cosa) - sqr(cosb) - sqr(cosg) + 2 * cosa * cosb * cosg);

    P.twin = in.twinned ? 1 : 0;
    P.lattice = (in.ltype == 12) ? 0 : 1;
    P.debyescherrer = in.debyescherrer ? 1 : 0;
    P.para = in.para ? 1 : 0;

    switch (in.particle) {
    case 0: P.part = 0; S.partdim = 3; S.cdim = 3; break;
    case 1: P.part = 1; S.partdim = 2; S.cdim = 1; break;
    case 2: P.part = 2; S.partdim = 1; S.cdim = 2; break;
    case 3: P.part = 3; S.partdim = 3; S.cdim = 3; break;
    case 4: P.part = 4; S.partdim = 4; S.cdim = 4; break;
    default:
        if (in.particle >= 5 && in.particle <= 10) {
            P.part = in.particle;
            S.partdim = in.particle;
            S.cdim = in.particle;
        }
        break;
    }
    P.cdim = S.cdim;
    P.partdim = S.partdim;
    switch (in.interior) {
    case 0: P.cs = 0; break;
    case 1: P.cs = 1; P.alphash1 = 0.0001; break;
    case 2: P.cs = 2; break;
    case 3: P.cs = 3; break;
    case 4: P.cs = 4; break;
    }

    switch (in.ltype) {
    case 5: case 13: case 17: case 19: S.dist = std::sqrt(2.0) * in.uca / 2.0; break;
    case 4: case 9: case 11: S.dist = std::sqrt(3.0) * in.uca / 2.0; break;
    default: S.dist = in.uca; break;
    }
    S.reldis = in.debyewaller / S.dist;
    P.dist = S.dist;
    P.reldis = S.reldis;

    if ((S.cdim != 9) && (S.cdim != 10)) {
        if (!S.coefficients()) {
            err = S.err.empty() ? "coefficients: no calculation done" : S.err;
            return CS_ERR_UNSUPPORTED;
        }
    } else {
        err = "chain particles are not implemented";
        return CS_ERR_UNSUPPORTED;
    }

    {
        // pixel-independent Gamma ratios of formfq_partCylinder's asymptote
        // (Source/sc_lib_formfq_partCylinder.h:209-210)
        const double zr = (1 - sqr(P.sigma)) / sqr(P.sigma);
        P.gamma_ratio[0] = ref_gamma(zr - 1 / 2.0) / ref_gamma(zr + 1);
        P.gamma_ratio[1] = ref_gamma(zr - 3 / 2.0) / ref_gamma(zr + 1);
    }

    {
        // limits and direction matrix of qrombdeltac for the cylinder and disk
        // orientation averages (Source/sc_calc_generic_gpu.cu:1394-1434), with
        // theta = polTheta and phi = 0 as formpq_partCylinder passes them
        // (Source/sc_lib_formpq_partCylinder.h:207), phi = polPhi as
        // formpq_partDisk does (Source/sc_lib_formpq_partDisk.h:183)
        const double dbeta = P.dbeta * M_PI / 180.0;
        const double theta = P.poltheta * M_PI / 180.0;
        const double phi = (P.particle == 2 ? P.polphi : 0) * M_PI / 180.0;
        double delmax = dbeta * std::sqrt(std::log(1.0 / 0.00001));
        if (delmax > M_PI / 2.0) delmax = M_PI / 2.0;
        float blim = delmax;
        float chib = 2 * M_PI;
        P.romb_delta_b = blim;
        P.romb_chi_b = chib;
        P.romb_dbeta = dbeta;
        float p11 = -std::cos(phi) * std::cos(theta);
        float p12 = std::sin(phi);
        float p13 = std::cos(phi) * std::sin(theta);
        float p21 = -std::cos(phi);
        float p22 = -std::sin(phi) * std::cos(theta);
        float p23 = std::sin(phi) * std::sin(theta);
        float p31 = -std::sin(theta);
        float p32 = 0;
        float p33 = -std::cos(theta);
        const float pm[9] = {p11, p12, p13, p21, p22, p23, p31, p32, p33};
        for (int i = 0; i < 9; i++) P.romb_p[i] = pm[i];
    }

    if (P.lattice) {
        std::string e = S.hkl_tables(in.ltype);
        if (!e.empty()) {
            err = "lattice type " + std::to_string(in.ltype) + ": " + e;
            return CS_ERR_UNSUPPORTED;
        }
        P.peakmax1 = P.latpar1[1][0];
        P.peakmax2 = P.latpar2[1][0];
        double ri11, ri12, ri13, ri21, ri22, ri23, ri31, ri32, ri33;
        double rt11, rt12, rt13, rt21, rt22, rt23, rt31, rt32, rt33;
        S.corotations(in.uca, in.ucb, in.ucc, in.ucalpha, in.ucbeta, in.ucgamma, in.ucn1, in.ucn2, in.ucn3, in.ucpsi,
                      S.lat1d, S.lat2d, ri11, ri12, ri13, ri21, ri22, ri23, ri31, ri32, ri33, rt11, rt12, rt13, rt21,
                      rt22, rt23, rt31, rt32, rt33, S.ucvol);

        double sphno = 1, qhkl0, fhkl, qhkl;
        for (int peakct1 = 1; peakct1 <= P.peakmax1; peakct1++) {
            int h = P.latpar1[peakct1][1], k = P.latpar1[peakct1][2], l = P.latpar1[peakct1][3];
            S.fhkl_c(in.ltype, h, k, l, sphno, fhkl, qhkl, qhkl0);
            P.latpar1[peakct1][5] = (int)std::round(fhkl);
            P.latpar[1] = S.ucvol;
            P.latpar[2] = sphno;
            P.latpar[3] = S.dwfactor;
        }
        if (P.peakmax1 == 0) {
            P.latpar[1] = S.ucvol;
            P.latpar[2] = 1;
            P.latpar[3] = S.dwfactor;
        }
        for (int peakct2 = 1; peakct2 <= P.peakmax2; peakct2++) {
            int h = P.latpar2[peakct2][1], k = P.latpar2[peakct2][2], l = P.latpar2[peakct2][3];
            int mhkl = 1;
            S.fhkl_c(in.ltype, h, k, l, sphno, fhkl, qhkl, qhkl0);
            P.latpar2[peakct2][5] = (int)std::round(fhkl);
            P.latpar2[peakct2][4] = mhkl;
            float *l3 = P.latpar3[peakct2];
            l3[1] = 2 * M_PI / in.uca;
            const double qxhkl = (2 * M_PI) * (ri11 * h + ri21 * k + ri31 * l);
            const double qyhkl = (2 * M_PI) * (ri12 * h + ri22 * k + ri32 * l);
            const double qzhkl = (2 * M_PI) * (ri13 * h + ri23 * k + ri33 * l);
            const double qxyhkl = (2 * M_PI) * std::sqrt(h * h * (ri11 * ri11 + ri12 * ri12 + ri13 * ri13) +
                                                         k * k * (ri21 * ri21 + ri22 * ri22 + ri23 * ri23));
            qhkl = std::sqrt(qxhkl * qxhkl + qyhkl * qyhkl + qzhkl * qzhkl);
            if (std::isnan(qhkl)) {
                if (peakct2 > 5) break;
            }
            l3[2] = qxhkl;
            l3[3] = qyhkl;
            l3[4] = qzhkl;
            l3[5] = qhkl;
            l3[6] = qhkl / (2.0 * M_PI);
            l3[7] = (2 * M_PI) * (rt11 * h + rt21 * k + rt31 * l);
            l3[8] = (2 * M_PI) * (rt12 * h + rt22 * k + rt32 * l);
            l3[9] = (2 * M_PI) * (rt13 * h + rt23 * k + rt33 * l);
            const double g3 = 4 * M_PI * M_PI / (2.0 * M_PI * qhkl * qhkl);
            const double x2phihkl = 4 * qhkl * qhkl / (M_PI * S.phiwidth * S.phiwidth);
            double peaknorm1 = 0, peaknorm2 = 0;
            const double beta = in.peakpar;
            switch (shp) {
            case 1: peaknorm1 = lorentznorm3(x2phihkl); break;
            case 2: peaknorm1 = gaussnorm3(x2phihkl); break;
            case 3: peaknorm1 = pearsonnorm3(x2phihkl, 2); break;
            case 4: peaknorm1 = pearsonnorm3(x2phihkl, 3 / 2.0); break;
            case 5: peaknorm1 = lorentznorm3(x2phihkl); break;
            case 6: peaknorm1 = pearsonnorm3(x2phihkl, beta); break;
            case 7: peaknorm1 = gaussnorm3(x2phihkl); break;
            case 8: peaknorm1 = 0; peaknorm2 = 0; break;
            }
            l3[10] = g3;
            l3[11] = peaknorm1;
            l3[12] = peaknorm2;
            l3[13] = qxyhkl;
        }
    }

    // :904-910 (uses polPhi after coefficients() may have reset it)
    P.sinphic = std::sin(-P.polphi * M_PI / 180.);
    P.cosphic = std::cos(-P.polphi * M_PI / 180.);

    // the anisotropic Gaussian peak on a lattice replaces norm by the
    // distribution's norm integral (qrombdeltac i0 = 2, :967-973), which
    // the particle's form factor then divides by as well
    if (shp == 8 && P.lattice) P.norm = qromb_delta_1d(2, 0, P.dbeta);

    // the anisotropic Gaussian peak: perfect orientation (z-direction or
    // dbeta = 0) and isotropic particles; the fiber pattern and the other
    // orientations (the unit-cell rotation integrals) are not built
    if (shp == 8 && P.lattice && !(P.ordis == 6 || std::fabs(P.dbeta) < kEps9 || P.ordis == 7)) {
        err = "anisotropic Gaussian peak shape: only the perfect and isotropic orientations are implemented";
        return CS_ERR_UNSUPPORTED;
    }

    if (expand) {
        P.xmin = -P.zmax;
        P.xmax = P.zmax;
        P.ymin = -P.zmax;
        P.ymax = P.zmax;
    } else {
        P.xmin = P.zzmin;
        P.xmax = P.zzmax;
        P.ymin = P.iimin;
        P.ymax = P.iimax;
    }

    // peak-shape constants, :585-590 (c0 = 1 is written as a literal), and
    // setPeakPar (eta = peakpar/100, beta = peakpar)
    P.pk_c1 = 4;
    P.pk_c2 = 4 * (std::sqrt(2.0) - 1);
    P.pk_c3 = 4 * (std::exp(2 * std::log(2.0) / 3.0) - 1);
    P.pk_beta = in.peakpar;
    P.pk_c4 = (P.pk_beta == 0) ? 1 : std::exp(std::log(2.) / P.pk_beta) - 1;
    P.pk_eta = in.peakpar / 100.;
    P.pk_gbeta = P.pk_gbeta_h = 0;
    if (shp == 6) {
        P.pk_gbeta = ref_gamma(P.pk_beta);
        P.pk_gbeta_h = ref_gamma(P.pk_beta - 0.5);
    }

    // dispatch key, Source/sc_calc_generic_gpu.cu:113: the specialised pixel
    // functions, else calc_GENERIC (also for every combination when the new
    // switch is ignored)
    P.key = (P.particle << 24) | (P.ltype == 12 ? 0 : (shp << 16)) | (P.ltype << 8) | P.ordis;
    const bool special = !P.ign_switch &&
                         (P.key == CS_KEY_SPHERE_NONE_ISO || P.key == CS_KEY_SPHERE_GAUSS_FCC_GAUSS ||
                          P.key == CS_KEY_CYL_NONE_GAUSS || P.key == CS_KEY_CYL_NONE_ZDIR ||
                          P.key == CS_KEY_CYL_GAUSS_BCT_ZDIR || P.key == CS_KEY_CUBE_NONE_ISO);
    if (!special) {
        // the generic pixel function covers the particles prepared above:
        // spheres, cylinders (z-direction, Gaussian orientation; isotropic,
        // homogeneous or core/shell), homogeneous
        // isotropic cubes, disks (isotropic, or z-direction or Gaussian along
        // an axis; homogeneous or core/shell),
        // isotropic or z-direction vesicles, and homogeneous isotropic
        // ellipsoids
        const bool ok = P.particle == 0 || (P.particle == 1 && (P.ordis == 6 || P.ordis == 0)) ||
                        (P.particle == 1 && P.ordis == 7 && (P.cs == 0 || P.cs == 1)) ||
                        (P.particle == 4 && P.ordis == 7 && P.cs == 0) ||
                        (P.particle == 2 && P.ordis == 6 && (P.cs == 0 || P.cs == 1) &&
                         P.orcase != CS_ORC_GENERAL) ||
                        (P.particle == 2 && P.ordis == 0 && (P.cs == 0 || P.cs == 1) &&
                         P.orcase != CS_ORC_GENERAL) ||
                        (P.particle == 2 && P.ordis == 7 && (P.cs == 0 || P.cs == 1)) ||
                        (P.particle == 3 && (P.ordis == 7 || P.ordis == 6)) ||
                        (P.particle == 5 && P.ordis == 7 && P.cs == 0);
        if (!ok) {
            err = "generic pixel function: particle " + std::to_string(P.particle) + " with ordis " +
                  std::to_string(P.ordis) + " is not implemented";
            return CS_ERR_UNSUPPORTED;
        }
        P.key = CS_KEY_GENERIC;
    }
    for (int i = 0; i < 4; i++) {
        P.nofit_x0[i] = P.nofit_x1[i] = P.nofit_y0[i] = P.nofit_y1[i] = -1;
    }
    return CS_OK;
}


// ---------------------------------------------------------------------------
// Orientation node tables (see cs_tables.h): node x of level j in the
// reference's order, x = a + del/2 then x += del, with a = 0. The chi table
// (CS_CHI_TABLE_LEN slots) also holds the FP32 copies after the FP64 nodes.
// ---------------------------------------------------------------------------
void build_chi_table(double chi_b, cs_chi_node *tab) {
    const double a = 0.0, b = chi_b;
    tab[0].c = std::cos(a);
    tab[0].s = std::sin(a);
    tab[1].c = std::cos(b);
    tab[1].s = std::sin(b);
    for (int j = 2; j <= CS_NODE_LEVELS; j++) {
        const int cnt = 1 << (j - 2);
        const double tnm = cnt;
        const double del = (b - a) / tnm;
        double x = a + 0.5 * del;
        cs_chi_node *nd = tab + CS_NODE_OFFSET(j);
        for (int k = 0; k < cnt; k++) {
            nd[k].c = std::cos(x);
            nd[k].s = std::sin(x);
            x += del;
        }
    }
    cs_chi_node_f *f = reinterpret_cast<cs_chi_node_f *>(tab + CS_NODE_COUNT);
    for (int k = 0; k < CS_NODE_COUNT; k++) {
        f[k].c = (float)tab[k].c;
        f[k].s = (float)tab[k].s;
    }
}

void build_delta_table(double delta_b, double dbeta, cs_delta_node *tab) {
    const double a = 0.0, b = delta_b;
    auto fill = [&](cs_delta_node &n, double x) {
        n.w = std::sin(x) * std::exp(-x * x / (dbeta * dbeta));
        n.c = std::cos(x);
        n.s = std::sin(x);
    };
    fill(tab[0], a);
    fill(tab[1], b);
    for (int j = 2; j <= CS_NODE_LEVELS; j++) {
        const int cnt = 1 << (j - 2);
        const double tnm = cnt;
        const double del = (b - a) / tnm;
        double x = a + 0.5 * del;
        cs_delta_node *nd = tab + CS_NODE_OFFSET(j);
        for (int k = 0; k < cnt; k++) {
            fill(nd[k], x);
            x = x + del;
        }
    }
}

bool needs_delta_table(const cs_prepared &P) { return P.ordis == 0 && (P.part == 1 || P.part == 2); }

}  // namespace cs
