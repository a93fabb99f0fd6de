// cs_simplex.cpp — the 2D simplex fit (include/crystalscatter.h, cs_simplex_fit).
//
// Restates SasCalc_SimplexFit2D::doSimplexFit2D, amotry and
// fehlerquadratsumme (Source/sc_simplexfit2d.cpp:19-611): a downhill simplex
// over the fitted parameters, each vertex judged by the chi^2 of
// doFitCalculation. Two reference behaviours that change the trajectory are
// kept: the initialisation loop that zeroes the first parameter of every
// initial vertex (its inner loop tests and increments the outer index,
// :375-380), and amotry's centroid factor over all parameters (fitted and
// fixed, :227-236), which also hands the fixed parameters' vertex sums to the
// evaluation.
//
// Evaluation schedules:
//   CS_FIT_SEQUENTIAL  one drop-in fit evaluation per vertex, in the
//                      reference's order (cs_fit_chi2 on a handle; the mixed
//                      mode uses a one-set batch);
//   CS_FIT_BATCHED     independent evaluations in one batch: the initial
//                      vertices, the shrink step, and per iteration the four
//                      candidates the reference may ask for next (reflection,
//                      expansion, contraction after an accepted or a rejected
//                      reflection), evaluated speculatively. Evaluations are
//                      pure functions of the parameters, so the decisions and
//                      the result equal the sequential schedule's.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/crystalscatter.h"
#include "cs_params_internal.h"

namespace {

const int kNap = 31;  // nap (Source/sc_simplexfit2d.h)
const int kMap = 30;  // map

struct Fit {
    // inputs
    cs_params base;
    const double *data = nullptr;
    int width = 0, height = 0;
    int nofit[16];
    int border = 0, bstop = 0, mode = CS_MODE_FP64, schedule = CS_FIT_SEQUENTIAL;
    // parameter table in the reference's order (fitted keys sorted, then fixed keys sorted)
    std::vector<std::string> keys;
    bool enabled[kNap];
    double values[kNap], minv[kNap], maxv[kNap];
    int numFit = 0, mmax = 0;
    // engines
    cs_handle *h = nullptr;
    cs_batch *b = nullptr;
    cs_objective_fn fn = nullptr;  // caller's objective instead of the image chi^2
    void *fn_ctx = nullptr;
    long images = 0;
    std::string err;
    int status = CS_OK;
    double chi2_stop = 0;  // stop once the best vertex reaches it (0: off)
};

// fehlerquadratsumme's limit check (Source/sc_simplexfit2d.cpp:24-42): true
// when the point is outside and its value is 1e20 without a calculation
bool out_of_limits(const Fit &F, const double *par) {
    for (int j = 0; j < F.numFit; j++) {
        if (!F.enabled[j]) continue;
        if (F.minv[j] == 0.0 && F.maxv[j] == 360.0) continue;
        if (par[j] < F.minv[j]) return true;
        if (par[j] > F.maxv[j]) return true;
    }
    return false;
}

// the parameter set of one evaluation: every parameter of the table set by key
// (updateParamValue for j < mmax, :43-50)
bool params_for(const Fit &F, const double *par, cs_params &p) {
    p = F.base;
    for (int j = 0; j < F.mmax; j++)
        if (!cs::set_param(&p, F.keys[j].c_str(), par[j])) return false;
    return true;
}

// chi^2 of several points (each kMap doubles); 1e20 outside the limits or on
// failure (the reference's value of a failed evaluation)
void evaluate(Fit &F, const std::vector<std::vector<double>> &pts, std::vector<double> &y) {
    y.assign(pts.size(), 1e20);
    if (F.status != CS_OK) return;
    std::vector<int> idx;
    std::vector<cs_params> sets;
    for (size_t k = 0; k < pts.size(); k++) {
        if (out_of_limits(F, pts[k].data())) continue;
        cs_params p;
        if (F.fn) {
            idx.push_back((int)k);
            continue;
        }
        if (!params_for(F, pts[k].data(), p)) {
            F.status = CS_ERR_PARAM;
            F.err = "unknown parameter key in the fit table";
            return;
        }
        idx.push_back((int)k);
        sets.push_back(p);
    }
    if (idx.empty()) return;
    if (F.fn) {
        // caller's objective: one call per batch (sequential: one point per call)
        const size_t step = F.schedule == CS_FIT_SEQUENTIAL ? 1 : idx.size();
        for (size_t n0 = 0; n0 < idx.size(); n0 += step) {
            const size_t n1 = std::min(idx.size(), n0 + step);
            std::vector<double> buf((n1 - n0) * (size_t)F.mmax), val(n1 - n0, 1e20);
            for (size_t n = n0; n < n1; n++)
                for (int j = 0; j < F.mmax; j++) buf[(n - n0) * F.mmax + j] = pts[idx[n]][j];
            F.fn(buf.data(), (int)(n1 - n0), F.mmax, val.data(), F.fn_ctx);
            F.images += (long)(n1 - n0);
            for (size_t n = n0; n < n1; n++) y[idx[n]] = val[n - n0];
        }
        return;
    }
    if (F.schedule == CS_FIT_SEQUENTIAL && F.mode == CS_MODE_FP64) {
        for (size_t n = 0; n < idx.size(); n++) {
            cs_set_params(F.h, &sets[n]);
            double chi2 = 1e20;
            long cnt = 0, nan = 0;
            const int rc = cs_fit_chi2(F.h, 0, F.bstop, F.border, CS_MODE_FP64, &chi2, &cnt, &nan);
            F.images++;
            if (rc != CS_OK && rc != CS_ERR_PARAM) {
                F.status = rc;
                F.err = cs_last_error(F.h);
                return;
            }
            y[idx[n]] = chi2;
        }
        return;
    }
    // batched (and the sequential mixed mode, one set at a time)
    const size_t step = F.schedule == CS_FIT_SEQUENTIAL ? 1 : idx.size();
    for (size_t n0 = 0; n0 < idx.size(); n0 += step) {
        const size_t n1 = std::min(idx.size(), n0 + step);
        int rc = cs_batch_prepare(F.b, sets.data() + n0, (int)(n1 - n0), 0, 1, 0);
        std::vector<double> chi2(n1 - n0, 1e20);
        std::vector<long> cnt(n1 - n0), nan(n1 - n0);
        if (rc == CS_OK) rc = cs_batch_fit_chi2(F.b, F.mode, chi2.data(), cnt.data(), nan.data());
        F.images += (long)(n1 - n0);
        if (rc != CS_OK && rc != CS_ERR_PARAM) {
            F.status = rc;
            F.err = cs_batch_last_error(F.b);
            return;
        }
        for (size_t n = n0; n < n1; n++) y[idx[n]] = chi2[n - n0];
    }
}

// amotry's test vertex (Source/sc_simplexfit2d.cpp:224-236)
std::vector<double> try_point(const Fit &F, const double p[kNap][kMap], const double *sum, int ihi, double fac) {
    std::vector<double> ptry(kMap, 0.0);
    for (int j = 0; j < F.mmax; j++) ptry[j] = sum[j];
    const double fac1 = (1.0 - fac) / F.mmax;
    const double fac2 = fac1 - fac;
    for (int j = 0; j < F.numFit; j++) ptry[j] = sum[j] * fac1 - p[ihi][j] * fac2;
    return ptry;
}

// amotry's acceptance (:238-248)
double accept(const Fit &F, double p[kNap][kMap], double *y, double *sum, int ihi, const std::vector<double> &ptry,
              double ytry) {
    if (ytry < y[ihi]) {
        y[ihi] = ytry;
        for (int j = 0; j < F.numFit; j++) {
            sum[j] += ptry[j] - p[ihi][j];
            p[ihi][j] = ptry[j];
        }
    }
    return ytry;
}

int run_simplex(Fit &F, cs_fit_param *params, int nparams, double stp, int maxit, double ftol,
                cs_fit_report *report);

}  // namespace

extern "C" {

int cs_simplex_fit(const cs_params *base, const double *data, int width, int height, const int *nofit,
                   cs_fit_param *params, int nparams, double stp, int maxit, double ftol, int borderpix, int bstoppix,
                   int mode, int schedule, double chi2_stop, cs_fit_report *report) {
    if (!base || !data || width <= 0 || height <= 0 || !params || nparams <= 0 || !report) return CS_ERR_PARAM;
    std::memset(report, 0, sizeof(*report));
    if (mode != CS_MODE_FP64 && mode != CS_MODE_MIXED) return CS_ERR_PARAM;
    if (schedule != CS_FIT_SEQUENTIAL && schedule != CS_FIT_BATCHED) return CS_ERR_PARAM;
    Fit F;
    F.base = *base;
    F.data = data;
    F.width = width;
    F.height = height;
    for (int i = 0; i < 16; i++) F.nofit[i] = nofit ? nofit[i] : -1;
    F.border = borderpix;
    F.bstop = bstoppix;
    F.mode = mode;
    F.schedule = schedule;
    F.chi2_stop = chi2_stop;
    return run_simplex(F, params, nparams, stp, maxit, ftol, report);
}

int cs_simplex_minimize(cs_objective_fn fn, void *ctx, cs_fit_param *params, int nparams, double stp, int maxit,
                        double ftol, int schedule, double chi2_stop, cs_fit_report *report) {
    if (!fn || !params || nparams <= 0 || !report) return CS_ERR_PARAM;
    std::memset(report, 0, sizeof(*report));
    if (schedule != CS_FIT_SEQUENTIAL && schedule != CS_FIT_BATCHED) return CS_ERR_PARAM;
    Fit F;
    F.fn = fn;
    F.fn_ctx = ctx;
    F.schedule = schedule;
    F.chi2_stop = chi2_stop;
    return run_simplex(F, params, nparams, stp, maxit, ftol, report);
}

}  // extern "C"

namespace {

int run_simplex(Fit &F, cs_fit_param *params, int nparams, double stp, int maxit, double ftol,
                cs_fit_report *report) {
    const int schedule = F.schedule, mode = F.mode;
    const auto t0 = std::chrono::steady_clock::now();

    // the parameter table: fitted keys in sorted order, then fixed keys sorted
    // (:283-321)
    std::vector<int> order(nparams);
    for (int i = 0; i < nparams; i++) order[i] = i;
    std::sort(order.begin(), order.end(), [&](int a, int c) { return std::strcmp(params[a].key, params[c].key) < 0; });
    std::vector<int> table;
    for (int pass = 0; pass < 2; pass++)
        for (int k : order) {
            if ((params[k].used != 0) != (pass == 0)) continue;
            const int i = (int)table.size();
            if (i >= kNap) break;
            table.push_back(k);
            F.keys.push_back(params[k].key);
            F.enabled[i] = pass == 0;
            F.values[i] = params[k].fitstart;
            F.minv[i] = params[k].min;
            F.maxv[i] = params[k].max;
            if (pass == 0) F.numFit = i + 1;
        }
    F.mmax = (int)F.keys.size();
    if (F.mmax >= kNap) {
        std::snprintf(report->info, sizeof report->info,
                      "The maximum array length (%d) was exeeded by the current number of fitable parameters (%d)", kNap,
                      F.mmax);
        return CS_ERR_PARAM;
    }
    // engines
    if (F.fn) {
        // the caller's objective needs none
    } else if (schedule == CS_FIT_SEQUENTIAL && mode == CS_MODE_FP64) {
        F.h = cs_create();
        if (!F.h) return CS_ERR_ALLOC;
        int rc = cs_set_fit_data(F.h, F.width, F.height, F.data);
        for (int r = 0; r < 4 && rc == CS_OK; r++)
            cs_set_nofit_rect(F.h, r, F.nofit[4 * r], F.nofit[4 * r + 1], F.nofit[4 * r + 2], F.nofit[4 * r + 3]);
        if (rc != CS_OK) {
            std::snprintf(report->info, sizeof report->info, "%s", cs_last_error(F.h));
            cs_destroy(F.h);
            return rc;
        }
    } else {
        F.b = cs_batch_create();
        if (!F.b) return CS_ERR_ALLOC;
        const int rc = cs_batch_set_fit(F.b, F.width, F.height, F.data, F.bstop, F.border, F.nofit);
        if (rc != CS_OK) {
            std::snprintf(report->info, sizeof report->info, "%s", cs_batch_last_error(F.b));
            cs_batch_destroy(F.b);
            return rc;
        }
    }

    const double alfa = 1.0, beta = 0.5, gamma = 2.0;
    double y[kNap], pp[kMap], q[kMap], step[kMap], psum[kMap];
    static thread_local double p[kNap][kMap];
    const int mmax = F.mmax, numFit = F.numFit;
    const double nmax = mmax + 1.0;
    const int ndim = mmax;
    const int mpts = numFit + 1;
    const double rootn1 = std::sqrt(nmax) - 1.0;
    const double mroot2 = 1.0 / (mmax * std::sqrt(2.0));
    for (int i = 0; i < kNap; i++)
        for (int j = 0; j < kMap; j++) p[i][j] = 0.0;
    for (int i = 0; i < mmax; i++) {
        psum[i] = F.values[i];
        p[0][i] = F.values[i];
        if (i < numFit) {
            if (F.values[i] == 0)
                step[i] = F.minv[i] == 0 ? stp : F.minv[i] * stp;
            else
                step[i] = F.values[i] * stp;
        } else
            step[i] = 0.0;
        pp[i] = step[i] * (rootn1 + mmax) * mroot2;
        q[i] = step[i] * rootn1 * mroot2;
    }
    for (int i = mmax; i < kMap; i++) psum[i] = p[0][i] = step[i] = pp[i] = q[i] = 0.0;
    // :375-380 as the reference executes it: y[0] = 0 and p[0..map-1][0] = 0
    y[0] = 0.0;
    for (int i = 0; i < kMap; i++) p[i][0] = 0.0;
    for (int i = 1; i < nmax; i++) {
        for (int j = 0; j < mmax; j++) p[i][j] = p[0][j] + q[j];
        p[i][i - 1] = p[i][i - 1] + pp[i - 1];
    }
    // first evaluations: the start values (y[0], from `values`) and vertices
    // 1 .. min(nmax-1, numFit+1); higher vertices copy y[numFit+1] (:404-411)
    {
        std::vector<std::vector<double>> pts;
        pts.push_back(std::vector<double>(F.values, F.values + kMap));
        std::vector<double> v(F.values, F.values + kMap);
        const int last = std::min((int)nmax - 1, numFit + 1);
        for (int i = 1; i <= last; i++) {
            for (int j = 0; j < numFit; j++) v[j] = p[i][j];
            pts.push_back(v);
        }
        std::vector<double> yy;
        if (schedule == CS_FIT_BATCHED) {
            evaluate(F, pts, yy);
        } else {
            yy.resize(pts.size());
            for (size_t k = 0; k < pts.size(); k++) {
                std::vector<double> one;
                evaluate(F, {pts[k]}, one);
                yy[k] = one[0];
            }
        }
        y[0] = yy[0];
        for (int i = 1; i < nmax; i++) y[i] = i > numFit + 1 ? y[numFit + 1] : yy[i];
    }
    for (int j = 0; j < ndim; j++) {
        double sum = 0.0;
        for (int i = 0; i < mpts; i++) sum += p[i][j];
        psum[j] = sum;
    }

    int ilo = 0, ihi = 0, inhi = 0, rep;
    bool aborted = false;
    for (rep = 0; rep < maxit && F.status == CS_OK; rep++) {
        ilo = 0;
        if (y[0] > y[1]) {
            ihi = 0;
            inhi = 1;
        } else {
            ihi = 1;
            inhi = 0;
        }
        for (int i = 0; i < mpts; i++) {
            if (y[i] < y[ilo]) ilo = i;
            if (y[i] > y[ihi]) {
                inhi = ihi;
                ihi = i;
            } else if (y[i] > y[inhi]) {
                if (i != ihi) inhi = i;
            }
        }
        if (F.chi2_stop > 0 && y[ilo] <= F.chi2_stop) break;  // (extension: target chi^2 reached)
        if (std::isnan(y[ihi]) || std::isnan(y[ilo]) || std::fabs(y[ihi]) + std::fabs(y[ilo]) == 0) {
            aborted = true;
            break;
        }
        const double rtol = 2.0 * std::fabs(y[ihi] - y[ilo]) / (std::fabs(y[ihi]) + std::fabs(y[ilo]));
        if (rtol <= ftol) break;

        // candidates: reflection; after it, expansion or contraction from the
        // simplex with or without the reflected vertex
        const std::vector<double> pr = try_point(F, p, psum, ihi, -alfa);
        double yr, ye = 0, yca = 0, ycr = 0;
        std::vector<double> pe, pca, pcr;
        if (schedule == CS_FIT_BATCHED) {
            double p2[kNap][kMap];
            double s2[kMap];
            std::memcpy(p2, p, sizeof p2);
            std::memcpy(s2, psum, sizeof s2);
            for (int j = 0; j < numFit; j++) {
                s2[j] += pr[j] - p2[ihi][j];
                p2[ihi][j] = pr[j];
            }
            pe = try_point(F, p2, s2, ihi, gamma);
            pca = try_point(F, p2, s2, ihi, beta);
            pcr = try_point(F, p, psum, ihi, beta);
            std::vector<double> yy;
            evaluate(F, {pr, pe, pca, pcr}, yy);
            yr = yy[0];
            ye = yy[1];
            yca = yy[2];
            ycr = yy[3];
        } else {
            std::vector<double> yy;
            evaluate(F, {pr}, yy);
            yr = yy[0];
        }
        const bool refl_accepted = yr < y[ihi];
        double ytry = accept(F, p, y, psum, ihi, pr, yr);
        if (ytry <= y[ilo]) {
            // (the speculative expansion assumed an accepted reflection; with
            // y[ilo] < y[ihi], which rtol > ftol >= 0 implies, it always is)
            const bool spec = schedule == CS_FIT_BATCHED && refl_accepted;
            const std::vector<double> pt = spec ? pe : try_point(F, p, psum, ihi, gamma);
            double yt = ye;
            if (!spec) {
                std::vector<double> yy;
                evaluate(F, {pt}, yy);
                yt = yy[0];
            }
            ytry = accept(F, p, y, psum, ihi, pt, yt);
        } else if (ytry >= y[inhi]) {
            const double ysave = y[ihi];
            std::vector<double> pt;
            double yt;
            if (schedule == CS_FIT_BATCHED) {
                pt = refl_accepted ? pca : pcr;
                yt = refl_accepted ? yca : ycr;
            } else {
                pt = try_point(F, p, psum, ihi, beta);
                std::vector<double> yy;
                evaluate(F, {pt}, yy);
                yt = yy[0];
            }
            ytry = accept(F, p, y, psum, ihi, pt, yt);
            if (ytry >= ysave) {
                // shrink towards the best vertex (:570-590)
                std::vector<std::vector<double>> pts;
                std::vector<int> who;
                for (int i = 0; i < mpts; i++)
                    if (i != ilo) {
                        for (int j = 0; j < ndim; j++) {
                            psum[j] = 0.5 * (p[i][j] + p[ilo][j]);
                            p[i][j] = psum[j];
                        }
                        pts.push_back(std::vector<double>(psum, psum + kMap));
                        who.push_back(i);
                    }
                std::vector<double> yy;
                if (schedule == CS_FIT_BATCHED) {
                    evaluate(F, pts, yy);
                } else {
                    yy.resize(pts.size());
                    for (size_t k = 0; k < pts.size(); k++) {
                        std::vector<double> one;
                        evaluate(F, {pts[k]}, one);
                        yy[k] = one[0];
                    }
                }
                for (size_t k = 0; k < who.size(); k++) y[who[k]] = yy[k];
                for (int j = 0; j < ndim; j++) {
                    double sum = 0.0;
                    for (int i = 0; i < mpts; i++) sum += p[i][j];
                    psum[j] = sum;
                }
            }
        }
    }
    // results: the best vertex (:598-603)
    for (int i = 0; i < mmax; i++) {
        params[table[i]].fitres = p[ilo][i];
        params[table[i]].fitvalid = 1;
    }
    report->repetitions = rep;
    report->images = F.images;
    report->chi2 = y[ilo];
    report->aborted = aborted ? 1 : 0;
    report->ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (F.status != CS_OK) std::snprintf(report->info, sizeof report->info, "%s", F.err.c_str());
    if (F.h) cs_destroy(F.h);
    if (F.b) cs_batch_destroy(F.b);
    return F.status;
}

}  // namespace
