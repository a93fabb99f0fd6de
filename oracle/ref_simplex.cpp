// C entry point to the reference's own downhill simplex
// (SasCalc_SimplexFit2D::doSimplexFit2D, Source/sc_simplexfit2d.cpp:254-611),
// compiled from the reference sources by oracle/build_ref.sh with the
// stand-in calculation class of ref_stubs/simplex_calc.h (test oracle only).
#include "simplex_calc.h"
#include "sc_simplexfit2d.h"

extern "C" int ref_simplex_run(int n, const char *const *names, const double *start, const double *mins,
                               const double *maxs, const int *used, double stp, int maxit, double ftol,
                               cs_ref_objective fn, void *ctx, double *fitres, int *repetitions, int *images,
                               int *aborted) {
    SC_CalcCons calc;
    calc.fn = fn;
    calc.ctx = ctx;
    std::vector<_fitLimits> lim(n);
    _param2fitval vals;
    for (int i = 0; i < n; i++) {
        lim[i].min = mins[i];
        lim[i].max = maxs[i];
        lim[i].fitstart = start[i];
        lim[i].fitres = start[i];
        lim[i].orgval = start[i];
        lim[i].fitType = fitNumeric;
        lim[i].used = used[i] != 0;
        lim[i].fitvalid = false;
        vals.insert(QString(names[i]), &lim[i]);
    }
    SasCalc_SimplexFit2D fit(&calc);
    static const double dummy = 0.0;
    fit.setImageInfo(0, 1, 0, 1, &dummy);
    QString info;
    fit.doSimplexFit2D(1, stp, maxit, ftol, 0, 0, false, nullptr, &vals, info);
    for (int i = 0; i < n; i++) fitres[i] = lim[i].fitres;
    *repetitions = fit.repetitions;
    *images = fit.numImgCalc;
    *aborted = fit.aborted ? 1 : 0;
    return info.empty() ? 0 : 1;
}
