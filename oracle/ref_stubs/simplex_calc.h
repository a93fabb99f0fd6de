// Forced-included (g++ -include) ahead of the reference's simplex unit
// (Source/sc_simplexfit2d.cpp) for the test oracle. It takes the place of the
// console calculation class SC_CalcCons (Source/sc_calcCons.h: its include
// guard is defined here, so the real header, and with it the whole
// calculation class, is skipped): the parameter values the simplex hands to
// updateParamValue() are collected in call order, and doFitCalculation()
// passes them to the objective the test installs. Nothing of the image
// calculation is involved; the simplex's own arithmetic and control flow are
// the reference's.
#ifndef CS_REF_SIMPLEX_CALC_H
#define CS_REF_SIMPLEX_CALC_H
#define SC_CALCCONS_H
#include <chrono>
#include <cmath>
#include <cstdio>
#include <vector>
#include "QDebug"
#include "QHash"
#include "QString"
#include "QStringList"
#include "sc_math.h"  // sqr, progressLogging

typedef double (*cs_ref_objective)(const double *values, int n, void *ctx);

struct CsRefImage {
    double xyIntensity(int, int) const { return 0.0; }
};

class SC_CalcCons {
public:
    cs_ref_objective fn = nullptr;
    void *ctx = nullptr;
    std::vector<double> vals;   // values of the current evaluation, call order
    bool collecting = false;
    CsRefImage img;

    bool updateParamValue(QString, double v) {
        if (!collecting) {
            vals.clear();
            collecting = true;
        }
        vals.push_back(v);
        return true;
    }
    void prepareData(bool, bool) { collecting = false; }
    double doFitCalculation(int, int, int, long &cnt, long &nancnt) {
        cnt = 1;
        nancnt = 0;
        return fn(vals.data(), (int)vals.size(), ctx);
    }
    void doCalculation(int, bool) {}
    bool setFitData(int, int, const double *) { return true; }
    int minX() { return 0; }
    int maxX() { return 0; }
    int minY() { return 0; }
    int maxY() { return 0; }
    CsRefImage *getCalcPtr() { return &img; }
    CsRefImage *getMemPtr() { return &img; }
};
#endif
