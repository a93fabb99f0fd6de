// C entry for the reference's r-phi transform (SasCalc_PostProc::generateRphi,
// Source/sc_postproc.cpp:53-334), test oracle only. The reference's output
// array is allocated once per size and never cleared, so entries the
// transform does not write keep old contents: the wrapper runs it once to
// allocate, fills the array with NaN and runs it again, which leaves NaN
// exactly where nothing was written.
#include <cmath>
#include <cstring>
#include <limits>
#include "sc_postproc.h"

extern "C" int ref_rphi(int x0, int x1, int y0, int y1, int xc, int yc, int s, const double *d, int scale, int clip,
                        int clip40, double *out) {
    SasCalc_PostProc *pp = SasCalc_PostProc::inst();
    double *a = pp->generateRphi(x0, x1, y0, y1, xc, yc, s, d, false, false, false);
    if (!a) return 1;
    for (int i = 0; i < s * s; i++) a[i] = std::numeric_limits<double>::quiet_NaN();
    a = pp->generateRphi(x0, x1, y0, y1, xc, yc, s, d, scale != 0, clip != 0, clip40 != 0);
    std::memcpy(out, a, sizeof(double) * s * s);
    return 0;
}
