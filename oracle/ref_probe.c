/* One-ulp perturbation of the math library for the probe build of the
 * reference (oracle/_ref/libscref_probe.so, TEST INFRASTRUCTURE): the
 * reference's objects are compiled without builtins and linked with
 * --wrap=<fn>, so each call below returns the library's result moved one ulp
 * up (mode bit set) or down (bit clear). Bit k of the mode selects function k
 * in the order sin cos atan atan2 pow exp sqrt log acos (sqrt is correctly
 * rounded everywhere and is not wrapped). A negative mode leaves the results
 * untouched. Used to measure how far the reference's own result moves under
 * last-bit differences of the math library (golden "cond" maps). */
#include <math.h>

static int g_mode = -1;

void ref_set_probe(int mode) { g_mode = mode; }

static double nudge(double r, int bit) {
    if (g_mode < 0 || !isfinite(r)) return r;
    return nextafter(r, ((g_mode >> bit) & 1) ? INFINITY : -INFINITY);
}

double __real_sin(double);
double __real_cos(double);
double __real_atan(double);
double __real_atan2(double, double);
double __real_pow(double, double);
double __real_exp(double);
double __real_log(double);
double __real_acos(double);

double __wrap_sin(double x) { return nudge(__real_sin(x), 0); }
double __wrap_cos(double x) { return nudge(__real_cos(x), 1); }
double __wrap_atan(double x) { return nudge(__real_atan(x), 2); }
double __wrap_atan2(double y, double x) { return nudge(__real_atan2(y, x), 3); }
double __wrap_pow(double x, double y) { return nudge(__real_pow(x, y), 4); }
double __wrap_exp(double x) { return nudge(__real_exp(x), 5); }
double __wrap_log(double x) { return nudge(__real_log(x), 7); }
double __wrap_acos(double x) { return nudge(__real_acos(x), 8); }
