/* Stop test of the reference's power series, decided cheaply.
 *
 * The formpq/formfq series of the reference (e.g.
 * Source/sc_lib_formpq_partCylinder.h:103-111,
 * Source/sc_lib_formfq_partCylinder.h:32-40, Source/sc_lib_formpq_partSphere.h:52)
 * add terms until the relative increment falls below 1e-4:
 *
 *     delser = fabs((pqsum - oldpqsum) / pqsum);  if (delser < 0.0001) break;
 *
 * That is a discrete decision on a sum that can cancel by many orders of
 * magnitude, so it is taken here exactly as the reference takes it, but
 * without the FP64 division on almost every term:
 *
 * 1. Exponent screen (integer ALU only). With the binary exponents E_s of s
 *    and E_d of d = fl(s - old): |s| < 2^(E_s+1) and |d| >= 2^E_d, so
 *    E_d >= E_s - 12 gives |d / s| > 2^-13 = 1.22e-4. 2^-13 is a double, so the
 *    rounded quotient is >= 2^-13 > 0.0001 too: not converged. An infinite or
 *    NaN d has the largest exponent and is not converged either, as in the
 *    reference (inf or NaN compared with < is false).
 * 2. Band test. With A = fl(0.0001 |s|), an increment below fl(A (1 - 2^-50))
 *    has an exact quotient below 0.0001 (1 - 2^-52), whose rounding stays
 *    below 0.0001; one above fl(A (1 + 2^-50)) stays above.
 * 3. Only inside that band, and for |s| outside [2^-962, 2^963) (zero,
 *    subnormal, NaN, inf, or products that could underflow), is the quotient
 *    computed as the reference computes it.
 *
 * The decision is the reference's in every case. The same function compiles
 * for the host, where a brute-force test compares it with the plain quotient
 * test. */
#ifndef CS_SERIES_STOP_H
#define CS_SERIES_STOP_H

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define CS_SERIES_HD __host__ __device__ __forceinline__
#else
#define CS_SERIES_HD inline
#endif

namespace cs_series {

/* biased binary exponent field of x (0 for zero / subnormal, 0x7FF for inf / NaN) */
CS_SERIES_HD int exp_field(double x) {
#ifdef __CUDA_ARCH__
    return (__double2hiint(x) >> 20) & 0x7FF;
#else
    std::uint64_t u;
    std::memcpy(&u, &x, sizeof u);
    return (int)((u >> 52) & 0x7FF);
#endif
}

CS_SERIES_HD double add_rn(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}

CS_SERIES_HD double mul_rn(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}

CS_SERIES_HD bool series_converged(double s, double old) {
    const double d = add_rn(s, -old);
    const int es = exp_field(s);
    if (es >= 1023 - 962 && es <= 1023 + 962) { /* 2^-962 <= |s| < 2^963 */
        if (exp_field(d) >= es - 12) return false;
        const double ad = fabs(d), a = mul_rn(0.0001, fabs(s));
        if (ad < mul_rn(a, 1.0 - 0x1p-50)) return true;
        if (ad > mul_rn(a, 1.0 + 0x1p-50)) return false;
    }
    return fabs(d / s) < 0.0001;
}

} /* namespace cs_series */

#endif
