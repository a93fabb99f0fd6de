// cs_ff.cuh — float-pair ("double-float") arithmetic and elementary
// functions for the mixed-precision kernels.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2:
// 48 significand bits (relative precision ~4e-15) carried on the FP32 pipe,
// which GB300 issues 64 times as fast as FP64. The basic operations are the
// error-free transformations of Dekker and Knuth (two-sum, and the product's
// error from one fused multiply-add); the functions reduce their argument
// with float-pair tables and finish with short Taylor series, whose leading
// terms are float pairs and whose small trailing terms are plain floats:
//   exp_ff    x = k ln2/64 + r, |r| <= ln2/128: 2^(k/64) from a table,
//             e^r = 1 + r + r^2/2 + r^3 (1/6 + r/24 + r^2/120 + r^3/720)
//             (Tang, ACM TOMS 15, 1989);
//   log_ff    one Newton step y0 + (x e^(-y0) - 1) - (.)^2/2 from the float
//             logarithm y0 (its error is cubic in the step); log1p of small
//             arguments from its series;
//   atan_ff   atan x = atan c + atan((x - c)/(1 + x c)), c = j/8, and
//             atan(1/x) = pi/2 - atan x beyond 1; series through r^13;
//   sincos_ff Cody-Waite reduction by pi/2 in three float parts, then
//             r = j/16 + s with the sines and cosines of j/16 from a table and
//             series through s^9.
// Accuracy (tests/test_ff.py, against long double on random arguments):
// relative ~1e-14 for exp/log/atan, absolute ~1e-14 plus |x| 1e-18 for
// sin/cos. Every function compiles for the host too (the tests).
#ifndef CS_FF_CUH
#define CS_FF_CUH

#include <math.h>

#ifdef __CUDACC__
#define CS_FF_HD __host__ __device__ __forceinline__
// the closed forms are called once per pixel: out of line, so that their
// registers do not add to the calling kernel's
#define CS_FF_OUTLINE __host__ __device__ __noinline__
#else
#define CS_FF_HD inline
#define CS_FF_OUTLINE inline
#endif

#if defined(__CUDA_ARCH__)
#define CS_FF_TABLE __device__ const
#define CS_FF_LD(p) __ldg(p)
#else
#define CS_FF_TABLE static const
#define CS_FF_LD(p) (*(p))
#endif

namespace csff {

struct ff {
    float hi, lo;
};
// table entries load as one 8-byte word on the device
struct alignas(8) cs_ff_pair {
    float x, y;
};

// atan(j/8), j = 0..8
CS_FF_TABLE cs_ff_pair kAtanTab[9] = {{0x0.0p+0f, 0x0.0p+0f}, {0x1.fd5baa0000000p-4f, -0x1.54f4240000000p-30f}, {0x1.f5b7600000000p-3f, -0x1.b4dfc80000000p-29f}, {0x1.6f61940000000p-2f, 0x1.e4def00000000p-30f}, {0x1.dac6700000000p-2f, 0x1.586ed40000000p-28f}, {0x1.1e00ba0000000p-1f, 0x1.7bdfd60000000p-26f}, {0x1.4978fa0000000p-1f, 0x1.934f700000000p-28f}, {0x1.700a7c0000000p-1f, 0x1.5e118c0000000p-27f}, {0x1.921fb60000000p-1f, -0x1.777a5c0000000p-26f}};
// sin(j/16), cos(j/16), j = 0..13
CS_FF_TABLE cs_ff_pair kSinTab[14] = {{0x0.0p+0f, 0x0.0p+0f}, {0x1.ffaaae0000000p-5f, 0x1.dda9dc0000000p-30f}, {0x1.feaaee0000000p-4f, 0x1.d0ddc60000000p-29f}, {0x1.7dc1020000000p-3f, 0x1.f75e560000000p-28f}, {0x1.faaeee0000000p-3f, -0x1.619d520000000p-28f}, {0x1.3ad12a0000000p-2f, -0x1.12c5840000000p-27f}, {0x1.7710260000000p-2f, -0x1.5137be0000000p-27f}, {0x1.b1d8300000000p-2f, 0x1.4c85860000000p-28f}, {0x1.eaee880000000p-2f, -0x1.769f420000000p-27f}, {0x1.110d0c0000000p-1f, 0x1.2da70e0000000p-27f}, {0x1.2b91de0000000p-1f, 0x1.5108440000000p-26f}, {0x1.44eb380000000p-1f, 0x1.cf386a0000000p-29f}, {0x1.5cffc20000000p-1f, -0x1.280e1e0000000p-26f}, {0x1.73b7680000000p-1f, 0x1.bd4af00000000p-30f}};
CS_FF_TABLE cs_ff_pair kCosTab[14] = {{0x1.0000000000000p+0f, 0x0.0p+0f}, {0x1.ff00160000000p-1f, -0x1.56c1660000000p-26f}, {0x1.fc01560000000p-1f, -0x1.b054860000000p-26f}, {0x1.f706be0000000p-1f, -0x1.84c7920000000p-31f}, {0x1.f0154a0000000p-1f, -0x1.0422be0000000p-30f}, {0x1.e733ea0000000p-1f, 0x1.93d3fa0000000p-33f}, {0x1.dc6b7e0000000p-1f, 0x1.732b220000000p-26f}, {0x1.cfc6d00000000p-1f, -0x1.6b54980000000p-27f}, {0x1.c152800000000p-1f, 0x1.96df540000000p-27f}, {0x1.b11d040000000p-1f, 0x1.62a4c60000000p-29f}, {0x1.9f368e0000000p-1f, 0x1.b225f00000000p-26f}, {0x1.8bb1060000000p-1f, -0x1.688dc00000000p-27f}, {0x1.769fec0000000p-1f, 0x1.9548480000000p-27f}, {0x1.6018520000000p-1f, 0x1.bd58f80000000p-27f}};
// 2^(-j/64), j = 0..63
CS_FF_TABLE cs_ff_pair kExp2m64[64] = {{0x1.0000000000000p+0f, 0x0.0p+0f}, {0x1.fa7c180000000p-1f, 0x1.9e90d80000000p-29f}, {0x1.f507660000000p-1f, -0x1.246eb00000000p-27f}, {0x1.efa1be0000000p-1f, 0x1.cc2b440000000p-26f}, {0x1.ea4afa0000000p-1f, 0x1.52486c0000000p-28f}, {0x1.e502ee0000000p-1f, 0x1.e2cffe0000000p-27f}, {0x1.dfc9740000000p-1f, -0x1.908c940000000p-26f}, {0x1.da9e600000000p-1f, 0x1.ed99420000000p-28f}, {0x1.d5818e0000000p-1f, -0x1.822dbc0000000p-28f}, {0x1.d072d40000000p-1f, 0x1.40f1300000000p-26f}, {0x1.cb720e0000000p-1f, -0x1.8837cc0000000p-28f}, {0x1.c67f120000000p-1f, 0x1.cafa2a0000000p-26f}, {0x1.c199be0000000p-1f, -0x1.3d56b20000000p-28f}, {0x1.bcc1ea0000000p-1f, -0x1.f687c60000000p-26f}, {0x1.b7f7700000000p-1f, -0x1.a094380000000p-26f}, {0x1.b33a2c0000000p-1f, -0x1.ec3a820000000p-27f}, {0x1.ae89fa0000000p-1f, -0x1.a94b140000000p-27f}, {0x1.a9e6b60000000p-1f, -0x1.50c0480000000p-26f}, {0x1.a5503c0000000p-1f, -0x1.b83b540000000p-26f}, {0x1.a0c6680000000p-1f, -0x1.2886a60000000p-27f}, {0x1.9c49180000000p-1f, 0x1.51f8480000000p-28f}, {0x1.97d82a0000000p-1f, -0x1.0d8d840000000p-32f}, {0x1.93737c0000000p-1f, -0x1.e647440000000p-26f}, {0x1.8f1aea0000000p-1f, -0x1.baa2320000000p-27f}, {0x1.8ace540000000p-1f, 0x1.15506e0000000p-28f}, {0x1.868d9a0000000p-1f, -0x1.2edb440000000p-27f}, {0x1.82589a0000000p-1f, -0x1.accc7c0000000p-27f}, {0x1.7e2f340000000p-1f, -0x1.2616340000000p-26f}, {0x1.7a11480000000p-1f, -0x1.829fd00000000p-26f}, {0x1.75feb60000000p-1f, -0x1.37b3060000000p-26f}, {0x1.71f75e0000000p-1f, 0x1.1d8bee0000000p-26f}, {0x1.6dfb240000000p-1f, -0x1.cd72e80000000p-28f}, {0x1.6a09e60000000p-1f, 0x1.9fcef40000000p-27f}, {0x1.6623880000000p-1f, 0x1.2a91120000000p-28f}, {0x1.6247ec0000000p-1f, -0x1.f8b5500000000p-26f}, {0x1.5e76f20000000p-1f, -0x1.4a5bd60000000p-26f}, {0x1.5ab07e0000000p-1f, -0x1.5bd5ec0000000p-28f}, {0x1.56f4740000000p-1f, -0x1.295b040000000p-26f}, {0x1.5342b60000000p-1f, -0x1.2c56100000000p-26f}, {0x1.4f9b280000000p-1f, -0x1.2c5a6c0000000p-26f}, {0x1.4bfdae0000000p-1f, -0x1.593abc0000000p-26f}, {0x1.486a2c0000000p-1f, -0x1.47d8660000000p-26f}, {0x1.44e0860000000p-1f, 0x1.8624b40000000p-31f}, {0x1.4160a20000000p-1f, 0x1.f72e2a0000000p-29f}, {0x1.3dea640000000p-1f, 0x1.8246840000000p-26f}, {0x1.3a7db40000000p-1f, -0x1.634c020000000p-26f}, {0x1.371a740000000p-1f, -0x1.18aac60000000p-26f}, {0x1.33c08c0000000p-1f, -0x1.b37d200000000p-26f}, {0x1.306fe00000000p-1f, 0x1.4636e20000000p-26f}, {0x1.2d285a0000000p-1f, 0x1.b900c20000000p-27f}, {0x1.29e9e00000000p-1f, -0x1.5c04240000000p-26f}, {0x1.26b4560000000p-1f, 0x1.789f380000000p-27f}, {0x1.2387a60000000p-1f, 0x1.ceac480000000p-26f}, {0x1.2063b80000000p-1f, 0x1.0c519a0000000p-26f}, {0x1.1d48740000000p-1f, -0x1.d2e8ca0000000p-26f}, {0x1.1a35be0000000p-1f, 0x1.6df96e0000000p-26f}, {0x1.172b840000000p-1f, -0x1.c157420000000p-28f}, {0x1.1429aa0000000p-1f, 0x1.d525bc0000000p-26f}, {0x1.11301e0000000p-1f, -0x1.fdb4960000000p-26f}, {0x1.0e3ec40000000p-1f, -0x1.a585cc0000000p-26f}, {0x1.0b55860000000p-1f, 0x1.9f31220000000p-26f}, {0x1.0874520000000p-1f, -0x1.e2990e0000000p-27f}, {0x1.059b0e0000000p-1f, -0x1.9d4f520000000p-26f}, {0x1.02c9a40000000p-1f, -0x1.887fa00000000p-29f}};

CS_FF_HD ff make(float h, float l) { return ff{h, l}; }
CS_FF_HD ff from_double(double d) {
    const float h = (float)d;
    return ff{h, (float)(d - (double)h)};
}
CS_FF_HD double to_double(ff a) { return (double)a.hi + (double)a.lo; }
CS_FF_HD ff from_pair(const cs_ff_pair *p) {
#if defined(__CUDA_ARCH__)
    const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
    return ff{v.x, v.y};
#else
    return ff{p->x, p->y};
#endif
}

// s + e = a + b exactly
CS_FF_HD void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
// s + e = a + b exactly, for |a| >= |b| (or a = 0)
CS_FF_HD void quick_two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    e = b - (s - a);
}
CS_FF_HD ff renorm(float a, float b) {
    ff r;
    quick_two_sum(a, b, r.hi, r.lo);
    return r;
}
CS_FF_HD ff neg(ff a) { return ff{-a.hi, -a.lo}; }
CS_FF_HD ff add(ff a, ff b) {
    float s, e, t, f;
    two_sum(a.hi, b.hi, s, e);
    two_sum(a.lo, b.lo, t, f);
    e += t;
    quick_two_sum(s, e, s, e);
    e += f;
    return renorm(s, e);
}
CS_FF_HD ff sub(ff a, ff b) { return add(a, neg(b)); }
CS_FF_HD ff add_f(ff a, float b) {
    float s, e;
    two_sum(a.hi, b, s, e);
    e += a.lo;
    return renorm(s, e);
}
CS_FF_HD ff mul(ff a, ff b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return renorm(p, e);
}
CS_FF_HD ff mul_f(ff a, float b) {
    const float p = a.hi * b;
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    return renorm(p, e);
}
// exact product of two floats as a pair
CS_FF_HD ff prod(float a, float b) {
    const float p = a * b;
    return ff{p, fmaf(a, b, -p)};
}
CS_FF_HD ff sqr(ff a) { return mul(a, a); }
CS_FF_HD ff div(ff a, ff b) {
    const float q1 = a.hi / b.hi;
    ff r = sub(a, mul_f(b, q1));
    const float q2 = r.hi / b.hi;
    r = sub(r, mul_f(b, q2));
    const float q3 = r.hi / b.hi;
    ff q = renorm(q1, q2);
    return add_f(q, q3);
}
CS_FF_HD ff sqrt_ff(ff a) {
    if (!(a.hi > 0.0f)) return ff{sqrtf(a.hi), 0.0f};
    const float y = sqrtf(a.hi);
    const ff r = sub(a, prod(y, y));
    return renorm(y, r.hi / (2.0f * y));
}
CS_FF_HD ff ldexp_ff(ff a, int e) { return ff{ldexpf(a.hi, e), ldexpf(a.lo, e)}; }

// e^x; 0 below -104 (FP32 underflows), +inf above 88
CS_FF_HD ff exp_ff(ff x) {
    if (x.hi < -104.0f) return ff{0.0f, 0.0f};
    if (x.hi > 88.0f) return ff{INFINITY, 0.0f};
    const ff k64ln2 = ff{0x1.715476p+6f, 0x1.4ae0cp-20f};   // 64/ln 2
    // ln 2/64 in three float parts: k times each of the first two is exact
    // as a pair, the third's product error is below 1e-22 relative
    const float L0 = 0x1.62e43p-7f, L1 = -0x1.05c61p-35f, L2 = -0x1.950d88p-60f;
    const float kf = rintf(x.hi * k64ln2.hi);
    // r = x - k ln2/64
    ff r = sub(x, prod(kf, L0));
    r = sub(r, prod(kf, L1));
    r = add_f(r, -kf * L2);
    const int k = (int)kf;
    const int q = k >> 6;  // floor
    const int j = k & 63;  // 2^(k/64) = 2^q 2^(j/64) = 2^(q+1) 2^(-(64-j)/64)
    const ff t = j == 0 ? ff{1.0f, 0.0f} : ldexp_ff(from_pair(&kExp2m64[64 - j]), 1);
    // e^r - 1 = r + r^2/2 + r^3 (1/6 + r/24 + r^2/120 + r^3/720)
    const float rh = r.hi;
    const float tail = rh * rh * rh * fmaf(rh, fmaf(rh, fmaf(rh, 1.0f / 720.0f, 1.0f / 120.0f), 1.0f / 24.0f), 1.0f / 6.0f);
    const ff em1 = add_f(add(r, mul_f(sqr(r), 0.5f)), tail);
    const ff e = add(t, mul(t, em1));
    return ldexp_ff(e, q);
}

// log(1 + v) for |v| < 1/64 from its series (through v^9: remainder < 1e-17
// relative; the terms through v^4 as pairs)
CS_FF_HD ff log1p_small(ff v) {
    const float vh = v.hi;
    // v - v^2/2 + v^3/3 - v^4/4 + v^5 (1/5 - v/6 + v^2/7 - v^3/8 + v^4/9)
    const float p = fmaf(vh, fmaf(vh, fmaf(vh, fmaf(vh, 1.0f / 9.0f, -0.125f), 1.0f / 7.0f), -1.0f / 6.0f), 0.2f);
    const ff v2 = sqr(v);
    const ff v3 = mul(v2, v);
    const ff v4 = sqr(v2);
    ff s = sub(v, mul_f(v2, 0.5f));
    s = add(s, div(v3, ff{3.0f, 0.0f}));
    s = sub(s, mul_f(v4, 0.25f));
    return add_f(s, v4.hi * vh * p);
}

// log x, x > 0 (near 1 from the series of log(1 + (x - 1)), where the
// difference is exact and carries the result's relative precision)
CS_FF_HD ff log_ff(ff x) {
    if (fabsf(x.hi - 1.0f) < 1.0f / 64.0f) return log1p_small(add_f(x, -1.0f));
    const float y0 = logf(x.hi);
    // u = x e^(-y0) - 1, log x = y0 + log(1 + u)
    const ff u = add_f(mul(x, exp_ff(ff{-y0, 0.0f})), -1.0f);
    return add(ff{y0, 0.0f}, log1p_small(u));
}

// log(1 + v), v > -1 given as a pair
CS_FF_HD ff log1p_ff(ff v) {
    if (fabsf(v.hi) < 1.0f / 64.0f) return log1p_small(v);
    return log_ff(add_f(v, 1.0f));
}

// atan x for 0 <= x <= 1
CS_FF_HD ff atan01(ff x) {
    const int j = (int)rintf(x.hi * 8.0f);
    const float c = 0.125f * (float)j;
    // r = (x - c)/(1 + x c), |r| <= 1/16
    const ff r = div(add_f(x, -c), add_f(mul_f(x, c), 1.0f));
    const float rh = r.hi, r2 = rh * rh;
    // atan r = r - r^3/3 + r^5/5 + r^7 (-1/7 + r^2/9 - r^4/11 + r^6/13)
    const float p = fmaf(r2, fmaf(r2, fmaf(r2, 1.0f / 13.0f, -1.0f / 11.0f), 1.0f / 9.0f), -1.0f / 7.0f);
    const ff rr = sqr(r);
    const ff r3 = mul(rr, r);
    const ff r5 = mul(r3, rr);
    ff s = sub(r, div(r3, ff{3.0f, 0.0f}));
    s = add(s, div(r5, ff{5.0f, 0.0f}));
    s = add_f(s, r5.hi * r2 * p);
    return add(from_pair(&kAtanTab[j]), s);
}

CS_FF_HD ff atan_ff(ff x) {
    const bool negx = x.hi < 0.0f;
    const ff ax = negx ? neg(x) : x;
    ff r;
    if (ax.hi <= 1.0f) {
        r = atan01(ax);
    } else {
        const ff half_pi = ff{0x1.921fb6p+0f, -0x1.777a5cp-25f};
        r = sub(half_pi, atan01(div(ff{1.0f, 0.0f}, ax)));
    }
    return negx ? neg(r) : r;
}

// sin and cos of a pair of moderate size (|x| < 2^20)
CS_FF_HD void sincos_ff(ff x, ff &s, ff &c) {
    // k = nearest integer to x/(pi/2); r = x - k pi/2 with pi/2 in three parts
    const float kf = rintf(x.hi * 0x1.45f306p-1f);  // 2/pi
    const float P0 = 0x1.921fb6p+0f, P1 = -0x1.777a5cp-25f, P2 = -0x1.ee59dap-50f;
    ff r = sub(x, prod(kf, P0));
    r = sub(r, prod(kf, P1));
    r = add_f(r, -kf * P2);
    // r = j/16 + t, |t| <= 1/32
    const int j = (int)rintf(r.hi * 16.0f);
    const ff t = add_f(r, -(float)j * 0.0625f);
    const float th = t.hi, t2 = th * th;
    // sin t = t - t^3/6 + t^5 (1/120 - t^2/5040 + t^4/362880)
    const ff tt = sqr(t);
    const ff t3 = mul(tt, t);
    ff st = sub(t, div(t3, ff{6.0f, 0.0f}));
    st = add_f(st, t3.hi * t2 * fmaf(t2, fmaf(t2, 1.0f / 362880.0f, -1.0f / 5040.0f), 1.0f / 120.0f));
    // cos t = 1 - t^2/2 + t^4 (1/24 - t^2/720 + t^4/40320)
    ff ct = sub(ff{1.0f, 0.0f}, mul_f(tt, 0.5f));
    ct = add_f(ct, t2 * t2 * fmaf(t2, fmaf(t2, 1.0f / 40320.0f, -1.0f / 720.0f), 1.0f / 24.0f));
    const int aj = j < 0 ? -j : j;
    ff sj = from_pair(&kSinTab[aj]);
    const ff cj = from_pair(&kCosTab[aj]);
    if (j < 0) sj = neg(sj);
    const ff sr = add(mul(sj, ct), mul(cj, st));
    const ff cr = sub(mul(cj, ct), mul(sj, st));
    switch (((int)kf) & 3) {
    case 0: s = sr; c = cr; break;
    case 1: s = cr; c = neg(sr); break;
    case 2: s = neg(sr); c = neg(cr); break;
    default: s = neg(cr); c = sr; break;
    }
}

// ---- closed forms of the Schulz-averaged cylinder in float pairs -----------

// Length factor (1/(2z(z-1)a^2)) (1 - cos(m atan 2a) (1+4a^2)^(-m/2)), m = z-1
// (the reference's ordis-6 closed form, Source/sc_lib_formpq_partCylinder.h:115-119),
// for |m a| >= 0.05 or |a| >= 0.05 (below, its series applies). rel: a bound
// on the relative error, from the angle's (|m atan 2a| ~4e-15) and the power's
// (m ~1e-14) absolute errors over the bracket, with a factor 2 to spare.
CS_FF_OUTLINE double cyl_len_closed(double a_d, double z_d, float &rel) {
    const ff a = from_double(a_d);
    const ff m = from_double(z_d - 1.0);
    const ff a2 = sqr(a);
    const ff th = mul(m, atan_ff(mul_f(a, 2.0f)));
    ff sn, cs;
    sincos_ff(th, sn, cs);
    const ff L = log1p_ff(mul_f(a2, 4.0f));
    const ff E = exp_ff(neg(mul(mul_f(m, 0.5f), L)));
    const ff ce = mul(cs, E);
    const ff br = sub(ff{1.0f, 0.0f}, ce);
    const ff k = div(ff{1.0f, 0.0f}, mul_f(mul(from_double(z_d), m), 2.0f));
    const ff v = mul(k, div(br, a2));
    const float ebr = fabsf(E.hi) * (fabsf(th.hi) + fabsf(m.hi) + 1.0f) * 4e-14f;
    rel = ebr / fabsf(br.hi) + 4e-14f;
    return to_double(v);
}

// Cross-section asymptote of the Schulz cylinder's P(q),
//   (4/pi) (T1 - T2 - (9/8) T3),  T1 = 1/(z(z-1)(z-2) a^3),
//   T2 = T1 sin((z-2) t) (1+4a^2)^(-(z-2)/2),
//   T3 = cos((z-3) t) (1+4a^2)^(-(z-3)/2) / (z(z-1)(z-2)(z-3) a^4),  t = atan 2a
// (Source/sc_lib_formpq_partCylinder.h:217-257), with cos((z-3)t) and the
// (z-3) power from the (z-2) ones: cos t = (1+4a^2)^(-1/2), sin t = 2a cos t.
// rel as above, over the terms' sum.
CS_FF_OUTLINE double cyl_cross_asym(double a_d, double z_d, float &rel) {
    const ff a = from_double(a_d);
    const ff n2 = from_double(z_d - 2.0);
    const ff v4 = mul_f(sqr(a), 4.0f);
    const ff tt = atan_ff(mul_f(a, 2.0f));
    const ff L = log1p_ff(v4);
    const ff th = mul(n2, tt);
    ff s2, c2;
    sincos_ff(th, s2, c2);
    const ff E2 = exp_ff(neg(mul(mul_f(n2, 0.5f), L)));
    const ff root = sqrt_ff(add_f(v4, 1.0f));             // (1+4a^2)^(1/2)
    const ff ct = div(ff{1.0f, 0.0f}, root);               // cos t
    const ff c3 = mul(ct, add(c2, mul(mul_f(a, 2.0f), s2)));  // cos((z-3)t)
    const ff E3 = mul(E2, root);
    const double zz = z_d * (z_d - 1) * (z_d - 2);
    const ff ia = div(ff{1.0f, 0.0f}, a);
    const ff ia3 = mul(sqr(ia), ia);
    const ff T1 = div(ia3, from_double(zz));
    const ff T2 = mul(T1, mul(s2, E2));
    const ff T3 = div(mul(mul(ia3, ia), mul(c3, E3)), from_double(zz * (z_d - 3)));
    const ff sum = sub(sub(T1, T2), mul_f(T3, 1.125f));
    const double v = to_double(sum) * (4.0 / M_PI);
    const float err = (fabsf(T1.hi) + (fabsf(T2.hi) + fabsf(T3.hi)) * (fabsf(th.hi) + fabsf(n2.hi) + 2.0f)) * 2e-14f;
    rel = err / fabsf(sum.hi) + 2e-14f;
    return v;
}

}  // namespace csff

#endif
