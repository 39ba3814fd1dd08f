// pmath.h — portable single-precision transcendentals.
//
// The path tracer calls four transcendental functions: sincosf (lens disk
// and unit-sphere sampling), powf (cube-root radius, Schlick's fifth power,
// gamma), acosf and atan2f (sphere UVs).  CUDA's device libm and the host's
// glibc disagree in the last bits of these functions, and one flipped bit is
// enough to send a Monte-Carlo path a different way.  This header gives one
// implementation that returns the same bits on an x86-64 host, an aarch64
// host and sm_103a, so a CPU restatement and the GPU kernel can produce
// bit-identical images from the same RNG stream.
//
// Determinism rules: only IEEE-754 operations that every target rounds
// correctly are used — +, -, *, /, sqrtf, fmaf (written out wherever a
// product feeds an add), floorf/rintf and integer bit manipulation.  Callers
// must compile with contraction disabled (-ffp-contract=off on the host,
// -fmad=false for nvcc) and without fast-math.
//
// Methods (textbook, from the mathematics; no vendor library code):
//   sin/cos   Cody–Waite reduction by pi/2 with a three-part constant, then
//             Taylor polynomials on |r| <= pi/4 (truncation < 1e-11).
//   atan2     octant folding, atan(z) = pi/6 + atan((sqrt3*z-1)/(z+sqrt3))
//             for z > tan(pi/12), Taylor series to z^13 on |z| <= tan(pi/12).
//   acos      acos(x) = atan2(sqrt((1-x)(1+x)), x).
//   pow       x = m*2^e, log2(m) from the atanh series in f=(m-1)/(m+1),
//             y*log2(x) = y*e + y*log2(m) kept as a float-float sum (fmaf
//             product errors, TwoSum), exp2 by integer part
//             plus Taylor series of e^(r ln2) on |r| <= 1/2, then 2^n by
//             exponent construction.
// Accuracy (checked against glibc in tests/test_pmath.py): sincos and atan2
// within 2 ulp, acos within 3 ulp, pow within 6 ulp on the domains the
// tracer uses.
#pragma once

#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#define PM_FN __host__ __device__ __forceinline__
#else
#define PM_FN static inline
#endif

PM_FN uint32_t pm_f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
PM_FN float pm_u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
PM_FN bool pm_isnan(float x) { return x != x; }
PM_FN bool pm_isinf(float x) { return (pm_f2u(x) & 0x7fffffffu) == 0x7f800000u; }
PM_FN float pm_fabs(float x) { return pm_u2f(pm_f2u(x) & 0x7fffffffu); }
PM_FN float pm_copysign(float x, float s) {
    return pm_u2f((pm_f2u(x) & 0x7fffffffu) | (pm_f2u(s) & 0x80000000u));
}
PM_FN bool pm_signbit(float x) { return (pm_f2u(x) >> 31) != 0u; }
PM_FN float pm_nan() { return pm_u2f(0x7fc00000u); }
PM_FN float pm_inf() { return pm_u2f(0x7f800000u); }
// 2^k for k in [-126, 127], exact.
PM_FN float pm_pow2i(int k) { return pm_u2f((uint32_t)(k + 127) << 23); }

// ---- sin / cos ---------------------------------------------------------
PM_FN void pm_sincosf(float x, float* s, float* c) {
    if (pm_isnan(x) || pm_isinf(x)) { *s = pm_nan(); *c = pm_nan(); return; }
    const float two_over_pi = 6.366197467e-01f;
    // pi/2 = P1 + P2 + P3 (each the float nearest the remaining tail)
    const float P1 = 1.570796371e+00f;
    const float P2 = -4.371138829e-08f;
    const float P3 = -1.715124510e-15f;
    float k = rintf(x * two_over_pi);
    float r = fmaf(-k, P1, x);
    r = fmaf(-k, P2, r);
    r = fmaf(-k, P3, r);
    int q = ((int)k) & 3;
    float r2 = r * r;
    // sin r = r + r^3 * (-1/3! + r^2/5! - r^4/7! + r^6/9! - r^8/11!)
    float ps = fmaf(r2, -2.505210794e-08f, 2.755731884e-06f);
    ps = fmaf(r2, ps, -1.984127011e-04f);
    ps = fmaf(r2, ps, 8.333333768e-03f);
    ps = fmaf(r2, ps, -1.666666716e-01f);
    float r3 = r2 * r;
    float sr = fmaf(r3, ps, r);
    // cos r = 1 - r^2/2 + r^4 * (1/4! - r^2/6! + r^4/8! - r^6/10! + r^8/12!)
    float pc = fmaf(r2, 2.087675588e-09f, -2.755731998e-07f);
    pc = fmaf(r2, pc, 2.480158764e-05f);
    pc = fmaf(r2, pc, -1.388888923e-03f);
    pc = fmaf(r2, pc, 4.166666791e-02f);
    float r4 = r2 * r2;
    float cr = fmaf(r4, pc, fmaf(r2, -0.5f, 1.0f));
    switch (q) {
        case 0: *s = sr; *c = cr; break;
        case 1: *s = cr; *c = -sr; break;
        case 2: *s = -sr; *c = -cr; break;
        default: *s = -cr; *c = sr; break;
    }
}

// ---- atan2 / acos --------------------------------------------------------
// atan(z) for z in [0, 1].
PM_FN float pm_atan_unit(float z) {
    const float tan_pi_12 = 2.679491937e-01f;
    const float sqrt3 = 1.732050776e+00f;
    const float pi_6 = 5.235987902e-01f;
    bool reduced = z > tan_pi_12;
    if (reduced) z = fmaf(z, sqrt3, -1.0f) / (z + sqrt3);
    float z2 = z * z;
    // atan z = z + z^3 * (-1/3 + z^2/5 - z^4/7 + z^6/9 - z^8/11 + z^10/13)
    float p = fmaf(z2, 7.692307979e-02f, -9.090909362e-02f);
    p = fmaf(z2, p, 1.111111119e-01f);
    p = fmaf(z2, p, -1.428571492e-01f);
    p = fmaf(z2, p, 2.000000030e-01f);
    p = fmaf(z2, p, -3.333333433e-01f);
    float z3 = z2 * z;
    float a = fmaf(z3, p, z);
    if (reduced) a = a + pi_6;
    return a;
}

PM_FN float pm_atan2f(float y, float x) {
    const float pi = 3.141592741e+00f;
    const float pi_2 = 1.570796371e+00f;
    if (pm_isnan(x) || pm_isnan(y)) return x + y;
    float ax = pm_fabs(x), ay = pm_fabs(y);
    float a;
    if (ax == 0.0f && ay == 0.0f) {
        a = pm_signbit(x) ? pi : 0.0f;
    } else if (pm_isinf(ax) && pm_isinf(ay)) {
        a = pm_signbit(x) ? 2.356194496e+00f : 7.853981853e-01f;
    } else {
        bool swap = ay > ax;
        float num = swap ? ax : ay;
        float den = swap ? ay : ax;
        float z = num / den;  // den > 0; inf den gives 0
        a = pm_atan_unit(z);
        if (swap) a = pi_2 - a;
        if (pm_signbit(x)) a = pi - a;
    }
    return pm_copysign(a, y);
}

PM_FN float pm_acosf(float x) {
    if (pm_isnan(x)) return x + x;
    if (pm_fabs(x) > 1.0f) return pm_nan();
    float s = sqrtf((1.0f - x) * (1.0f + x));
    return pm_atan2f(s, x);
}

// ---- pow -------------------------------------------------------------------
// 2^(n + r) for integer-valued n and |r| <= ~0.5
PM_FN float pm_exp2_split(float n, float r) {
    const float ln2 = 6.931471825e-01f;
    if (n > 128.0f) return pm_inf();
    if (n < -151.0f) return 0.0f;
    float w = r * ln2;
    // e^w = 1 + w + w^2/2! + ... + w^9/9!
    float p = fmaf(w, 2.755731884e-06f, 2.480158764e-05f);
    p = fmaf(w, p, 1.984127011e-04f);
    p = fmaf(w, p, 1.388888923e-03f);
    p = fmaf(w, p, 8.333333768e-03f);
    p = fmaf(w, p, 4.166666791e-02f);
    p = fmaf(w, p, 1.666666716e-01f);
    p = fmaf(w, p, 0.5f);
    p = fmaf(w, p, 1.0f);
    p = fmaf(w, p, 1.0f);
    int k = (int)n;
    if (k > 127) return (p * pm_pow2i(127)) * pm_pow2i(k - 127);
    if (k < -126) return (p * pm_pow2i(-126)) * pm_pow2i(k + 126);
    return p * pm_pow2i(k);
}

PM_FN float pm_powf(float x, float y) {
    if (y == 0.0f) return 1.0f;
    if (x == 1.0f) return 1.0f;
    if (pm_isnan(x) || pm_isnan(y)) return x + y;
    float ax = pm_fabs(x);
    bool y_inf = pm_isinf(y);
    bool y_int = !y_inf && floorf(y) == y;
    bool y_odd = false;
    if (y_int && pm_fabs(y) < 16777216.0f) y_odd = (((int32_t)y) & 1) != 0;
    if (y_inf) {
        if (ax == 1.0f) return 1.0f;
        return ((ax > 1.0f) == (y > 0.0f)) ? pm_inf() : 0.0f;
    }
    if (ax == 0.0f) {
        if (y < 0.0f) return y_odd ? pm_copysign(pm_inf(), x) : pm_inf();
        return y_odd ? x : 0.0f;
    }
    if (pm_isinf(ax)) {
        float r = (y < 0.0f) ? 0.0f : pm_inf();
        return (pm_signbit(x) && y_odd) ? -r : r;
    }
    if (pm_signbit(x) && !y_int) return pm_nan();

    // log2(ax) = e + log2(m), m in [sqrt(1/2), sqrt(2))
    uint32_t bits = pm_f2u(ax);
    int e = 0;
    if (bits < 0x00800000u) {          // subnormal: scale by 2^24
        bits = pm_f2u(ax * 16777216.0f);
        e = -24;
    }
    e += (int)(bits >> 23) - 127;
    float m = pm_u2f((bits & 0x007fffffu) | 0x3f800000u);  // [1, 2)
    if (m > 1.414213538e+00f) { m = m * 0.5f; e += 1; }
    float f = (m - 1.0f) / (m + 1.0f);
    float s = f * f;
    // ln m = 2f * (1 + s/3 + s^2/5 + s^3/7 + s^4/9 + s^5/11)
    float t = fmaf(s, 9.090909362e-02f, 1.111111119e-01f);
    t = fmaf(s, t, 1.428571492e-01f);
    t = fmaf(s, t, 2.000000030e-01f);
    t = fmaf(s, t, 3.333333433e-01f);
    float fs = f * s;
    float ln_m_half = fmaf(fs, t, f);                 // ln(m) / 2
    float log2_m = ln_m_half * 2.885390043e+00f;      // * 2*log2(e)
    // y * (e + log2_m) as an unevaluated sum: both products with their exact
    // rounding errors (fmaf), the two large parts combined by TwoSum.
    float fe = (float)e;
    float p1 = y * fe, p1e = fmaf(y, fe, -p1);
    float p2 = y * log2_m, p2e = fmaf(y, log2_m, -p2);
    float ph = p1 + p2;
    if (ph > 200.0f) return (pm_signbit(x) && y_odd) ? -pm_inf() : pm_inf();
    if (ph < -200.0f) return (pm_signbit(x) && y_odd) ? -0.0f : 0.0f;
    float bb = ph - p1;
    float pl = ((p1 - (ph - bb)) + (p2 - bb)) + (p1e + p2e);
    float n = rintf(ph);
    float r = (ph - n) + pl;
    float res = pm_exp2_split(n, r);
    return (pm_signbit(x) && y_odd) ? -res : res;
}
