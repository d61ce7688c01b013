// Float results of the reference's double-precision expressions without the
// FP64 pipe in the common case.
//
// The reference evaluates a few expressions in double and rounds the result
// to float: (float)(1 / Math.Sqrt(x)) in Vector3/Quaternion.Normalize,
// (float)(Math.Sqrt(e) / y) in the stabilization boost (EntityBase.cs:931)
// and (float)Math.Pow(c, dt) in the damping (EntityBase.cs:943,952).  GB300
// runs FP64 at a small fraction of its FP32 rate, and one double pow per body
// and step cost a quarter of the pile's step time.  Each routine here first
// computes the exact value in double-float arithmetic (an unevaluated sum of
// two floats, ~44 significant bits; Dekker 1971, error-free sums and
// products with a fused multiply-add), then rounds it to float.  The double
// expression's own error is below 2^-52 relative, so when the double-float
// value lies farther than its error bound (2^-42 relative and more) from the
// midpoint between two floats, the double expression rounds to the same
// float.  Inside that margin -- about one argument in 2^15 -- the routine
// evaluates the double expression itself.  So every result is the float the
// double expression gives, and nearly all of them cost FP32 work only.
//
// Host and device compile the same code (the host with std::fma and
// -ffp-contract=off), so the host tests cover the routines' logic.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define BEPU_HD __host__ __device__ __forceinline__
#else
#define BEPU_HD inline
#endif

namespace bepugpu {
namespace dr {

BEPU_HD float Fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}
BEPU_HD float Sqrt(float x) {
#ifdef __CUDA_ARCH__
    return __fsqrt_rn(x);
#else
    return std::sqrt(x);
#endif
}
BEPU_HD uint32_t Bits(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    uint32_t u;
    std::memcpy(&u, &x, 4);
    return u;
#endif
}
BEPU_HD float FromBits(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float x;
    std::memcpy(&x, &u, 4);
    return x;
#endif
}
// 2^k for k in [-126, 127].
BEPU_HD float Pow2(int k) { return FromBits((uint32_t)(k + 127) << 23); }

// A double-float value hi + lo with |lo| <= half an ulp of hi.
struct DF {
    float hi, lo;
};
// a + b exactly, when |a| >= |b| or a == 0 (Dekker's fast two-sum).
BEPU_HD DF QuickTwoSum(float a, float b) {
    float s = a + b;
    return {s, b - (s - a)};
}
// a + b exactly (Knuth's two-sum).
BEPU_HD DF TwoSum(float a, float b) {
    float s = a + b;
    float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
// a * b exactly.
BEPU_HD DF TwoProd(float a, float b) {
    float p = a * b;
    return {p, Fma(a, b, -p)};
}
BEPU_HD DF Add(DF x, DF y) {
    DF s = TwoSum(x.hi, y.hi);
    DF t = TwoSum(x.lo, y.lo);
    s.lo = s.lo + t.hi;
    s = QuickTwoSum(s.hi, s.lo);
    s.lo = s.lo + t.lo;
    return QuickTwoSum(s.hi, s.lo);
}
BEPU_HD DF Mul(DF x, DF y) {
    DF p = TwoProd(x.hi, y.hi);
    p.lo = p.lo + (x.hi * y.lo + x.lo * y.hi);
    return QuickTwoSum(p.hi, p.lo);
}
BEPU_HD DF MulF(DF x, float y) {
    DF p = TwoProd(x.hi, y);
    p.lo = p.lo + x.lo * y;
    return QuickTwoSum(p.hi, p.lo);
}

// Whether a value within `bound` of y could round to a float other than
// y.hi: y lies within `bound` of a midpoint between y.hi and a neighbour, or
// y.hi is a power of two (its neighbours' spacing differs on each side).
BEPU_HD bool NearMidpoint(DF y, float bound) {
    const uint32_t b = Bits(y.hi) & 0x7fffffffu;
    if ((b & 0x007fffffu) == 0u || b < 0x0c800000u || b >= 0x7f000000u) return true;  // 2^-102 .. 2^127
    const float halfUlp = Pow2((int)(b >> 23) - 127 - 24);
    return std::fabs(y.lo) + bound >= halfUlp;
}

// (float)(1 / Math.Sqrt((double)x)): the double-float value, when it
// decides the rounding (TryInvSqrt returns false otherwise).
BEPU_HD bool TryInvSqrt(float x, float& out) {
    if (!(x >= 0x1p-100f && x <= 0x1p100f)) return false;
    const float s0 = Sqrt(x);
    const float s1 = Fma(-s0, s0, x) / (2.f * s0);  // sqrt(x) = s0 + s1 to ~2^-48
    const float y0 = 1.f / s0;
    const float e = Fma(-y0, s0, 1.f);               // 1 - y0 s0, exact
    // 1 / (s0 + s1) = y0 (1 + e - s1 / s0) to second order
    const DF y = QuickTwoSum(y0, y0 * (e - s1 * y0));
    out = y.hi;
    return !NearMidpoint(y, y0 * 0x1p-42f);
}
BEPU_HD float InvSqrtAsDouble(float x) {
    float r;
    if (TryInvSqrt(x, r)) return r;
    return (float)(1.0 / std::sqrt((double)x));
}

// (float)(Math.Sqrt((double)e) / (double)y).
BEPU_HD bool TrySqrtQuotient(float e, float y, float& out) {
    if (e == 0.f && y > 0.f) {
        out = 0.f;
        return true;
    }
    if (!(e >= 0x1p-100f && e <= 0x1p100f && y >= 0x1p-60f && y <= 0x1p60f)) return false;
    const float s0 = Sqrt(e);
    const float s1 = Fma(-s0, s0, e) / (2.f * s0);
    const float q0 = s0 / y;
    const float q1 = (Fma(-q0, y, s0) + s1) / y;  // (s0 + s1 - q0 y) / y
    const DF q = QuickTwoSum(q0, q1);
    out = q.hi;
    return !NearMidpoint(q, q0 * 0x1p-42f);
}
BEPU_HD float SqrtQuotientAsDouble(float e, float y) {
    float r;
    if (TrySqrtQuotient(e, y, r)) return r;
    return (float)(std::sqrt((double)e) / (double)y);
}

// Constants of the double-float logarithm and exponential: hi + lo of ln 2,
// 1 / (2k + 1) for the atanh series and 1 / n! for the exponential series,
// each hi the float nearest the value and lo the float nearest the rest.
#define BEPU_POW_TABLES                                                                                           \
    {                                                                                                             \
        {0x1.62e43p-1f, -0x1.05c61p-29f},                                                                        \
        {{0x1p+0f, 0x0p+0f}, {0x1.555556p-2f, -0x1.555556p-27f}, {0x1.99999ap-3f, -0x1.99999ap-29f},            \
         {0x1.24924ap-3f, -0x1.b6db6ep-28f}, {0x1.c71c72p-4f, -0x1.c71c72p-31f},                                 \
         {0x1.745d18p-4f, -0x1.745d18p-29f}, {0x1.3b13b2p-4f, -0x1.89d89ep-29f},                                 \
         {0x1.111112p-4f, -0x1.dddddep-29f}, {0x1.e1e1e2p-5f, -0x1.e1e1e2p-33f},                                 \
         {0x1.af286cp-5f, -0x1.af286cp-32f}, {0x1.861862p-5f, -0x1.e79e7ap-31f}},                                \
        {{0x1p+0f, 0x0p+0f}, {0x1p+0f, 0x0p+0f}, {0x1p-1f, 0x0p+0f}, {0x1.555556p-3f, -0x1.555556p-28f},        \
         {0x1.555556p-5f, -0x1.555556p-30f}, {0x1.111112p-7f, -0x1.dddddep-32f},                                 \
         {0x1.6c16c2p-10f, -0x1.27d27ep-35f}, {0x1.a01a02p-13f, -0x1.7f97fap-39f},                               \
         {0x1.a01a02p-16f, -0x1.7f97fap-42f}, {0x1.71de3ap-19f, 0x1.55b1ccp-45f},                                \
         {0x1.27e4fcp-22f, -0x1.10ec14p-47f}, {0x1.ae6456p-26f, 0x1.fd5138p-52f},                                \
         {0x1.1eed8ep-29f, 0x1.ff1b12p-54f}, {0x1.612462p-33f, -0x1.8af25ep-58f}},                               \
    }
struct PowTables {
    float ln2[2];
    float odd[11][2];   // 1 / (2k + 1), k = 0..10
    float fact[14][2];  // 1 / n!, n = 0..13
};
#ifdef __CUDACC__
__constant__ const PowTables kPowTablesDevice = BEPU_POW_TABLES;
#endif
static const PowTables kPowTablesHost = BEPU_POW_TABLES;
BEPU_HD const PowTables& Tables() {
#ifdef __CUDA_ARCH__
    return kPowTablesDevice;
#else
    return kPowTablesHost;
#endif
}

// (float)Math.Pow((double)c, (double)dt) for the damping factor: c in [0, 1]
// (a clamped 1 - damping), dt a time step.  ln c from the atanh series of
// (m - 1) / (m + 1) with c = m 2^k, m in [0.70, 1.42) (|s| <= 0.172, eleven
// terms), exp by 2^j e^r with |r| <= ln 2 / 2 (fourteen terms).
BEPU_HD bool TryPow(float c, float dt, float& out) {
    if (c == 1.f || (c == 0.f && dt > 0.f)) {
        out = c;
        return true;
    }
    if (!(c >= 0x1p-126f && c < 1.f && dt >= 0x1p-40f && dt <= 16.f)) return false;
    const PowTables& T = Tables();
    const uint32_t cb = Bits(c);
    int k = (int)(cb >> 23) - 127;                       // c = m 2^k, m in [1, 2)
    float m = FromBits((cb & 0x007fffffu) | 0x3f800000u);
    if (m > 0x1.6a09e6p+0f) {                            // above sqrt 2: m in [0.70, 1.42)
        m = m * 0.5f;
        k += 1;
    }
    const float num = m - 1.f;                           // exact (Sterbenz)
    const DF den = TwoSum(m, 1.f);
    const float s0 = num / den.hi;
    const float s1 = (Fma(-s0, den.hi, num) - s0 * den.lo) / den.hi;
    const DF s = QuickTwoSum(s0, s1);                    // (m - 1) / (m + 1)
    const DF t = Mul(s, s);
    DF p = {T.odd[10][0], T.odd[10][1]};
    for (int i = 9; i >= 0; i--) p = Add(Mul(p, t), DF{T.odd[i][0], T.odd[i][1]});
    DF lnc = Mul(s, p);                                  // ln m = 2 s sum t^i / (2i + 1)
    lnc.hi = lnc.hi * 2.f;
    lnc.lo = lnc.lo * 2.f;
    const DF ln2 = {T.ln2[0], T.ln2[1]};
    lnc = Add(lnc, MulF(ln2, (float)k));
    const DF x = MulF(lnc, dt);                          // dt ln c <= 0
    if (!(x.hi > -80.f)) return false;
    const float j = std::rint(x.hi * 0x1.715476p+0f);    // nearest x / ln 2, in [-116, 0]
    const DF jl = MulF(ln2, j);
    const DF r = Add(x, DF{-jl.hi, -jl.lo});             // |r| <= ln 2 / 2 + rounding
    DF e = {T.fact[13][0], T.fact[13][1]};
    for (int n = 12; n >= 0; n--) e = Add(Mul(e, r), DF{T.fact[n][0], T.fact[n][1]});
    const float scale = Pow2((int)j);
    const DF y = {e.hi * scale, e.lo * scale};
    out = y.hi;
    return y.hi >= 0x1p-100f && !NearMidpoint(y, (std::fabs(x.hi) + 1.f) * 0x1p-41f * y.hi);
}
BEPU_HD float PowAsDouble(float c, float dt) {
    float r;
    if (TryPow(c, dt, r)) return r;
    return (float)std::pow((double)c, (double)dt);
}

}  // namespace dr
}  // namespace bepugpu
