// nesf_df.cuh -- double-float arithmetic for the adaptive solver's deferred passes.
//
// A value is the unevaluated sum hi + lo of two FP32 numbers with |lo| <= ulp(hi) / 2:
// 48 significant bits (relative rounding ~3.6e-15), FP32's exponent range. On this GPU
// an FP64 instruction holds its SM sub-partition's FP64 pipe for ~64 cycles (one warp
// instruction per ~64 cycles, whatever the active lanes: measured), and a dependent FP64
// instruction waits as long, while FP32 instructions issue every cycle at ~5 cycles of
// latency. The replays and polishes of the few cells whose FP32 sweep is not kept are
// chains of dependent arithmetic of one cell, so double-float arithmetic on the FP32
// pipes runs them faster than FP64 and leaves the FP64 pipe to nobody.
//
// Methods (published; the constants below are computed from their definitions):
//   two_sum (Knuth, TAOCP vol. 2, 4.2.2), fast_two_sum and two_prod with a fused
//   multiply-add (Dekker 1971), the accurate double-double addition and the
//   multiplication of Hida, Li and Bailey (QD library paper, 2001); division by three
//   quotient digits from one reciprocal, square root by one correction of an FP32 estimate
//   (Karp and Markstein 1997); cube root by one
//   Newton step; exp by the reduction x = k ln2 / 64 + r (Tang 1989) with a table of
//   2^(j/64) and a Taylor polynomial of e^r - 1 (|r| <= ln2 / 128); log by the reduction
//   x = 2^e m and one Newton step y + m e^-y - 1 from an FP32 estimate; atan by the reduction atan(x) = atan(c) +
//   atan((x - c) / (1 + x c)), c = j / 32, and a Taylor polynomial (|t| <= 1 / 64).
// The error-free transformations use the IEEE-rounded FP32 intrinsics, so the files'
// fast-math flags leave them exact; the corrections' own divisions are approximate
// (__fdividef: a few ulps of a term already ~2^-24 of the result).
// Accuracy: a few units of 2^-48 for + - * / sqrt, ~1e-14 relative for cbrt, exp, log,
// pow and atan over the arguments the interface solves produce (tested against FP64).
#pragma once

#include <cstdint>

namespace nesf {

struct df {
    float hi, lo;
    df() = default;
    __host__ __device__ constexpr df(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ constexpr df(float f) : hi(f), lo(0.0f) {}
    __host__ __device__ constexpr df(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
    __host__ __device__ constexpr df(int i) : df((double)i) {}
    __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
    __host__ __device__ explicit operator float() const { return hi + lo; }
};

namespace dfx {

__device__ __forceinline__ df two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df(s, e);
}
// |a| >= |b| (or a = 0)
__device__ __forceinline__ df fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return df(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ df two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return df(p, __fmaf_rn(a, b, -p));
}
__device__ __forceinline__ df add(df a, df b) {
    const df s = two_sum(a.hi, b.hi);
    const df t = two_sum(a.lo, b.lo);
    df u = fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
    return fast_two_sum(u.hi, __fadd_rn(u.lo, t.lo));
}
__device__ __forceinline__ df neg(df a) { return df(-a.hi, -a.lo); }
__device__ __forceinline__ df mul(df a, df b) {
    const df p = two_prod(a.hi, b.hi);
    return fast_two_sum(p.hi, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo)));
}
__device__ __forceinline__ df mul_f(df a, float b) {
    const df p = two_prod(a.hi, b);
    return fast_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}
// a * 2^k for an exact power of two b (no rounding)
__device__ __forceinline__ df scale(df a, float b) { return df(__fmul_rn(a.hi, b), __fmul_rn(a.lo, b)); }
// Three quotient digits from one approximate reciprocal (its error of a few ulps is
// corrected by the next digit: the residuals r are exact to 2^-48 of a).
__device__ __forceinline__ df div(df a, df b) {
    const float inv = __fdividef(1.0f, b.hi);
    const float q1 = __fmul_rn(a.hi, inv);
    const df r = add(a, neg(mul_f(b, q1)));
    const float q2 = __fmul_rn(r.hi, inv);
    const df r2 = add(r, neg(mul_f(b, q2)));
    const float q3 = __fmul_rn(r2.hi, inv);
    return add(fast_two_sum(q1, q2), df(q3));
}
__device__ __forceinline__ bool lt(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool eq(df a, df b) { return a.hi == b.hi && a.lo == b.lo; }

}  // namespace dfx

__device__ __forceinline__ df operator+(df a, df b) { return dfx::add(a, b); }
__device__ __forceinline__ df operator-(df a, df b) { return dfx::add(a, dfx::neg(b)); }
__device__ __forceinline__ df operator-(df a) { return dfx::neg(a); }
__device__ __forceinline__ df operator*(df a, df b) { return dfx::mul(a, b); }
__device__ __forceinline__ df operator/(df a, df b) { return dfx::div(a, b); }
__device__ __forceinline__ df& operator+=(df& a, df b) { return a = a + b; }
__device__ __forceinline__ df& operator-=(df& a, df b) { return a = a - b; }
__device__ __forceinline__ df& operator*=(df& a, df b) { return a = a * b; }
__device__ __forceinline__ df& operator/=(df& a, df b) { return a = a / b; }
__device__ __forceinline__ bool operator<(df a, df b) { return dfx::lt(a, b); }
__device__ __forceinline__ bool operator>(df a, df b) { return dfx::lt(b, a); }
__device__ __forceinline__ bool operator<=(df a, df b) { return !dfx::lt(b, a) && !::isnan(a.hi) && !::isnan(b.hi); }
__device__ __forceinline__ bool operator>=(df a, df b) { return !dfx::lt(a, b) && !::isnan(a.hi) && !::isnan(b.hi); }
__device__ __forceinline__ bool operator==(df a, df b) { return dfx::eq(a, b); }
__device__ __forceinline__ bool operator!=(df a, df b) { return !dfx::eq(a, b); }
// Overloads for df beside the global ones, which the using-declarations keep visible to
// the FP32 and FP64 code of this namespace (an overload of the same name here would
// otherwise hide them and convert their arguments to df).
using ::isnan;
using ::signbit;
using ::__shfl_xor_sync;
__device__ __forceinline__ bool isnan(df a) { return ::isnan(a.hi); }
__device__ __forceinline__ bool signbit(df a) { return ::signbit(a.hi); }
__device__ __forceinline__ df __shfl_xor_sync(unsigned mask, df v, int lane) {
    return df(::__shfl_xor_sync(mask, v.hi, lane), ::__shfl_xor_sync(mask, v.lo, lane));
}

namespace dfx {

// 2^(j/64), j = 0..63, rounded to double then split (Tang's table)
__device__ constexpr df kExp2Tab[64] = {
    df(1.0), df(1.0108892860517005), df(1.0218971486541166), df(1.0330248790212284), df(1.0442737824274138),
    df(1.0556451783605572), df(1.0671404006768237), df(1.0787607977571199), df(1.0905077326652577),
    df(1.102382583307841), df(1.1143867425958924), df(1.1265216186082418), df(1.1387886347566916),
    df(1.1511892299529827), df(1.1637248587775775), df(1.1763969916502812), df(1.189207115002721),
    df(1.202156731452703), df(1.215247359980469), df(1.22848053610687), df(1.241857812073484),
    df(1.255380757024691), df(1.2690509571917332), df(1.2828700160787783), df(1.2968395546510096),
    df(1.3109612115247644), df(1.3252366431597413), df(1.339667524053303), df(1.3542555469368927),
    df(1.3690024229745905), df(1.383909881963832), df(1.3989796725383112), df(1.4142135623730951),
    df(1.42961333839197), df(1.4451808069770467), df(1.460917794180647), df(1.4768261459394993),
    df(1.4929077282912648), df(1.5091644275934228), df(1.5255981507445384), df(1.5422108254079407),
    df(1.559004400237837), df(1.5759808451078865), df(1.593142151342267), df(1.6104903319492543),
    df(1.6280274218573478), df(1.645755478153965), df(1.6636765803267364), df(1.681792830507429),
    df(1.7001063537185235), df(1.718619298122478), df(1.7373338352737062), df(1.7562521603732995),
    df(1.7753764925265212), df(1.7947090750031072), df(1.8142521755003989), df(1.8340080864093424),
    df(1.8539791250833855), df(1.8741676341103), df(1.8945759815869656), df(1.9152065613971474),
    df(1.9360617934922943), df(1.9571441241754002), df(1.978456026387951)};

// atan(j / 32), j = 0..32
__device__ constexpr df kAtanTab[33] = {
    df(0.0), df(0.031239833430268277), df(0.06241880999595735), df(0.09347678115858947), df(0.12435499454676144),
    df(0.15499674192394097), df(0.18534794999569476), df(0.21535769969773805), df(0.24497866312686414),
    df(0.2741674511196588), df(0.3028848683749714), df(0.3310960767041321), df(0.35877067027057225),
    df(0.38588266939807375), df(0.4124104415973873), df(0.43833655985795783), df(0.4636476090008061),
    df(0.48833395105640554), df(0.5123894603107377), df(0.5358112379604637), df(0.5585993153435624),
    df(0.5807563535676704), df(0.6022873461349642), df(0.6231993299340659), df(0.6435011087932844),
    df(0.6632029927060933), df(0.6823165548747481), df(0.7008544078844502), df(0.7188299996216245),
    df(0.7362574289814281), df(0.7531512809621944), df(0.7695264804056583), df(0.7853981633974483)};

// ln2 / 64 = kL1 + kL2 + kL3: kL1 has 11 significant bits (k kL1 exact for |k| < 2^13)
constexpr float kL1 = 0.01082611083984375f;
constexpr float kL2 = 4.313856607041089e-06f;
constexpr float kL3 = -2.0164599157102003e-13f;
constexpr float kInvL = 92.33248261689366f;   // 64 / ln2
constexpr df kLn2 = df(0.6931471805599453);
constexpr df kPiHalf = df(1.5707963267948966);

// e^x = 2^e T (1 + m): T = 2^(j/64) from the table, m = e^r - 1, x = (64 e + j) ln2 / 64 + r,
// |r| <= ln2 / 128 (k = 64 e + j). Returns e, T and m for |x| below FP32's overflow.
__device__ __forceinline__ int exp_parts(df x, df& T, df& m) {
    const float kf = rintf(__fmul_rn(x.hi, kInvL));
    const int k = (int)kf;
    // r = x - k ln2 / 64 (k kL1 exact; the other two parts' products rounded at 2^-24 of
    // terms already ~2^-24 of r at most)
    df r = add(two_sum(x.hi, -__fmul_rn(kf, kL1)), df(x.lo));
    r = add(r, neg(two_prod(kf, kL2)));
    r = add(r, df(-__fmul_rn(kf, kL3)));
    // e^r - 1 = r + r^2 / 2 + r^3 (1/6 + r/24 + r^2/120 + r^3/720), the last group in FP32
    // (its terms are below 2^-23 of the sum's)
    const float rh = r.hi;
    const float tail = __fmul_rn(__fmul_rn(__fmul_rn(rh, rh), rh),
                                 __fmaf_rn(rh, __fmaf_rn(rh, __fmaf_rn(rh, 1.0f / 720.0f, 1.0f / 120.0f), 1.0f / 24.0f),
                                           1.0f / 6.0f));
    m = add(r, add(scale(mul(r, r), 0.5f), df(tail)));
    const int j = k & 63;
    T = kExp2Tab[j];
    return (k - j) / 64;                                 // exact: k - j is a multiple of 64
}

static __device__ __noinline__ df exp(df x) {
    if (::isnan(x.hi)) return x;
    if (x.hi > 88.7f) return df(__int_as_float(0x7f800000), 0.0f);
    if (x.hi < -87.0f) return df(0.0f, 0.0f);            // below FP32's normal range
    df T, m;
    const int e = exp_parts(x, T, m);
    const df v = add(T, mul(T, m));
    return scale(v, __int_as_float((127 + e) << 23));   // e in [-126, 127]
}

// e^x - 1 with a relative error of a few units of 2^-48 for |x| <= 1 (the log's correction)
__device__ __forceinline__ df expm1_small(df x) {
    df T, m;
    const int e = exp_parts(x, T, m);                    // e in {-2, -1, 0, 1}
    const float s = __int_as_float((127 + e) << 23);
    const df sT = scale(T, s);
    // 2^e T - 1 (the high part's difference exact by Sterbenz: 2^e T.hi in [1/4, 4)) + 2^e T m
    const df a = add(two_sum(sT.hi, -1.0f), df(sT.lo));
    return add(a, mul(sT, m));
}

static __device__ __noinline__ df log(df x) {
    if (!(x.hi > 0.0f)) {
        if (x.hi == 0.0f) return df(-__int_as_float(0x7f800000), 0.0f);
        return df(__int_as_float(0x7fffffff), 0.0f);
    }
    if (::isinf(x.hi)) return x;
    // x = 2^e m, m in [sqrt(1/2), sqrt(2)): log x = e ln2 + log m. log m from an FP32
    // estimate y0 = log1p(m - 1) and one Newton step on e^y = m in relative form:
    // d = m e^-y0 - 1 = t + E + t E (t = m - 1 exact, E = e^-y0 - 1), log m = y0 + d - d^2 / 2
    // + O(d^3), d ~ y0's error of a few ulps of |log m| <= 0.35: the result keeps a few units
    // of 2^-48 relative to log m also where it is small (x near 1)
    int e = 0;
    float mh = frexpf(x.hi, &e);                         // mh in [1/2, 1)
    if (mh < 0.70710678f) { mh = __fmul_rn(mh, 2.0f); e -= 1; }
    const df t = add(df(__fsub_rn(mh, 1.0f)), df(ldexpf(x.lo, -e)));   // x 2^-e - 1
    const float y0 = log1pf(t.hi);
    const df E = expm1_small(df(-y0));
    const df d = add(add(t, E), mul(t, E));
    const df lm = add(df(y0), add(d, df(-0.5f * d.hi * d.hi)));
    return e == 0 ? lm : add(mul_f(kLn2, (float)e), lm);
}

__device__ __forceinline__ df sqrt(df a) {
    if (!(a.hi > 0.0f)) return a.hi == 0.0f ? df(0.0f, 0.0f) : df(__int_as_float(0x7fffffff), 0.0f);
    if (::isinf(a.hi)) return a;
    const float y = __fsqrt_rn(a.hi);
    const df r = add(a, neg(two_prod(y, y)));
    return fast_two_sum(y, __fdividef(r.hi, __fmul_rn(2.0f, y)));
}

static __device__ __noinline__ df cbrt(df a) {
    if (a.hi == 0.0f || ::isnan(a.hi) || ::isinf(a.hi)) return df(a.hi, 0.0f);
    const float y = cbrtf(a.hi);
    const df y3 = mul_f(two_prod(y, y), y);
    const df r = add(a, neg(y3));
    return fast_two_sum(y, __fdividef(r.hi, __fmul_rn(3.0f, __fmul_rn(y, y))));
}

static __device__ __noinline__ df pow(df x, df y) {
    if (y.hi == 0.0f) return df(1.0f, 0.0f);
    if (x.hi == 1.0f && x.lo == 0.0f) return df(1.0f, 0.0f);
    if (!(x.hi > 0.0f)) return df(__int_as_float(0x7fffffff), 0.0f);   // the solves take positive bases
    return exp(mul(y, log(x)));
}

// atan on |t| <= 1/64: t - t^3 (1/3 - t^2 / 5 + t^4 / 7 - t^6 / 9); the bracket's part after
// 1/3 is below 5e-5 of it, so it is summed in FP32 against 1/3 in double-float
__device__ __forceinline__ df atan_small(df t) {
    const df u = mul(t, t);
    const float uh = u.hi;
    const float rest = __fmul_rn(uh, __fmaf_rn(uh, __fmaf_rn(uh, -1.0f / 9.0f, 1.0f / 7.0f), -1.0f / 5.0f));
    const df q = add(df(1.0 / 3.0), df(rest));
    return add(t, neg(mul(mul(t, u), q)));
}

static __device__ __noinline__ df atan(df x) {
    if (::isnan(x.hi)) return x;
    const bool negx = x.hi < 0.0f;
    df a = negx ? neg(x) : x;
    const bool big = a.hi > 1.0f;
    if (big) {
        if (::isinf(a.hi)) return negx ? neg(kPiHalf) : kPiHalf;
        a = div(df(1.0f), a);
    }
    const int j = (int)rintf(__fmul_rn(a.hi, 32.0f));   // 0..32
    const float c = __fmul_rn((float)j, 1.0f / 32.0f);
    // t = (a - c) / (1 + a c), |t| <= 1/64
    const df t = div(add(a, df(-c)), add(df(1.0f), mul_f(a, c)));
    df y = add(kAtanTab[j], atan_small(t));
    if (big) y = add(kPiHalf, neg(y));
    return negx ? neg(y) : y;
}

}  // namespace dfx
}  // namespace nesf
