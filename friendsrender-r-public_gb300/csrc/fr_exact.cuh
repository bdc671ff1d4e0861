// Float results of the reference's double-precision expressions without the
// FP64 pipe (GB300 runs FP64 at 1/64 of the FP32 rate).
//
// Each function returns exactly the float that the reference gets by
// evaluating its expression in double and rounding the result to float.  It
// evaluates the expression in float-float arithmetic (a value is the unevaluated
// sum hi + lo of two floats, about 48 significant bits) together with a bound b
// on the distance between that value and the reference's double result.  When
// every real number within b of the float-float value rounds to the same float,
// that float is the reference's result; otherwise (a result within about 2^-40
// relative of a rounding boundary, or an input outside the ranges the bounds
// were derived for) the function evaluates the reference's expression in double
// instead.  This is Ziv's rounding test (A. Ziv, "Fast evaluation of elementary
// mathematical functions with correctly rounded last bit", ACM TOMS 17(3),
// 1991); the float-float operations are the error-free transformations of
// Knuth (two-sum) and Dekker (two-product, here with an FMA) and the usual
// division and square root refinements (T. J. Dekker, "A floating-point
// technique for extending the available precision", Numer. Math. 18, 1971).
//
// Error bounds: every float-float operation below is accurate to better than
// 2^-45 relative; the bounds charge 2^-44 per operation, and each double
// operation of the reference contributes its rounding (2^-53 relative)
// amplified by any cancellation after it.  fr_check_exact_math compares every
// function with its double expression on the device.
#pragma once
#include <cstdint>

namespace fr {
namespace xf {

struct ff {
  float h, l;
};

// Knuth's two-sum: s + e == a + b exactly.
__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

// s + e == a + b exactly when |a| >= |b|.
__device__ __forceinline__ ff fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// p + e == a * b exactly (no underflow in the inputs' ranges used here).
__device__ __forceinline__ ff two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ ff add_f(ff a, float b) {
  const ff s = two_sum(a.h, b);
  return fast_two_sum(s.h, __fadd_rn(s.l, a.l));
}

__device__ __forceinline__ ff add(ff a, ff b) {
  const ff s = two_sum(a.h, b.h);
  return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}

__device__ __forceinline__ ff mul_f(ff a, float b) {
  const ff p = two_prod(a.h, b);
  return fast_two_sum(p.h, __fmaf_rn(a.l, b, p.l));
}

__device__ __forceinline__ ff mul(ff a, ff b) {
  const ff p = two_prod(a.h, b.h);
  const float t = __fmaf_rn(a.h, b.l, __fmul_rn(a.l, b.h));
  return fast_two_sum(p.h, __fadd_rn(p.l, t));
}

// a / b for a float-float a and a float b.  The remainder a.h - q1*b of the
// correctly rounded quotient q1 is a float, so the FMA gives it exactly.
__device__ __forceinline__ ff div_f(ff a, float b) {
  const float q1 = __fdiv_rn(a.h, b);
  const float r = __fadd_rn(__fmaf_rn(-q1, b, a.h), a.l);
  return fast_two_sum(q1, __fdiv_rn(r, b));
}

// a / b for a float a and a float-float b.
__device__ __forceinline__ ff f_div(float a, ff b) {
  const float q1 = __fdiv_rn(a, b.h);
  const float r = __fsub_rn(__fmaf_rn(-q1, b.h, a), __fmul_rn(q1, b.l));
  return fast_two_sum(q1, __fdiv_rn(r, b.h));
}

__device__ __forceinline__ ff div(ff a, ff b) {
  const float q1 = __fdiv_rn(a.h, b.h);
  const float r = __fsub_rn(__fadd_rn(__fmaf_rn(-q1, b.h, a.h), a.l), __fmul_rn(q1, b.l));
  return fast_two_sum(q1, __fdiv_rn(r, b.h));
}

// sqrt(a); the remainder a.h - s*s of the correctly rounded root s is a float.
__device__ __forceinline__ ff sqrt(ff a) {
  const float s = __fsqrt_rn(a.h);
  const float r = __fadd_rn(__fmaf_rn(-s, s, a.h), a.l);
  return fast_two_sum(s, __fdiv_rn(r, __fmul_rn(2.0f, s)));
}

// Ziv's test: true (and the float in `out`) when every real within b of
// y.h + y.l rounds to nearest to the same float.
__device__ __forceinline__ bool round_ok(ff y, float b, float& out) {
  const float ah = fabsf(y.h);
  if (!(ah >= 0x1p-100f && ah <= 0x1p100f)) return false;  // also rejects NaN
  const float al = y.h < 0.0f ? -y.l : y.l;
  const int bits = __float_as_int(ah);
  const float up = __fmul_rn(__fsub_rn(__int_as_float(bits + 1), ah), 0.5f);  // half gap above |y.h|
  const float dn = __fmul_rn(__fsub_rn(ah, __int_as_float(bits - 1)), 0.5f);  // half gap below
  if (!(__fadd_ru(al, b) < up) || !(__fadd_ru(-al, b) < dn)) return false;
  out = y.h;
  return true;
}

// Absolute bound e * |y| (+ extra), rounded up.
__device__ __forceinline__ float bound(ff y, float e, float extra = 0.0f) {
  return __fadd_ru(__fmul_ru(e, fabsf(y.h)), extra);
}

__device__ __forceinline__ bool in_range(float x, float lo, float hi) {
  const float a = fabsf(x);
  return a >= lo && a <= hi;  // false for NaN
}

}  // namespace xf

// ---------------------------------------------------------------- functions
// Each *_d function is the reference's expression in double (the fallback);
// the public function tries the float-float path first.

// (float)(1.0 / ((double)x * (double)x)): powf(x, -2.0f) of the reference.
static __device__ __noinline__ float pow_m2_d(float x) {
  const double xd = (double)x;
  return (float)(1.0 / (xd * xd));
}
__device__ __forceinline__ bool pow_m2_fast(float x, float& r) {
  if (xf::in_range(x, 0x1p-40f, 0x1p40f)) {
    // x*x is exact in double; one double rounding (2^-53); two float-float
    // operations.
    const xf::ff y = xf::f_div(1.0f, xf::two_prod(x, x));
    return xf::round_ok(y, xf::bound(y, 0x1p-42f), r);
  }
  return false;
}
__device__ __forceinline__ float pow_m2(float x) {
  float r;
  return pow_m2_fast(x, r) ? r : pow_m2_d(x);
}

// (float)sqrt((1.0 - (double)e) / (double)den), Sampling.cpp:129 (GGX_Sampling).
static __device__ __noinline__ float ggx_cth_d(float e, float den) { return (float)sqrt((1.0 - (double)e) / (double)den); }
__device__ __forceinline__ bool ggx_cth_fast(float e, float den, float& r) {
  const xf::ff n = xf::two_sum(1.0f, -e);  // 1 - e, exact as in double
  if (n.h > 0x1p-30f && n.h <= 2.0f && den > 0x1p-30f && den <= 0x1p30f) {
    // double: divide, square root: |d - sqrt(n/den)| <= 1.51 * 2^-53 * sqrt.
    const xf::ff y = xf::sqrt(xf::div_f(n, den));
    return xf::round_ok(y, xf::bound(y, 0x1p-42f), r);
  }
  return false;
}
__device__ __forceinline__ float ggx_cth(float e, float den) {
  float r;
  return ggx_cth_fast(e, den, r) ? r : ggx_cth_d(e, den);
}

// (float)((double)a2 / ((double)PI * ((double)x * (double)x)) * (double)wm_N / (double)f4),
// Sampling.cpp:154 (GGX_Sampling's pdf; f4 = 4 * wo_wm in float).
static __device__ __noinline__ float ggx_pdf_d(float a2, float x, float wm_N, float f4, float pi) {
  return (float)((double)a2 / ((double)pi * ((double)x * (double)x)) * (double)wm_N / (double)f4);
}
__device__ __forceinline__ bool ggx_pdf_fast(float a2, float x, float wm_N, float f4, float pi, float& r) {
  if (xf::in_range(a2, 0x1p-40f, 0x1p20f) && xf::in_range(x, 0x1p-30f, 0x1p30f) &&
      xf::in_range(wm_N, 0x1p-40f, 0x1p20f) && xf::in_range(f4, 0x1p-40f, 0x1p20f)) {
    // double: 4 roundings (x*x exact) -> 2^-51; float-float: 4 operations.
    const xf::ff D = xf::mul_f(xf::two_prod(x, x), pi);
    const xf::ff y = xf::div_f(xf::mul_f(xf::f_div(a2, D), wm_N), f4);
    return xf::round_ok(y, xf::bound(y, 0x1p-41f), r);
  }
  return false;
}
__device__ __forceinline__ float ggx_pdf(float a2, float x, float wm_N, float f4, float pi) {
  float r;
  return ggx_pdf_fast(a2, x, wm_N, f4, pi, r) ? r : ggx_pdf_d(a2, x, wm_N, f4, pi);
}

// GGXGlass_Sampling's cos(theta), Sampling.cpp:193:
//   den = (double)e * ((double)a2 - 0.99999) + 1.0
//   (float)sqrt((1.0000001 - (double)e) / den)
static __device__ __noinline__ float glass_cth_d(float e, float a2) {
  const double den = (double)e * ((double)a2 - 0.99999) + 1.0;
  return (float)sqrt((1.0000001 - (double)e) / den);
}
__device__ __forceinline__ bool glass_cth_fast(float e, float a2, float& r) {
  if (a2 >= 0x1p-40f && a2 <= 0.25f) {
    // The double constants as float-float, each within 2^-48 of the double.
    constexpr float c1h = 0.99999f, c1l = (float)(0.99999 - (double)0.99999f);
    constexpr float c2h = 1.0000001f, c2l = (float)(1.0000001 - (double)1.0000001f);
    // diff = a2 - 0.99999 in [-1, -0.74]: no cancellation.
    const xf::ff diff = xf::add_f(xf::two_sum(a2, -c1h), -c1l);
    const xf::ff m = xf::mul_f(diff, e);          // in (-1, 0]
    const xf::ff den = xf::add_f(m, 1.0f);        // >= 1e-5 + a2 * e
    const xf::ff num = xf::add_f(xf::two_sum(c2h, -e), c2l);  // >= 1.5e-7
    if (den.h > 0x1p-30f && num.h > 0x1p-30f) {
      const xf::ff y = xf::sqrt(xf::div(num, den));
      // Relative bound: the constants' error amplified by the cancellation in
      // num (2^-47 / num), both evaluations' errors in m amplified by
      // K = |m| / den, and 2^-42 for the rest.
      const float K = __fdiv_ru(fabsf(m.h), den.h);
      const float e_rel = __fadd_ru(__fadd_ru(__fdiv_ru(0x1p-46f, num.h), __fmul_ru(0x1p-45f, K)), 0x1p-41f);
            return xf::round_ok(y, xf::bound(y, e_rel), r);
    }
  }
  return false;
}
__device__ __forceinline__ float glass_cth(float e, float a2) {
  float r;
  return glass_cth_fast(e, a2, r) ? r : glass_cth_d(e, a2);
}

// GGXGlass_Sampling's refraction pdf, Sampling.cpp:242:
//   q = (double)B / ((double)s * (double)s)
//   (float)((double)A * q * (double)alpha * (double)alpha / (double)D)
static __device__ __noinline__ float glass_pdf_d(float A, float B, float s, float alpha, float D) {
  const double q = (double)B / ((double)s * (double)s);
  return (float)((double)A * q * (double)alpha * (double)alpha / (double)D);
}
__device__ __forceinline__ bool glass_pdf_fast(float A, float B, float s, float alpha, float D, float& r) {
  if (xf::in_range(A, 0x1p-40f, 0x1p20f) && xf::in_range(B, 0x1p-40f, 0x1p20f) && xf::in_range(s, 0x1p-30f, 0x1p30f) &&
      xf::in_range(alpha, 0x1p-20f, 0x1p10f) && xf::in_range(D, 0x1p-40f, 0x1p20f)) {
    // double: 5 roundings -> 2^-50.4; float-float: 6 operations.
    const xf::ff q = xf::f_div(B, xf::two_prod(s, s));
    const xf::ff y = xf::div_f(xf::mul_f(xf::mul_f(xf::mul_f(q, A), alpha), alpha), D);
    return xf::round_ok(y, xf::bound(y, 0x1p-41f), r);
  }
  return false;
}
__device__ __forceinline__ float glass_pdf(float A, float B, float s, float alpha, float D) {
  float r;
  return glass_pdf_fast(A, B, s, alpha, D, r) ? r : glass_pdf_d(A, B, s, alpha, D);
}

// MetalSurface::BRDF's value, material.h:410:
//   (float)((double)DeltaPDF / ((double)c + 0.00001)), c = dot(out, n) > 1e-4
static __device__ __noinline__ float metal_brdf_d(float c, float delta) { return (float)((double)delta / ((double)c + 0.00001)); }
__device__ __forceinline__ bool metal_brdf_fast(float c, float delta, float& r) {
  if (c >= 0x1p-14f && c <= 0x1p20f && xf::in_range(delta, 0x1p-40f, 0x1p40f)) {
    constexpr float c3h = 0.00001f, c3l = (float)(0.00001 - (double)0.00001f);
    // c + 1e-5 with c > 6e-5: no cancellation; double: 2 roundings.
    const xf::ff d = xf::add_f(xf::two_sum(c, c3h), c3l);
    const xf::ff y = xf::f_div(delta, d);
    return xf::round_ok(y, xf::bound(y, 0x1p-42f), r);
  }
  return false;
}
__device__ __forceinline__ float metal_brdf(float c, float delta) {
  float r;
  return metal_brdf_fast(c, delta, r) ? r : metal_brdf_d(c, delta);
}

// Roughconductor::BRDF's masking term, material.h:255-256:
//   (float)((-1.0f + sqrt(1.0f + (double)a2 * ((double)inv - 1.0))) * 0.5)
// with a2 = alpha * alpha and inv = 1 / (l * l) in float.
static __device__ __noinline__ float conductor_lambda_d(float a2, float inv) {
  return (float)((-1.0f + sqrt(1.0f + (double)a2 * ((double)inv - 1.0))) * 0.5);
}
__device__ __forceinline__ bool conductor_lambda_fast(float a2, float inv, float& r) {
  if (inv >= 1.0f && inv < 0x1p24f && a2 >= 0x1p-40f && a2 <= 0x1p10f) {
    // inv - 1 is exact in float for inv in [1, 2^24); w = a2 * (inv - 1) is
    // exact in double (two_prod here).  The reference rounds 1 + w, the square
    // root and (above 2) the subtraction: |d - L| <= 2^-52 * sqrt(1 + w), an
    // absolute term that the cancellation in sqrt(1 + w) - 1 makes large
    // relative to a small L.  L = w / (2 (sqrt(1 + w) + 1)) has no
    // cancellation: 6 float-float operations.
    const xf::ff w = xf::two_prod(a2, inv - 1.0f);
    if (w.h == 0.0f) { r = 0.0f; return true; }  // inv == 1: the reference computes (-1 + sqrt(1)) * 0.5 = 0
    const xf::ff s = xf::sqrt(xf::add_f(w, 1.0f));
    const xf::ff y = xf::mul_f(xf::div(w, xf::add_f(s, 1.0f)), 0.5f);
    return xf::round_ok(y, xf::bound(y, 0x1p-41f, __fmul_ru(0x1p-52f, __fmul_ru(s.h, 1.0001f))), r);
  }
  return false;
}
__device__ __forceinline__ float conductor_lambda(float a2, float inv) {
  float r;
  return conductor_lambda_fast(a2, inv, r) ? r : conductor_lambda_d(a2, inv);
}

// Roughconductor::BRDF's tm3, material.h:266:
//   (float)((double)(A) + (double)(B) * (1.0 - (double)f2))
// with A = apb * fcos * fcos, B = 1.0f - f2 and f2 = fcos * fcos in float.
static __device__ __noinline__ float conductor_tm3_d(float A, float B, float f2) {
  return (float)((double)A + (double)B * (1.0 - (double)f2));
}
__device__ __forceinline__ bool conductor_tm3_fast(float A, float B, float f2, float& r) {
  if (A >= 0.0f && A <= 0x1p40f && B >= 0x1p-40f && B <= 0x1p40f && f2 >= 0x1p-28f && f2 <= 1.0f) {
    // 1 - f2 is exact in double for f2 >= 2^-28 and as a float-float (two_sum);
    // every term is non-negative, so the reference's 2 roundings give 2^-52 and
    // the float-float sum of products 3 operations.
    const xf::ff c = xf::two_sum(1.0f, -f2);
    const xf::ff y = xf::add_f(xf::mul(xf::ff{B, 0.0f}, c), A);
    return xf::round_ok(y, xf::bound(y, 0x1p-42f), r);
  }
  return false;
}
__device__ __forceinline__ float conductor_tm3(float A, float B, float f2) {
  float r;
  return conductor_tm3_fast(A, B, f2, r) ? r : conductor_tm3_d(A, B, f2);
}

// (float)sqrt((double)x * 0.5), Roughconductor::BRDF's a (material.h:262):
// x * 0.5 is exact in double, and rounding the
// double square root of a float to float gives the correctly rounded float
// square root (double rounding is innocuous for square root when the wider
// format has at least 2p + 2 bits: S. Figueroa, "When is double rounding
// innocuous?", SIGNUM Newsl. 30(3), 1995).  x * 0.5f is exact in float for
// x >= 2^-125 (below, the halved value is subnormal and can round, even up to
// 2^-126).
static __device__ __noinline__ float sqrt_half_d(float x) { return (float)sqrt((double)x * 0.5); }
__device__ __forceinline__ bool sqrt_half_fast(float x, float& r) {
  if (!(x >= 0x1p-125f || x == 0.0f)) return false;
  r = __fsqrt_rn(__fmul_rn(x, 0.5f));
  return true;
}
__device__ __forceinline__ float sqrt_half(float x) {
  float r;
  return sqrt_half_fast(x, r) ? r : sqrt_half_d(x);
}

}  // namespace fr
