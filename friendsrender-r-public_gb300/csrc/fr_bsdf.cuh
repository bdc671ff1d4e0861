// Surfaces, sampling routines and texture fetch of the reference's SPPM path,
// as device functions.
//
// Each function restates the reference's arithmetic in its own evaluation
// order and precision.  Where the reference's expression is promoted to
// double (a double literal or a double-returning libm call: sqrt, sincos) the
// restatement returns the same float without FP64 arithmetic in all but rare
// cases (fr_exact.cuh), or reads a table of the exact result; where it calls
// powf(x, -2.0f) the restatement uses pow_m2; pow(x, 2) is an exact square
// (the compiler folds it in the reference's build); comparisons of a float
// with a double constant use the equivalent float threshold.
#pragma once
#include "fr_exact.cuh"
#include "fr_layout.h"
#include "fr_math.cuh"

namespace fr {

constexpr float kSMin = 1e-16f;                    // Sampling::sMin (Sampling.h:8)
constexpr float kDeltaPDF = 1.0f;                  // Sampling::DeltaPDF (Sampling.h:7)

__device__ __forceinline__ V3 invalid_dir() { return V3{1e-3f, 1e-3f, 1e-3f}; }  // RUtil::INVALID_DIR
__device__ __forceinline__ bool is_valid_direction(V3 d) { return norm2(d) > 0.9999f; }  // RayUtility.cpp:36-38

// FUNCTION_PARAM (material.h:12-34)
struct FParam {
  V3 in, out, n;
  float from, to, rough, absorb, refl;
};

// Orthonormal frame around e1 used by Cos/GGX sampling (Sampling.cpp:10-18, 132-138).
__device__ __forceinline__ void frame(V3 e1, V3& e2, V3& e3) {
  if (fabsf(e1.x) > kGt1e6) e2 = normalized(cross(v3(0.f, 1.f, 0.f), e1));
  else e2 = normalized(cross(v3(1.f, 0.f, 0.f), e1));
  e3 = normalized(cross(e1, e2));
}

// Tables of the two double-precision functions of a single 24-bit draw u
// that the sampling routines use, filled on the host with the host's libm:
//   c_sincos_tab[u] = {(float)cos(x), (float)sin(x)}, x = (float)((u*2^-24) * 2 * PI)
//                     (Sampling.cpp:65, 127, 191 evaluate u*2.0f*PI in double and round it once)
//   c_sqrt1m_tab[u] = (float)sqrt(1.000000001 - u*2^-24)          (Sampling.cpp:24)
// GB300's FP64 rate is 1/64 of FP32; a table read replaces ~50 FP64
// instructions per bounce and returns the reference's exact floats.
constexpr uint32_t kU24 = 1u << 24;
__constant__ const float2* c_sincos_tab;
__constant__ const float* c_sqrt1m_tab;

__device__ __forceinline__ float unit24(uint32_t u) { return (float)u * (1.0f / 16777216.0f); }

// Sampling::Cos_Sampling (Sampling.cpp:7-28)
__device__ __forceinline__ V3 cos_sampling(Rng& rng, V3 normal, float* pdf) {
  V3 e2, e3;
  const V3 e1 = normal;
  frame(e1, e2, e3);
  const uint32_t uph = rng.next_u24();
  const uint32_t uth = rng.next_u24();
  const float th2 = sqrtf(unit24(uth));
  const float2 cs = __ldg(c_sincos_tab + uph);
  const float r1 = __ldg(c_sqrt1m_tab + uth);
  V3 result = e1 * r1 + e2 * cs.x * th2 + e3 * cs.y * th2;
  result = normalized(result);
  if (pdf) *pdf = fmaxf(kSMin, dot(result, normal) / kPI);
  return result;
}

// Sampling::Reflect_Sampling (Sampling.cpp:293-295)
__device__ __forceinline__ V3 reflect_sampling(V3 n, V3 in) { return normalized(in - 2.0f * dot(n, in) * n); }

// Sampling::Fresnel_Reflectance (Sampling.cpp:297-313)
__device__ __forceinline__ float fresnel_reflectance(V3 n, V3 in, float ni, float no) {
  const float n1_div_n2 = ni / no;
  const float cosA = fabsf(dot(n, in));
  const float sinA = sqrtf(1.0000001f - cosA * cosA);
  const float sinB = n1_div_n2 * sinA;
  if (sinB > kGt0_999999) return 1.0f;
  const float cosB = sqrtf(1.0000001f - sinB * sinB);
  const float rp = (no * cosA - ni * cosB) / (no * cosA + ni * cosB);
  const float rs = (ni * cosA - no * cosB) / (ni * cosA + no * cosB);
  return (0.5f * rs * rs) + (0.5f * rp * rp);
}

// RUtil::Refract (RayUtility.cpp:10-17)
__device__ __forceinline__ V3 refract(V3 in, V3 n, float from, float into) {
  const V3 NN = dot(in, n) < 0.0f ? n : -n;
  const float eta = from / into;
  const float LN = -dot(in, NN);
  const float sq = fmaxf(0.0f, 1.0f - eta * eta * (1.0f - LN * LN));
  return normalized(-NN * sqrtf(sq) - eta * (-in - LN * NN));
}

// RUtil::IsReflect (RayUtility.cpp:34-36)
__device__ __forceinline__ bool is_reflect(V3 in, V3 out, V3 n) { return dot(n, in) * dot(n, out) < 0.0f; }

// RUtil::GetMicrofacetNormal_FromRefraction (RayUtility.cpp:21-33)
__device__ __forceinline__ V3 microfacet_from_refraction(V3 in, V3 out, float from, float into) {
  const float c = fabsf(dot(in, out));
  const float eta = into / from;
  const float isq = eta * eta - 2.0f * eta * c + 1.0f;
  if (isq < kLt1e8) return v3(0.f, 0.f, 0.f);
  const float ss = 1.0f / sqrtf(isq);
  const V3 h = normalized(-eta * ss * out + ss * in);
  return into > from ? h : -h;
}

// Sampling::GGX_Sampling (Sampling.cpp:123-157)
__device__ __forceinline__ V3 ggx_sampling(Rng& rng, V3 normal, V3 in, float alpha, float* pdf) {
  const V3 e1 = normal;
  const float2 cs = __ldg(c_sincos_tab + rng.next_u24());
  const float e = rng.next();
  const float den = e * (alpha * alpha - 1.0f) + 1.0f;
  const float cth = ggx_cth(e, den);
  V3 e2, e3;
  frame(e1, e2, e3);
  const float cph = cs.x, sph = cs.y;
  const float sth = sqrtf(1.0f - cth * cth);
  const V3 mN = normalized(e3 * sth * cph + e2 * sth * sph + e1 * cth);
  if (dot(mN, in) > 0.0f) { *pdf = kSMin; return invalid_dir(); }
  const V3 result = reflect_sampling(mN, in);
  if (dot(result, normal) < 0.0f) { *pdf = kSMin; return invalid_dir(); }
  const float wm_N = dot(mN, normal);
  const float wo_wm = dot(result, mN);
  const float x = 1.0f - (1.0f - alpha * alpha) * wm_N * wm_N;
  *pdf = ggx_pdf(alpha * alpha, x, wm_N, 4.0f * wo_wm, kPI);
  return result;
}

// Sampling::GGX_Sampling_PDF (Sampling.cpp:158-180)
__device__ __forceinline__ float ggx_sampling_pdf(V3 out, V3 normal, V3 in, float a) {
  if (!is_reflect(in, out, normal)) return kSMin;
  const V3 h = normalized(-in + out);
  const float h_n = dot(h, normal);
  if (h_n < 0.0f) return kSMin;
  const float wi_h = -dot(in, h);
  if (wi_h < 0.0f) return kSMin;
  const float wo_h = dot(out, h);
  if (wo_h < 0.0f) return kSMin;
  const float jc = 1.0f / (4.0f * wo_h);
  return (a * a / kPI * pow_m2(1.0f - (1.0f - a * a) * h_n * h_n)) * h_n * jc;
}

// Sampling::GGXGlass_Sampling (Sampling.cpp:181-248)
__device__ __forceinline__ V3 ggxglass_sampling(Rng& rng, V3 normal, V3 in, float alpha, float ii, float io, float* pdf) {
  constexpr float kSmall = 1e-12f;
  const V3 NN = dot(in, normal) < 0.0f ? normal : -normal;
  *pdf = 1.0f;
  const V3 e1 = NN;
  const float2 cs = __ldg(c_sincos_tab + rng.next_u24());
  const float e = rng.next();
  const float cth = glass_cth(e, alpha * alpha);
  V3 e2, e3;
  frame(e1, e2, e3);
  const float cph = cs.x, sph = cs.y;
  const float sth = sqrtf(1.00000001f - cth * cth);
  const V3 mN = normalized(e3 * sth * cph + e2 * sth * sph + e1 * cth);
  const float wi_wm = -dot(in, mN);
  const float wm_N = dot(mN, NN);
  const float wi_N = -dot(in, NN);
  if (wi_N < kSmall) { *pdf = kSMin; return invalid_dir(); }
  if (wi_wm < kSmall) { *pdf = kSMin; return invalid_dir(); }
  if (wm_N < kSmall) { *pdf = kSMin; return invalid_dir(); }
  const float reflectance = fresnel_reflectance(mN, in, ii, io);
  const float y = 1.0f - (1.0f - alpha * alpha) * wm_N * wm_N;
  if (reflectance > rng.next()) {
    *pdf = reflectance;
    const V3 result = reflect_sampling(mN, in);
    const float wo_wm = dot(result, mN);
    if (wo_wm < kSmall) return invalid_dir();
    if (dot(result, NN) * dot(in, NN) > kSmall) { *pdf = kSMin; return invalid_dir(); }
    *pdf = reflectance * (wm_N / (4.0f * wo_wm) * alpha * alpha / (kPI * (y * y)));
    return result;
  }
  const V3 result = refract(in, mN, ii, io);
  const float wo_wm = -dot(result, mN);
  const float wo_N = -dot(result, NN);
  if (wi_N * wo_N < kSmall || wo_N < kSmall || wo_wm < kSmall) { *pdf = kSMin; return invalid_dir(); }
  const float A = (1.0f - reflectance) * wm_N;
  const float B = io * io * wo_wm;
  const float s = ii * wi_wm + io * wo_wm;
  *pdf = glass_pdf(A, B, s, alpha, kPI * (y * y));
  return result;
}

// Sampling::GGXGlass_Sampling_PDF (Sampling.cpp:249-288)
__device__ __forceinline__ float ggxglass_sampling_pdf(V3 out, V3 normal, V3 in, float a, float ii, float io) {
  if (is_reflect(in, out, normal)) {
    const V3 h = normalized(-in + out);
    const float h_n = dot(h, normal);
    if (h_n < 0.0f) return kSMin;
    const float wi_h = -dot(in, h);
    if (wi_h < 0.0f) return kSMin;
    const float wo_h = dot(out, h);
    if (wo_h < 0.0f) return kSMin;
    const float reflectance = fresnel_reflectance(h, in, ii, io);
    const float jc = 1.0f / (4.0f * wo_h);
    return reflectance * h_n * (a * a / kPI * pow_m2(1.0f - (1.0f - a * a) * h_n * h_n)) * jc;
  }
  const V3 h = microfacet_from_refraction(in, out, ii, io);
  const float h_n = dot(h, normal);
  if (h_n < 0.0f) return kSMin;
  const float wi_h = -dot(in, h);
  if (wi_h < 0.0f) return kSMin;
  const float wo_h = -dot(out, h);
  if (wo_h < 0.0f) return kSMin;
  const float reflectance = fresnel_reflectance(h, in, ii, io);
  const float jc = io * io * wo_h * pow_m2(ii * wi_h + io * wo_h);
  return (1.0f - reflectance) * h_n * (a * a / kPI * pow_m2(1.0f - (1.0f - a * a) * h_n * h_n)) * jc;
}

// Surface::OpeqeReflect (material.h:139-141)
__device__ __forceinline__ bool opaque_reflect(const FParam& p) {
  return dot(p.in, -p.n) > kGt1e4 && dot(p.out, p.n) > kGt1e4;
}

// Roughconductor::BRDF (material.h:227-274)
__device__ __forceinline__ float roughconductor_brdf(const FParam& p) {
  constexpr float kSmall = 1e-10f;
  if (dot(p.in, p.n) > -kSmall || dot(p.out, p.n) < kSmall) return 0.0f;
  const float k = p.absorb;
  const float eta = p.to / p.from;
  const float alpha = p.rough;
  const V3 h = normalized(-p.in + p.out);
  const float ccs = dot(h, p.n);
  if (ccs < kSmall || dot(h, p.in) > -kSmall || dot(h, p.out) < kSmall) return 0.0f;
  const float dd = 1.0001f - (1.0f - alpha * alpha) * ccs * ccs;
  const float D = fmaxf(kSMin, (alpha * alpha) / (kPI * (dd * dd)));
  const float lc = fmaxf(0.0f, fminf(0.9999f, dot(p.in, -p.n)));
  const float lv = fmaxf(0.0f, fminf(0.9999f, dot(p.out, p.n)));
  if (lc < kSMin || lv < kSMin) return 0.0f;
  const float L_l = conductor_lambda(alpha * alpha, 1.0f / (lc * lc));
  const float L_v = conductor_lambda(alpha * alpha, 1.0f / (lv * lv));
  const float G = 1.0f / ((1.0f + L_l) * (1.0f + L_v));
  const float fcos = dot(p.n, -p.in);
  const float temp = eta * eta - k * k - (1.0f - fcos * fcos);
  const float apb = sqrtf(temp * temp + k * k * eta * eta);
  const float a = sqrt_half(apb + temp);
  const float tm1 = apb + fcos * fcos;
  const float tm2 = a * 2.0f * fcos;
  const float rs2 = (tm1 - tm2) / (tm1 + tm2);
  const float tm3 = conductor_tm3(apb * fcos * fcos, 1.0f - fcos * fcos, fcos * fcos);
  const float tm4 = tm2 * (1.0f - fcos * fcos);
  const float rp2 = rs2 * (tm3 - tm4) / (tm3 + tm4);
  const float F = 0.5f * (rp2 + rs2);  // (float)(0.5 * (double)x) rounds 0.5 * x once, as this does
  const float fx = (4.0f * dot(p.in, -p.n) * dot(p.out, p.n));
  return (F * G * D) / fx;
}

// GGXGlass::EstimateN (material.h:297-309)
__device__ __forceinline__ V3 ggxglass_estimate_n(V3 in, V3 out, float I_i, float I_o) {
  const float c = fabsf(dot(in, out));
  const float eta = I_o / I_i;
  const float isq = eta * eta - 2.0f * eta * c + 1.0f;
  if (isq < kSMin) return v3(0.f, 0.f, 0.f);
  const float ss = 1.0f / sqrtf(isq);
  const V3 h = normalized(-eta * ss * out + ss * in);
  return I_o > I_i ? h : -h;
}

// GGXGlass::BRDF (material.h:314-390)
__device__ __forceinline__ float ggxglass_brdf(const FParam& p) {
  constexpr float kSmall = 1e-8f;
  const bool reflect = dot(p.n, p.in) * dot(p.n, p.out) < 0.0f;
  const float a = p.rough;
  const float Ii = p.from, Io = p.to;
  if (reflect) {
    const V3 h = normalized(-p.in + p.out);
    const float n_h = dot(p.n, h);
    if (n_h < 0.0f) return 0.0f;
    const float D = (a * a) * pow_m2(1.0f - (1.0f - a * a) * n_h * n_h) / kPI;
    const float L_l = (-1.0f + sqrtf(1.0001f + a * a * (pow_m2(dot(p.n, -p.in)) - 1.0f))) * 0.5f;
    const float L_v = (-1.0f + sqrtf(1.0001f + a * a * (pow_m2(dot(p.n, p.out)) - 1.0f))) * 0.5f;
    const float G = 1.0f / (L_l + L_v + 1.0f);
    const float F = fresnel_reflectance(h, p.in, Ii, Io);
    const float wo_n = fmaxf(0.0f, fminf(1.0f, dot(p.out, h)));
    const float wi_n = fmaxf(0.0f, fminf(1.0f, -dot(p.in, h)));
    if (wo_n < kSmall || wi_n < kSmall) return 0.0f;
    return F * G * D / (4.0f * wo_n * wi_n);
  }
  const float eta = Io / Ii;
  if (fabsf(eta - 1.0f) < kSmall) return 1.0f;
  if (dot(p.in, p.out) < 0.0f) return 0.0f;
  const V3 h = ggxglass_estimate_n(p.in, p.out, p.from, p.to);
  if (norm(h) < kSmall) return 0.0f;
  const float n_h = dot(h, p.n);
  if (n_h < kSmall) return 0.0f;
  const float D = (a * a) * pow_m2(1.0f - (1.0f - a * a) * n_h * n_h) / kPI;
  const float L_l = (-1.0f + sqrtf(1.0001f + a * a * (pow_m2(dot(p.n, -p.in)) - 1.0f))) * 0.5f;
  const float L_v = (-1.0f + sqrtf(1.0001f + a * a * (pow_m2(dot(p.n, -p.out)) - 1.0f))) * 0.5f;
  const float G = 1.0f / (L_l + L_v + 1.0f);
  const float F = fresnel_reflectance(h, p.in, Ii, Io);
  const float wi_wm = -dot(p.in, h);
  const float wo_wm = -dot(p.out, h);
  const float wi_n = -dot(p.in, p.n);
  const float wo_n = -dot(p.out, p.n);
  if (wo_wm < kSmall || wi_wm < kSmall) return 0.0f;
  if (wi_n < kSmall || wo_n < kSmall) return 0.0f;
  return (wi_wm * wo_wm) / (wi_n * wo_n) * (Io * Io) * (1.0f - F) * G * D * pow_m2(Ii * wo_wm + Io * wi_wm);
}

// ------------------------------------------- the demo's further surfaces
// BiMetalSurface, GlassSurface, GlossTransmitSurface, DiffuseTransmitSurface
// (material.h:427-531, 637-766).  Where the reference promotes to double (a
// double literal), the restatement computes in double: these surfaces are
// rare enough that FP64 costs nothing measurable, and IEEE double gives the
// reference's bits.

// The surface normal facing the incoming ray's side (material.h:429, 485, 698).
__device__ __forceinline__ V3 facing(V3 n, V3 in) { return dot(n, in) < 0.0f ? n : -n; }

// Sampling::Refract_Sampling (Sampling.cpp:329-337)
__device__ __forceinline__ V3 refract_sampling(V3 n, V3 in, float ii, float io) {
  const float eta = ii / io;
  const V3 NN = dot(in, n) > 0.0f ? -n : n;
  const float LN = -dot(in, NN);
  const float sq = fmaxf(0.00000001f, 1.0f - eta * eta * (1.0f - LN * LN));
  return normalized(-NN * sqrtf(sq) - eta * (-in - LN * NN));
}

// GlassSurface::Refract (material.h:470-477): as Refract_Sampling.
__device__ __forceinline__ V3 glass_refract(float from, float to, V3 in, V3 n) { return refract_sampling(n, in, from, to); }

// GlossTransmitSurface::ReflectByN (material.h:683-686)
__device__ __forceinline__ V3 reflect_by_n(V3 r, V3 n) { return r - 2.0f * dot(n, r) * n; }

// BiMetalSurface (material.h:427-463)
__device__ __forceinline__ float bimetal_brdf(const FParam& p) {
  const V3 N = facing(p.n, p.in);
  if (!opaque_reflect(p)) return 0.0f;
  const V3 ref = reflect_sampling(N, p.in);
  if (dot(ref, p.out) > 1.0f - 1.0f / kDeltaPDF) return metal_brdf(dot(p.out, N), kDeltaPDF);
  return 0.0f;
}
__device__ __forceinline__ float bimetal_pdf(const FParam& p) {
  const V3 ref = reflect_sampling(facing(p.n, p.in), p.in);
  return dot(ref, p.out) > 1.0f - 1.0f / kDeltaPDF ? kDeltaPDF : kSMin;
}

// GlassSurface (material.h:465-531)
__device__ __forceinline__ V3 glass_sampling(Rng& rng, const FParam& p, float* pdf) {
  const V3 NN = facing(p.n, p.in);
  const float reflectance = fresnel_reflectance(NN, p.in, p.from, p.to);
  if (reflectance > rng.next()) {
    *pdf = reflectance;
    return reflect_sampling(NN, p.in);
  }
  *pdf = 1.0f - reflectance;
  const float eta = p.from / p.to;
  const float LN = -dot(p.in, NN);
  const float sq = (float)(1.0f - (double)(eta * eta) * (1.0 - (double)(LN * LN)));
  if (sq < kLt1e6) return reflect_sampling(p.n, p.in);
  return glass_refract(p.from, p.to, p.in, p.n);
}
__device__ __forceinline__ float glass_brdf(const FParam& p) {
  const V3 NN = facing(p.n, p.in);
  const float reflectance = fresnel_reflectance(NN, p.in, p.from, p.to);
  const float w = is_reflect(p.in, p.out, p.n) ? kDeltaPDF * reflectance : kDeltaPDF * (1.0f - reflectance);
  return (float)((double)w / ((double)fabsf(dot(p.out, NN)) + 0.0001));
}
__device__ __forceinline__ float glass_pdf_delta(const FParam& p) {
  const V3 NN = facing(p.n, p.in);
  const float reflectance = fresnel_reflectance(NN, p.in, p.from, p.to);
  if (is_reflect(p.in, p.out, p.n)) {
    const V3 ref = reflect_sampling(NN, p.in);
    return fabsf(dot(ref, p.out)) > kGt0_99 ? kDeltaPDF * reflectance : kSMin;
  }
  const V3 rac = refract_sampling(NN, p.in, p.from, p.to);
  return fabsf(dot(rac, p.out)) > kGt0_99 ? kDeltaPDF * (1.0f - reflectance) : kSMin;
}

// DiffuseTransmitSurface (material.h:637-675)
__device__ __forceinline__ V3 diffuse_transmit_sampling(Rng& rng, const FParam& p, float* pdf) {
  const V3 n = dot(p.n, p.in) > 0.0f ? p.n : -p.n;
  if (p.refl > rng.next()) {
    const V3 rs = cos_sampling(rng, -n, pdf);
    *pdf *= p.refl;
    return rs;
  }
  const V3 rs = cos_sampling(rng, n, pdf);
  *pdf *= (1.0f - p.refl);
  return rs;
}
__device__ __forceinline__ float diffuse_transmit_brdf(const FParam& p) {
  return is_reflect(p.in, p.out, p.n) ? p.refl / kPI : (1.0f - p.refl) / kPI;
}
__device__ __forceinline__ float diffuse_transmit_pdf(const FParam& p) {
  const float c = (float)fabs((double)dot(p.out, p.n) + 0.00001);
  return is_reflect(p.in, p.out, p.n) ? p.refl * c / kPI : (1.0f - p.refl) * c / kPI;
}

// GlossTransmitSurface (material.h:677-766)
__device__ __forceinline__ V3 gloss_transmit_sampling(Rng& rng, const FParam& p, float* pdf) {
  const V3 n = facing(p.n, p.in);
  if (p.refl > rng.next()) {
    const V3 rs = ggx_sampling(rng, n, p.in, p.rough, pdf);
    *pdf *= p.refl;
    return rs;
  }
  const V3 rs = reflect_by_n(ggx_sampling(rng, n, p.in, p.rough, pdf), n);
  *pdf *= (1.0f - p.refl);
  return rs;
}
__device__ __forceinline__ float gloss_transmit_brdf(const FParam& p) {
  constexpr float kSmall = 1e-10f;
  const float power = is_reflect(p.in, p.out, p.n) ? p.refl : 1.0f - p.refl;
  const V3 in = p.in;
  const V3 N = facing(p.n, in);
  V3 out = p.out;
  if (dot(out, N) < 0.0f) out = reflect_by_n(out, N);
  if (dot(in, N) > -kSmall || dot(out, N) < kSmall) return 0.0f;
  const float alpha = p.rough;
  const V3 h = normalized(-in + out);
  const float ccs = dot(h, N);
  if (ccs < kSmall || dot(h, in) > -kSmall || dot(h, out) < kSmall) return 0.0f;
  const float dd = 1.0001f - (1.0f - alpha * alpha) * ccs * ccs;
  const float D = fmaxf(kSMin, (alpha * alpha) / (kPI * (dd * dd)));
  const float lc = fmaxf(0.0f, fminf(0.9999f, dot(in, -N)));
  const float lv = fmaxf(0.0f, fminf(0.9999f, dot(out, N)));
  if (lc < kSMin || lv < kSMin) return 0.0f;
  const float L_l = conductor_lambda(alpha * alpha, 1.0f / (lc * lc));
  const float L_v = conductor_lambda(alpha * alpha, 1.0f / (lv * lv));
  const float G = 1.0f / ((1.0f + L_l) * (1.0f + L_v));
  const float fx = (4.0f * dot(in, -N) * dot(out, N));
  return power * (G * D) / fx;
}
__device__ __forceinline__ float gloss_transmit_pdf(const FParam& p) {
  if (is_reflect(p.in, p.out, p.n)) return p.refl * ggx_sampling_pdf(p.out, p.n, p.in, p.rough);
  return (1.0f - p.refl) * ggx_sampling_pdf(reflect_by_n(p.out, p.n), p.n, p.in, p.rough);
}

// Virtual Surface dispatch (material.h:137-146) for the eight surfaces.
__device__ __forceinline__ V3 surface_sample(int type, Rng& rng, const FParam& p, float* pdf) {
  switch (type) {
    case kSurfDiffuse: return cos_sampling(rng, p.n, pdf);                                 // DiffuseSurface
    case kSurfMetal: *pdf = kDeltaPDF; return reflect_sampling(p.n, p.in);                 // MetalSurface
    case kSurfConductor: return ggx_sampling(rng, p.n, p.in, p.rough, pdf);                // Roughconductor
    case kSurfGGXGlass: return ggxglass_sampling(rng, p.n, p.in, p.rough, p.from, p.to, pdf);  // GGXGlass
    case kSurfBiMetal: *pdf = kDeltaPDF; return reflect_sampling(facing(p.n, p.in), p.in);
    case kSurfGlass: return glass_sampling(rng, p, pdf);
    case kSurfGlossTransmit: return gloss_transmit_sampling(rng, p, pdf);
    default: return diffuse_transmit_sampling(rng, p, pdf);                               // DiffuseTransmit
  }
}

__device__ __forceinline__ float surface_brdf(int type, const FParam& p) {
  switch (type) {
    case kSurfDiffuse: return opaque_reflect(p) ? 1.0f / kPI : 0.0f;
    case kSurfMetal: {
      if (!opaque_reflect(p)) return 0.0f;
      const V3 ref = reflect_sampling(p.n, p.in);
      if (dot(ref, p.out) > 1.0f - 1.0f / kDeltaPDF) return metal_brdf(dot(p.out, p.n), kDeltaPDF);
      return 0.0f;
    }
    case kSurfConductor: return roughconductor_brdf(p);
    case kSurfGGXGlass: return ggxglass_brdf(p);
    case kSurfBiMetal: return bimetal_brdf(p);
    case kSurfGlass: return glass_brdf(p);
    case kSurfGlossTransmit: return gloss_transmit_brdf(p);
    default: return diffuse_transmit_brdf(p);
  }
}

__device__ __forceinline__ float surface_pdf(int type, const FParam& p) {
  switch (type) {
    case kSurfDiffuse: return fmaxf(kSMin, dot(p.out, p.n) / kPI);
    case kSurfMetal: {
      const V3 ref = reflect_sampling(p.n, p.in);
      return dot(ref, p.out) > 1.0f - 1.0f / kDeltaPDF ? kDeltaPDF : kSMin;
    }
    case kSurfConductor: return ggx_sampling_pdf(p.out, p.n, p.in, p.rough);
    case kSurfGGXGlass: return ggxglass_sampling_pdf(p.out, p.n, p.in, p.rough, p.from, p.to);
    case kSurfBiMetal: return bimetal_pdf(p);
    case kSurfGlass: return glass_pdf_delta(p);
    case kSurfGlossTransmit: return gloss_transmit_pdf(p);
    default: return diffuse_transmit_pdf(p);
  }
}

// ---------------------------------------------------------------- textures
struct F4 { float x, y, z, w; };

__constant__ float c_byte_to_unit[256];  // b / 255.0f (TextureUtility.cpp:28)

__device__ __forceinline__ F4 texel(const TextureGPU& t, int idx) {
  const uint32_t v = __ldg(t.texels + idx);
  return F4{c_byte_to_unit[v & 255u], c_byte_to_unit[(v >> 8) & 255u], c_byte_to_unit[(v >> 16) & 255u],
            c_byte_to_unit[v >> 24]};
}
__device__ __forceinline__ F4 lerp4(F4 a, float wa, F4 b, float wb) {
  return F4{a.x * wa + b.x * wb, a.y * wa + b.y * wb, a.z * wa + b.z * wb, a.w * wa + b.w * wb};
}

// LinearSampler::Sample (TextureSampler.h:61-79) with its wrap rule.
__device__ __forceinline__ F4 tex_bilinear(const TextureGPU& t, float u, float v) {
  const int W = t.width, H = t.height;
  const int iu = (int)((float)W * u), iv = (int)((float)H * v);
  const int x1 = abs(iu) % W;
  const int y1 = abs(iv) % H;
  const int x2 = min(W - 1, x1 + 1), y2 = min(H - 1, y1 + 1);
  const F4 t00 = texel(t, x1 + y1 * W), t10 = texel(t, x2 + y1 * W);
  const F4 t01 = texel(t, x1 + y2 * W), t11 = texel(t, x2 + y2 * W);
  const float w = fabsf(u * (float)W) - (float)abs(iu);
  const float h = fabsf(v * (float)H) - (float)abs(iv);
  const F4 up = lerp4(t00, 1.0f - w, t10, w);
  const F4 down = lerp4(t01, 1.0f - w, t11, w);
  return lerp4(up, 1.0f - h, down, h);
}

}  // namespace fr
