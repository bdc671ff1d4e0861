// ORACLE — test infrastructure only.  Nothing in the product links, loads or
// calls this file; tests/, smoke() and bench.py's CPU baseline use it as the
// checker and the timed CPU reference.
//
// A CPU restatement (C++17 + OpenMP) of the reference's SPPM render loop,
// SPPM/SPPM/SPPM.cpp of tabochans/FriendsRender-R-public, with the Philox
// stream of the oracle overlay (oracle/ref/overlay/MT.h) in place of its
// mt19937.  Its results are pinned to the reference's own outputs by the
// golden fixtures (tests/golden/, made by running the reference).  Each
// function names the reference lines it restates.
//
// Differences from the reference, all documented there too:
//  * closest hit: the reference's BVH (bvh8.h) is replaced by a binary BVH;
//    of equal-t hits the larger facet index wins (the reference keeps the one
//    its traversal visits last, bvh8.h:591);
//  * the photon kd-tree (kdtree.h) is a median-split kd-tree; the query keeps
//    the reference's box test and sphere filter;
//  * camera sampler: three draws from the pixel's own stream.
#include <omp.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

namespace port {

// The arithmetic type of the restatement.  float (the default) is the
// reference's arithmetic, bit for bit; FR_PORT_REAL=double builds the FP64
// oracle: the same estimator with every float evaluated in double (the
// random draws, the reference's constants and the scene data are the same).
#ifndef FR_PORT_REAL
#define FR_PORT_REAL float
#endif
using Real = FR_PORT_REAL;

constexpr Real PI = 3.14159f;           // Vec.h:10
constexpr Real RAY_OFFSET = 1e-4f;      // Primitive.h:31
constexpr Real sMin = 1e-16f;           // Sampling.h:8
constexpr int NUM_SAMPLE = 1000;         // LightSampler.h:17
constexpr int SLOTS = 32;                // SPPM.cpp:753

// ------------------------------------------------------------------ Vec3
struct V {
  Real x = 0, y = 0, z = 0;
  V() = default;
  V(Real a, Real b, Real c) : x(a), y(b), z(c) {}
  Real operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
// Vec.h:179-243, 303-323
inline V operator+(V a, V b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V operator-(V a, V b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V operator*(V a, V b) { return V(a.x * b.x, a.y * b.y, a.z * b.z); }
inline V operator/(V a, V b) { return V(a.x / b.x, a.y / b.y, a.z / b.z); }
inline V operator-(V a) { return V(-a.x, -a.y, -a.z); }
inline V operator*(Real s, V a) { return V(s * a.x, s * a.y, s * a.z); }
inline V operator*(V a, Real s) { return V(s * a.x, s * a.y, s * a.z); }
inline V operator/(V a, Real s) { return V(a.x / s, a.y / s, a.z / s); }
inline Real dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V cross(V a, V b) { return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline Real norm2(V a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline Real norm(V a) { return std::sqrt(norm2(a)); }
inline V normalized(V a) {
  const Real d = norm(a);
  return V(a.x / d, a.y / d, a.z / d);
}
template <typename T>
inline V vp(const T* p) { return V(p[0], p[1], p[2]); }

// ------------------------------------------------------------------ RNG
// Philox4x32-10 (Salmon et al., SC'11) keyed by the reference's integer seed.
struct Rng {
  uint32_t key, key_hi, draw = 0, buf[4];
  // key_hi: the second key word of every stream (the overlay's 0x5350504D);
  // another value gives streams that share nothing with those.
  explicit Rng(uint32_t seed, uint32_t hi = 0x5350504Du) : key(seed), key_hi(hi) {}
  static void philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t o[4]) {
    for (int r = 0; r < 10; ++r) {
      if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
      const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
      const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
      c0 = n0; c1 = (uint32_t)p1; c2 = n2; c3 = (uint32_t)p0;
    }
    o[0] = c0; o[1] = c1; o[2] = c2; o[3] = c3;
  }
  uint32_t u24() {
    const uint32_t lane = draw & 3u;
    if (!lane) philox(draw >> 2, 0, 0, 0, key, key_hi, buf);
    ++draw;
    return buf[lane] >> 8;
  }
  // RandomMT::genrand64_real1/real2 (MT.h:30-37)
  double real() { return (double)((Real)u24() * (1.0f / 16777216.0f)); }
};

// ------------------------------------------------------------------ scene
struct Texture {
  int w = 0, h = 0;
  std::vector<Real> c;  // RGBA, value / 255.0f (TextureUtility.cpp:28)
};
struct Material {
  int type, sppm, opaque, tex_albedo, tex_rough, tex_bump;
  V albedo, radiance;
  Real index, roughness, extinction, reflectance;
};
struct Facet {
  V p[3], n[3];
  Real uv[3][2];
  int attr;
};
struct AliasBin { Real prob = 1.0f; int left = -1, right = -1; };
struct Table {  // TableSampler<T> (TableSampler.h:9-169)
  std::vector<AliasBin> bins;
  std::vector<Real> values;
  Real average = 0;
  int n = 0;
  // TableSampler::Init (TableSampler.h:44-120)
  void init(const std::vector<Real>& v) {
    n = (int)v.size();
    values = v;
    bins.assign(n, AliasBin());
    average = 0.0f;
    for (int i = 0; i < n; ++i) average += std::max<Real>(0.0f, v[i]);
    average /= n;
    std::vector<std::pair<Real, int>> bigger, smaller;
    for (int i = 0; i < n; ++i) {
      const Real x = std::max<Real>(0.0f, v[i]);
      if (x >= average) bigger.push_back({x / average, i});
      else smaller.push_back({x / average, i});
    }
    size_t s = 0, b = 0;
    for (int i = 0; i < n; ++i) {
      if (s < smaller.size()) {
        bins[i].left = smaller[s].second;
        bins[i].prob = smaller[s].first;
        ++s;
        if (b < bigger.size()) {
          bins[i].right = bigger[b].second;
          bigger[b].first -= (1.0f - bins[i].prob);
          if (bigger[b].first < 1.0f) smaller.push_back(bigger[b++]);
        } else if (smaller.size() == s) {
          bins[i].right = -1;
          bins[i].prob = 1.0f;
        } else {
          bins[i].right = smaller[s].second;
        }
      } else {
        bins[i].left = bigger[b].second;
        bins[i].prob = 1.0f;
        bigger[b].first -= 1.0f;
        if (bigger[b].first < 1.0f) smaller.push_back(bigger[b++]);
      }
    }
  }
  Real pdf(int i) const { return values[i] / average / (Real)n; }  // TableSampler.h:122-124
  // TableSampler::Sample (TableSampler.h:126-129)
  int sample(Rng& mt) const {
    const AliasBin& bin = bins[(size_t)((double)n * mt.real())];
    return mt.real() < bin.prob ? bin.left : bin.right;
  }
};
struct Light {
  Facet f;
  V flux;
  bool textured;
  Table table;
  std::vector<V> uvw, L;
};

struct Camera {
  int type, W, H;
  V pos, dir, e1, e2;
  Real fov, pw, ph, lw, lh, F, dist;
};

struct Ray {
  V o, d;
  Real index;
};

// --------------------------------------------------------------- texture
// LinearSampler::Sample (TextureSampler.h:61-79)
inline void tex_sample(const Texture& t, Real u, Real v, Real out[4]) {
  const int W = t.w, H = t.h;
  const int x1 = std::abs(int(W * u)) % W;
  const int y1 = std::abs(int(H * v)) % H;
  const Real* c00 = &t.c[4 * (size_t)(x1 + y1 * W)];
  const Real* c10 = &t.c[4 * (size_t)(std::min(W - 1, x1 + 1) + y1 * W)];
  const Real* c01 = &t.c[4 * (size_t)(x1 + std::min(H - 1, y1 + 1) * W)];
  const Real* c11 = &t.c[4 * (size_t)(std::min(W - 1, x1 + 1) + std::min(H - 1, y1 + 1) * W)];
  const Real w = (std::abs(u * W) - std::abs(int(W * u)));
  const Real h = (std::abs(v * H) - std::abs(int(H * v)));
  for (int k = 0; k < 4; ++k) {
    const Real up = c00[k] * (Real)(1.0 - w) + c10[k] * w;
    const Real down = c01[k] * (Real)(1.0 - w) + c11[k] * w;
    out[k] = up * (Real)(1.0 - h) + down * h;
  }
}

// ------------------------------------------------------------------- BVH
struct BNode { Real lo[3], hi[3]; int left, right, first, count; };
struct BVH {
  std::vector<BNode> nodes;
  std::vector<int> idx;
  void build(const std::vector<Facet>& F) {
    const int T = (int)F.size();
    idx.resize(T);
    std::vector<V> cen(T);
    for (int t = 0; t < T; ++t) {
      idx[t] = t;
      cen[t] = (F[t].p[0] + F[t].p[1] + F[t].p[2]) * (1.0f / 3.0f);
    }
    nodes.clear();
    nodes.reserve(2 * (size_t)T);
    rec(F, cen, 0, T);
  }
  int rec(const std::vector<Facet>& F, const std::vector<V>& cen, int first, int count) {
    BNode n;
    for (int a = 0; a < 3; ++a) { n.lo[a] = FLT_MAX; n.hi[a] = -FLT_MAX; }
    Real clo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, chi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int i = first; i < first + count; ++i) {
      const Facet& f = F[idx[i]];
      for (int k = 0; k < 3; ++k)
        for (int a = 0; a < 3; ++a) { n.lo[a] = std::min(n.lo[a], f.p[k][a]); n.hi[a] = std::max(n.hi[a], f.p[k][a]); }
      for (int a = 0; a < 3; ++a) { clo[a] = std::min(clo[a], cen[idx[i]][a]); chi[a] = std::max(chi[a], cen[idx[i]][a]); }
    }
    // Padded like the reference's triangle boxes (Intersect.cpp:572-573) so
    // culling is conservative.
    for (int a = 0; a < 3; ++a) { n.lo[a] -= 0.001f + std::fabs(n.lo[a]) * 1e-6f; n.hi[a] += 0.001f + std::fabs(n.hi[a]) * 1e-6f; }
    n.left = n.right = -1;
    n.first = first;
    n.count = count;
    const int id = (int)nodes.size();
    nodes.push_back(n);
    if (count <= 4) return id;
    int axis = 0;
    for (int a = 1; a < 3; ++a)
      if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
    const int mid = first + count / 2;
    std::nth_element(idx.begin() + first, idx.begin() + mid, idx.begin() + first + count,
                     [&](int a, int b) { return cen[a][axis] < cen[b][axis]; });
    const int l = rec(F, cen, first, mid - first);
    const int r = rec(F, cen, mid, first + count - mid);
    nodes[id].left = l;
    nodes[id].right = r;
    nodes[id].count = 0;
    return id;
  }
};

// Isc::Intersect(Ray, Triangle_ID) (Intersect.cpp:67-89)
inline bool intersect(const Ray& ray, const Facet& p, Real& t, Real& u, Real& v) {
  const V dd = ray.d;
  const V e1 = p.p[1] - p.p[0];
  const V e2 = p.p[2] - p.p[0];
  const V ps = cross(dd, e2);
  const Real a = dot(e1, ps);
  if (a > -FLT_MIN && a < FLT_MIN) return false;
  const Real f = 1.0f / a;
  const V s = ray.o - p.p[0];
  u = f * dot(s, ps);
  if (u < 0.0 || u > 1.0) return false;
  const V q = cross(s, e1);
  v = f * dot(dd, q);
  if (v < 0.0 || u + v > 1.0) return false;
  t = f * dot(e2, q);
  return true;
}

// Watertight ray-triangle test (Woop, Benthin and Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013), the precision mode's test:
// the same float and double operations, in the same order, as the GPU's
// intersect_watertight (csrc/fr_trace.cuh).  u, v are the weights of p[1]
// and p[2], as Moller-Trumbore's.
inline Real axis_of(const V& a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

inline bool intersect_watertight(const Ray& ray, const Facet& p, Real& t, Real& u, Real& v) {
  const V dir = ray.d;
  const Real adx = std::fabs(dir.x), ady = std::fabs(dir.y), adz = std::fabs(dir.z);
  const int kz = adx > ady ? (adx > adz ? 0 : 2) : (ady > adz ? 1 : 2);
  int kx = kz == 2 ? 0 : kz + 1;
  int ky = kx == 2 ? 0 : kx + 1;
  const Real dz = axis_of(dir, kz);
  if (dz < 0.0f) std::swap(kx, ky);
  const Real Sx = axis_of(dir, kx) / dz, Sy = axis_of(dir, ky) / dz, Sz = 1.0f / dz;
  const V A = p.p[0] - ray.o, B = p.p[1] - ray.o, C = p.p[2] - ray.o;
  const Real Az0 = axis_of(A, kz), Bz0 = axis_of(B, kz), Cz0 = axis_of(C, kz);
  const Real Ax = axis_of(A, kx) - Sx * Az0, Ay = axis_of(A, ky) - Sy * Az0;
  const Real Bx = axis_of(B, kx) - Sx * Bz0, By = axis_of(B, ky) - Sy * Bz0;
  const Real Cx = axis_of(C, kx) - Sx * Cz0, Cy = axis_of(C, ky) - Sy * Cz0;
  Real U = Cx * By - Cy * Bx, W2 = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
  if (U == 0.0f || W2 == 0.0f || W == 0.0f) {
    U = (Real)((double)Cx * (double)By - (double)Cy * (double)Bx);
    W2 = (Real)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (Real)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0.0f || W2 < 0.0f || W < 0.0f) && (U > 0.0f || W2 > 0.0f || W > 0.0f)) return false;
  const Real det = U + W2 + W;
  if (det == 0.0f) return false;
  const Real T = U * (Sz * Az0) + W2 * (Sz * Bz0) + W * (Sz * Cz0);
  const Real rcp = 1.0f / det;
  t = T * rcp;
  u = W2 * rcp;
  v = W * rcp;
  return true;
}

// The triangle test of a renderer's mode.
inline bool intersect(const Ray& ray, const Facet& p, Real& t, Real& u, Real& v, bool watertight) {
  return watertight ? intersect_watertight(ray, p, t, u, v) : intersect(ray, p, t, u, v);
}

inline bool box_hit(const BNode& n, const Ray& r, Real tmin, Real tmax) {
  Real t0 = tmin, t1 = tmax;
  for (int a = 0; a < 3; ++a) {
    const double inv = 1.0 / (double)r.d[a];
    double ta = ((double)n.lo[a] - r.o[a]) * inv, tb = ((double)n.hi[a] - r.o[a]) * inv;
    if (ta > tb) std::swap(ta, tb);
    if (std::isnan(ta) || std::isnan(tb)) continue;
    t0 = (Real)std::max((double)t0, ta);
    t1 = (Real)std::min((double)t1, tb);
  }
  return t0 <= t1;
}

struct Hit { Real t, u, v; int facet; };

// N_BVH8::findClosestElement semantics (bvh8.h:568-641): nearest t > MinT.
bool closest(const BVH& b, const std::vector<Facet>& F, const Ray& ray, Hit& h, bool wt = false) {
  Real best = FLT_MAX;
  int bf = -1;
  Real bu = 0, bv = 0;
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const BNode& n = b.nodes[stack[--sp]];
    if (!box_hit(n, ray, RAY_OFFSET, best)) continue;
    if (n.left < 0) {
      for (int i = n.first; i < n.first + n.count; ++i) {
        const int f = b.idx[i];
        Real t, u, v;
        if (intersect(ray, F[f], t, u, v, wt) && t > RAY_OFFSET && (t < best || (t == best && f > bf))) {
          best = t; bf = f; bu = u; bv = v;
        }
      }
    } else {
      stack[sp++] = n.right;
      stack[sp++] = n.left;
    }
  }
  if (bf < 0) return false;
  h = Hit{best, bu, bv, bf};
  return true;
}

// findAnyElement (bvh8.h:643-707)
bool any_hit(const BVH& b, const std::vector<Facet>& F, const Ray& ray, Real tmin, Real tmax, bool wt = false) {
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const BNode& n = b.nodes[stack[--sp]];
    if (!box_hit(n, ray, tmin, tmax)) continue;
    if (n.left < 0) {
      for (int i = n.first; i < n.first + n.count; ++i) {
        Real t, u, v;
        if (intersect(ray, F[b.idx[i]], t, u, v, wt) && tmax >= t && t > tmin) return true;
      }
    } else {
      stack[sp++] = n.right;
      stack[sp++] = n.left;
    }
  }
  return false;
}

// ------------------------------------------------------------- sampling
const V INVALID_DIR(1e-3, 1e-3, 1e-3);  // RayUtility.h:8
inline bool valid_dir(V d) { return norm2(d) > 0.9999f; }  // RayUtility.cpp:36-38

struct FP { V in, out, n; Real from, to, rough, absorb, refl; };  // material.h:12-34

inline void basis(V e1, V& e2, V& e3) {
  if (std::abs(e1.x) > 0.000001) e2 = normalized(cross(V(0, 1, 0), e1));
  else e2 = normalized(cross(V(1, 0, 0), e1));
  e3 = normalized(cross(e1, e2));
}

// Sampling::Cos_Sampling (Sampling.cpp:7-28)
V cos_sampling(Rng& mt, V normal, Real* pdf) {
  V e2, e3;
  const V e1 = normal;
  basis(e1, e2, e3);
  const Real ph = mt.real() * 2.0f * PI;
  const Real th = mt.real();
  const Real th2 = std::sqrt(th);
  V r = e1 * (Real)std::sqrt(1.000000001 - th) + e2 * (Real)std::cos((double)ph) * th2 +
        e3 * (Real)std::sin((double)ph) * th2;
  r = normalized(r);
  if (pdf) *pdf = std::max(sMin, dot(r, normal) / PI);
  return r;
}
// Sampling::Reflect_Sampling (Sampling.cpp:293-295)
V reflect(V n, V in) { return normalized(in - 2.0f * (dot(n, in)) * n); }
// Sampling::Fresnel_Reflectance (Sampling.cpp:297-313)
Real fresnel(V n, V in, Real ni, Real no) {
  const Real r12 = ni / no;
  const Real cosA = std::abs(dot(n, in));
  const Real sinA = std::sqrt(1.0000001f - cosA * cosA);
  const Real sinB = r12 * sinA;
  if (sinB > 0.999999) return 1.0f;
  const Real cosB = std::sqrt(1.0000001f - sinB * sinB);
  const Real rp = (no * cosA - ni * cosB) / (no * cosA + ni * cosB);
  const Real rs = (ni * cosA - no * cosB) / (ni * cosA + no * cosB);
  return (0.5f * rs * rs) + (0.5f * rp * rp);
}
// RUtil::Refract (RayUtility.cpp:10-17)
V refract(V in, V n, Real from, Real into) {
  const V NN = dot(in, n) < 0 ? n : -n;
  const Real eta = from / into;
  const Real LN = -dot(in, NN);
  const Real sq = std::max<Real>(0.0f, 1.0f - eta * eta * (1.0f - LN * LN));
  return normalized(-NN * std::sqrt(sq) - eta * (-in - LN * NN));
}
inline bool is_reflect(V in, V out, V n) { return dot(n, in) * dot(n, out) < 0.0f; }  // RayUtility.cpp:34-36
// RUtil::GetMicrofacetNormal_FromRefraction (RayUtility.cpp:21-33)
V mfn_refraction(V in, V out, Real from, Real into) {
  const Real c = std::abs(dot(in, out));
  const Real eta = into / from;
  const Real isq = eta * eta - 2.0f * eta * c + 1.0f;
  if (isq < 1e-8) return V(0, 0, 0);
  const Real ss = 1.0f / std::sqrt(isq);
  const V h = normalized(-eta * ss * out + ss * in);
  return into > from ? h : -h;
}
inline Real powm2(Real x) { return std::pow(x, -2.0f); }

// Sampling::GGX_Sampling (Sampling.cpp:123-157)
V ggx_sampling(Rng& mt, V normal, V in, Real alpha, Real* pdf) {
  const V e1 = normal;
  const Real phi = mt.real() * 2.0f * PI;
  const Real e = mt.real();
  const Real cth = (Real)std::sqrt((1.0 - e) / (e * (alpha * alpha - 1.0f) + 1.0f));
  V e2, e3;
  basis(e1, e2, e3);
  const Real cph = (Real)std::cos((double)phi), sph = (Real)std::sin((double)phi);
  const Real sth = std::sqrt(1.0f - cth * cth);
  const V mN = normalized(e3 * sth * cph + e2 * sth * sph + e1 * cth);
  if (dot(mN, in) > 0.0) { *pdf = sMin; return INVALID_DIR; }
  const V r = reflect(mN, in);
  if (dot(r, normal) < 0.0) { *pdf = sMin; return INVALID_DIR; }
  const Real wm_N = dot(mN, normal), wo_wm = dot(r, mN);
  const double x = 1.0f - (1.0f - alpha * alpha) * wm_N * wm_N;
  *pdf = (Real)((alpha * alpha) / (PI * (x * x)) * wm_N / (4.0f * wo_wm));
  return r;
}
// Sampling::GGX_Sampling_PDF (Sampling.cpp:158-180)
Real ggx_pdf(V out, V normal, V in, Real a) {
  if (!is_reflect(in, out, normal)) return sMin;
  const V h = normalized(-in + out);
  const Real h_n = dot(h, normal);
  if (h_n < 0.0f) return sMin;
  if (-dot(in, h) < 0.0f) return sMin;
  const Real wo_h = dot(out, h);
  if (wo_h < 0.0f) return sMin;
  const Real jc = 1.0f / (4.0f * wo_h);
  return (a * a / PI * powm2(1.0f - (1.0f - a * a) * h_n * h_n)) * h_n * jc;
}
// Sampling::GGXGlass_Sampling (Sampling.cpp:181-248)
V glass_sampling(Rng& mt, V normal, V in, Real alpha, Real Ii, Real Io, Real* pdf) {
  constexpr Real small = 1e-12f;
  const V NN = dot(in, normal) < 0 ? normal : -normal;
  *pdf = 1.0f;
  const V e1 = NN;
  const Real phi = mt.real() * 2.0f * PI;
  const Real e = mt.real();
  const Real cth = (Real)std::sqrt((1.0000001 - e) / (e * (alpha * alpha - 0.99999) + 1.0f));
  V e2, e3;
  basis(e1, e2, e3);
  const Real cph = (Real)std::cos((double)phi), sph = (Real)std::sin((double)phi);
  const Real sth = std::sqrt(1.00000001f - cth * cth);
  const V mN = normalized(e3 * sth * cph + e2 * sth * sph + e1 * cth);
  const Real wi_wm = -dot(in, mN), wm_N = dot(mN, NN), wi_N = -dot(in, NN);
  if (wi_N < small || wi_wm < small || wm_N < small) { *pdf = sMin; return INVALID_DIR; }
  const Real refl = fresnel(mN, in, Ii, Io);
  const Real y = 1.0f - (1.0f - alpha * alpha) * wm_N * wm_N;
  if (refl > mt.real()) {
    *pdf = refl;
    const V r = reflect(mN, in);
    const Real wo_wm = dot(r, mN);
    if (wo_wm < small) return INVALID_DIR;
    if (dot(r, NN) * dot(in, NN) > small) { *pdf = sMin; return INVALID_DIR; }
    *pdf = refl * (wm_N / (4.0f * wo_wm) * alpha * alpha / (PI * (y * y)));
    return r;
  }
  const V r = refract(in, mN, Ii, Io);
  const Real wo_wm = -dot(r, mN), wo_N = -dot(r, NN);
  if (wi_N * wo_N < small || wo_N < small || wo_wm < small) { *pdf = sMin; return INVALID_DIR; }
  const double s = Ii * wi_wm + Io * wo_wm;
  *pdf = (Real)((1.0f - refl) * wm_N * (Io * Io * wo_wm / (s * s)) * alpha * alpha / (PI * (y * y)));
  return r;
}
// Sampling::GGXGlass_Sampling_PDF (Sampling.cpp:249-288)
Real glass_pdf(V out, V normal, V in, Real a, Real Ii, Real Io) {
  if (is_reflect(in, out, normal)) {
    const V h = normalized(-in + out);
    const Real h_n = dot(h, normal);
    if (h_n < 0.0f) return sMin;
    if (-dot(in, h) < 0.0f) return sMin;
    const Real wo_h = dot(out, h);
    if (wo_h < 0.0f) return sMin;
    const Real refl = fresnel(h, in, Ii, Io);
    const Real jc = 1.0f / (4.0f * wo_h);
    return refl * h_n * (a * a / PI * powm2(1.0f - (1.0f - a * a) * h_n * h_n)) * jc;
  }
  const V h = mfn_refraction(in, out, Ii, Io);
  const Real h_n = dot(h, normal);
  if (h_n < 0.0f) return sMin;
  const Real wi_h = -dot(in, h);
  if (wi_h < 0.0f) return sMin;
  const Real wo_h = -dot(out, h);
  if (wo_h < 0.0f) return sMin;
  const Real refl = fresnel(h, in, Ii, Io);
  const Real jc = Io * Io * wo_h * powm2(Ii * wi_h + Io * wo_h);
  return (1.0f - refl) * h_n * (a * a / PI * powm2(1.0f - (1.0f - a * a) * h_n * h_n)) * jc;
}
inline bool opaque_reflect(const FP& p) { return dot(p.in, -p.n) > 1e-4 && dot(p.out, p.n) > 1e-4; }  // material.h:139-141

// Roughconductor::BRDF (material.h:227-274)
Real conductor_brdf(const FP& p) {
  constexpr Real small = 1e-10f;
  if (dot(p.in, p.n) > -small || dot(p.out, p.n) < small) return 0.0f;
  const Real k = p.absorb, eta = p.to / p.from, alpha = p.rough;
  const V h = normalized(-p.in + p.out);
  const Real ccs = dot(h, p.n);
  if (ccs < small || dot(h, p.in) > -small || dot(h, p.out) < small) return 0.0f;
  const Real dd = 1.0001f - (1.0f - alpha * alpha) * ccs * ccs;
  const Real D = std::max(sMin, (alpha * alpha) / (PI * (dd * dd)));
  const Real lc = std::max<Real>(0.0f, std::min<Real>(0.9999f, dot(p.in, -p.n)));
  const Real lv = std::max<Real>(0.0f, std::min<Real>(0.9999f, dot(p.out, p.n)));
  if (lc < sMin || lv < sMin) return 0.0f;
  const Real L_l = (-1.0f + std::sqrt(1.0f + alpha * alpha * (1.0f / (lc * lc) - 1.0))) * 0.5;
  const Real L_v = (-1.0f + std::sqrt(1.0f + alpha * alpha * (1.0f / (lv * lv) - 1.0))) * 0.5;
  const Real G = 1.0f / ((1.0f + L_l) * (1.0f + L_v));
  const Real fcos = dot(p.n, -p.in);
  const Real temp = eta * eta - k * k - (1.0f - fcos * fcos);
  const Real apb = std::sqrt(temp * temp + k * k * eta * eta);
  const Real a = std::sqrt((apb + temp) * 0.5);
  const Real tm1 = apb + fcos * fcos;
  const Real tm2 = a * 2.0f * fcos;
  const Real rs2 = (tm1 - tm2) / (tm1 + tm2);
  const Real tm3 = apb * fcos * fcos + (1.0f - fcos * fcos) * (1.0 - fcos * fcos);
  const Real tm4 = tm2 * (1.0f - fcos * fcos);
  const Real rp2 = rs2 * (tm3 - tm4) / (tm3 + tm4);
  const Real F = 0.5 * (rp2 + rs2);
  const Real fx = (4.0f * dot(p.in, -p.n) * dot(p.out, p.n));
  return (F * G * D) / fx;
}
// GGXGlass::EstimateN (material.h:297-309)
V estimate_n(V in, V out, Real Ii, Real Io) {
  const Real c = std::abs(dot(in, out));
  const Real eta = Io / Ii;
  const Real isq = eta * eta - 2.0f * eta * c + 1.0f;
  if (isq < sMin) return V(0, 0, 0);
  const Real ss = 1.0f / std::sqrt(isq);
  const V h = normalized(-eta * ss * out + ss * in);
  return Io > Ii ? h : -h;
}
// GGXGlass::BRDF (material.h:314-390)
Real glass_brdf(const FP& p) {
  constexpr Real small = 1e-8f;
  const bool refl = dot(p.n, p.in) * dot(p.n, p.out) < 0;
  const Real a = p.rough, Ii = p.from, Io = p.to;
  if (refl) {
    const V h = normalized(-p.in + p.out);
    const Real n_h = dot(p.n, h);
    if (n_h < 0) return 0.0f;
    const Real D = (a * a) * powm2(1.0f - (1.0f - a * a) * n_h * n_h) / PI;
    const Real L_l = (-1.0f + std::sqrt(1.0001f + a * a * (powm2(dot(p.n, -p.in)) - 1.0f))) * 0.5f;
    const Real L_v = (-1.0f + std::sqrt(1.0001f + a * a * (powm2(dot(p.n, p.out)) - 1.0f))) * 0.5f;
    const Real G = 1.0f / (L_l + L_v + 1.0f);
    const Real F = fresnel(h, p.in, Ii, Io);
    const Real wo_n = std::max<Real>(0.0f, std::min<Real>(1.0f, dot(p.out, h)));
    const Real wi_n = std::max<Real>(0.0f, std::min<Real>(1.0f, -dot(p.in, h)));
    if (wo_n < small || wi_n < small) return 0.0f;
    return F * G * D / (4.0f * wo_n * wi_n);
  }
  const Real eta = Io / Ii;
  if (std::abs(eta - 1.0f) < small) return 1.0;
  if (dot(p.in, p.out) < 0.0) return 0.0f;
  const V h = estimate_n(p.in, p.out, p.from, p.to);
  if (norm(h) < small) return 0.0f;
  const Real n_h = dot(h, p.n);
  if (n_h < small) return 0.0f;
  const Real D = (a * a) * powm2(1.0f - (1.0f - a * a) * n_h * n_h) / PI;
  const Real L_l = (-1.0f + std::sqrt(1.0001f + a * a * (powm2(dot(p.n, -p.in)) - 1.0f))) * 0.5f;
  const Real L_v = (-1.0f + std::sqrt(1.0001f + a * a * (powm2(dot(p.n, -p.out)) - 1.0f))) * 0.5f;
  const Real G = 1.0f / (L_l + L_v + 1.0f);
  const Real F = fresnel(h, p.in, Ii, Io);
  const Real wi_wm = -dot(p.in, h), wo_wm = -dot(p.out, h);
  const Real wi_n = -dot(p.in, p.n), wo_n = -dot(p.out, p.n);
  if (wo_wm < small || wi_wm < small) return 0.0f;
  if (wi_n < small || wo_n < small) return 0.0f;
  return (wi_wm * wo_wm) / (wi_n * wo_n) * (Io * Io) * (1.0f - F) * G * D * powm2(Ii * wo_wm + Io * wi_wm);
}

// ------------------------------------------- the demo's further surfaces
inline V facing(V n, V in) { return dot(n, in) < 0 ? n : -n; }
// Sampling::Refract_Sampling (Sampling.cpp:329-337)
V refract_sampling(V n, V in, Real ii, Real io) {
  const Real eta = ii / io;
  const V NN = (dot(in, n) > 0) ? -n : n;
  const Real LN = -dot(in, NN);
  const Real sq = std::max<Real>(0.00000001f, 1.0f - eta * eta * (1.0f - LN * LN));
  return normalized(-NN * std::sqrt(sq) - eta * (-in - LN * NN));
}
inline bool if_reflect(V n, V in, V out) { return dot(n, in) * dot(n, out) < 0.0f; }
inline V reflect_by_n(V r, V n) { return r - 2.0f * dot(n, r) * n; }  // material.h:683-686

// BiMetalSurface (material.h:427-463)
Real bimetal_brdf(const FP& p) {
  const V N = facing(p.n, p.in);
  if (!opaque_reflect(p)) return 0.0f;
  const V r = reflect(N, p.in);
  if (dot(r, p.out) > 1.0f - 1.0f / 1.0f) return 1.0f / (dot(p.out, N) + 0.00001);
  return 0.0f;
}
// GlassSurface (material.h:465-531); its Reflect is Reflect_Sampling's
// expression, its Refract Refract_Sampling's.
V glasssurf_sample(Rng& mt, const FP& p, Real* pdf) {
  const V NN = facing(p.n, p.in);
  const Real reflectance = fresnel(NN, p.in, p.from, p.to);
  if (reflectance > mt.real()) {
    *pdf = reflectance;
    return reflect(NN, p.in);
  }
  *pdf = 1.0f - reflectance;
  const Real eta = p.from / p.to;
  const Real LN = -dot(p.in, NN);
  const Real sq = 1.0f - eta * eta * (1.0 - LN * LN);
  if (sq < 0.000001) return reflect(p.n, p.in);
  return refract_sampling(p.n, p.in, p.from, p.to);
}
Real glasssurf_brdf(const FP& p) {
  const V NN = facing(p.n, p.in);
  const Real reflectance = fresnel(NN, p.in, p.from, p.to);
  if (if_reflect(p.n, p.in, p.out)) return 1.0f * reflectance / (std::abs(dot(p.out, NN)) + 0.0001);
  return 1.0f * (1.0f - reflectance) / (std::abs(dot(p.out, NN)) + 0.0001);
}
Real glasssurf_pdf(const FP& p) {
  const V NN = facing(p.n, p.in);
  const Real reflectance = fresnel(NN, p.in, p.from, p.to);
  if (if_reflect(p.n, p.in, p.out)) {
    const V r = reflect(NN, p.in);
    return std::abs(dot(r, p.out)) > 0.99 ? 1.0f * reflectance : sMin;
  }
  const V rac = refract_sampling(NN, p.in, p.from, p.to);
  return std::abs(dot(rac, p.out)) > 0.99 ? 1.0f * (1.0f - reflectance) : sMin;
}
// DiffuseTransmitSurface (material.h:637-675)
V difftrans_sample(Rng& mt, const FP& p, Real* pdf) {
  const V n = dot(p.n, p.in) > 0 ? p.n : -p.n;
  V rs;
  if (p.refl > mt.real()) {
    rs = cos_sampling(mt, -n, pdf);
    *pdf *= p.refl;
  } else {
    rs = cos_sampling(mt, n, pdf);
    *pdf *= (1.0f - p.refl);
  }
  return rs;
}
Real difftrans_brdf(const FP& p) { return if_reflect(p.n, p.in, p.out) ? p.refl / PI : (1.0f - p.refl) / PI; }
Real difftrans_pdf(const FP& p) {
  const Real c = std::abs(dot(p.out, p.n) + 0.00001);
  return if_reflect(p.n, p.in, p.out) ? p.refl * c / PI : (1.0f - p.refl) * c / PI;
}
// GlossTransmitSurface (material.h:677-766)
V glosstrans_sample(Rng& mt, const FP& p, Real* pdf) {
  const V n = facing(p.n, p.in);
  V rs;
  if (p.refl > mt.real()) {
    rs = ggx_sampling(mt, n, p.in, p.rough, pdf);
    *pdf *= p.refl;
  } else {
    rs = reflect_by_n(ggx_sampling(mt, n, p.in, p.rough, pdf), n);
    *pdf *= (1.0f - p.refl);
  }
  return rs;
}
Real glosstrans_brdf(const FP& p) {
  const Real power = if_reflect(p.n, p.in, p.out) ? p.refl : 1.0f - p.refl;
  const V in = p.in;
  const V N = facing(p.n, in);
  V out = p.out;
  if (dot(out, N) < 0) out = reflect_by_n(out, N);
  constexpr Real small = 1e-10;
  if (dot(in, N) > -small || dot(out, N) < small) return 0.0f;
  const Real alpha = p.rough;
  const V h = normalized(-in + out);
  const Real ccs = dot(h, N);
  if (ccs < small || dot(h, in) > -small || dot(h, out) < small) return 0.0f;
  const Real dd = 1.0001f - (1.0f - alpha * alpha) * ccs * ccs;
  const Real D = std::max(sMin, (alpha * alpha) / (PI * (dd * dd)));  // pow(x, 2.0f): folded to x * x
  const Real lc = std::max<Real>(0.0f, std::min<Real>(0.9999f, dot(in, -N)));
  const Real lv = std::max<Real>(0.0f, std::min<Real>(0.9999f, dot(out, N)));
  if (lc < sMin || lv < sMin) return 0.0f;
  const Real L_l = (-1.0f + std::sqrt(1.0f + alpha * alpha * (1.0f / (lc * lc) - 1.0))) * 0.5;
  const Real L_v = (-1.0f + std::sqrt(1.0f + alpha * alpha * (1.0f / (lv * lv) - 1.0))) * 0.5;
  const Real G = 1.0f / ((1.0f + L_l) * (1.0f + L_v));
  const Real fx = (4.0f * dot(in, -N) * dot(out, N));
  return power * (G * D) / fx;
}
Real glosstrans_pdf(const FP& p) {
  if (if_reflect(p.n, p.in, p.out)) return p.refl * ggx_pdf(p.out, p.n, p.in, p.rough);
  return (1.0f - p.refl) * ggx_pdf(reflect_by_n(p.out, p.n), p.n, p.in, p.rough);
}

// Surface virtual interface (material.h:137-146) over the eight surfaces.
V surf_sample(int type, Rng& mt, const FP& p, Real* pdf) {
  switch (type) {
    case 0: return cos_sampling(mt, p.n, pdf);                          // DiffuseSurface (material.h:165-167)
    case 1: *pdf = 1.0f; return reflect(p.n, p.in);                     // MetalSurface (material.h:398-403)
    case 2: return ggx_sampling(mt, p.n, p.in, p.rough, pdf);           // Roughconductor (material.h:224-226)
    case 3: return glass_sampling(mt, p.n, p.in, p.rough, p.from, p.to, pdf);  // GGXGlass (material.h:311-313)
    case 4: *pdf = 1.0f; return reflect(facing(p.n, p.in), p.in);       // BiMetalSurface (material.h:429-436)
    case 5: return glasssurf_sample(mt, p, pdf);
    case 6: return glosstrans_sample(mt, p, pdf);
    default: return difftrans_sample(mt, p, pdf);
  }
}
Real surf_brdf(int type, const FP& p) {
  switch (type) {
    case 0: return opaque_reflect(p) ? 1.0f / PI : 0.0f;  // material.h:168-173
    case 1: {                                             // material.h:404-415
      if (!opaque_reflect(p)) return 0.0f;
      const V r = reflect(p.n, p.in);
      if (dot(r, p.out) > 1.0f - 1.0f / 1.0f) return 1.0f / (dot(p.out, p.n) + 0.00001);
      return 0.0f;
    }
    case 2: return conductor_brdf(p);
    case 3: return glass_brdf(p);
    case 4: return bimetal_brdf(p);
    case 5: return glasssurf_brdf(p);
    case 6: return glosstrans_brdf(p);
    default: return difftrans_brdf(p);
  }
}
Real surf_pdf(int type, const FP& p) {
  switch (type) {
    case 0: return std::max(sMin, dot(p.out, p.n) / PI);  // material.h:174-176
    case 1: return dot(reflect(p.n, p.in), p.out) > 1.0f - 1.0f / 1.0f ? 1.0f : sMin;  // material.h:416-424
    case 2: return ggx_pdf(p.out, p.n, p.in, p.rough);
    case 3: return glass_pdf(p.out, p.n, p.in, p.rough, p.from, p.to);
    case 4: return dot(reflect(facing(p.n, p.in), p.in), p.out) > 1.0f - 1.0f / 1.0f ? 1.0f : sMin;  // material.h:452-462
    case 5: return glasssurf_pdf(p);
    case 6: return glosstrans_pdf(p);
    default: return difftrans_pdf(p);
  }
}

// ------------------------------------------------------------- renderer
struct Geometry {  // SPPM.h:56-68
  V pos, normal;
  Real uvx, uvy;
  const Material* m;
  V albedo, radiance;
  Real rough, translucency;
};
struct HitPoint {  // SPPM.h:83-110
  int type = 0;    // 0 NONE, 1 HIT, 2 ONLY_DIRECTLIGHT
  V pos, normal, out, weight;
  V dl;            // DirectLight: environment light at the path's end
  Real rough = 0;
  int facet = -1;
  const Material* m = nullptr;
};
struct Photon { V pos, flux, dir; Real index, pdf; bool valid = false; };  // SPPM.h:128-143
// SPPM.h:112-126; nf is N as a float (FR_FLAG_FLOAT_PHOTON_COUNT).
struct Shared { V rad; int n = 0; Real r = 0; int g = 0; V dl; int ndl = 0; float nf = 0.0f; };

struct KdNode { int photon, axis, left, right; };

struct Renderer {
  std::vector<Facet> F;
  std::vector<Material> mats;
  std::vector<Texture> texs;
  std::vector<Light> lights;
  Table light_table;
  Camera cam;
  BVH bvh;
  Texture ibl;            // environment map, converted as LightSampler.cpp:24 does
  bool has_ibl = false;
  int P = 0;
  Real alpha = 0.9f, r0 = 0.015f;
  bool fix_stale = false;
  bool watertight = false;  // FR_FLAG_WATERTIGHT: the watertight triangle test
  // FR_FLAG_END_DEGENERATE_PATHS: end a path whose sampled BSDF value or pdf
  // is NaN or whose pdf is zero, and a photon path whose flux or PDF product
  // is no longer finite.
  bool end_degenerate = false;
  bool float_count = false;  // FR_FLAG_FLOAT_PHOTON_COUNT
  uint32_t stream_key = 0x5350504Du;  // second Philox key word of every stream
  // Pixels the eye pass and the gather cover: [x0, x1) x [y0, y1); the rest
  // get no hitpoint (for oracle images of a window of the frame).
  int win_x0 = 0, win_y0 = 0, win_x1 = 1 << 30, win_y1 = 1 << 30;
  int step = 0;
  long long total_photons = 0;
  std::vector<Shared> sp;
  std::vector<HitPoint> hp;
  std::vector<Photon> slots;  // P x SLOTS
  std::vector<Photon> photons;
  std::vector<int> ph_path, ph_slot;
  std::vector<KdNode> kd;
  std::vector<int> gather_m;
  std::vector<V> gather_phi;
  // Closest-hit rays kept for measurement: every ray_stride-th traced ray (in
  // the order the threads reach the counter), up to ray_cap; 8 floats each:
  // origin, direction, index, pass (0 eye, 1 photon).
  mutable std::atomic<long long> ray_count{0};
  long long ray_stride = 0;
  size_t ray_cap = 0;
  mutable std::mutex ray_mu;
  mutable std::vector<Real> ray_sample;

  bool trace(const Ray& r, Hit& h, int pass) const {
    if (ray_stride > 0 && ray_count.fetch_add(1) % ray_stride == 0) {
      std::lock_guard<std::mutex> lock(ray_mu);
      if (ray_sample.size() < ray_cap * 8)
        ray_sample.insert(ray_sample.end(), {r.o.x, r.o.y, r.o.z, r.d.x, r.d.y, r.d.z, r.index, (Real)pass});
    }
    return closest(bvh, F, r, h, watertight);
  }

  // calculateGeometry (SPPM.cpp:36-77)
  void geometry(const Hit& h, Geometry& g) const {
    const Facet& f = F[h.facet];
    g.pos = h.u * (f.p[1] - f.p[0]) + h.v * (f.p[2] - f.p[0]) + f.p[0];
    g.normal = normalized(h.u * (f.n[1] - f.n[0]) + h.v * (f.n[2] - f.n[0]) + f.n[0]);
    g.uvx = h.u * (f.uv[1][0] - f.uv[0][0]) + h.v * (f.uv[2][0] - f.uv[0][0]) + f.uv[0][0];
    g.uvy = h.u * (f.uv[1][1] - f.uv[0][1]) + h.v * (f.uv[2][1] - f.uv[0][1]) + f.uv[0][1];
    const Material& m = mats[f.attr];
    g.m = &m;
    g.albedo = m.albedo;
    g.radiance = m.radiance;
    g.rough = m.roughness;
    g.translucency = 0.0f;
    if (norm2(g.radiance) > 1e-6) g.albedo = V(1, 1, 1);
    Real c[4];
    if (m.tex_rough >= 0) {
      tex_sample(texs[m.tex_rough], g.uvx, g.uvy, c);
      g.rough = std::min<Real>(0.8f, std::max<Real>(0.05f, 0.5f * c[0]));
    }
    if (m.tex_albedo >= 0) {
      tex_sample(texs[m.tex_albedo], g.uvx, g.uvy, c);
      g.albedo = V(c[0], c[1], c[2]);
      g.radiance = g.radiance * g.albedo;
      g.translucency = 1.0 - c[3];
    }
    if (m.tex_bump >= 0) {
      tex_sample(texs[m.tex_bump], g.uvx, g.uvy, c);  // GetNormalFromNormalmap (TextureUtility.cpp:161-164)
      V nm = normalized(V(2.0f * c[0] - 1.0f, 2.0f * c[1] - 1.0f, 2.0f * c[2] - 1.0f));
      nm = normalized(V(nm.x, nm.z, nm.y));
      const V e2 = g.normal;
      const V e1 = std::abs(e2.y) > 0.9 ? cross(e2, V(1, 0, 0)) : cross(e2, V(0, 1, 0));
      const V e3 = normalized(cross(e1, e2));
      // CreateMatrixFromColumns({e1, e2, e3}).inv() (Matrix.h:180-184, Matrix.cpp:22-34)
      const Real M[3][3] = {{e1.x, e2.x, e3.x}, {e1.y, e2.y, e3.y}, {e1.z, e2.z, e3.z}};
      Real C[3][3];
      for (int r = 0; r < 3; ++r)
        for (int col = 0; col < 3; ++col) {
          Real m2[2][2];
          for (int i = 0, rr = 0; i < 3; ++i) {
            if (i == r) continue;
            for (int j = 0, cc = 0; j < 3; ++j) {
              if (j == col) continue;
              m2[rr][cc++] = M[i][j];
            }
            ++rr;
          }
          C[r][col] = (m2[0][0] * m2[1][1] - m2[0][1] * m2[1][0]) * ((r + col) % 2 ? -1 : 1);
        }
      const Real det = M[0][0] * C[0][0] + M[1][0] * C[1][0] + M[2][0] * C[2][0];
      const Real ix = 1.0f / det;
      V rows[3];
      for (int i = 0; i < 3; ++i) rows[i] = V(ix * C[0][i], ix * C[1][i], ix * C[2][i]);
      g.normal = normalized(V(dot(rows[0], nm), dot(rows[1], nm), dot(rows[2], nm)));
    }
  }

  // Camera::SampleCameraRay (Camera.h:73-83 pinhole, 103-129 thin lens)
  Ray camera_ray(Real u, Real v, Rng& mt, Real& pdf) const {
    const Real s0 = mt.real(), s1 = mt.real(), s2 = mt.real();
    if (cam.type == 0) {
      const V off = V(s0, s1, s2) * V(cam.pw, cam.ph, 0) / V((Real)cam.W, (Real)cam.H, 1.0f);
      const V image = cam.pos - cam.dir * cam.dist + (u - 0.5f + off.x) * cam.e1 * cam.pw + (v - 0.5f + off.y) * cam.e2 * cam.ph;
      pdf = 1.0f;
      return Ray{image, normalized(normalized(cam.pos - image)), 1.0f};
    }
    const Real pdf_area = 1.0f / (cam.lw * cam.lh);
    const V lens = cam.pos + (s0 - 0.5f) * cam.e1 * cam.lw + (s1 - 0.5f) * cam.e2 * cam.lh;
    const V image = cam.pos - cam.dir * cam.dist + (u - 0.5f) * cam.e1 * cam.pw + (v - 0.5f) * cam.e2 * cam.ph;
    const Real A = cam.dist, B = (A * cam.F) / (A - cam.F);
    const V target = image + (cam.pos - image) * (A + B) / A;
    const Real cs = dot(cam.dir, normalized(lens - image));
    const Real d2 = norm2(lens - image);
    pdf = pdf_area * (d2 / cam.F / cam.F) / cs;
    return Ray{lens, normalized(normalized(target - lens)), 1.0f};
  }

  static bool near1(Real s) { return std::abs(s - 1.0f) < 0.00001; }  // SPPM.h:27-29

  // IBL::GetIBLColorFromDirection (IBL.h:122-129) with the SPHERE mapping of
  // GetUVFromDirection (IBL.h:96-104): acos of a float is the double ::acos.
  V ibl_color(V dir) const {
    Real u = 0.0f, v = 0.0f;
    if (!(std::abs(dir.x) < 1e-6 && std::abs(dir.z) < 1e-6)) {
      const V xz = normalized(V(dir.x, 0.0f, dir.z));
      const double ax = ::acos((double)xz.x);
      u = (Real)((xz.z >= 0 ? ax : (double)(2.0f * PI) - ax) / (double)(2.0f * PI));
      v = (Real)(::acos((double)dir.y) / (double)PI);
    }
    Real c[4];
    tex_sample(ibl, u, v, c);
    return V(c[0], c[1], c[2]);
  }

  // getHitpointInfo (SPPM.cpp:98-306); stops at the first hitpoint (nothing
  // after it reaches the image without an environment light).
  HitPoint eye(int i) const {
    const int W = cam.W, H = cam.H;
    Rng mt((uint32_t)i + (uint32_t)(W * H) * (uint32_t)step, stream_key);  // SPPM.cpp:334
    const int w = i % W, h = i / W;
    const Real u = w / (Real)W, v = h / (Real)H;
    Real cam_pdf = 1.0f;
    Ray cur = camera_ray(u, v, mt, cam_pdf), nxt = cur;
    Real PDF = 1.0f;
    V thr(1, 1, 1);
    int depth = 0;
    HitPoint hp;
    bool stored = false;  // isStoredPhoton
    while (true) {
      if (depth > 6) break;
      if (depth > 4) {
        const Real rus = std::exp(4 - depth);
        if (mt.real() > rus) break;
        PDF *= rus;
      }
      Hit hit;
      if (!trace(cur, hit, 0)) {
        // Sample IBL (SPPM.cpp:290-300)
        if (has_ibl) hp.dl = hp.dl + ibl_color(cur.d) * thr / PDF;
        if (hp.type == 0) hp.type = 2;
        break;
      }
      Geometry g;
      geometry(hit, g);
      g.normal = dot(g.normal, cur.d) > 0 ? -g.normal : g.normal;
      nxt.o = g.pos;
      if (g.translucency > 0.5f) {
        thr = thr * V(g.translucency, g.translucency, g.translucency);
        cur.o = g.pos + cur.d * RAY_OFFSET;
        continue;
      }
      if (g.m->sppm && !stored) {  // makeHitPoint (SPPM.cpp:79-96), once per path (SPPM.cpp:170-173)
        hp.type = 1;
        hp.pos = g.pos;
        hp.normal = g.normal;
        hp.out = -cur.d;
        hp.weight = (thr / PDF) / cam_pdf;
        hp.rough = g.rough;
        hp.facet = hit.facet;
        hp.m = g.m;
        hp.dl = V(0, 0, 0);
        stored = true;
        // The path goes on only for the environment light: without one,
        // nothing after the hitpoint reaches the image.
        if (!has_ibl) return hp;
      }
      Real Ii, Io;
      if (near1(cur.index)) { Ii = 1.0f; Io = g.m->index; }
      else { Ii = cur.index; Io = 1.0f; }
      FP p{cur.d, nxt.d, g.normal, Ii, Io, g.rough, g.m->extinction, g.m->reflectance};
      Real pdf = 1.0f;
      nxt.d = surf_sample(g.m->type, mt, p, &pdf);
      if (!valid_dir(nxt.d)) break;
      if (g.m->opaque) {
        if (dot(nxt.d, g.normal) < 1e-6) break;
      } else {
        nxt.index = dot(nxt.d, g.normal) < 0.0f ? Io : cur.index;
      }
      p.out = nxt.d;
      pdf = surf_pdf(g.m->type, p);
      const V on = dot(g.normal, nxt.d) > 0 ? g.normal : -g.normal;
      nxt.o = nxt.o + on * RAY_OFFSET;
      const Real brdf = surf_brdf(g.m->type, p);
      const Real cs = std::max<Real>(0.0f, std::min<Real>(1.0f, dot(nxt.d, on)));
      if (brdf < 1e-8) break;
      if (pdf < 0) break;
      if (end_degenerate && !(brdf >= 1e-8 && pdf > 0)) break;
      thr = thr * (g.albedo * cs * brdf);
      PDF *= pdf;
      cur = nxt;
      ++depth;
    }
    hp.dl = hp.dl / cam_pdf;  // createHitpoints (SPPM.cpp:345)
    return hp;
  }

  // createPhotonMap body for path i (SPPM.cpp:508-673)
  void photon_path(int i) {
    Rng mt((uint32_t)i + 135u + (uint32_t)step * (uint32_t)P, stream_key);  // SPPM.cpp:520
    Photon* arr = &slots[(size_t)i * SLOTS];
    // generateLightRay (SPPM.cpp:453-471)
    const Light& L = lights[light_table.sample(mt)];
    V pos, rad;
    Real pdf_area;
    const Real area = 0.5f * norm(cross(L.f.p[1] - L.f.p[0], L.f.p[2] - L.f.p[0]));
    if (L.textured) {  // SamplePointOnAreaLight (LightSampler.cpp:68-75)
      const int e = L.table.sample(mt);
      const V w = L.uvw[e];
      pos = w.x * L.f.p[0] + w.y * L.f.p[1] + (1.0f - w.x - w.y) * L.f.p[2];
      rad = L.L[e];
      pdf_area = (L.table.pdf(e) * NUM_SAMPLE) / area;
    } else {  // PointOnTriangle (Sampling.cpp:339-349), LightSampler.cpp:76-79
      Real u = mt.real(), v = mt.real();
      if (v > u) { u *= 0.5f; v -= u; }
      else { v *= 0.5f; u -= v; }
      pdf_area = 2.0f / std::abs(norm(cross(L.f.p[1] - L.f.p[0], L.f.p[2] - L.f.p[0])));
      pos = u * L.f.p[0] + v * L.f.p[1] + (1.0f - u - v) * L.f.p[2];
      rad = L.flux / (2.0f * PI * area);
    }
    pdf_area *= light_table.pdf((int)(&L - &lights[0]));
    const V ln = normalized(L.f.n[0] + L.f.n[1] + L.f.n[2]);
    Real pdf_dir = 1.0f;
    const V od = cos_sampling(mt, ln, &pdf_dir);
    rad = rad * std::min<Real>(1.0f, std::max<Real>(0.0f, dot(ln, od)));
    Ray cur{pos + ln * RAY_OFFSET, normalized(od), 1.0f}, nxt = cur;
    const V flux = rad;
    Real PDF = pdf_area * pdf_dir;
    V thr(1, 1, 1);
    arr[0] = Photon{cur.o, flux * thr * PI, cur.d, cur.index, PDF, true};
    int k = 0, loop = 0, depth = 0;
    while (true) {
      if (loop++ > 32 || k >= 32 - 1) break;
      if (thr.x < 1e-8 || thr.y < 1e-8 || thr.z < 1e-8) break;
      Hit hit;
      if (!trace(cur, hit, 1)) break;
      Geometry g;
      geometry(hit, g);
      g.normal = dot(g.normal, cur.d) > 0 ? -g.normal : g.normal;
      nxt.o = g.pos;
      if (norm2(g.radiance) > 0.00001) break;
      if (g.translucency > 0.5f) {
        thr = thr * V(g.translucency, g.translucency, g.translucency);
        cur.o = g.pos + cur.d * RAY_OFFSET;
        continue;
      }
      // russianRulette_PhotonMapping (SPPM.h:33-52)
      if (depth > 16) break;
      const V a = g.albedo;
      const Real pdf_rus = 0.98f * (a.x > a.y ? (a.x > a.z ? a.x : a.z) : (a.y > a.z ? a.y : a.z));
      if (mt.real() > pdf_rus) break;
      PDF *= pdf_rus;
      Real Ii, Io;
      if (near1(cur.index)) { Ii = 1.0f; Io = g.m->index; }
      else { Ii = cur.index; Io = 1.0f; }
      FP p{cur.d, nxt.d, g.normal, Ii, Io, g.rough, g.m->extinction, g.m->reflectance};
      if (g.m->sppm) arr[k++] = Photon{g.pos, flux * thr * g.albedo, cur.d, cur.index, PDF, true};
      Real pdf = 1.0f;
      nxt.d = surf_sample(g.m->type, mt, p, &pdf);
      if (!valid_dir(nxt.d)) break;
      if (g.m->opaque) {
        if (dot(nxt.d, g.normal) < 1e-6) break;
      } else {
        nxt.index = is_reflect(cur.d, nxt.d, g.normal) ? cur.index : Io;
      }
      p.out = nxt.d;
      pdf = surf_pdf(g.m->type, p);
      const V on = dot(g.normal, nxt.d) > 0 ? g.normal : -g.normal;
      nxt.o = nxt.o + on * RAY_OFFSET;
      const Real brdf = surf_brdf(g.m->type, p);
      const Real cs = std::max<Real>(0.0f, std::min<Real>(1.0f, dot(nxt.d, on)));
      if (brdf < 1e-8) break;
      if (pdf < 0) break;
      if (end_degenerate && !(brdf >= 1e-8 && pdf > 0)) break;
      thr = thr * (g.albedo * cs * brdf);
      PDF *= pdf;
      if (end_degenerate) {
        const V f = flux * thr;
        if (!(std::isfinite(PDF) && std::isfinite(f.x) && std::isfinite(f.y) && std::isfinite(f.z))) break;
      }
      cur = nxt;
      ++depth;
    }
    // SPPM.cpp:672 (terminator one past the last stored photon).
    const int term = fix_stale ? std::max(k, 1) : k + 1;
    if (term < SLOTS) arr[term].valid = false;
  }

  // Median-split kd-tree over photons (replaces kdtree.h:348-431).
  int kd_build(std::vector<int>& ids, int lo, int hi) {
    if (lo >= hi) return -1;
    Real mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int i = lo; i < hi; ++i)
      for (int a = 0; a < 3; ++a) {
        mn[a] = std::min(mn[a], photons[ids[i]].pos[a]);
        mx[a] = std::max(mx[a], photons[ids[i]].pos[a]);
      }
    int axis = 0;
    for (int a = 1; a < 3; ++a)
      if (mx[a] - mn[a] > mx[axis] - mn[axis]) axis = a;
    const int mid = (lo + hi) / 2;
    std::nth_element(ids.begin() + lo, ids.begin() + mid, ids.begin() + hi,
                     [&](int a, int b) { return photons[a].pos[axis] < photons[b].pos[axis]; });
    const int node = (int)kd.size();
    kd.push_back(KdNode{ids[mid], axis, -1, -1});
    const int l = kd_build(ids, lo, mid);
    const int r = kd_build(ids, mid + 1, hi);
    kd[node].left = l;
    kd[node].right = r;
    return node;
  }

  // GetElementsInsideBox (kdtree.h:457-482) then the sphere filter
  // (SPPM.cpp:432); left subtree holds coordinates <= the split.
  template <typename Fn>
  void query(int node, V bmin, V bmax, V x, Real R2, Fn&& fn) const {
    if (node < 0) return;
    const KdNode& n = kd[node];
    const Photon& p = photons[n.photon];
    bool in = true;
    for (int a = 0; a < 3; ++a)
      if (bmin[a] > p.pos[a] || bmax[a] < p.pos[a]) in = false;  // isIncludePoint (kdtree.h:78-88)
    if (in && norm2(p.pos - x) < R2) fn(n.photon);
    if (bmin[n.axis] <= p.pos[n.axis]) query(n.left, bmin, bmax, x, R2, fn);
    if (bmax[n.axis] >= p.pos[n.axis]) query(n.right, bmin, bmax, x, R2, fn);
  }

  void iterate() {
    ++step;
    const int npix = cam.W * cam.H;
    // Photon pass (SPPM.cpp:771-774, 798): slot 0 reset, then every path.
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < P; ++i) {
      slots[(size_t)i * SLOTS].valid = false;
      photon_path(i);
    }
    // Compaction up to the first invalid slot (SPPM.cpp:812-822).
    photons.clear(); ph_path.clear(); ph_slot.clear();
    for (int i = 0; i < P; ++i)
      for (int k = 0; k < SLOTS; ++k) {
        const Photon& p = slots[(size_t)i * SLOTS + k];
        if (!p.valid) break;
        photons.push_back(p); ph_path.push_back(i); ph_slot.push_back(k);
      }
    kd.clear();
    std::vector<int> ids(photons.size());
    for (size_t i = 0; i < ids.size(); ++i) ids[i] = (int)i;
    kd.reserve(ids.size());
    kd_build(ids, 0, (int)ids.size());
    // Eye pass (SPPM.cpp:776-779, 836).
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < npix; ++i) {
      const int x = i % cam.W, y = i / cam.W;
      hp[i] = (x >= win_x0 && x < win_x1 && y >= win_y0 && y < win_y1) ? eye(i) : HitPoint();
    }
    // Gather and update (applyHitPointInfo, SPPM.cpp:395-451).
#pragma omp parallel for schedule(dynamic, 64)
    for (int v = 0; v < npix; ++v) {
      const HitPoint& h = hp[v];
      gather_m[v] = 0;
      gather_phi[v] = V(0, 0, 0);
      if (h.type == 0) continue;
      Shared& s = sp[v];
      if (norm2(h.dl) > 1e-8) {  // SPPM.cpp:411-414
        s.dl = s.dl + h.dl;
        s.ndl++;
      }
      if (h.type != 1) continue;
      const V bmin = h.pos - s.r * V(1, 1, 1), bmax = h.pos + s.r * V(1, 1, 1);
      V add(0, 0, 0);
      int m = 0;
      query(kd.empty() ? -1 : 0, bmin, bmax, h.pos, s.r * s.r, [&](int j) {
        const Photon& p = photons[j];
        const Real Ii = p.index;
        const Real Io = near1(p.index) ? h.m->index : 1.0f;
        const V nn = dot(p.dir, h.normal) < 0 ? h.normal : -h.normal;
        const FP fp{p.dir, h.out, nn, Ii, Io, h.rough, h.m->extinction, h.m->reflectance};
        add = add + h.weight * surf_brdf(h.m->type, fp) * p.flux / p.pdf;
        ++m;
      });
      gather_m[v] = m;
      gather_phi[v] = add;
      if (m > 0) {
        if (float_count) {  // N as a float: nothing truncated
          const Real a = s.nf + alpha * m, b = s.nf + (Real)m;
          s.rad = (s.rad + add) * a / b;
          s.r *= std::sqrt(a / b);
          s.nf = (float)(s.nf + m * alpha);
        } else {
          const Real a = s.n + alpha * m, b = (Real)(s.n + m);
          s.rad = (s.rad + add) * a / b;
          s.r *= std::sqrt(a / b);
          s.n += m * alpha;
        }
        s.g++;
      }
    }
    total_photons += P;
  }

  // reconstructImageFromSharedPoints (SPPM.cpp:473-493)
  void resolve(Real* out) const {
    const int npix = cam.W * cam.H;
    for (int i = 0; i < npix; ++i) {
      const Shared& s = sp[i];
      const Real d = ((Real)total_photons * (s.g + 0.0001f) / (0.0001f + (Real)step)) * PI * s.r * s.r;
      const V L = s.dl / (Real)(s.ndl + 0.0001f) + s.rad / d;
      out[4 * i] = std::pow(L.x, 1.0f / 1.2f);
      out[4 * i + 1] = std::pow(L.y, 1.0f / 1.2f);
      out[4 * i + 2] = std::pow(L.z, 1.0f / 1.2f);
      out[4 * i + 3] = 1.0f;
    }
  }
};

// QRandSequence::HaltonCore (QRandSequence.h:10-25)
Real halton(int n, int B) {
  Real result = 0.0f;
  if (n <= 0) return result;
  const int keta = std::log2(n) / std::log2(B) + 1;
  for (int i = 0; i < keta; ++i) {
    result += (n % B) * std::pow(B, -(i + 1));
    n /= B;
  }
  return result;
}

}  // namespace port

using namespace port;

extern "C" {

// Material and camera parameters stay float in every build (the scene's own
// values); arrays and scalars of the calls below are Real.
struct port_material {
  int32_t type, sppm, opaque, tex_albedo, tex_rough, tex_bump;
  float albedo[3], emission[3], index, roughness, extinction, reflectance;
};
struct port_camera {
  int32_t type, width, height;
  float pos[3], target[3], fov, focal, dist, aspect, lens;
};

void* port_create(int32_t T, const Real* pos, const Real* nrm, const Real* uv, const int32_t* mat, int32_t nm,
                  const port_material* mats, int32_t nt, const int32_t* tex_wh, const uint8_t* const* texels,
                  const port_camera* c, int32_t photons, Real alpha, Real r0, int32_t fix_stale) {
  Renderer* r = new Renderer();
  r->F.resize(T);
  for (int t = 0; t < T; ++t) {
    Facet& f = r->F[t];
    for (int k = 0; k < 3; ++k) {
      f.p[k] = vp(pos + 9 * (size_t)t + 3 * k);
      f.n[k] = vp(nrm + 9 * (size_t)t + 3 * k);
      f.uv[k][0] = uv[6 * (size_t)t + 2 * k];
      f.uv[k][1] = uv[6 * (size_t)t + 2 * k + 1];
    }
    f.attr = mat[t];
  }
  for (int m = 0; m < nm; ++m) {
    const port_material& d = mats[m];
    r->mats.push_back(Material{d.type, d.sppm, d.opaque, d.tex_albedo, d.tex_rough, d.tex_bump, vp(d.albedo),
                               vp(d.emission), d.index, d.roughness, d.extinction, d.reflectance});
  }
  for (int t = 0; t < nt; ++t) {
    Texture tx;
    tx.w = tex_wh[2 * t];
    tx.h = tex_wh[2 * t + 1];
    tx.c.resize(4 * (size_t)tx.w * tx.h);
    for (size_t i = 0; i < tx.c.size(); ++i) tx.c[i] = texels[t][i] / 255.0f;
    r->texs.push_back(std::move(tx));
  }
  // Scene::CreateScene lights (Scene.cpp:145-154), LightSampler (LightSampler.cpp:6-66).
  std::vector<Real> fl;
  for (int t = 0; t < T; ++t) {
    const Material& m = r->mats[r->F[t].attr];
    if (!(m.radiance.x + m.radiance.y + m.radiance.z > 0.00001f)) continue;
    Light L;
    L.f = r->F[t];
    const Facet& f = L.f;
    const Real area = 0.5f * norm(cross(f.p[1] - f.p[0], f.p[2] - f.p[0]));
    if (m.tex_albedo >= 0) {
      L.textured = true;
      V total(0, 0, 0);
      std::vector<Real> vals;
      for (int i = 0; i < NUM_SAMPLE; ++i) {
        V w(i / (Real)NUM_SAMPLE, halton(i, 2), halton(i, 3));
        if (w.y > w.x) { w.x *= 0.5f; w.y -= w.x; }
        else { w.y *= 0.5f; w.x -= w.y; }
        const Real u = w.x * f.uv[0][0] + w.y * f.uv[1][0] + (1.0f - w.x - w.y) * f.uv[2][0];
        const Real v = w.x * f.uv[0][1] + w.y * f.uv[1][1] + (1.0f - w.x - w.y) * f.uv[2][1];
        Real c4[4];
        tex_sample(r->texs[m.tex_albedo], u, v, c4);
        V l = V(c4[0], c4[1], c4[2]) * m.radiance;
        if (norm2(l) < 0.01f) l = V(0, 0, 0);
        L.uvw.push_back(w);
        L.L.push_back(l);
        total = total + l;
      }
      if (norm2(total) < 1e-6) {
        L.L[0] = 1e-6 * V(1, 1, 1);
        L.uvw[0] = V(0, 0, 0);
      } else {
        total = total * (2.0f * PI * area / (Real)NUM_SAMPLE);
      }
      for (int i = 0; i < NUM_SAMPLE; ++i) vals.push_back(norm(L.L[i]));
      L.table.init(vals);
      L.flux = total;
    } else {
      L.textured = false;
      L.flux = m.radiance * 2.0f * PI * area;
    }
    fl.push_back(norm(L.flux));
    r->lights.push_back(std::move(L));
  }
  if (r->lights.empty()) { delete r; return nullptr; }
  r->light_table.init(fl);
  // iCamera constructor (Camera.h:132-151)
  Camera& cam = r->cam;
  cam.type = c->type;
  cam.W = c->width;
  cam.H = c->height;
  cam.pos = vp(c->pos);
  cam.dir = normalized(vp(c->target) - cam.pos);
  cam.fov = PI * c->fov / 360.0f;
  cam.pw = 2.0 * c->dist * std::tan((double)cam.fov) * c->aspect;
  cam.ph = 2.0 * c->dist * std::tan((double)cam.fov);
  cam.lw = c->lens > 0 ? c->lens : cam.pw;
  cam.lh = c->lens > 0 ? c->lens : cam.ph;
  cam.F = c->focal;
  cam.dist = c->dist;
  if (cam.dir.y > 0.99) { cam.e1 = V(1, 0, 0); cam.e2 = V(0, 0, 1); }
  else { cam.e1 = normalized(cross(V(0, 1, 0), cam.dir)); cam.e2 = normalized(cross(cam.dir, cam.e1)); }
  r->bvh.build(r->F);
  r->P = photons;
  r->alpha = alpha;
  r->r0 = r0;
  r->fix_stale = fix_stale != 0;
  const int npix = cam.W * cam.H;
  r->sp.assign(npix, Shared());
  for (auto& s : r->sp) s.r = r0;  // initializeSharedPoints (SPPM.cpp:356-373)
  r->hp.assign(npix, HitPoint());
  r->slots.assign((size_t)photons * SLOTS, Photon());
  r->gather_m.assign(npix, 0);
  r->gather_phi.assign(npix, V());
  return r;
}

void port_destroy(void* h) { delete static_cast<Renderer*>(h); }

void port_set_threads(int32_t n) { omp_set_num_threads(n > 0 ? n : omp_get_num_procs()); }
int32_t port_max_threads(void) { return omp_get_max_threads(); }

void port_iterate(void* h, int32_t n) {
  Renderer* r = static_cast<Renderer*>(h);
  for (int k = 0; k < n; ++k) r->iterate();
}

// The next iteration runs step first_step + 1 (its seeds, SPPM.cpp:334,520);
// for checking one step's eye pass without running the steps before it.  The
// resolve then counts the skipped steps as iterations.
// Starts (stride > 0) or stops keeping every stride-th closest-hit ray, up
// to cap rays; clears the kept ones.
void port_sample_rays(void* h, int64_t stride, int64_t cap) {
  Renderer* r = static_cast<Renderer*>(h);
  r->ray_stride = stride;
  r->ray_cap = (size_t)std::max<int64_t>(0, cap);
  r->ray_count = 0;
  r->ray_sample.clear();
}
// Copies the kept rays (8 floats each) to out when out is not NULL; returns their count.
int64_t port_read_ray_sample(void* h, Real* out) {
  Renderer* r = static_cast<Renderer*>(h);
  if (out) std::memcpy(out, r->ray_sample.data(), r->ray_sample.size() * sizeof(Real));
  return (int64_t)(r->ray_sample.size() / 8);
}

void port_seek(void* h, int32_t first_step) { static_cast<Renderer*>(h)->step = first_step; }

// The precision mode's watertight triangle test (FR_FLAG_WATERTIGHT) on or off.
void port_set_watertight(void* h, int32_t on) { static_cast<Renderer*>(h)->watertight = on != 0; }

// FR_FLAG_FLOAT_PHOTON_COUNT on or off.
void port_set_float_count(void* h, int32_t on) { static_cast<Renderer*>(h)->float_count = on != 0; }

// FR_FLAG_END_DEGENERATE_PATHS on or off.
void port_set_end_degenerate(void* h, int32_t on) { static_cast<Renderer*>(h)->end_degenerate = on != 0; }

// Second Philox key word of every stream (default 0x5350504D).
void port_set_stream_key(void* h, uint32_t key) { static_cast<Renderer*>(h)->stream_key = key; }

// Eye pass and gather only for pixels [x0, x1) x [y0, y1).
void port_set_window(void* h, int32_t x0, int32_t y0, int32_t x1, int32_t y1) {
  Renderer* r = static_cast<Renderer*>(h);
  r->win_x0 = x0; r->win_y0 = y0; r->win_x1 = x1; r->win_y1 = y1;
}

// Photon pass only (for a bounded CPU timing sample).
void port_photon_pass(void* h, int32_t first, int32_t count) {
  Renderer* r = static_cast<Renderer*>(h);
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = first; i < first + count; ++i) r->photon_path(i);
}

void port_resolve(void* h, Real* out) { static_cast<Renderer*>(h)->resolve(out); }

void port_trace_closest(void* h, const Real* rays, int32_t n, int32_t* facet, Real* tuv) {
  Renderer* r = static_cast<Renderer*>(h);
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < n; ++i) {
    const Real* q = rays + 7 * (size_t)i;
    Ray ray{vp(q), vp(q + 3), q[6]};
    Hit hit;
    if (closest(r->bvh, r->F, ray, hit, r->watertight)) {
      facet[i] = hit.facet;
      tuv[3 * i] = hit.t; tuv[3 * i + 1] = hit.u; tuv[3 * i + 2] = hit.v;
    } else {
      facet[i] = -1;
      tuv[3 * i] = FLT_MAX; tuv[3 * i + 1] = 0; tuv[3 * i + 2] = 0;
    }
  }
}

void port_trace_any(void* h, const Real* rays, int32_t n, int32_t* hit) {
  Renderer* r = static_cast<Renderer*>(h);
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < n; ++i) {
    const Real* q = rays + 8 * (size_t)i;
    hit[i] = any_hit(r->bvh, r->F, Ray{vp(q), vp(q + 3), 1.0f}, q[6], q[7], r->watertight) ? 1 : 0;
  }
}

// Hitpoints of the last iteration: type, facet; pos/nrm/out/w (3 floats each), rough.
void port_read_hitpoints(void* h, int32_t* type, int32_t* facet, Real* pos, Real* nrm, Real* out, Real* w,
                         Real* rough) {
  Renderer* r = static_cast<Renderer*>(h);
  for (size_t i = 0; i < r->hp.size(); ++i) {
    const HitPoint& p = r->hp[i];
    type[i] = p.type;
    facet[i] = p.facet;
    const V* src[4] = {&p.pos, &p.normal, &p.out, &p.weight};
    Real* dst[4] = {pos, nrm, out, w};
    for (int k = 0; k < 4; ++k) { dst[k][3 * i] = src[k]->x; dst[k][3 * i + 1] = src[k]->y; dst[k][3 * i + 2] = src[k]->z; }
    rough[i] = p.rough;
  }
}

int64_t port_num_photons(void* h) { return (int64_t) static_cast<Renderer*>(h)->photons.size(); }

// Compacted photons of the last iteration: N x 11 {pos, flux, dir, index, pdf}, path, slot.
void port_read_photons(void* h, Real* ph, int32_t* path, int32_t* slot) {
  Renderer* r = static_cast<Renderer*>(h);
  for (size_t i = 0; i < r->photons.size(); ++i) {
    const Photon& p = r->photons[i];
    Real* d = ph + 11 * i;
    d[0] = p.pos.x; d[1] = p.pos.y; d[2] = p.pos.z;
    d[3] = p.flux.x; d[4] = p.flux.y; d[5] = p.flux.z;
    d[6] = p.dir.x; d[7] = p.dir.y; d[8] = p.dir.z;
    d[9] = p.index; d[10] = p.pdf;
    path[i] = r->ph_path[i];
    slot[i] = r->ph_slot[i];
  }
}

void port_read_gather(void* h, int32_t* m, Real* phi) {
  Renderer* r = static_cast<Renderer*>(h);
  for (size_t i = 0; i < r->gather_m.size(); ++i) {
    m[i] = r->gather_m[i];
    phi[3 * i] = r->gather_phi[i].x; phi[3 * i + 1] = r->gather_phi[i].y; phi[3 * i + 2] = r->gather_phi[i].z;
  }
}

// Environment map (RGBA8, w x h) as the IBL texture: each texel value / 255.0f
// (TextureUtility.cpp:28), converted by 0.4 * (c^2, c^2, c^2, 0)
// (LightSampler.cpp:24: the literal 0.4 meets operator*(float, Vec4)).
void port_set_ibl(void* h, int32_t w, int32_t hh, const uint8_t* texels) {
  Renderer* r = static_cast<Renderer*>(h);
  r->ibl.w = w;
  r->ibl.h = hh;
  r->ibl.c.resize((size_t)w * hh * 4);
  for (size_t i = 0; i < (size_t)w * hh; ++i)
    for (int k = 0; k < 4; ++k) {
      const Real c = k < 3 ? texels[4 * i + k] / 255.0f : 0.0f;
      r->ibl.c[4 * i + k] = 0.4f * (c * c);
    }
  r->has_ibl = true;
}

// Per-hitpoint direct light of the last iteration and per-pixel sums and counts.
void port_read_direct(void* h, Real* hp_dl, Real* sp_dl, int32_t* sp_ndl) {
  Renderer* r = static_cast<Renderer*>(h);
  for (size_t i = 0; i < r->sp.size(); ++i) {
    const HitPoint& p = r->hp[i];
    const Shared& s = r->sp[i];
    hp_dl[3 * i] = p.dl.x; hp_dl[3 * i + 1] = p.dl.y; hp_dl[3 * i + 2] = p.dl.z;
    sp_dl[3 * i] = s.dl.x; sp_dl[3 * i + 1] = s.dl.y; sp_dl[3 * i + 2] = s.dl.z;
    sp_ndl[i] = s.ndl;
  }
}

void port_read_state(void* h, Real* rad, int32_t* n, Real* rr, int32_t* g) {
  Renderer* r = static_cast<Renderer*>(h);
  for (size_t i = 0; i < r->sp.size(); ++i) {
    const Shared& s = r->sp[i];
    rad[3 * i] = s.rad.x; rad[3 * i + 1] = s.rad.y; rad[3 * i + 2] = s.rad.z;
    if (r->float_count) std::memcpy(&n[i], &s.nf, 4);  // the float's bits, as the GPU returns them
    else n[i] = s.n;
    rr[i] = s.r;
    g[i] = s.g;
  }
}

// Radius query over given hitpoints (x, y, z, R) and photons (x, y, z): counts.
void port_radius_count(const Real* hp, int32_t nh, const Real* ph, int32_t np, int32_t* counts) {
  Renderer r;
  r.photons.resize(np);
  for (int i = 0; i < np; ++i) r.photons[i].pos = vp(ph + 3 * (size_t)i);
  std::vector<int> ids(np);
  for (int i = 0; i < np; ++i) ids[i] = i;
  r.kd.reserve(np);
  r.kd_build(ids, 0, np);
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < nh; ++i) {
    const V x = vp(hp + 4 * (size_t)i);
    const Real R = hp[4 * (size_t)i + 3];
    int m = 0;
    r.query(r.kd.empty() ? -1 : 0, x - R * V(1, 1, 1), x + R * V(1, 1, 1), x, R * R, [&](int) { ++m; });
    counts[i] = m;
  }
}

// Philox4x32-10 block, for known-answer tests.
void port_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  Rng::philox(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1], out);
}

}  // extern "C"
