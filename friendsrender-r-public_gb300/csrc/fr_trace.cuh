// Ray traversal of the 8-wide BVH and surface geometry at a hit.
//
// The BVH only culls: a child box is entered when the slab interval meets
// [tmin, tbest], and boxes are padded on the host, so every triangle the
// reference's exhaustive test would accept is reached.  The triangle test is
// the reference's Moller-Trumbore (Intersect.cpp:67-89) with its acceptance
// rule t > MinT (bvh8.h:591); of equal-t candidates the larger facet index
// wins, where the reference keeps the one its own traversal visits last.
#pragma once
#include <cfloat>
#include "fr_bsdf.cuh"
#include "fr_layout.h"
#include "fr_math.cuh"

namespace fr {

constexpr int kTraversalStack = kTraversalStackEntries;

struct Hit {
  float t, u, v;
  int32_t tri;    // triangle slot in leaf order
  int32_t facet;  // facet (OBJ face) index
};

// Isc::Intersect(Ray, Triangle_ID) (Intersect.cpp:67-89).
__device__ __forceinline__ bool intersect_triangle(const V3 org, const V3 dir, const TriGPU& tr, float& t,
                                                   float& u, float& v) {
  const V3 v0 = v3(tr.v0), e1 = v3(tr.e1), e2 = v3(tr.e2);
  const V3 ps = cross(dir, e2);
  const float a = dot(e1, ps);
  if (a > -FLT_MIN && a < FLT_MIN) return false;
  const float f = 1.0f / a;
  const V3 s = org - v0;
  u = f * dot(s, ps);
  if (u < 0.0f || u > 1.0f) return false;
  const V3 q = cross(s, e1);
  v = f * dot(dir, q);
  if (v < 0.0f || u + v > 1.0f) return false;
  t = f * dot(e2, q);
  return true;
}

// Watertight ray-triangle test (Woop, Benthin and Wald, JCGT 2(1), 2013):
// the vertices are moved into a ray-aligned frame (kz the direction's
// largest axis, the frame sheared so the ray is its z axis) and the three
// 2-D edge functions decide; an edge function that is exactly zero in float
// is evaluated again in double, so an edge shared by two triangles is never
// missed by both.  No backface culling.  u, v are the weights of p1 and p2
// (as Moller-Trumbore's), t the distance along dir.  The CPU oracle runs the
// same float and double operations in the same order.
__device__ __forceinline__ float axis_of(V3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

__device__ __forceinline__ bool intersect_watertight(const V3 org, const V3 dir, const V3 p0, const V3 p1,
                                                     const V3 p2, float& t, float& u, float& v) {
  const float adx = fabsf(dir.x), ady = fabsf(dir.y), adz = fabsf(dir.z);
  const int kz = adx > ady ? (adx > adz ? 0 : 2) : (ady > adz ? 1 : 2);
  int kx = kz == 2 ? 0 : kz + 1;
  int ky = kx == 2 ? 0 : kx + 1;
  const float dz = axis_of(dir, kz);
  if (dz < 0.0f) {  // keep the winding
    const int k = kx;
    kx = ky;
    ky = k;
  }
  const float Sx = axis_of(dir, kx) / dz, Sy = axis_of(dir, ky) / dz, Sz = 1.0f / dz;
  const V3 A = p0 - org, B = p1 - org, C = p2 - org;
  const float Az0 = axis_of(A, kz), Bz0 = axis_of(B, kz), Cz0 = axis_of(C, kz);
  const float Ax = axis_of(A, kx) - Sx * Az0, Ay = axis_of(A, ky) - Sy * Az0;
  const float Bx = axis_of(B, kx) - Sx * Bz0, By = axis_of(B, ky) - Sy * Bz0;
  const float Cx = axis_of(C, kx) - Sx * Cz0, Cy = axis_of(C, ky) - Sy * Cz0;
  float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
  const float det = U + V + W;
  if (det == 0.0f) return false;
  const float T = U * (Sz * Az0) + V * (Sz * Bz0) + W * (Sz * Cz0);
  const float rcp = 1.0f / det;
  t = T * rcp;
  u = V * rcp;
  v = W * rcp;
  return true;
}

__device__ __forceinline__ TriGPU load_tri(const TriGPU* tris, int i) {
  const float4* p = reinterpret_cast<const float4*>(tris + i);
  const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
  TriGPU t;
  t.v0[0] = a.x; t.v0[1] = a.y; t.v0[2] = a.z; t.v0[3] = a.w;
  t.e1[0] = b.x; t.e1[1] = b.y; t.e1[2] = b.z; t.e1[3] = b.w;
  t.e2[0] = c.x; t.e2[1] = c.y; t.e2[2] = c.z; t.e2[3] = c.w;
  return t;
}

// The scene's triangle test for triangle slot i (already loaded as tr): the
// reference's Moller-Trumbore, or (kWT, a scene with FR_FLAG_WATERTIGHT) the
// watertight test on the exact vertices.  The traversal kernels are
// instantiated for both, so the reference's mode keeps its registers.
template <bool kWT>
__device__ __forceinline__ bool tri_test(const SceneGPU& sc, const V3 org, const V3 dir, const TriGPU& tr, int i,
                                         float& t, float& u, float& v) {
  if constexpr (!kWT) {
    return intersect_triangle(org, dir, tr, t, u, v);
  } else {
    const float4* q = reinterpret_cast<const float4*>(sc.tri_v12) + 2 * (size_t)i;
    const float4 a = __ldg(q), b = __ldg(q + 1);
    return intersect_watertight(org, dir, v3(tr.v0), v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), t, u, v);
  }
}

struct RayPre {
  float idx, idy, idz;  // inverse direction
  float ox, oy, oz;     // origin
};

__device__ __forceinline__ float safe_inv(float d) {
  const float m = 1e-20f;
  return 1.0f / (fabsf(d) < m ? copysignf(m, d) : d);
}

// Entry distances of the 8 children of a node, as sort keys (float bits of
// the entry distance with the slot in the low 3 bits; entry distances are
// positive, so the integer order is the distance order), and the node's child
// bookkeeping.  Missed and empty children get 0xFFFFFFFF.
struct NodeVisit {
  uint32_t key[8];
  uint32_t child_base, tri_base, imask;
  uint32_t meta_lo, meta_hi;
};

// Child slab tests.  With FR_NEAR_FAR (the default) each axis reads its near
// plane from the lo array and its far plane from the hi array when the ray's
// inverse direction on that axis is positive, and the other way round when
// it is negative: fma(b, idir, -o*idir) is monotonic in b, so these are the
// min and the max of the two plane distances without computing both and
// comparing (the same t0 and t1 bit for bit, for boxes with lo <= hi; empty
// slots are masked out by their meta byte).  FR_MINMAX3 takes the entry and
// exit distances with three-input min/max instructions.
#ifndef FR_NEAR_FAR
#define FR_NEAR_FAR 1
#endif
#ifndef FR_MINMAX3
#define FR_MINMAX3 0
#endif

__device__ __forceinline__ float max3f(float a, float b, float c) {
#if FR_MINMAX3
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
#else
  return fmaxf(fmaxf(a, b), c);
#endif
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
#if FR_MINMAX3
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
#else
  return fminf(fminf(a, b), c);
#endif
}

__device__ __forceinline__ void visit_node(const BVHNodeW* nodes, uint32_t ni, const RayPre& r, float tmin,
                                           float tmax, NodeVisit& nv) {
  const float4* q = reinterpret_cast<const float4*>(nodes + ni);
  float lx[8], ly[8], lz[8], hx[8], hy[8], hz[8];
#define FR_LD8(arr, i0)                                   \
  {                                                       \
    const float4 a_ = __ldg(q + (i0)), b_ = __ldg(q + (i0) + 1); \
    arr[0] = a_.x; arr[1] = a_.y; arr[2] = a_.z; arr[3] = a_.w;   \
    arr[4] = b_.x; arr[5] = b_.y; arr[6] = b_.z; arr[7] = b_.w;   \
  }
#if FR_NEAR_FAR
  // lx/ly/lz: near planes, hx/hy/hz: far planes (float4 offsets: lo x 0, lo y
  // 2, lo z 4, hi x 6, hi y 8, hi z 10).
  const int nx = r.idx < 0.0f ? 6 : 0, ny = r.idy < 0.0f ? 8 : 2, nz = r.idz < 0.0f ? 10 : 4;
  FR_LD8(lx, nx) FR_LD8(ly, ny) FR_LD8(lz, nz) FR_LD8(hx, 6 - nx) FR_LD8(hy, 10 - ny) FR_LD8(hz, 14 - nz)
#else
  FR_LD8(lx, 0) FR_LD8(ly, 2) FR_LD8(lz, 4) FR_LD8(hx, 6) FR_LD8(hy, 8) FR_LD8(hz, 10)
#endif
#undef FR_LD8
  const uint4 m0 = __ldg(reinterpret_cast<const uint4*>(q + 12));
  const uint4 m1 = __ldg(reinterpret_cast<const uint4*>(q + 13));
  nv.child_base = m0.x;
  nv.tri_base = m0.y;
  nv.imask = m0.z;
  nv.meta_lo = m1.x;
  nv.meta_hi = m1.y;
  // t = (b - o) * idir, with the products fused (the boxes are padded far
  // beyond the rounding of the fused form).
  const float ox = r.ox * r.idx, oy = r.oy * r.idy, oz = r.oz * r.idz;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const float ax = fmaf(lx[c], r.idx, -ox), bx = fmaf(hx[c], r.idx, -ox);
    const float ay = fmaf(ly[c], r.idy, -oy), by = fmaf(hy[c], r.idy, -oy);
    const float az = fmaf(lz[c], r.idz, -oz), bz = fmaf(hz[c], r.idz, -oz);
#if FR_NEAR_FAR
    const float t0 = max3f(ax, ay, fmaxf(az, tmin));
    const float t1 = min3f(bx, by, fminf(bz, tmax));
#else
    const float t0 = max3f(fminf(ax, bx), fminf(ay, by), fmaxf(fminf(az, bz), tmin));
    const float t1 = min3f(fmaxf(ax, bx), fmaxf(ay, by), fminf(fmaxf(az, bz), tmax));
#endif
#if FR_NEAR_FAR
    // An empty slot's box is lo = +inf, hi = -inf (collapse_bvh8), so its near
    // plane distance is +inf and its far one -inf: t0 > t1 culls it without
    // reading its meta byte.
    nv.key[c] = t0 <= t1 ? ((__float_as_uint(t0) & ~7u) | (uint32_t)c) : 0xFFFFFFFFu;
#else
    const uint32_t mw = c < 4 ? m1.x : m1.y;
    const bool valid = ((mw >> (8 * (c & 3))) & 0xFFu) != 0u;
    nv.key[c] = (valid && t0 <= t1) ? ((__float_as_uint(t0) & ~7u) | (uint32_t)c) : 0xFFFFFFFFu;
#endif
  }
}

// Ascending order of the 8 keys (19-comparator sorting network), in registers.
__device__ __forceinline__ void sort8(uint32_t k[8]) {
#define FR_CX(i, j)                              \
  {                                              \
    const uint32_t a_ = min(k[i], k[j]);         \
    k[j] = max(k[i], k[j]);                      \
    k[i] = a_;                                   \
  }
  FR_CX(0, 1) FR_CX(2, 3) FR_CX(4, 5) FR_CX(6, 7) FR_CX(0, 2) FR_CX(1, 3) FR_CX(4, 6) FR_CX(5, 7)
  FR_CX(1, 2) FR_CX(5, 6) FR_CX(0, 4) FR_CX(3, 7) FR_CX(1, 5) FR_CX(2, 6) FR_CX(1, 4) FR_CX(3, 6)
  FR_CX(2, 4) FR_CX(3, 5) FR_CX(3, 4)
#undef FR_CX
}

// Stack reference of slot c of a visited node.
__device__ __forceinline__ uint32_t child_ref(const NodeVisit& nv, uint32_t c) {
  if ((nv.imask >> c) & 1u) return nv.child_base + (uint32_t)__popc(nv.imask & ((1u << c) - 1u));
  const uint32_t m = ((c < 4 ? nv.meta_lo : nv.meta_hi) >> (8 * (c & 3))) & 0xFFu;
  return kLeafBit | (((m >> 5) & 3u) << kLeafCountShift) | (nv.tri_base + (m & 31u));
}

__device__ __forceinline__ RayPre ray_pre(V3 org, V3 dir) {
  RayPre r;
  r.idx = safe_inv(dir.x); r.idy = safe_inv(dir.y); r.idz = safe_inv(dir.z);
  r.ox = org.x; r.oy = org.y; r.oz = org.z;
  return r;
}

// Closest hit on (tmin, +inf).  Returns false on a miss; sets *err on stack overflow.
template <bool kWT>
__device__ bool trace_closest(const SceneGPU& sc, V3 org, V3 dir, float tmin, Hit& hit, int* err) {
  const RayPre r = ray_pre(org, dir);
  float tbest = FLT_MAX;
  int32_t best_tri = -1, best_facet = -1;
  float bu = 0.0f, bv = 0.0f;
  uint2 stack[kTraversalStack];
  int sp = 0;
  uint32_t ref = 0;
  float tref = tmin;
  while (true) {
    if (tref <= tbest) {
      if (!(ref & kLeafBit)) {
        NodeVisit nv;
        visit_node(sc.nodes, ref, r, tmin, tbest, nv);
        sort8(nv.key);
        if (nv.key[0] != 0xFFFFFFFFu) {
          // Nearest child next; the others stacked far to near.
          int n = 1;
#pragma unroll
          for (int k = 1; k < 8; ++k) n += nv.key[k] != 0xFFFFFFFFu;
          if (sp + n - 1 > kTraversalStack) {
            atomicOr(err, kErrStack);
            return false;
          }
#pragma unroll
          for (int k = 7; k >= 1; --k)
            if (k < n) stack[sp++] = make_uint2(child_ref(nv, nv.key[k] & 7u), nv.key[k] & ~7u);
          ref = child_ref(nv, nv.key[0] & 7u);
          tref = __uint_as_float(nv.key[0] & ~7u);
          continue;
        }
      } else {
        const int first = (int)(ref & kLeafFirstMask);
        const int count = (int)((ref >> kLeafCountShift) & 0xFu) + 1;
        for (int k = 0; k < count; ++k) {
          const TriGPU tr = load_tri(sc.tris, first + k);
          float t, u, v;
          if (tri_test<kWT>(sc, org, dir, tr, first + k, t, u, v) && t > tmin) {
            const int32_t facet = __float_as_int(tr.v0[3]);
            if (t < tbest || (t == tbest && facet > best_facet)) {
              tbest = t; bu = u; bv = v; best_tri = first + k; best_facet = facet;
            }
          }
        }
      }
    }
    if (sp == 0) break;
    const uint2 e = stack[--sp];
    ref = e.x;
    tref = __uint_as_float(e.y);
  }
  if (best_tri < 0) return false;
  hit.t = tbest; hit.u = bu; hit.v = bv; hit.tri = best_tri; hit.facet = best_facet;
  return true;
}

// Any hit with t in (tmin, tmax] (findAnyElement, bvh8.h:643-707).
template <bool kWT>
__device__ bool trace_any(const SceneGPU& sc, V3 org, V3 dir, float tmin, float tmax, int* err) {
  const RayPre r = ray_pre(org, dir);
  uint32_t stack[kTraversalStack];
  int sp = 0;
  uint32_t ref = 0;
  while (true) {
    if (!(ref & kLeafBit)) {
      NodeVisit nv;
      visit_node(sc.nodes, ref, r, tmin, tmax, nv);
      int n = 0;
#pragma unroll
      for (int k = 0; k < 8; ++k) n += nv.key[k] != 0xFFFFFFFFu;
      if (sp + n > kTraversalStack) {
        atomicOr(err, kErrStack);
        return false;
      }
#pragma unroll
      for (int k = 0; k < 8; ++k)
        if (nv.key[k] != 0xFFFFFFFFu) stack[sp++] = child_ref(nv, (uint32_t)k);
    } else {
      const int first = (int)(ref & kLeafFirstMask);
      const int count = (int)((ref >> kLeafCountShift) & 0xFu) + 1;
      for (int k = 0; k < count; ++k) {
        const TriGPU tr = load_tri(sc.tris, first + k);
        float t, u, v;
        if (tri_test<kWT>(sc, org, dir, tr, first + k, t, u, v) && tmax >= t && t > tmin) return true;
      }
    }
    if (sp == 0) return false;
    ref = stack[--sp];
  }
}

// Geometry at a hit (StochasticProgressivePhotonMapping::Geometry, SPPM.h:56-68).
struct Geom {
  V3 pos, normal;
  float uvx, uvy;
  int32_t mat;
  int32_t type, flags;
  V3 albedo, radiance;
  float index, rough, extinction, reflectance;
  float translucency;
};

// calculateGeometry (SPPM.cpp:36-77).
__device__ __forceinline__ void calc_geometry(const SceneGPU& sc, const Hit& h, Geom& g) {
  const TriGPU tr = load_tri(sc.tris, h.tri);
  const V3 P0 = v3(tr.v0), E1 = v3(tr.e1), E2 = v3(tr.e2);
  const FacetShade& fs = sc.shade[h.facet];
  const V3 N0 = v3(fs.n0), N1 = v3(fs.n1), N2 = v3(fs.n2);
  g.pos = h.u * E1 + h.v * E2 + P0;
  g.normal = normalized(h.u * (N1 - N0) + h.v * (N2 - N0) + N0);
  g.uvx = h.u * (fs.uv1[0] - fs.uv0[0]) + h.v * (fs.uv2[0] - fs.uv0[0]) + fs.uv0[0];
  g.uvy = h.u * (fs.uv1[1] - fs.uv0[1]) + h.v * (fs.uv2[1] - fs.uv0[1]) + fs.uv0[1];
  g.mat = fs.attr;
  const MaterialGPU& m = sc.mats[fs.attr];
  g.type = m.type;
  g.flags = m.flags;
  g.albedo = v3(m.albedo);
  g.radiance = v3(m.radiance);
  g.index = m.index;
  g.rough = m.roughness;
  g.extinction = m.extinction;
  g.reflectance = m.reflectance;
  g.translucency = 0.0f;
  if (norm2(g.radiance) > kGt1e6) g.albedo = v3(1.f, 1.f, 1.f);
  if (m.tex_rough >= 0) {
    const F4 c = tex_bilinear(sc.texs[m.tex_rough], g.uvx, g.uvy);
    g.rough = fminf(0.8f, fmaxf(0.05f, 0.5f * c.x));
  }
  if (m.tex_albedo >= 0) {
    const F4 c = tex_bilinear(sc.texs[m.tex_albedo], g.uvx, g.uvy);
    g.albedo = v3(c.x, c.y, c.z);
    g.radiance = g.radiance * g.albedo;
    g.translucency = 1.0f - c.w;
  }
  if (m.tex_bump >= 0) {
    // GetNormalFromNormalmap (TextureUtility.cpp:161-164), swizzle (x, z, y),
    // then the inverse of the column basis {e1, e2, e3} (Matrix.h:180-184).
    const F4 c = tex_bilinear(sc.texs[m.tex_bump], g.uvx, g.uvy);
    const V3 nm = normalized(v3(2.0f * c.x - 1.0f, 2.0f * c.y - 1.0f, 2.0f * c.z - 1.0f));
    const V3 nrm = normalized(v3(nm.x, nm.z, nm.y));
    const V3 e2 = g.normal;
    const V3 e1 = fabsf(e2.y) > kGt0_9 ? cross(e2, v3(1.f, 0.f, 0.f)) : cross(e2, v3(0.f, 1.f, 0.f));
    const V3 e3 = normalized(cross(e1, e2));
    // M[i][j] = component i of column j.
    const float M[3][3] = {{e1.x, e2.x, e3.x}, {e1.y, e2.y, e3.y}, {e1.z, e2.z, e3.z}};
    float C[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float m2[2][2];
        int rr = 0;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          if (i == r) continue;
          int cc = 0;
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            if (j == c) continue;
            m2[rr][cc] = M[i][j];
            ++cc;
          }
          ++rr;
        }
        const float d2 = m2[0][0] * m2[1][1] - m2[0][1] * m2[1][0];
        C[r][c] = d2 * (float)(((r + c) % 2) ? -1 : 1);
      }
    }
    const float det = M[0][0] * C[0][0] + M[1][0] * C[1][0] + M[2][0] * C[2][0];
    const float ix = 1.0f / det;
    // inverse = adjugate * (1/det), adjugate[i][j] = C[j][i]
    float I[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) I[i][j] = ix * C[j][i];
    const V3 out = v3(dot(v3(I[0][0], I[0][1], I[0][2]), nrm), dot(v3(I[1][0], I[1][1], I[1][2]), nrm),
                      dot(v3(I[2][0], I[2][1], I[2][2]), nrm));
    g.normal = normalized(out);
  }
}

}  // namespace fr
