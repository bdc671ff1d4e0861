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

__device__ __forceinline__ TriGPU load_tri(const TriGPU* tris, int i) {
  const float4* p = reinterpret_cast<const float4*>(tris + i);
  const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
  TriGPU t;
  t.v0[0] = a.x; t.v0[1] = a.y; t.v0[2] = a.z; t.v0[3] = a.w;
  t.e1[0] = b.x; t.e1[1] = b.y; t.e1[2] = b.z; t.e1[3] = b.w;
  t.e2[0] = c.x; t.e2[1] = c.y; t.e2[2] = c.z; t.e2[3] = c.w;
  return t;
}

struct RayBoxPre {
  float idx, idy, idz, ox, oy, oz;  // inverse direction and origin * inverse direction
};

__device__ __forceinline__ float safe_inv(float d) {
  const float m = 1e-20f;
  return 1.0f / (fabsf(d) < m ? copysignf(m, d) : d);
}

// Test the 8 children of a node; returns a bit mask of entered children and
// their entry distances.
__device__ __forceinline__ uint32_t node_hits(const BVHNode8* nodes, uint32_t ni, const RayBoxPre& r, float tmin,
                                              float tmax, float tn[8], uint32_t ch[8]) {
  const float4* p = reinterpret_cast<const float4*>(nodes + ni);
  float lx[8], ly[8], lz[8], hx[8], hy[8], hz[8];
  {
    float4 q;
    q = __ldg(p + 0); lx[0] = q.x; lx[1] = q.y; lx[2] = q.z; lx[3] = q.w;
    q = __ldg(p + 1); lx[4] = q.x; lx[5] = q.y; lx[6] = q.z; lx[7] = q.w;
    q = __ldg(p + 2); ly[0] = q.x; ly[1] = q.y; ly[2] = q.z; ly[3] = q.w;
    q = __ldg(p + 3); ly[4] = q.x; ly[5] = q.y; ly[6] = q.z; ly[7] = q.w;
    q = __ldg(p + 4); lz[0] = q.x; lz[1] = q.y; lz[2] = q.z; lz[3] = q.w;
    q = __ldg(p + 5); lz[4] = q.x; lz[5] = q.y; lz[6] = q.z; lz[7] = q.w;
    q = __ldg(p + 6); hx[0] = q.x; hx[1] = q.y; hx[2] = q.z; hx[3] = q.w;
    q = __ldg(p + 7); hx[4] = q.x; hx[5] = q.y; hx[6] = q.z; hx[7] = q.w;
    q = __ldg(p + 8); hy[0] = q.x; hy[1] = q.y; hy[2] = q.z; hy[3] = q.w;
    q = __ldg(p + 9); hy[4] = q.x; hy[5] = q.y; hy[6] = q.z; hy[7] = q.w;
    q = __ldg(p + 10); hz[0] = q.x; hz[1] = q.y; hz[2] = q.z; hz[3] = q.w;
    q = __ldg(p + 11); hz[4] = q.x; hz[5] = q.y; hz[6] = q.z; hz[7] = q.w;
    const uint4 c0 = __ldg(reinterpret_cast<const uint4*>(p + 12));
    const uint4 c1 = __ldg(reinterpret_cast<const uint4*>(p + 13));
    ch[0] = c0.x; ch[1] = c0.y; ch[2] = c0.z; ch[3] = c0.w;
    ch[4] = c1.x; ch[5] = c1.y; ch[6] = c1.z; ch[7] = c1.w;
  }
  uint32_t mask = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    // Boxes are padded on the host, so fused rounding here only moves the
    // slab bounds by far less than the padding.
    const float ax = fmaf(lx[c], r.idx, -r.ox), bx = fmaf(hx[c], r.idx, -r.ox);
    const float ay = fmaf(ly[c], r.idy, -r.oy), by = fmaf(hy[c], r.idy, -r.oy);
    const float az = fmaf(lz[c], r.idz, -r.oz), bz = fmaf(hz[c], r.idz, -r.oz);
    const float t0 = fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fmaxf(fminf(az, bz), tmin));
    const float t1 = fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fminf(fmaxf(az, bz), tmax));
    tn[c] = t0;
    if (t0 <= t1 && ch[c] != kEmptyChild) mask |= 1u << c;
  }
  return mask;
}

// Closest hit on (tmin, +inf).  Returns false on a miss; sets *err on stack overflow.
__device__ bool trace_closest(const SceneGPU& sc, V3 org, V3 dir, float tmin, Hit& hit, int* err) {
  RayBoxPre r;
  r.idx = safe_inv(dir.x); r.idy = safe_inv(dir.y); r.idz = safe_inv(dir.z);
  r.ox = org.x * r.idx; r.oy = org.y * r.idy; r.oz = org.z * r.idz;
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
        float tn[8];
        uint32_t ch[8];
        uint32_t mask = node_hits(sc.nodes, ref, r, tmin, tbest, tn, ch);
        // Visit the nearest entered child next; stack the others far to near.
        int n = 0;
        uint32_t ord_c[8];
        float ord_t[8];
        while (mask) {
          const int c = __ffs(mask) - 1;
          mask &= mask - 1;
          float t = tn[c];
          uint32_t cc = ch[c];
          int j = n++;
          while (j > 0 && ord_t[j - 1] < t) {
            ord_t[j] = ord_t[j - 1];
            ord_c[j] = ord_c[j - 1];
            --j;
          }
          ord_t[j] = t;
          ord_c[j] = cc;
        }
        if (n > 0) {
          if (sp + n - 1 > kTraversalStack) {
            atomicOr(err, kErrStack);
            return false;
          }
          for (int k = 0; k < n - 1; ++k) stack[sp++] = make_uint2(ord_c[k], __float_as_uint(ord_t[k]));
          ref = ord_c[n - 1];
          tref = ord_t[n - 1];
          continue;
        }
      } else {
        const int first = (int)(ref & kLeafFirstMask);
        const int count = (int)((ref >> kLeafCountShift) & 0xFu) + 1;
        for (int k = 0; k < count; ++k) {
          const TriGPU tr = load_tri(sc.tris, first + k);
          float t, u, v;
          if (intersect_triangle(org, dir, tr, t, u, v) && t > tmin) {
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
__device__ bool trace_any(const SceneGPU& sc, V3 org, V3 dir, float tmin, float tmax, int* err) {
  RayBoxPre r;
  r.idx = safe_inv(dir.x); r.idy = safe_inv(dir.y); r.idz = safe_inv(dir.z);
  r.ox = org.x * r.idx; r.oy = org.y * r.idy; r.oz = org.z * r.idz;
  uint32_t stack[kTraversalStack];
  int sp = 0;
  uint32_t ref = 0;
  while (true) {
    if (!(ref & kLeafBit)) {
      float tn[8];
      uint32_t ch[8];
      uint32_t mask = node_hits(sc.nodes, ref, r, tmin, tmax, tn, ch);
      if (sp + __popc(mask) > kTraversalStack) {
        atomicOr(err, kErrStack);
        return false;
      }
      while (mask) {
        const int c = __ffs(mask) - 1;
        mask &= mask - 1;
        stack[sp++] = ch[c];
      }
    } else {
      const int first = (int)(ref & kLeafFirstMask);
      const int count = (int)((ref >> kLeafCountShift) & 0xFu) + 1;
      for (int k = 0; k < count; ++k) {
        const TriGPU tr = load_tri(sc.tris, first + k);
        float t, u, v;
        if (intersect_triangle(org, dir, tr, t, u, v) && tmax >= t && t > tmin) return true;
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
