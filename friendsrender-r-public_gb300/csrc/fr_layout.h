// Device-resident data layouts shared by the host library and the kernels.
// Plain structs only: no CUDA or C++ library types, so the host side
// (g++) and the device side (nvcc) agree on every offset.
#pragma once
#include <cstdint>

namespace fr {

// Constants of the reference's SPPM path.
constexpr float kPI = 3.14159f;                 // PTUtility::PI (SPPM/SPPM/Vec.h:10)
constexpr float kRayOffset = 1e-4f;             // Ray::RAY_OFFSET (SPPM/SPPM/Primitive.h:31)
constexpr int kPhotonSlots = 32;                // photon deque length per path (SPPM.cpp:753)
constexpr int kEmitSamples = 1000;              // LightSampler::NumSample (LightSampler.h:17)
constexpr uint32_t kPhiloxKeyHi = 0x5350504Du;  // second Philox key word of every stream

// Hitpoint types (SPPM.h:85-89).
constexpr int kHitNone = 0, kHitHit = 1, kHitOnlyDirect = 2;
// Surface types (FR_MAT_*).
constexpr int kSurfDiffuse = 0, kSurfMetal = 1, kSurfConductor = 2, kSurfGGXGlass = 3, kSurfBiMetal = 4,
              kSurfGlass = 5, kSurfGlossTransmit = 6, kSurfDiffuseTransmit = 7;

// Material flags.
constexpr int kMatSPPM = 1;    // SURFACE_PARAM::isSPPMSurface
constexpr int kMatOpaque = 2;  // SURFACE_PARAM::IfOpeque

// One attribute (Normal_Facet.h:67-113): the Surface subclass and its SURFACE_PARAM.
struct MaterialGPU {
  int32_t type;        // kSurf*
  int32_t flags;       // kMatSPPM | kMatOpaque
  int32_t tex_albedo;  // texture index or -1 (map_Kd)
  int32_t tex_rough;   // (map_d)
  int32_t tex_bump;    // (map_bump)
  int32_t pad0;
  float albedo[3];
  float radiance[3];
  float index, roughness, extinction, reflectance;
};

// RGBA8 texture, texels packed r | g<<8 | b<<16 | a<<24, row-major with
// row j at j*width (the reference's layout after stbi_load,
// TextureUtility.cpp:12-35).
struct TextureGPU {
  const uint32_t* texels;
  int32_t width, height;
  int32_t pad0, pad1;
};

// One area light (LightSampler.h:19-41) with everything the photon emitter
// needs precomputed on the host in the reference's float order.
struct LightGPU {
  float p0[3], p1[3], p2[3];
  float normal[3];      // (N0 + N1 + N2).normalized()       (SPPM.cpp:465)
  float radiance[3];    // untextured: Flux / (2*PI*Area)    (LightSampler.cpp:78)
  float pdf_point;      // untextured: 2 / |e1 x e2|         (Sampling.cpp:347)
  float pdf_light;      // alias pdf of this light           (LightSampler.h:87)
  float alias_prob;     // bin of the light alias table      (TableSampler.h:14-20)
  int32_t alias_left, alias_right;
  int32_t textured;
  int32_t emit_offset;  // first entry of its 1000-point emission table
};

// One entry of a textured light's emission table (LightSampler.cpp:30-66).
struct EmitEntry {
  float prob;
  int32_t left, right;
  float uvw[3];
  float L[3];
  float pdf;            // (GetPDF(uvl) * 1000) / Area       (LightSampler.cpp:73)
  float pad0;
};

struct CameraGPU {
  int32_t type;         // 0 pinhole (Camera.h:70-86), 1 thin lens (Camera.h:87-157)
  int32_t width, height;
  int32_t pad0;
  float pos[3], dir[3], e1[3], e2[3];
  float plane_w, plane_h, lens_w, lens_h, F, dist;
};

// 8-wide BVH node (224 bytes, fourteen 16-byte loads): child boxes as float
// SoA, then the child bookkeeping.  Internal children are stored contiguously
// from child_base in slot order; the triangles of leaf children contiguously
// from tri_base.
//   meta[c] == 0                : empty slot
//   imask bit c set             : internal child child_base + popc(imask & ((1<<c)-1))
//   otherwise (meta[c] & 0x80)  : leaf of ((meta[c] >> 5) & 3) + 1 triangles at
//                                 tri_base + (meta[c] & 31)
struct alignas(16) BVHNodeW {
  float lox[8], loy[8], loz[8];
  float hix[8], hiy[8], hiz[8];
  uint32_t child_base;
  uint32_t tri_base;
  uint32_t imask;
  uint32_t pad0;
  uint8_t meta[8];
  uint32_t pad1[2];
};
static_assert(sizeof(BVHNodeW) == 224, "node is fourteen 16-byte words");

// Traversal-stack reference: an internal node index, or a leaf run
// kLeafBit | (count-1) << kLeafCountShift | first triangle.
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr int kLeafCountShift = 27;
constexpr uint32_t kLeafFirstMask = (1u << kLeafCountShift) - 1u;
constexpr int kMaxLeafTris = 4;

// Triangle in leaf order: v0, e1 = v1 - v0, e2 = v2 - v0 (the exact floats
// the reference's Moller-Trumbore test forms, Intersect.cpp:67-89);
// v0.w carries the facet index.
struct alignas(16) TriGPU {
  float v0[4];
  float e1[4];
  float e2[4];
};

// Per-facet shading data in facet (OBJ face) order.
struct alignas(16) FacetShade {
  float n0[3], n1[3], n2[3];
  float uv0[2], uv1[2], uv2[2];
  int32_t attr;
};
static_assert(sizeof(FacetShade) == 64, "facet record is 64 bytes");

struct SceneGPU {
  const BVHNodeW* nodes;
  const TriGPU* tris;
  const FacetShade* shade;
  const MaterialGPU* mats;
  const TextureGPU* texs;
  const LightGPU* lights;
  const EmitEntry* emit;
  int32_t num_nodes, num_tris, num_facets, num_lights;
  float lo[3], hi[3];   // scene bounds
  const float* env;     // environment map: 4 floats per converted texel, 16-byte aligned; or null
  int32_t env_w, env_h;
  // Watertight mode: per triangle in leaf order 8 floats, the exact vertices
  // v1 and v2 (xyz, w unused; 16-byte aligned); v0 is TriGPU::v0.  Null in
  // the reference's mode.
  const float* tri_v12;
  int32_t watertight;
  int32_t pad0;
};

// Per-iteration parameters read by the kernels.
struct IterParams {
  const uint32_t* step;       // device word: reference iteration number (starts at 1)
  int32_t photons;            // photon paths this iteration
  int32_t width, height;
  float alpha;                // ppm_Alpha (SPPM.cpp:20)
  uint32_t flags;
};

constexpr uint32_t kFlagFixStaleSlot = 1u;  // drop the stale photon slot quirk (SPPM.cpp:672)
constexpr uint32_t kFlagStandardResolve = 2u;  // resolve with tau / (pi R^2 * photons emitted)
constexpr uint32_t kFlagEndDegenerate = 4u;    // end paths with a NaN BSDF value or pdf, or a zero pdf
constexpr uint32_t kFlagWatertight = 8u;       // watertight triangle test instead of Moller-Trumbore
constexpr uint32_t kFlagFloatPhotonCount = 16u;  // per-pixel N kept as float bits, not a truncated int

// Entries of the per-thread traversal stack (a wide node pushes at most 7).
constexpr int kTraversalStackEntries = 96;

// Device error word bits.
constexpr int kErrStack = 1;        // traversal stack overflow
constexpr int kErrQuery = 64;       // a radius query ball refused by query_ball_ok

// A radius query visits every grid cell its box (x - R, x + R) overlaps.  A
// ball that is not finite, or that spans more than kMaxQuerySpan cells along
// an axis, is refused: its loop over cells would take minutes, or never end
// once a cell index saturates.  Cell coordinates are bounded by
// kMaxQueryCellCoord so that the float-to-int conversion is exact.
constexpr int kMaxQuerySpan = 128;
constexpr float kMaxQueryCellCoord = 1.0e9f;

#if defined(__CUDACC__)
#define FR_HOST_DEVICE __host__ __device__
#else
#define FR_HOST_DEVICE
#endif

// The same float operations as the grid's cell_of on the box's corners
// ((x - R - origin) * inv_cell on each axis, no contraction).
FR_HOST_DEVICE inline bool query_ball_ok(float x, float y, float z, float R, const float origin[3], float inv_cell) {
  if (!(R >= 0.0f) || !(R <= 3.0e38f)) return false;  // NaN, negative or infinite radius
  const float c[3] = {x, y, z};
  for (int a = 0; a < 3; ++a) {
    const float f0 = (c[a] - R - origin[a]) * inv_cell;
    const float f1 = (c[a] + R - origin[a]) * inv_cell;
    if (!(f0 >= -kMaxQueryCellCoord) || !(f1 <= kMaxQueryCellCoord) || !(f1 - f0 <= (float)kMaxQuerySpan))
      return false;
  }
  return true;
}

}  // namespace fr
