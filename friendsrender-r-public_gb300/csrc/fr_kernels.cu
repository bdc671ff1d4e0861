// SPPM iteration kernels for sm_103a.
//
// One iteration (StochasticProgressivePhotonMapping, SPPM/SPPM/SPPM.cpp:768-848):
//   k_eye_pass       createHitpoints + getHitpointInfo  (SPPM.cpp:98-353)
//   k_photon_pass    createPhotonMap + generateLightRay (SPPM.cpp:453-680)
//   k_grid_setup / k_photon_count / scan / k_photon_scatter
//                    photon cell grid, replacing the photon kd-tree
//                    (SPPM.cpp:809-833, kdtree.h:348-431)
//   k_gather_update  applyHitPointInfo                  (SPPM.cpp:395-451)
//   k_resolve        reconstructImageFromSharedPoints   (SPPM.cpp:473-493)
// The eye and photon passes draw from independent per-pixel / per-path
// streams, so running the eye pass first gives the same numbers as the
// reference's photon-first order; it lets the grid size its cells from this
// iteration's hitpoint radii.
#include <cuda_runtime.h>
#include <algorithm>
#include <cfloat>
#include <cstdint>
#include "fr_bsdf.cuh"
#include "fr_grid.cuh"
#include "fr_kernels.h"
#include "fr_layout.h"
#include "fr_math.cuh"
#include "fr_trace.cuh"

namespace fr {

namespace {

__device__ __forceinline__ bool near1(float s) { return fabsf(s - 1.0f) < kLt1e5; }  // SPPM.h:27-29

__device__ __forceinline__ float max3(V3 a) {
  return a.x > a.y ? (a.x > a.z ? a.x : a.z) : (a.y > a.z ? a.y : a.z);
}

__device__ __forceinline__ void store_float4(float4* p, V3 v, float w) { *p = make_float4(v.x, v.y, v.z, w); }

// ----------------------------------------------------------------- camera
// PinholeCamera / ThinLensCamera::SampleCameraRay (Camera.h:73-83, 103-129).
// s0..s2: the three sampler draws (the first draws of the pixel's stream).
__device__ __forceinline__ void camera_ray(const CameraGPU& c, float u, float v, float s0, float s1, float s2,
                                           V3& org, V3& dir, float& pdf) {
  const V3 pos = v3(c.pos), cdir = v3(c.dir), e1 = v3(c.e1), e2 = v3(c.e2);
  if (c.type == 0) {
    const V3 off = v3(s0, s1, s2) * v3(c.plane_w, c.plane_h, 0.0f) / v3((float)c.width, (float)c.height, 1.0f);
    const V3 image = pos - cdir * c.dist + (u - 0.5f + off.x) * e1 * c.plane_w + (v - 0.5f + off.y) * e2 * c.plane_h;
    pdf = 1.0f;
    org = image;
    dir = normalized(normalized(pos - image));
  } else {
    const float pdf_area = 1.0f / (c.lens_w * c.lens_h);
    const V3 lens = pos + (s0 - 0.5f) * e1 * c.lens_w + (s1 - 0.5f) * e2 * c.lens_h;
    const V3 image = pos - cdir * c.dist + (u - 0.5f) * e1 * c.plane_w + (v - 0.5f) * e2 * c.plane_h;
    const float A = c.dist;
    const float B = (A * c.F) / (A - c.F);
    const V3 target = image + (pos - image) * (A + B) / A;
    const float cs = dot(cdir, normalized(lens - image));
    const float d2 = norm2(lens - image);
    pdf = pdf_area * (d2 / c.F / c.F) / cs;
    org = lens;
    dir = normalized(normalized(target - lens));
  }
}

// ------------------------------------------------------------------ eye pass
__global__ void __launch_bounds__(128) k_eye_pass(SceneGPU sc, CameraGPU cam, IterParams it, float rr5, float rr6,
                                                  HitpointBuf hp, PixelState st, GridInfo* gi, int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int npix = it.width * it.height;
  int hit_type = kHitNone;
  float radius = 0.0f;
  if (i < npix) {
    const int w = i % it.width, h = i / it.width;
    const float u = (float)w / (float)it.width;
    const float v = (float)h / (float)it.height;
    Rng rng((uint32_t)i + (uint32_t)npix * it.step);
    const float s0 = rng.next(), s1 = rng.next(), s2 = rng.next();
    V3 org, dir;
    float cam_pdf;
    camera_ray(cam, u, v, s0, s1, s2, org, dir, cam_pdf);

    V3 cur_o = org, cur_d = dir, nxt_o = org, nxt_d = dir;
    float cur_ix = 1.0f, nxt_ix = 1.0f;
    float PDF = 1.0f;
    V3 thr = v3(1.f, 1.f, 1.f);
    int depth = 0;
    while (true) {
      if (depth > 6) break;
      if (depth > 4) {
        const float rus = depth == 5 ? rr5 : rr6;
        if (rng.next() > rus) break;
        PDF *= rus;
      }
      Hit hit;
      if (!trace_closest(sc, cur_o, cur_d, kRayOffset, hit, err)) {
        hit_type = kHitOnlyDirect;  // miss: ONLY_DIRECTLIGHT with no IBL (SPPM.cpp:290-300)
        break;
      }
      Geom g;
      calc_geometry(sc, hit, g);
      g.normal = dot(g.normal, cur_d) > 0.0f ? -g.normal : g.normal;
      nxt_o = g.pos;
      if (g.translucency > 0.5f) {
        thr = thr * v3(g.translucency, g.translucency, g.translucency);
        cur_o = g.pos + cur_d * kRayOffset;
        continue;
      }
      if (g.flags & kMatSPPM) {
        // makeHitPoint (SPPM.cpp:79-96); with no IBL nothing after the first
        // hitpoint reaches the image, so the path stops here.
        const V3 wgt = (thr / PDF) / cam_pdf;
        store_float4(hp.pos + i, g.pos, __int_as_float(kHitHit));
        store_float4(hp.nrm + i, g.normal, g.rough);
        store_float4(hp.out + i, -cur_d, __int_as_float(g.mat));
        store_float4(hp.wgt + i, wgt, __int_as_float(hit.facet));
        hit_type = kHitHit;
        radius = st.r[i];
        break;
      }
      float Ii, Io;
      if (near1(cur_ix)) { Ii = 1.0f; Io = g.index; }
      else { Ii = cur_ix; Io = 1.0f; }
      FParam p{cur_d, nxt_d, g.normal, Ii, Io, g.rough, g.extinction, g.reflectance};
      float pdf = 1.0f;
      nxt_d = surface_sample(g.type, rng, p, &pdf);
      if (!is_valid_direction(nxt_d)) break;
      if (g.flags & kMatOpaque) {
        if (dot(nxt_d, g.normal) < kLt1e6) break;
      } else {
        const bool reflect = !(dot(nxt_d, g.normal) < 0.0f);
        nxt_ix = reflect ? cur_ix : Io;
      }
      p.out = nxt_d;
      pdf = surface_pdf(g.type, p);
      const V3 on = dot(g.normal, nxt_d) > 0.0f ? g.normal : -g.normal;
      nxt_o = nxt_o + on * kRayOffset;
      const float brdf = surface_brdf(g.type, p);
      const float cs = fmaxf(0.0f, fminf(1.0f, dot(nxt_d, on)));
      if (brdf < kLt1e8) break;
      if (pdf < 0.0f) break;
      thr = thr * (g.albedo * cs * brdf);
      PDF *= pdf;
      cur_o = nxt_o; cur_d = nxt_d; cur_ix = nxt_ix;
      ++depth;
    }
    if (hit_type != kHitHit) store_float4(hp.pos + i, v3(0.f, 0.f, 0.f), __int_as_float(hit_type));
  }
  // Radii of this iteration's hitpoints, for the grid's cell size.
  float rs = radius;
  unsigned cnt = hit_type == kHitHit ? 1u : 0u;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    rs += __shfl_down_sync(0xffffffffu, rs, o);
    cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  }
  if ((threadIdx.x & 31) == 0 && cnt) {
    atomicAdd(&gi->r_sum, rs);
    atomicAdd(&gi->r_count, cnt);
  }
}

// --------------------------------------------------------------- photon pass
// One photon path (createPhotonMap body, SPPM.cpp:508-673) as a state that
// advances one loop iteration at a time, so a persistent thread can start a
// new path as soon as its current one ends.
struct PhotonPath {
  Rng rng;
  V3 cur_o, cur_d, nxt_o, nxt_d, thr, flux0;
  float cur_ix, nxt_ix, PDF;
  int k, loop, depth;
  size_t base;
  int idx;

  __device__ __forceinline__ PhotonPath() : rng(0u) {}

  // generateLightRay (SPPM.cpp:453-471) and the light-surface photon (SPPM.cpp:530-540).
  __device__ __forceinline__ void start(const SceneGPU& sc, const IterParams& it, const PhotonSlots& ph, int i) {
    idx = i;
    rng = Rng((uint32_t)i + 135u + it.step * (uint32_t)it.photons);
    base = (size_t)i * kPhotonSlots;
    const uint32_t lb = (uint32_t)(((uint64_t)(uint32_t)sc.num_lights * rng.next_u24()) >> 24);
    const LightGPU& bin = sc.lights[lb];
    const int li = rng.next() < bin.alias_prob ? bin.alias_left : bin.alias_right;
    const LightGPU& L = sc.lights[li];
    const V3 P0 = v3(L.p0), P1 = v3(L.p1), P2 = v3(L.p2);
    V3 pos, rad;
    float pdf_area;
    if (L.textured) {
      const EmitEntry* tab = sc.emit + L.emit_offset;
      const uint32_t eb = (uint32_t)(((uint64_t)kEmitSamples * rng.next_u24()) >> 24);
      const int ei = rng.next() < tab[eb].prob ? tab[eb].left : tab[eb].right;
      const EmitEntry& e = tab[ei];
      pos = e.uvw[0] * P0 + e.uvw[1] * P1 + (1.0f - e.uvw[0] - e.uvw[1]) * P2;
      rad = v3(e.L);
      pdf_area = e.pdf;
    } else {
      float u = rng.next(), v = rng.next();
      if (v > u) { u *= 0.5f; v -= u; }
      else { v *= 0.5f; u -= v; }
      pos = u * P0 + v * P1 + (1.0f - u - v) * P2;
      rad = v3(L.radiance);
      pdf_area = L.pdf_point;
    }
    pdf_area *= L.pdf_light;
    const V3 ln = v3(L.normal);
    float pdf_dir = 1.0f;
    const V3 d = cos_sampling(rng, ln, &pdf_dir);
    rad = rad * fminf(1.0f, fmaxf(0.0f, dot(ln, d)));
    cur_o = pos + ln * kRayOffset;
    cur_d = normalized(d);
    flux0 = rad;
    PDF = pdf_area * pdf_dir;
    thr = v3(1.f, 1.f, 1.f);
    store_float4(ph.pos + base, cur_o, 1.0f);
    store_float4(ph.flux + base, flux0 * thr * kPI, PDF);
    store_float4(ph.dir + base, cur_d, 1.0f);
    nxt_o = cur_o;
    nxt_d = cur_d;
    cur_ix = nxt_ix = 1.0f;
    k = loop = depth = 0;
  }

  // One pass of the bounce loop (SPPM.cpp:548-671); false when the path ends.
  __device__ __forceinline__ bool step(const SceneGPU& sc, const PhotonSlots& ph, int* err) {
    if (loop++ > 32 || k >= kPhotonSlots - 1) return false;
    if (thr.x < kLt1e8 || thr.y < kLt1e8 || thr.z < kLt1e8) return false;
    Hit hit;
    if (!trace_closest(sc, cur_o, cur_d, kRayOffset, hit, err)) return false;
    Geom g;
    calc_geometry(sc, hit, g);
    g.normal = dot(g.normal, cur_d) > 0.0f ? -g.normal : g.normal;
    nxt_o = g.pos;
    if (norm2(g.radiance) > kGt1e5) return false;
    if (g.translucency > 0.5f) {
      thr = thr * v3(g.translucency, g.translucency, g.translucency);
      cur_o = g.pos + cur_d * kRayOffset;
      return true;
    }
    // russianRulette_PhotonMapping (SPPM.h:33-52)
    if (depth > 16) return false;
    const float pdf_rus = 0.98f * max3(g.albedo);
    if (rng.next() > pdf_rus) return false;
    PDF *= pdf_rus;
    float Ii, Io;
    if (near1(cur_ix)) { Ii = 1.0f; Io = g.index; }
    else { Ii = cur_ix; Io = 1.0f; }
    FParam p{cur_d, nxt_d, g.normal, Ii, Io, g.rough, g.extinction, g.reflectance};
    if (g.flags & kMatSPPM) {
      const size_t s = base + k;
      store_float4(ph.pos + s, g.pos, cur_ix);
      store_float4(ph.flux + s, flux0 * thr * g.albedo, PDF);
      store_float4(ph.dir + s, cur_d, 1.0f);
      ++k;
    }
    float pdf = 1.0f;
    nxt_d = surface_sample(g.type, rng, p, &pdf);
    if (!is_valid_direction(nxt_d)) return false;
    if (g.flags & kMatOpaque) {
      if (dot(nxt_d, g.normal) < kLt1e6) return false;
    } else {
      nxt_ix = is_reflect(cur_d, nxt_d, g.normal) ? cur_ix : Io;
    }
    p.out = nxt_d;
    pdf = surface_pdf(g.type, p);
    const V3 on = dot(g.normal, nxt_d) > 0.0f ? g.normal : -g.normal;
    nxt_o = nxt_o + on * kRayOffset;
    const float brdf = surface_brdf(g.type, p);
    const float cs = fmaxf(0.0f, fminf(1.0f, dot(nxt_d, on)));
    if (brdf < kLt1e8) return false;
    if (pdf < 0.0f) return false;
    thr = thr * (g.albedo * cs * brdf);
    PDF *= pdf;
    cur_o = nxt_o; cur_d = nxt_d; cur_ix = nxt_ix;
    ++depth;
    return true;
  }

  // Terminator (SPPM.cpp:672): written one past the last stored photon, which
  // leaves slot k as it was; the compactor (SPPM.cpp:812-822) takes slots up to
  // the first invalid one, so a valid stale slot k joins this iteration.
  __device__ __forceinline__ void finish(const IterParams& it, const PhotonSlots& ph, uint32_t* counts) {
    uint32_t n;
    if (it.flags & kFlagFixStaleSlot) {
      const int term = k > 0 ? k : 1;
      if (term < kPhotonSlots) ph.dir[base + term].w = 0.0f;
      n = (uint32_t)term;
    } else {
      const int term = k + 1;
      if (term < kPhotonSlots) ph.dir[base + term].w = 0.0f;
      n = (k == 0 || ph.dir[base + k].w == 0.0f) ? (uint32_t)(k > 0 ? k : 1) : (uint32_t)(k + 1);
    }
    counts[idx] = n;
  }
};

// Persistent photon pass: every lane runs paths back to back, taking the next
// path index (a warp-aggregated atomic on *work) as soon as its path ends, so
// warps stay full however unequal the path lengths.
__global__ void __launch_bounds__(128) k_photon_pass(SceneGPU sc, IterParams it, PhotonSlots ph,
                                                     uint32_t* counts, uint32_t* work, int* err) {
  const unsigned lane = threadIdx.x & 31u;
  PhotonPath path;
  bool active = false, done = false;
  while (true) {
    const unsigned need = __ballot_sync(0xffffffffu, !active && !done);
    if (need) {
      const int leader = __ffs(need) - 1;
      uint32_t first = 0;
      if ((int)lane == leader) first = atomicAdd(work, (uint32_t)__popc(need));
      first = __shfl_sync(0xffffffffu, first, leader);
      if (!active && !done) {
        const uint32_t i = first + (uint32_t)__popc(need & ((1u << lane) - 1u));
        if (i < (uint32_t)it.photons) {
          path.start(sc, it, ph, (int)i);
          active = true;
        } else {
          done = true;
        }
      }
    }
    if (__all_sync(0xffffffffu, done)) break;
    if (active && !path.step(sc, ph, err)) {
      path.finish(it, ph, counts);
      active = false;
    }
  }
}

// ------------------------------------------------------------- photon grid
// Cell edge for this iteration from the mean radius of its hitpoints; resets
// the accumulators for the next iteration's eye pass.
__global__ void k_grid_setup(GridInfo* gi, SceneGPU sc, float cell_scale, float r0) {
  const float mean = gi->r_count ? gi->r_sum / (float)gi->r_count : r0;
  float cell = fmaxf(cell_scale * mean, 1e-6f);
  gi->cell = cell;
  gi->inv_cell = 1.0f / cell;
  gi->origin[0] = sc.lo[0] - cell;
  gi->origin[1] = sc.lo[1] - cell;
  gi->origin[2] = sc.lo[2] - cell;
  gi->r_sum = 0.0f;
  gi->r_count = 0;
}

__global__ void __launch_bounds__(256) k_photon_count(PhotonSlots ph, const uint32_t* counts, int paths, int stride,
                                                      PhotonGrid g, const GridInfo* gi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= paths) return;
  const float ox = gi->origin[0], oy = gi->origin[1], oz = gi->origin[2], inv = gi->inv_cell;
  const uint32_t mask = g.table - 1u;
  const size_t base = (size_t)i * stride;
  const uint32_t n = counts[i];
  for (uint32_t k = 0; k < n; ++k) {
    const float4 p = ph.pos[base + k];
    const uint32_t h = cell_hash(cell_of(p.x, ox, inv), cell_of(p.y, oy, inv), cell_of(p.z, oz, inv), mask);
    g.slot_key[base + k] = h;
    g.slot_rank[base + k] = atomicAdd(g.cell_count + h, 1u);
  }
}

__global__ void __launch_bounds__(256) k_photon_scatter(PhotonSlots ph, const uint32_t* counts, int paths,
                                                        int stride, PhotonGrid g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= paths) return;
  const size_t base = (size_t)i * stride;
  const uint32_t n = counts[i];
  for (uint32_t k = 0; k < n; ++k) {
    const size_t s = base + k;
    const uint32_t dst = g.cell_start[g.slot_key[s]] + g.slot_rank[s];
    g.pos[dst] = ph.pos[s];
    g.flux[dst] = ph.flux[s];
    float4 d = ph.dir[s];
    d.w = __uint_as_float((uint32_t)s);
    g.dir[dst] = d;
  }
}

// ---------------------------------------------------------------- scan
constexpr int kScanBlock = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanBlock * kScanItems;

__global__ void __launch_bounds__(kScanBlock) k_scan_tile(const uint32_t* in, uint32_t* out, uint32_t n,
                                                          uint32_t* block_sums) {
  __shared__ uint32_t warp_tot[kScanBlock / 32];
  const uint32_t tile = blockIdx.x * kScanTile;
  uint32_t v[kScanItems];
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const uint32_t idx = tile + threadIdx.x * kScanItems + k;
    v[k] = idx < n ? in[idx] : 0u;
    sum += v[k];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    uint32_t w = lane < kScanBlock / 32 ? warp_tot[lane] : 0u;
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < kScanBlock / 32) warp_tot[lane] = wi - w;
    if (lane == kScanBlock / 32 - 1 && block_sums) block_sums[blockIdx.x] = wi;
  }
  __syncthreads();
  uint32_t run = warp_tot[wid] + incl - sum;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const uint32_t idx = tile + threadIdx.x * kScanItems + k;
    if (idx < n) out[idx] = run;
    run += v[k];
  }
}

__global__ void __launch_bounds__(kScanBlock) k_scan_add(uint32_t* out, uint32_t n, const uint32_t* block_offsets) {
  const uint32_t tile = blockIdx.x * kScanTile;
  const uint32_t add = block_offsets[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const uint32_t idx = tile + threadIdx.x * kScanItems + k;
    if (idx < n) out[idx] += add;
  }
}

// ----------------------------------------------------------- gather/update
// Query of one hitpoint: photons p with isIncludePoint(p, x - R, x + R)
// (kdtree.h:78-88, SPPM.cpp:424-428) and |p - x|^2 < R^2 (SPPM.cpp:432).
// Each visited cell only counts photons whose own cell it is, so buckets
// shared by several cells through hash collisions are never counted twice.
template <typename F>
__device__ __forceinline__ void for_each_photon_in_ball(const PhotonGrid& g, const GridInfo& gi, V3 x, float R, F&& f) {
  const V3 bmin = x - R * v3(1.f, 1.f, 1.f);
  const V3 bmax = x + R * v3(1.f, 1.f, 1.f);
  const float R2 = R * R;
  const float inv = gi.inv_cell;
  const int x0 = cell_of(bmin.x, gi.origin[0], inv), x1 = cell_of(bmax.x, gi.origin[0], inv);
  const int y0 = cell_of(bmin.y, gi.origin[1], inv), y1 = cell_of(bmax.y, gi.origin[1], inv);
  const int z0 = cell_of(bmin.z, gi.origin[2], inv), z1 = cell_of(bmax.z, gi.origin[2], inv);
  const uint32_t mask = g.table - 1u;
  for (int cz = z0; cz <= z1; ++cz)
    for (int cy = y0; cy <= y1; ++cy)
      for (int cx = x0; cx <= x1; ++cx) {
        const uint32_t h = cell_hash(cx, cy, cz, mask);
        const uint32_t b = __ldg(g.cell_start + h), e = __ldg(g.cell_start + h + 1);
        for (uint32_t j = b; j < e; ++j) {
          const float4 p4 = __ldg(g.pos + j);
          if (cell_of(p4.x, gi.origin[0], inv) != cx || cell_of(p4.y, gi.origin[1], inv) != cy ||
              cell_of(p4.z, gi.origin[2], inv) != cz)
            continue;
          if (bmin.x > p4.x || bmax.x < p4.x || bmin.y > p4.y || bmax.y < p4.y || bmin.z > p4.z || bmax.z < p4.z)
            continue;
          const V3 p = v3(p4.x, p4.y, p4.z);
          if (!(norm2(p - x) < R2)) continue;
          f(j, p4);
        }
      }
}

__global__ void __launch_bounds__(128) k_gather_update(SceneGPU sc, IterParams it, HitpointBuf hp, PhotonGrid g,
                                                       const GridInfo* gip, PixelState st, int32_t* dbg_m,
                                                       float4* dbg_phi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= it.width * it.height) return;
  const float4 hp0 = hp.pos[i];
  if (__float_as_int(hp0.w) != kHitHit) {
    if (dbg_m) { dbg_m[i] = 0; dbg_phi[i] = make_float4(0.f, 0.f, 0.f, 0.f); }
    return;
  }
  const GridInfo gi = *gip;
  const float4 hn = hp.nrm[i], ho = hp.out[i], hw = hp.wgt[i];
  const V3 x = v3(hp0.x, hp0.y, hp0.z), n = v3(hn.x, hn.y, hn.z), out = v3(ho.x, ho.y, ho.z);
  const V3 W = v3(hw.x, hw.y, hw.z);
  const MaterialGPU& m = sc.mats[__float_as_int(ho.w)];
  const int type = m.type;
  const float R = st.r[i];
  int M = 0;
  // Compensated (Kahan) FP32 sum of this iteration's flux.
  float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
  for_each_photon_in_ball(g, gi, x, R, [&](uint32_t j, float4 p4) {
    const float4 f4 = __ldg(g.flux + j);
    const float4 d4 = __ldg(g.dir + j);
    const V3 indir = v3(d4.x, d4.y, d4.z);
    const float Ii = p4.w;
    const float Io = near1(p4.w) ? m.index : 1.0f;
    const V3 nn = dot(indir, n) < 0.0f ? n : -n;
    const FParam p{indir, out, nn, Ii, Io, hn.w, m.extinction, m.reflectance};
    const float brdf = surface_brdf(type, p);
    const V3 add = W * brdf * v3(f4.x, f4.y, f4.z) / f4.w;
    float y, t;
    y = add.x - cx; t = sx + y; cx = (t - sx) - y; sx = t;
    y = add.y - cy; t = sy + y; cy = (t - sy) - y; sy = t;
    y = add.z - cz; t = sz + y; cz = (t - sz) - y; sz = t;
    ++M;
  });
  if (dbg_m) { dbg_m[i] = M; dbg_phi[i] = make_float4(sx, sy, sz, 0.f); }
  if (M > 0) {
    // N/tau/R update (SPPM.cpp:444-449); tau kept in FP64.
    const int N = st.n[i];
    const float a = (float)N + it.alpha * (float)M;
    const float b = (float)(N + M);
    double* tau = st.tau + 3 * (size_t)i;
    const double ad = (double)a, bd = (double)b;
    tau[0] = (tau[0] + (double)sx) * ad / bd;
    tau[1] = (tau[1] + (double)sy) * ad / bd;
    tau[2] = (tau[2] + (double)sz) * ad / bd;
    st.r[i] = R * sqrtf(a / b);
    st.n[i] = (int)((float)N + (float)M * it.alpha);
    st.g[i] += 1;
  }
}

// ---------------------------------------------------------------- resolve
// reconstructImageFromSharedPoints (SPPM.cpp:473-493): normalisation in FP64,
// gamma 1/1.2 in FP32 as the reference applies it.
__global__ void k_resolve(PixelState st, int pixels, double photons_total, double iterations, float4* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= pixels) return;
  const double R = (double)st.r[i];
  const double denom = (photons_total * ((double)st.g[i] + 1e-4) / (1e-4 + iterations)) * (double)kPI * R * R;
  const double* tau = st.tau + 3 * (size_t)i;
  const float lr = (float)(tau[0] / denom), lg = (float)(tau[1] / denom), lb = (float)(tau[2] / denom);
  const float gm = 1.0f / 1.2f;
  out[i] = make_float4(powf(lr, gm), powf(lg, gm), powf(lb, gm), 1.0f);
}

// ------------------------------------------------------------ parity kernels
__global__ void k_trace_closest(SceneGPU sc, const float* rays, int n, int32_t* facet, float* tuv, int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* r = rays + 7 * (size_t)i;
  Hit h;
  if (trace_closest(sc, v3(r[0], r[1], r[2]), v3(r[3], r[4], r[5]), kRayOffset, h, err)) {
    facet[i] = h.facet;
    tuv[3 * i] = h.t; tuv[3 * i + 1] = h.u; tuv[3 * i + 2] = h.v;
  } else {
    facet[i] = -1;
    tuv[3 * i] = FLT_MAX; tuv[3 * i + 1] = 0.f; tuv[3 * i + 2] = 0.f;
  }
}

// rays: N x 8 {org, dir, minT, maxT}
__global__ void k_trace_any(SceneGPU sc, const float* rays, int n, int32_t* hit, int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* r = rays + 8 * (size_t)i;
  hit[i] = trace_any(sc, v3(r[0], r[1], r[2]), v3(r[3], r[4], r[5]), r[6], r[7], err) ? 1 : 0;
}

// hp: xyz position, w radius
__global__ void k_radius_count(const float4* hp, int nh, PhotonGrid g, const GridInfo* gip, int32_t* m,
                               uint32_t* pairs, uint32_t cap, uint32_t* pair_count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nh) return;
  const GridInfo gi = *gip;
  const float4 h = hp[i];
  int M = 0;
  for_each_photon_in_ball(g, gi, v3(h.x, h.y, h.z), h.w, [&](uint32_t j, float4) {
    ++M;
    if (pairs) {
      const uint32_t slot = atomicAdd(pair_count, 1u);
      if (slot < cap) {
        pairs[2 * (size_t)slot] = (uint32_t)i;
        pairs[2 * (size_t)slot + 1] = __float_as_uint(__ldg(g.dir + j).w);
      }
    }
  });
  m[i] = M;
}

inline unsigned blocks_for(size_t n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

void upload_byte_lut(cudaStream_t s) {
  float lut[256];
  for (int b = 0; b < 256; ++b) lut[b] = (float)b / 255.0f;
  cudaMemcpyToSymbolAsync(c_byte_to_unit, lut, sizeof(lut), 0, cudaMemcpyHostToDevice, s);
}

void launch_eye_pass(const SceneGPU& sc, const CameraGPU& cam, const IterParams& it, const float* rr_eye,
                     HitpointBuf hp, PixelState st, GridInfo* gi, int* err, cudaStream_t s) {
  const int n = it.width * it.height;
  k_eye_pass<<<blocks_for(n, 128), 128, 0, s>>>(sc, cam, it, rr_eye[0], rr_eye[1], hp, st, gi, err);
}

void launch_photon_pass(const SceneGPU& sc, const IterParams& it, PhotonSlots ph, uint32_t* counts, uint32_t* work,
                        int resident_blocks, int* err, cudaStream_t s) {
  const unsigned need = blocks_for(it.photons, 128);
  const unsigned grid = resident_blocks > 0 ? std::min<unsigned>(need, (unsigned)resident_blocks) : need;
  cudaMemsetAsync(work, 0, sizeof(uint32_t), s);
  k_photon_pass<<<grid, 128, 0, s>>>(sc, it, ph, counts, work, err);
}

int photon_pass_blocks_per_sm() {
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_photon_pass, 128, 0);
  return b;
}

void upload_tables(const float2* sincos_tab, const float* sqrt1m_tab, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(c_sincos_tab, &sincos_tab, sizeof(sincos_tab), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_sqrt1m_tab, &sqrt1m_tab, sizeof(sqrt1m_tab), 0, cudaMemcpyHostToDevice, s);
}

void launch_grid_setup(GridInfo* gi, const SceneGPU& sc, float cell_scale, float r0, cudaStream_t s) {
  k_grid_setup<<<1, 1, 0, s>>>(gi, sc, cell_scale, r0);
}

void launch_photon_count(PhotonSlots ph, const uint32_t* counts, int paths, int stride, PhotonGrid g,
                         const GridInfo* gi, cudaStream_t s) {
  k_photon_count<<<blocks_for(paths, 256), 256, 0, s>>>(ph, counts, paths, stride, g, gi);
}

void launch_photon_scatter(PhotonSlots ph, const uint32_t* counts, int paths, int stride, PhotonGrid g,
                           cudaStream_t s) {
  k_photon_scatter<<<blocks_for(paths, 256), 256, 0, s>>>(ph, counts, paths, stride, g);
}

uint32_t scan_temp_words(uint32_t n, ScanTemp& t) {
  uint32_t words = 0;
  t.levels = 0;
  uint32_t m = n;
  while (true) {
    const uint32_t nb = (m + kScanTile - 1) / kScanTile;
    t.level_n[t.levels++] = nb;
    words += nb + 1;
    if (nb <= 1) break;
    m = nb;
  }
  return words;
}

int launch_scan(uint32_t* in, uint32_t* out, uint32_t n, ScanTemp& t, cudaStream_t s) {
  int launches = 1;
  // Exclusive scan: tiles, then the tile sums (recursively), then the add-back.
  const uint32_t nb = (n + kScanTile - 1) / kScanTile;
  k_scan_tile<<<nb, kScanBlock, 0, s>>>(in, out, n, t.level[0]);
  uint32_t cur_n = nb;
  int lvl = 0;
  while (cur_n > 1) {
    const uint32_t nb2 = (cur_n + kScanTile - 1) / kScanTile;
    k_scan_tile<<<nb2, kScanBlock, 0, s>>>(t.level[lvl], t.level[lvl], cur_n, t.level[lvl + 1]);
    ++launches;
    cur_n = nb2;
    ++lvl;
  }
  // Level lvl-1 was scanned as one tile and is final; push its offsets down.
  for (int l = lvl - 2; l >= 0; --l) {
    const uint32_t nn = t.level_n[l];
    k_scan_add<<<(nn + kScanTile - 1) / kScanTile, kScanBlock, 0, s>>>(t.level[l], nn, t.level[l + 1]);
    ++launches;
  }
  if (nb > 1) {
    k_scan_add<<<nb, kScanBlock, 0, s>>>(out, n, t.level[0]);
    ++launches;
  }
  return launches;
}

void launch_gather_update(const SceneGPU& sc, const IterParams& it, HitpointBuf hp, PhotonGrid g, const GridInfo* gi,
                          PixelState st, int32_t* dbg_m, float4* dbg_phi, cudaStream_t s) {
  const int n = it.width * it.height;
  k_gather_update<<<blocks_for(n, 128), 128, 0, s>>>(sc, it, hp, g, gi, st, dbg_m, dbg_phi);
}

void launch_resolve(PixelState st, int pixels, double photons_total, double iterations, float4* out, cudaStream_t s) {
  k_resolve<<<blocks_for(pixels, 256), 256, 0, s>>>(st, pixels, photons_total, iterations, out);
}

void launch_trace_closest(const SceneGPU& sc, const float* rays, int n, int32_t* facet, float* tuv, int* err,
                          cudaStream_t s) {
  k_trace_closest<<<blocks_for(n, 128), 128, 0, s>>>(sc, rays, n, facet, tuv, err);
}

void launch_trace_any(const SceneGPU& sc, const float* rays, int n, int32_t* hit, int* err, cudaStream_t s) {
  k_trace_any<<<blocks_for(n, 128), 128, 0, s>>>(sc, rays, n, hit, err);
}

void launch_radius_count(const float4* hp, int nh, PhotonGrid g, const GridInfo* gi, int32_t* m, uint32_t* pairs,
                         uint32_t cap, uint32_t* pair_count, cudaStream_t s) {
  k_radius_count<<<blocks_for(nh, 128), 128, 0, s>>>(hp, nh, g, gi, m, pairs, cap, pair_count);
}

}  // namespace fr
