// SPPM iteration kernels for sm_103a.
//
// One iteration (StochasticProgressivePhotonMapping, SPPM/SPPM/SPPM.cpp:768-848):
//   k_ew_start / k_wave_trace / k_ew_shade / k_ew_tail
//                    createHitpoints + getHitpointInfo  (SPPM.cpp:98-353)
//                    as a wavefront over queues of live paths
//   k_pw_emit / k_wave_trace / k_pw_shade / k_pw_tail
//                    createPhotonMap + generateLightRay (SPPM.cpp:453-680)
//                    as a wavefront over queues of live paths
//   k_grid_setup / k_photon_count / scan / k_photon_scatter
//                    photon cell grid, replacing the photon kd-tree
//                    (SPPM.cpp:809-833, kdtree.h:348-431)
//   k_gather         applyHitPointInfo                  (SPPM.cpp:395-451)
//   k_resolve        reconstructImageFromSharedPoints   (SPPM.cpp:473-493)
// The eye and photon passes draw from independent per-pixel / per-path
// streams, so running the eye pass first gives the same numbers as the
// reference's photon-first order; it lets the grid size its cells from this
// iteration's hitpoint radii.
#include <cuda_runtime.h>
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cstdint>
#include "fr_bsdf.cuh"
#include "fr_grid.cuh"
#include "fr_guide.cuh"
#include "fr_kernels.h"
#include "fr_layout.h"
#include "fr_math.cuh"
#include "fr_trace.cuh"

namespace fr {

// Occupancy floor (blocks of 128 threads per SM) for the trace kernels'
// register allocation, as a __launch_bounds__ minimum: 7 blocks keep them at
// 72 registers with the near/far plane loads of visit_node, which take 80
// otherwise (6 blocks per SM; mixed materials 4.05 ms per iteration against
// 3.98 with the floor).  0 states only the block size.
#ifndef FR_TRACE_MIN_BLOCKS
#define FR_TRACE_MIN_BLOCKS 7
#endif
// k_wave_trace keeps its stack's top entry in registers (1) or pushes every
// entry to the local-memory stack (0).
#ifndef FR_STACK_TOP_REG
#define FR_STACK_TOP_REG 1
#endif
#if FR_TRACE_MIN_BLOCKS > 0
#define FR_TRACE_BOUNDS __launch_bounds__(128, FR_TRACE_MIN_BLOCKS)
#else
#define FR_TRACE_BOUNDS __launch_bounds__(128)
#endif
// The same for the photon pass's shade kernel, which waits on a chain of
// dependent loads (hit, facet record, material, textures).  More resident
// warps did not help: mixed materials 3.55-3.56 ms per iteration with no
// floor (90 registers, 5 blocks per SM), 3.56 with 6 (78), 3.54-3.56 with 7
// (72, 20-byte spills), 3.55-3.57 with 8 (64).  0 states only the block size.
#ifndef FR_PW_SHADE_MIN_BLOCKS
#define FR_PW_SHADE_MIN_BLOCKS 0
#endif
#if FR_PW_SHADE_MIN_BLOCKS > 0
#define FR_PW_SHADE_BOUNDS __launch_bounds__(128, FR_PW_SHADE_MIN_BLOCKS)
#else
#define FR_PW_SHADE_BOUNDS __launch_bounds__(128)
#endif

namespace {

__device__ __forceinline__ bool near1(float s) { return fabsf(s - 1.0f) < kLt1e5; }  // SPPM.h:27-29

// Round skipping (see kPhotonTailMin): the counters of a round are final
// before its kernels start, so every kernel of the round decides alike.
__device__ __forceinline__ bool round_skipped(const PathWave& w, int round) {
  return round > 0 && *(volatile const uint32_t*)(w.qcount + round) < w.min_live;
}
__device__ __forceinline__ int tail_round(const PathWave& w, int rounds) {
  int r = rounds > 0 ? 1 : 0;
  while (r < rounds && *(volatile const uint32_t*)(w.qcount + r) >= w.min_live) ++r;
  return r;
}

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

// Advances the device iteration counter: the first kernel of an iteration, so
// that a captured iteration graph replays unchanged.
__global__ void k_next_step(uint32_t* step) { *step += 1u; }

// ------------------------------------------------------------------ eye pass
// createHitpoints + getHitpointInfo (SPPM.cpp:98-353) as a wavefront: k_ew_start
// makes every camera ray, rounds of k_wave_trace and k_ew_shade advance the
// live paths, k_ew_tail finishes the rest.  Without an environment map a
// path ends at its first SPPM surface (makeHitPoint, SPPM.cpp:79-96): nothing
// after the first hitpoint reaches the image.  With one it goes on, as the
// reference's does (SPPM.cpp:170-173), until it ends or misses the scene.
//
// Path state between kernels (one entry per pixel):
//   a: origin.xyz, ray index of refraction   b: direction.xyz, PDF
//   c: throughput.xyz, camera PDF            d: draw counter, depth, hitpoint stored
struct EyeState {
  V3 o, d, thr;
  float ix, PDF, cam_pdf;
  uint32_t draw;
  int depth;
  int stored;  // isStoredPhoton (SPPM.cpp:170-173)
};

__device__ __forceinline__ uint32_t eye_seed(const IterParams& it, int i) {
  return (uint32_t)i + (uint32_t)(it.width * it.height) * *it.step;  // SPPM.cpp:334
}

__device__ __forceinline__ void load_eye(const PathWave& w, int i, EyeState& s) {
  const float4 a = w.a[i], b = w.b[i], c = w.c[i], d = w.d[i];
  s.o = v3(a.x, a.y, a.z); s.ix = a.w;
  s.d = v3(b.x, b.y, b.z); s.PDF = b.w;
  s.thr = v3(c.x, c.y, c.z); s.cam_pdf = c.w;
  s.draw = __float_as_uint(d.x);
  s.depth = __float_as_int(d.y);
  s.stored = __float_as_int(d.z);
}

__device__ __forceinline__ void store_eye(const PathWave& w, int i, const EyeState& s) {
  w.a[i] = make_float4(s.o.x, s.o.y, s.o.z, s.ix);
  w.b[i] = make_float4(s.d.x, s.d.y, s.d.z, s.PDF);
  w.c[i] = make_float4(s.thr.x, s.thr.y, s.thr.z, s.cam_pdf);
  w.d[i] = make_float4(__uint_as_float(s.draw), __int_as_float(s.depth), __int_as_float(s.stored), 0.f);
}

// Top of the bounce loop (SPPM.cpp:99-122): depth cap and Russian roulette
// with p = exp(4 - depth) above depth 4.  false ends the path.
__device__ __forceinline__ bool eye_top(EyeState& s, Rng& rng, float rr5, float rr6) {
  if (s.depth > 6) return false;
  if (s.depth > 4) {
    const float rus = s.depth == 5 ? rr5 : rr6;
    if (rng.next() > rus) return false;
    s.PDF *= rus;
  }
  return true;
}

// IBL::GetIBLColorFromDirection (IBL.h:122-129) with the SPHERE mapping
// (GetUVFromDirection, IBL.h:96-104; acos of a float there is the double
// ::acos) and LinearSampler::Sample (TextureSampler.h:61-79) on the converted
// texels.
__device__ __forceinline__ V3 env_color(const SceneGPU& sc, V3 dir) {
  float u = 0.0f, v = 0.0f;
  if (!(fabsf(dir.x) < kLt1e6 && fabsf(dir.z) < kLt1e6)) {
    const V3 xz = normalized(v3(dir.x, 0.0f, dir.z));
    const double ax = acos((double)xz.x);
    const double two_pi = (double)(2.0f * kPI);
    u = (float)((xz.z >= 0.0f ? ax : two_pi - ax) / two_pi);
    v = (float)(acos((double)dir.y) / (double)kPI);
  }
  const int W = sc.env_w, H = sc.env_h;
  const int iu = (int)((float)W * u), iv = (int)((float)H * v);
  const int x1 = abs(iu) % W, y1 = abs(iv) % H;
  const int x2 = min(W - 1, x1 + 1), y2 = min(H - 1, y1 + 1);
  const float4* env = reinterpret_cast<const float4*>(sc.env);
  const float4 t00 = env[x1 + y1 * W], t10 = env[x2 + y1 * W];
  const float4 t01 = env[x1 + y2 * W], t11 = env[x2 + y2 * W];
  const float w = fabsf(u * (float)W) - (float)abs(iu);
  const float h = fabsf(v * (float)H) - (float)abs(iv);
  const F4 up = lerp4(F4{t00.x, t00.y, t00.z, t00.w}, 1.0f - w, F4{t10.x, t10.y, t10.z, t10.w}, w);
  const F4 down = lerp4(F4{t01.x, t01.y, t01.z, t01.w}, 1.0f - w, F4{t11.x, t11.y, t11.z, t11.w}, w);
  const F4 c = lerp4(up, 1.0f - h, down, h);
  return v3(c.x, c.y, c.z);
}

// An eye path that leaves the scene (SPPM.cpp:290-300): with an environment
// map, its colour times the throughput over the path pdf and (createHitpoints,
// SPPM.cpp:345) the camera pdf is the pixel's direct light, added to the
// pixel's sum when its squared norm exceeds 1e-8 (applyHitPointInfo,
// SPPM.cpp:411-414).  Returns the hitpoint type the path ends with.
__device__ __forceinline__ int eye_miss(const SceneGPU& sc, const HitpointBuf& hp, const PixelState& st, int i,
                                        const EyeState& s) {
  if (sc.env) {
    const V3 dl = ((env_color(sc, s.d) * s.thr) / s.PDF) / s.cam_pdf;
    hp.dl[i] = make_float4(dl.x, dl.y, dl.z, 0.0f);
    if (norm2(dl) > kGt1e8) {
      const float4 a = st.dl[i];
      st.dl[i] = make_float4(a.x + dl.x, a.y + dl.y, a.z + dl.z, __int_as_float(__float_as_int(a.w) + 1));
    }
  }
  return s.stored ? kHitHit : kHitOnlyDirect;
}

// The rest of one pass after the closest hit (SPPM.cpp:123-305).  Returns
// kHitHit after writing a hitpoint, kHitNone when the path ends without one,
// and -1 when it goes on.
template <bool kEndDegenerate>
__device__ __forceinline__ int eye_shade(const SceneGPU& sc, const HitpointBuf& hp, int i, EyeState& s, Rng& rng,
                                         const Hit& hit, float rr5, float rr6) {
  Geom g;
  calc_geometry(sc, hit, g);
  g.normal = dot(g.normal, s.d) > 0.0f ? -g.normal : g.normal;
  V3 nxt_o = g.pos;
  if (g.translucency > 0.5f) {
    s.thr = s.thr * v3(g.translucency, g.translucency, g.translucency);
    s.o = g.pos + s.d * kRayOffset;
    return eye_top(s, rng, rr5, rr6) ? -1 : (s.stored ? kHitHit : kHitNone);
  }
  if ((g.flags & kMatSPPM) && !s.stored) {
    const V3 wgt = (s.thr / s.PDF) / s.cam_pdf;
    store_float4(hp.pos + i, g.pos, __int_as_float(kHitHit));
    store_float4(hp.nrm + i, g.normal, g.rough);
    store_float4(hp.out + i, -s.d, __int_as_float(g.mat));
    store_float4(hp.wgt + i, wgt, __int_as_float(hit.facet));
    s.stored = 1;
    if (!sc.env) return kHitHit;
  }
  // How the path ends from here: with its hitpoint if it made one.
  const int end = s.stored ? kHitHit : kHitNone;
  float Ii, Io;
  if (near1(s.ix)) { Ii = 1.0f; Io = g.index; }
  else { Ii = s.ix; Io = 1.0f; }
  FParam p{s.d, s.d, g.normal, Ii, Io, g.rough, g.extinction, g.reflectance};
  float pdf = 1.0f;
  const V3 nd = surface_sample(g.type, rng, p, &pdf);
  if (!is_valid_direction(nd)) return end;
  float nix = s.ix;
  if (g.flags & kMatOpaque) {
    if (dot(nd, g.normal) < kLt1e6) return end;
  } else {
    const bool reflect = !(dot(nd, g.normal) < 0.0f);
    nix = reflect ? s.ix : Io;
  }
  p.out = nd;
  pdf = surface_pdf(g.type, p);
  const V3 on = dot(g.normal, nd) > 0.0f ? g.normal : -g.normal;
  nxt_o = nxt_o + on * kRayOffset;
  const float brdf = surface_brdf(g.type, p);
  const float cs = fmaxf(0.0f, fminf(1.0f, dot(nd, on)));
  if (brdf < kLt1e8) return end;
  if (pdf < 0.0f) return end;
  // The reference goes on with a NaN BSDF value or pdf, or a zero pdf, which
  // gives the hitpoint a NaN or infinite weight; the flag ends such paths.
  if (kEndDegenerate && !(brdf >= kLt1e8 && pdf > 0.0f)) return end;
  s.thr = s.thr * (g.albedo * cs * brdf);
  s.PDF *= pdf;
  s.o = nxt_o; s.d = nd; s.ix = nix;
  ++s.depth;
  return eye_top(s, rng, rr5, rr6) ? -1 : end;
}

// Appends i to queue t of T (queue t starts at q + t * cap, its length is
// count[t]) when 0 <= t < T, with one global atomic per queue per block: the
// counters are few addresses that every block of a launch updates.  Every
// thread of the block calls it, the same number of times.
template <int T>
__device__ __forceinline__ void block_append(uint32_t* q, size_t cap, uint32_t* count, int t, uint32_t i) {
  __shared__ uint32_t s_warp[32][T];
  __shared__ uint32_t s_base[T];
  const unsigned lane = threadIdx.x & 31u, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned mine = 0;
#pragma unroll
  for (int u = 0; u < T; ++u) {
    const unsigned m = __ballot_sync(0xffffffffu, t == u);
    if (t == u) mine = m;
    if (lane == 0) s_warp[wid][u] = (uint32_t)__popc(m);
  }
  __syncthreads();
  if (threadIdx.x < (unsigned)T) {
    const int u = (int)threadIdx.x;
    uint32_t run = 0;
    for (unsigned v = 0; v < nw; ++v) {
      const uint32_t c = s_warp[v][u];
      s_warp[v][u] = run;
      run += c;
    }
    s_base[u] = run ? atomicAdd(count + u, run) : 0u;
  }
  __syncthreads();
  if (t >= 0 && t < T) q[(size_t)t * cap + s_base[t] + s_warp[wid][t] + (uint32_t)__popc(mine & ((1u << lane) - 1u))] = i;
  __syncthreads();
}

// Sum over the block of v and n into *sum and *cnt (one atomic pair per
// block).  Every thread of the block calls it.
__device__ __forceinline__ void block_add(float* sum, uint32_t* cnt, float v, uint32_t n) {
  __shared__ float s_v[32];
  __shared__ uint32_t s_n[32];
  const unsigned lane = threadIdx.x & 31u, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v += __shfl_down_sync(0xffffffffu, v, o);
    n += __shfl_down_sync(0xffffffffu, n, o);
  }
  if (lane == 0) {
    s_v[wid] = v;
    s_n[wid] = n;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float tv = 0.0f;
    uint32_t tn = 0;
    for (unsigned k = 0; k < nw; ++k) {
      tv += s_v[k];
      tn += s_n[k];
    }
    if (tn) {
      atomicAdd(sum, tv);
      atomicAdd(cnt, tn);
    }
  }
  __syncthreads();
}

// End of an eye path: the hit code of a pixel without a hitpoint, the list
// of this iteration's hitpoints, and their radius summed for the grid's cell
// size.  Every thread of the block calls it.
__device__ __forceinline__ void eye_finish(const HitpointBuf& hp, const PixelState& st, GridInfo* gi, bool ended,
                                           int i, int hit_type) {
  float rs = 0.0f;
  uint32_t cnt = 0;
  if (ended) {
    if (hit_type == kHitHit) {
      rs = st.r[i];
      cnt = 1;
    } else {
      store_float4(hp.pos + i, v3(0.f, 0.f, 0.f), __int_as_float(hit_type));
    }
  }
  block_append<1>(hp.list, 0, hp.list_count, cnt ? 0 : -1, (uint32_t)i);
  block_add(&gi->r_sum, &gi->r_count, rs, cnt);
}

// Every pixel's path is live after its camera ray, so the first queue is
// the identity (no atomics).
__global__ void __launch_bounds__(128) k_ew_start(CameraGPU cam, IterParams it, PathWave w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int npix = it.width * it.height;
  if (i == 0) w.qcount[0] = (uint32_t)npix;
  if (i < npix) {
    w.queue[0][i] = (uint32_t)i;
    const int px = i % it.width, py = i / it.width;
    const float u = (float)px / (float)it.width;
    const float v = (float)py / (float)it.height;
    Rng rng(eye_seed(it, i));
    const float s0 = rng.next(), s1 = rng.next(), s2 = rng.next();
    EyeState s;
    camera_ray(cam, u, v, s0, s1, s2, s.o, s.d, s.cam_pdf);
    s.ix = 1.0f;
    s.PDF = 1.0f;
    s.thr = v3(1.f, 1.f, 1.f);
    s.depth = 0;
    s.stored = 0;
    s.draw = rng.draw;
    store_eye(w, i, s);
  }
}

// Closest hit of every path in queue `round`, for queues of coherent rays
// (camera rays in pixel order): each warp takes 32 consecutive entries.
template <bool kWT>
__global__ void FR_TRACE_BOUNDS k_wave_trace_static(SceneGPU sc, PathWave w, int round, int* err) {
  if (round_skipped(w, round)) return;
  const uint32_t n = *(volatile uint32_t*)(w.qcount + round);
  const uint32_t* q = w.queue[round & 1];
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const uint32_t i = q[j];
    const float4 a = w.a[i], b = w.b[i];
    Hit h;
    if (trace_closest<kWT>(sc, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), kRayOffset, h, err))
      w.hit[i] = make_float4(h.u, h.v, __int_as_float(h.tri), __int_as_float(h.facet));
    else
      w.hit[i] = make_float4(0.f, 0.f, __int_as_float(-1), __int_as_float(-1));
  }
}

// Closest hit of every path in queue `round` (eye or photon wave), with
// dynamic ray fetch: a lane whose ray is done takes the next queue entry at
// once instead of idling until the warp's slowest ray ends.  A warp claims
// queue entries 32 at a time with one atomic and hands them to its idle lanes.
// The traversal is trace_closest's (fr_trace.cuh), one node visit or leaf per
// loop pass, so the hits are the same.
template <bool kWT>
__global__ void FR_TRACE_BOUNDS k_wave_trace(SceneGPU sc, PathWave w, int round, int* err) {
  if (round_skipped(w, round)) return;
  const uint32_t n = *(volatile uint32_t*)(w.qcount + round);
  const uint32_t* q = w.queue[round & 1];
  uint32_t* fetch = w.tfetch + round;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  // Warp-uniform batch of claimed queue entries [pool, pool + left).
  uint32_t pool = 0, left = 0;
  bool exhausted = false;
  // Per-lane traversal state.
  bool active = false;
  uint32_t i = 0;
  V3 org = v3(0.f, 0.f, 0.f), dir = org;
  RayPre r{};
  float tbest = FLT_MAX, bu = 0.f, bv = 0.f, tref = 0.f;
  int32_t best_tri = -1, best_facet = -1;
  uint32_t ref = 0;
  int sp = 0;
  uint2 stack[kTraversalStack];
#if FR_STACK_TOP_REG
  // The stack's top entry in registers: the entry pushed last is the nearest
  // of a node's remaining children, the one popped next after a leaf.
  uint2 top = make_uint2(0u, 0u);
  bool has_top = false;
#endif
  while (true) {
    unsigned idle = __ballot_sync(0xffffffffu, !active);
    while (idle && !exhausted) {
      if (left == 0) {
        uint32_t b = 0;
        if (lane == 0) b = atomicAdd(fetch, 32u);
        b = __shfl_sync(0xffffffffu, b, 0);
        if (b >= n) {
          exhausted = true;
          break;
        }
        pool = b;
        left = min(32u, n - b);
      }
      const unsigned take = min((unsigned)__popc(idle), left);
      const unsigned rank = (unsigned)__popc(idle & below);
      if (!active && rank < take) {
        i = q[pool + rank];
        const float4 a4 = w.a[i], b4 = w.b[i];
        org = v3(a4.x, a4.y, a4.z);
        dir = v3(b4.x, b4.y, b4.z);
        r = ray_pre(org, dir);
        tbest = FLT_MAX;
        best_tri = best_facet = -1;
        bu = bv = 0.f;
        ref = 0;
        tref = kRayOffset;
        sp = 0;
#if FR_STACK_TOP_REG
        has_top = false;
#endif
        active = true;
      }
      pool += take;
      left -= take;
      idle = __ballot_sync(0xffffffffu, !active);
    }
    if (!__any_sync(0xffffffffu, active)) break;
    if (!active) continue;
    // One pass of trace_closest's loop.
    bool pop = true;
    if (tref <= tbest) {
      if (!(ref & kLeafBit)) {
        NodeVisit nv;
        visit_node(sc.nodes, ref, r, kRayOffset, tbest, nv);
        sort8(nv.key);
        if (nv.key[0] != 0xFFFFFFFFu) {
          int cnt = 1;
#pragma unroll
          for (int k = 1; k < 8; ++k) cnt += nv.key[k] != 0xFFFFFFFFu;
#if FR_STACK_TOP_REG
          if (sp + (has_top ? 1 : 0) + cnt - 1 > kTraversalStack) {
            atomicOr(err, kErrStack);
            best_tri = -1;
            sp = 0;
            has_top = false;
          } else {
#pragma unroll
            for (int k = 7; k >= 1; --k)
              if (k < cnt) {
                if (has_top) stack[sp++] = top;
                top = make_uint2(child_ref(nv, nv.key[k] & 7u), nv.key[k] & ~7u);
                has_top = true;
              }
#else
          if (sp + cnt - 1 > kTraversalStack) {
            atomicOr(err, kErrStack);
            best_tri = -1;
            sp = 0;
          } else {
#pragma unroll
            for (int k = 7; k >= 1; --k)
              if (k < cnt) stack[sp++] = make_uint2(child_ref(nv, nv.key[k] & 7u), nv.key[k] & ~7u);
#endif
            ref = child_ref(nv, nv.key[0] & 7u);
            tref = __uint_as_float(nv.key[0] & ~7u);
            pop = false;
          }
        }
      } else {
        const int first = (int)(ref & kLeafFirstMask);
        const int count = (int)((ref >> kLeafCountShift) & 0xFu) + 1;
        for (int k = 0; k < count; ++k) {
          const TriGPU tr = load_tri(sc.tris, first + k);
          float t, u, v;
          if (tri_test<kWT>(sc, org, dir, tr, first + k, t, u, v) && t > kRayOffset) {
            const int32_t facet = __float_as_int(tr.v0[3]);
            if (t < tbest || (t == tbest && facet > best_facet)) {
              tbest = t; bu = u; bv = v; best_tri = first + k; best_facet = facet;
            }
          }
        }
      }
    }
    if (pop) {
#if FR_STACK_TOP_REG
      const bool empty = !has_top && sp == 0;
#else
      const bool empty = sp == 0;
#endif
      if (empty) {
        w.hit[i] = best_tri >= 0 ? make_float4(bu, bv, __int_as_float(best_tri), __int_as_float(best_facet))
                                 : make_float4(0.f, 0.f, __int_as_float(-1), __int_as_float(-1));
        active = false;
      } else {
#if FR_STACK_TOP_REG
        const uint2 e = has_top ? top : stack[--sp];
        has_top = false;
#else
        const uint2 e = stack[--sp];
#endif
        ref = e.x;
        tref = __uint_as_float(e.y);
      }
    }
  }
}

// The paths of queue `round` sorted into the queues of their hit surface's
// type (misses last), so that each warp of the shade kernel runs one
// surface's code.
__global__ void __launch_bounds__(256) k_wave_sort(SceneGPU sc, PathWave w, int round) {
  if (round_skipped(w, round)) return;  // its shade kernel then finds no paths
  const uint32_t n = *(volatile uint32_t*)(w.qcount + round);
  const uint32_t* q = w.queue[round & 1];
  uint32_t* mc = w.mcount + round * kShadeQueues;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t n_round = (n + stride - 1) / stride * stride;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_round; j += stride) {
    int type = -1;
    uint32_t i = 0;
    if (j < n) {
      i = q[j];
      const int facet = __float_as_int(w.hit[i].w);
      // The demo's further surfaces (types 4-7) share the four queues (type mod 4).
      type = facet >= 0 ? (sc.mats[sc.shade[facet].attr].type & 3) : kShadeQueues - 1;
    }
    block_append<kShadeQueues>(w.mq, w.cap, mc, type, i);
  }
}

// Entry k of this round's shade work: the queues of the surface types one
// after another.
struct ShadeQueues {
  uint32_t off[kShadeQueues + 1];
  __device__ __forceinline__ ShadeQueues(const PathWave& w, int round) {
    off[0] = 0;
#pragma unroll
    for (int t = 0; t < kShadeQueues; ++t)
      off[t + 1] = off[t] + *(volatile uint32_t*)(w.mcount + round * kShadeQueues + t);
  }
  __device__ __forceinline__ uint32_t total() const { return off[kShadeQueues]; }
  __device__ __forceinline__ uint32_t path(const PathWave& w, uint32_t k) const {
    int t = 0;
#pragma unroll
    for (int u = 1; u < kShadeQueues; ++u) t += k >= off[u];
    return w.mq[(size_t)t * w.cap + (k - off[t])];
  }
};

__device__ __forceinline__ bool wave_hit(const PathWave& w, uint32_t i, Hit& h) {
  const float4 hv = w.hit[i];
  h.t = 0.f; h.u = hv.x; h.v = hv.y; h.tri = __float_as_int(hv.z); h.facet = __float_as_int(hv.w);
  return h.tri >= 0;
}

template <bool kEndDegenerate>
__global__ void __launch_bounds__(128) k_ew_shade(SceneGPU sc, IterParams it, float rr5, float rr6, PathWave w,
                                                  HitpointBuf hp, PixelState st, GridInfo* gi, int round) {
  const ShadeQueues sq(w, round);
  const uint32_t n = sq.total();
  uint32_t* qn = w.queue[(round + 1) & 1];
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t n_round = (n + stride - 1) / stride * stride;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_round; j += stride) {
    bool keep = false, ended = false;
    int hit_type = kHitNone;
    uint32_t i = 0;
    if (j < n) {
      i = sq.path(w, j);
      EyeState s;
      load_eye(w, (int)i, s);
      Hit h;
      if (!wave_hit(w, i, h)) {
        hit_type = eye_miss(sc, hp, st, (int)i, s);  // SPPM.cpp:290-300
        ended = true;
      } else {
        Rng rng(eye_seed(it, (int)i));
        rng.seek(s.draw);
        const int r = eye_shade<kEndDegenerate>(sc, hp, (int)i, s, rng, h, rr5, rr6);
        if (r < 0) {
          s.draw = rng.draw;
          store_eye(w, (int)i, s);
          keep = true;
        } else {
          hit_type = r;
          ended = true;
        }
      }
    }
    eye_finish(hp, st, gi, ended, (int)i, hit_type);
    block_append<1>(qn, 0, w.qcount + round + 1, keep ? 0 : -1, i);
  }
}

// Eye paths alive after the last wavefront round, each run to its end.
template <bool kEndDegenerate, bool kWT>
__global__ void __launch_bounds__(128) k_ew_tail(SceneGPU sc, IterParams it, float rr5, float rr6, PathWave w,
                                                 HitpointBuf hp, PixelState st, GridInfo* gi, int rounds, int* err) {
  const int round = tail_round(w, rounds);
  const uint32_t n = *(volatile uint32_t*)(w.qcount + round);
  const uint32_t* q = w.queue[round & 1];
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t n_round = (n + stride - 1) / stride * stride;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_round; j += stride) {
    int hit_type = kHitNone;
    int i = 0;
    if (j < n) {
      i = (int)q[j];
      EyeState s;
      load_eye(w, i, s);
      Rng rng(eye_seed(it, i));
      rng.seek(s.draw);
      while (true) {
        Hit h;
        if (!trace_closest<kWT>(sc, s.o, s.d, kRayOffset, h, err)) {
          hit_type = eye_miss(sc, hp, st, i, s);
          break;
        }
        const int r = eye_shade<kEndDegenerate>(sc, hp, i, s, rng, h, rr5, rr6);
        if (r >= 0) {
          hit_type = r;
          break;
        }
      }
    }
    eye_finish(hp, st, gi, j < n, i, hit_type);
  }
}

// --------------------------------------------------------------- photon pass
// createPhotonMap (SPPM.cpp:495-680) as a wavefront.  k_pw_emit starts every
// path (generateLightRay, SPPM.cpp:453-471, and the light-surface photon,
// SPPM.cpp:530-540); then rounds of k_pw_trace (closest hit of every live
// path) and k_pw_shade (the rest of one pass of the bounce loop,
// SPPM.cpp:548-671) over a compacted queue of live paths; k_pw_tail finishes
// the few paths still alive after the last round.  Every path keeps its own
// Philox stream, so the order in which paths are processed changes nothing.
//
// Path state between kernels (one entry per path):
//   a: origin.xyz, ray index of refraction     b: direction.xyz, PDF
//   c: throughput.xyz, flux0.x                 d: flux0.yz, draw counter, k | loop << 8 | depth << 16
// At the top of each loop pass the reference's NextRay equals CurrentRay
// (SPPM.cpp:669), so only the current ray is kept.
struct PhotonState {
  V3 o, d, thr, flux0;
  float ix, PDF;
  uint32_t draw;
  int k, loop, depth;
};

__device__ __forceinline__ uint32_t photon_seed(const IterParams& it, int i) {
  return (uint32_t)i + 135u + *it.step * (uint32_t)it.photons;  // SPPM.cpp:520
}

__device__ __forceinline__ void load_state(const PathWave& w, int i, PhotonState& s) {
  const float4 a = w.a[i], b = w.b[i], c = w.c[i], d = w.d[i];
  s.o = v3(a.x, a.y, a.z); s.ix = a.w;
  s.d = v3(b.x, b.y, b.z); s.PDF = b.w;
  s.thr = v3(c.x, c.y, c.z);
  s.flux0 = v3(c.w, d.x, d.y);
  s.draw = __float_as_uint(d.z);
  const uint32_t m = __float_as_uint(d.w);
  s.k = (int)(m & 0xFFu); s.loop = (int)((m >> 8) & 0xFFu); s.depth = (int)(m >> 16);
}

__device__ __forceinline__ void store_state(const PathWave& w, int i, const PhotonState& s) {
  w.a[i] = make_float4(s.o.x, s.o.y, s.o.z, s.ix);
  w.b[i] = make_float4(s.d.x, s.d.y, s.d.z, s.PDF);
  w.c[i] = make_float4(s.thr.x, s.thr.y, s.thr.z, s.flux0.x);
  w.d[i] = make_float4(s.flux0.y, s.flux0.z, __uint_as_float(s.draw),
                       __uint_as_float((uint32_t)s.k | ((uint32_t)s.loop << 8) | ((uint32_t)s.depth << 16)));
}

// A point on a light (generateLightRay, SPPM.cpp:453-466): the light by its
// flux alias table (LightSampler.h:86), the point (textured: the 1000-point
// emission table, LightSampler.cpp:30-66; else uniform, Sampling.cpp:339-349),
// its radiance and area pdf; u, v are the point's barycentrics.
struct LightPoint {
  V3 pos, rad, ln;
  float pdf_area, u, v;
};

__device__ __forceinline__ void light_point(const SceneGPU& sc, Rng& rng, LightPoint& lp) {
  const uint32_t lb = (uint32_t)(((uint64_t)(uint32_t)sc.num_lights * rng.next_u24()) >> 24);
  const LightGPU& bin = sc.lights[lb];
  const int li = rng.next() < bin.alias_prob ? bin.alias_left : bin.alias_right;
  const LightGPU& L = sc.lights[li];
  const V3 P0 = v3(L.p0), P1 = v3(L.p1), P2 = v3(L.p2);
  if (L.textured) {
    const EmitEntry* tab = sc.emit + L.emit_offset;
    const uint32_t eb = (uint32_t)(((uint64_t)kEmitSamples * rng.next_u24()) >> 24);
    const int ei = rng.next() < tab[eb].prob ? tab[eb].left : tab[eb].right;
    const EmitEntry& e = tab[ei];
    lp.pos = e.uvw[0] * P0 + e.uvw[1] * P1 + (1.0f - e.uvw[0] - e.uvw[1]) * P2;
    lp.rad = v3(e.L);
    lp.pdf_area = e.pdf;
    lp.u = e.uvw[0];
    lp.v = e.uvw[1];
  } else {
    float u = rng.next(), v = rng.next();
    if (v > u) { u *= 0.5f; v -= u; }
    else { v *= 0.5f; u -= v; }
    lp.pos = u * P0 + v * P1 + (1.0f - u - v) * P2;
    lp.rad = v3(L.radiance);
    lp.pdf_area = L.pdf_point;
    lp.u = u;
    lp.v = v;
  }
  lp.pdf_area *= L.pdf_light;
  lp.ln = v3(L.normal);
}

// The photon path from its light point and direction (generateLightRay,
// SPPM.cpp:466-470) and the light-surface photon in slot 0 (SPPM.cpp:530-540).
__device__ __forceinline__ size_t slot_index(const PhotonSlots& ph, int i, int k) {
  return (size_t)k * ph.paths + (size_t)i;
}

__device__ __forceinline__ void photon_launch(const PhotonSlots& ph, int i, const LightPoint& lp, V3 d, float pdf_dir,
                                              const Rng& rng, PhotonState& s) {
  const size_t base = slot_index(ph, i, 0);
  const V3 rad = lp.rad * fminf(1.0f, fmaxf(0.0f, dot(lp.ln, d)));
  s.o = lp.pos + lp.ln * kRayOffset;
  s.d = normalized(d);
  s.flux0 = rad;
  s.PDF = lp.pdf_area * pdf_dir;
  s.thr = v3(1.f, 1.f, 1.f);
  store_float4(ph.pos + base, s.o, 1.0f);
  store_float4(ph.flux + base, s.flux0 * s.thr * kPI, s.PDF);
  store_float4(ph.dir + base, s.d, 1.0f);
  s.ix = 1.0f;
  s.k = s.loop = s.depth = 0;
  s.draw = rng.draw;
}

// generateLightRay (SPPM.cpp:453-471) with cosine-sampled direction.
__device__ __forceinline__ void photon_start(const SceneGPU& sc, const IterParams& it, const PhotonSlots& ph, int i,
                                             PhotonState& s) {
  Rng rng(photon_seed(it, i));
  LightPoint lp;
  light_point(sc, rng, lp);
  float pdf_dir = 1.0f;
  const V3 d = cos_sampling(rng, lp.ln, &pdf_dir);
  photon_launch(ph, i, lp, d, pdf_dir, rng, s);
}

// Checks at the top of each pass of the bounce loop (SPPM.cpp:549-554);
// false ends the path.
__device__ __forceinline__ bool photon_top(PhotonState& s) {
  if (s.loop++ > 32 || s.k >= kPhotonSlots - 1) return false;
  return !(s.thr.x < kLt1e8 || s.thr.y < kLt1e8 || s.thr.z < kLt1e8);
}

// The rest of one pass after the closest hit (SPPM.cpp:556-670); false ends
// the path.
template <bool kEndDegenerate>
__device__ __forceinline__ bool photon_shade(const SceneGPU& sc, const IterParams& it, const PhotonSlots& ph, int i,
                                             PhotonState& s, const Hit& hit) {
  Rng rng(photon_seed(it, i));
  rng.seek(s.draw);
  Geom g;
  calc_geometry(sc, hit, g);
  g.normal = dot(g.normal, s.d) > 0.0f ? -g.normal : g.normal;
  V3 nxt_o = g.pos;
  if (norm2(g.radiance) > kGt1e5) return false;
  if (g.translucency > 0.5f) {
    s.thr = s.thr * v3(g.translucency, g.translucency, g.translucency);
    s.o = g.pos + s.d * kRayOffset;
    return true;
  }
  // russianRulette_PhotonMapping (SPPM.h:33-52)
  if (s.depth > 16) return false;
  const float pdf_rus = 0.98f * max3(g.albedo);
  if (rng.next() > pdf_rus) return false;
  s.PDF *= pdf_rus;
  float Ii, Io;
  if (near1(s.ix)) { Ii = 1.0f; Io = g.index; }
  else { Ii = s.ix; Io = 1.0f; }
  FParam p{s.d, s.d, g.normal, Ii, Io, g.rough, g.extinction, g.reflectance};
  if (g.flags & kMatSPPM) {
    const size_t slot = slot_index(ph, i, s.k);
    store_float4(ph.pos + slot, g.pos, s.ix);
    store_float4(ph.flux + slot, s.flux0 * s.thr * g.albedo, s.PDF);
    store_float4(ph.dir + slot, s.d, 1.0f);
    ++s.k;
  }
  float pdf = 1.0f;
  const V3 nd = surface_sample(g.type, rng, p, &pdf);
  s.draw = rng.draw;
  if (!is_valid_direction(nd)) return false;
  float nix = s.ix;
  if (g.flags & kMatOpaque) {
    if (dot(nd, g.normal) < kLt1e6) return false;
  } else {
    nix = is_reflect(s.d, nd, g.normal) ? s.ix : Io;
  }
  p.out = nd;
  pdf = surface_pdf(g.type, p);
  const V3 on = dot(g.normal, nd) > 0.0f ? g.normal : -g.normal;
  nxt_o = nxt_o + on * kRayOffset;
  const float brdf = surface_brdf(g.type, p);
  const float cs = fmaxf(0.0f, fminf(1.0f, dot(nd, on)));
  if (brdf < kLt1e8) return false;
  if (pdf < 0.0f) return false;
  if (kEndDegenerate && !(brdf >= kLt1e8 && pdf > 0.0f)) return false;  // as in eye_shade
  s.thr = s.thr * (g.albedo * cs * brdf);
  s.PDF *= pdf;
  // The path's weight is kept as two running products (flux and PDF) that
  // grow together bounce by bounce: sharp glass lobes multiply both by ~1e3,
  // so a long path inside a cluster of rough dielectrics overflows both to
  // infinity and its photons then carry inf / inf.  Such a path ends here.
  if (kEndDegenerate) {
    const V3 f = s.flux0 * s.thr;
    if (!(isfinite(s.PDF) && isfinite(f.x) && isfinite(f.y) && isfinite(f.z))) return false;
  }
  s.o = nxt_o; s.d = nd; s.ix = nix;
  ++s.depth;
  return true;
}

// Terminator (SPPM.cpp:672): written one past the last stored photon, which
// leaves slot k as it was; the compactor (SPPM.cpp:812-822) takes slots up to
// the first invalid one, so a valid stale slot k joins this iteration.
__device__ __forceinline__ void photon_finish(const IterParams& it, const PhotonSlots& ph, uint32_t* counts, int i,
                                              int k) {
  uint32_t n;
  if (it.flags & kFlagFixStaleSlot) {
    const int term = k > 0 ? k : 1;
    if (term < kPhotonSlots) ph.dir[slot_index(ph, i, term)].w = 0.0f;
    n = (uint32_t)term;
  } else {
    const int term = k + 1;
    if (term < kPhotonSlots) ph.dir[slot_index(ph, i, term)].w = 0.0f;
    n = (k == 0 || ph.dir[slot_index(ph, i, k)].w == 0.0f) ? (uint32_t)(k > 0 ? k : 1) : (uint32_t)(k + 1);
  }
  counts[i] = n;
}

// A new path passes the bounce loop's first checks (loop 0, no photon
// stored, throughput 1), so every path is live and the first queue is the
// identity (no atomics).
__global__ void __launch_bounds__(128) k_pw_emit(SceneGPU sc, IterParams it, PhotonSlots ph, PathWave w,
                                                 uint32_t* counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) w.qcount[0] = (uint32_t)it.photons;
  if (i < it.photons) {
    PhotonState s;
    photon_start(sc, it, ph, i, s);
    photon_top(s);  // loop 0 -> 1; true for a new path
    store_state(w, i, s);
    w.queue[0][i] = (uint32_t)i;
  }
}

// Guided emission: the light point as in k_pw_emit, then the direction from
// the defensive mixture f * cosine + (1 - f) * guide, the guide's lobes coming
// from the MLP evaluated for the CTA's 128 paths on the tensor cores; the
// photon's pdf is the mixture's.  Also records each path's guide inputs and
// direction (training data) and clears its importance.
constexpr int kEmitSmW = 0;                                  // W2, W3, W4 tiles
constexpr int kEmitSmH = kTileW2T;                           // 128 x 64 activations
constexpr int kEmitSmP1 = kEmitSmH + 128 * 64 * 2;           // W1, b1
constexpr int kEmitSmB = kEmitSmP1 + kOffW2 * 4;             // b2, b3, b4
constexpr int kEmitSmMisc = kEmitSmB + (64 + 64 + 48) * 4;
constexpr int kEmitSmem = kEmitSmMisc + 64;

__global__ void __launch_bounds__(128) k_pw_emit_guided(SceneGPU sc, IterParams it, PhotonSlots ph, PathWave w,
                                                        uint32_t* counts, GuideGPU g) {
  extern __shared__ __align__(1024) uint8_t sm[];
  uint8_t* W = sm + kEmitSmW;
  uint8_t* H = sm + kEmitSmH;
  float* p1 = reinterpret_cast<float*>(sm + kEmitSmP1);
  float* bias = reinterpret_cast<float*>(sm + kEmitSmB);
  uint32_t* tbase = reinterpret_cast<uint32_t*>(sm + kEmitSmMisc);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + kEmitSmMisc + 8);
  const uint32_t t = threadIdx.x, warp = t >> 5;
  const int i = (int)(blockIdx.x * blockDim.x + t);
  const bool live = i < it.photons;
  if (i == 0) w.qcount[0] = (uint32_t)it.photons;
  for (uint32_t e = t; e < (uint32_t)kTileW2T / 16; e += 128)
    reinterpret_cast<uint4*>(W)[e] = reinterpret_cast<const uint4*>(g.emit_tiles)[e];
  for (uint32_t e = t; e < (uint32_t)kOffW2; e += 128) p1[e] = g.emit_params[e];
  for (uint32_t e = t; e < 64; e += 128) {
    bias[e] = g.emit_params[kOffB2 + e];
    bias[64 + e] = g.emit_params[kOffB3 + e];
  }
  for (uint32_t e = t; e < 48; e += 128) bias[128 + e] = g.emit_params[kOffB4 + e];
  Rng rng(photon_seed(it, i));
  LightPoint lp;
  float x[kGuideIn] = {0.f, 0.f, 0.f, 0.f, 0.f};
  if (live) {
    counts[i] = 0;
    light_point(sc, rng, lp);
    // Inputs: position scaled to [-1, 1] over the scene bounds, barycentrics.
    x[0] = 2.0f * (lp.pos.x - sc.lo[0]) / fmaxf(sc.hi[0] - sc.lo[0], 1e-20f) - 1.0f;
    x[1] = 2.0f * (lp.pos.y - sc.lo[1]) / fmaxf(sc.hi[1] - sc.lo[1], 1e-20f) - 1.0f;
    x[2] = 2.0f * (lp.pos.z - sc.lo[2]) / fmaxf(sc.hi[2] - sc.lo[2], 1e-20f) - 1.0f;
    x[3] = lp.u;
    x[4] = lp.v;
  }
  guide_layer1(p1, x, H, t);
  if (t == 0) tc::mbar_init(bar, 1);
  if (warp == 0) tc::tmem_alloc(tbase, 64);
  publish();
  const uint32_t tm = *tbase, lane_addr = tm + ((warp * 32u) << 16);
  const uint32_t aH = tc::smem_addr(H);
  TcSync sy{bar, 0u, true};
  float o[kGuideOut];
  if (t == 0) {
    tc::gemm_issue(tm, aH, tc::smem_addr(W + kTileW2), 64, 64, false);
    tc::mma_commit(bar);
  }
  if (sy.wait()) {
    guide_hidden_epilogue(lane_addr, bias, H, t);
    publish();
    if (t == 0) {
      tc::gemm_issue(tm, aH, tc::smem_addr(W + kTileW3), 64, 64, false);
      tc::mma_commit(bar);
    }
    if (sy.wait()) {
      guide_hidden_epilogue(lane_addr, bias + 64, H, t);
      publish();
      if (t == 0) {
        tc::gemm_issue(tm, aH, tc::smem_addr(W + kTileW4), kGuideOutPad, 64, false);
        tc::mma_commit(bar);
      }
      if (sy.wait()) guide_output_epilogue(lane_addr, bias + 128, o);
    }
  }
  if (!sy.ok && t == 0) atomicOr(g.err, kErrGuide);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tm, 64);
  if (!live) return;
  V3 d;
  float pdf_dir;
  if (sy.ok) {
    GuideMixture mix;
    guide_mixture(o, mix);
    const float f = g.plain_fraction;
    if (rng.next() < f) {
      d = cos_sampling(rng, lp.ln, nullptr);
    } else {
      const float xi = rng.next();
      int k = 0;
      float acc = mix.w[0];
      while (k < kGuideLobes - 1 && xi >= acc) acc += mix.w[++k];
      const float e1 = rng.next(), e2 = rng.next();
      d = vmf_sample(mix.mu[k], mix.kappa[k], e1, e2);
    }
    pdf_dir = f * fmaxf(0.0f, dot(lp.ln, d)) / kPI + (1.0f - f) * guide_pdf(mix, d);
  } else {
    d = cos_sampling(rng, lp.ln, &pdf_dir);
  }
  PhotonState s;
  photon_launch(ph, i, lp, d, pdf_dir, rng, s);
  photon_top(s);  // loop 0 -> 1; true for a new path
  store_state(w, i, s);
  w.queue[0][i] = (uint32_t)i;
  g.feat[i] = make_float4(x[0], x[1], x[2], x[3]);
  g.dir[i] = make_float4(x[4], s.d.x, s.d.y, s.d.z);
  reinterpret_cast<ulonglong2*>(g.importance)[i] = make_ulonglong2(0ull, 0ull);
}

template <bool kEndDegenerate>
__global__ void FR_PW_SHADE_BOUNDS k_pw_shade(SceneGPU sc, IterParams it, PhotonSlots ph, PathWave w,
                                                  uint32_t* counts, int round) {
  const ShadeQueues sq(w, round);
  const uint32_t n = sq.total();
  uint32_t* qn = w.queue[(round + 1) & 1];
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t n_round = (n + stride - 1) / stride * stride;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_round; j += stride) {
    bool keep = false;
    uint32_t i = 0;
    if (j < n) {
      i = sq.path(w, j);
      PhotonState s;
      load_state(w, (int)i, s);
      Hit h;
      const bool alive = wave_hit(w, i, h) && photon_shade<kEndDegenerate>(sc, it, ph, (int)i, s, h) && photon_top(s);
      if (alive) {
        store_state(w, (int)i, s);
        keep = true;
      } else {
        photon_finish(it, ph, counts, (int)i, s.k);
      }
    }
    block_append<1>(qn, 0, w.qcount + round + 1, keep ? 0 : -1, i);
  }
}

// Paths alive after the last wavefront round, each run to its end.
// At most kTailPathsPerWarp paths share a warp: a tail path's bounces are a
// chain of dependent traversals, and the fewer divergent paths a warp carries,
// the sooner each of its paths advances.
// Paths per warp in the photon tail: the fewest (a power of two) that give
// every path a lane of the resident grid, at most kTailPathsPerWarp.  Fewer
// paths per warp diverge less, and the tail's time is the latency of its
// longest path, so idle lanes cost nothing while every path has a lane.
#ifndef FR_TAIL_PATHS_PER_WARP
#define FR_TAIL_PATHS_PER_WARP 16
#endif
constexpr uint32_t kTailPathsPerWarp = FR_TAIL_PATHS_PER_WARP;
__device__ __forceinline__ uint32_t tail_paths_per_warp(uint32_t n, uint32_t nwarps) {
  uint32_t ppw = 1;
  while (ppw < kTailPathsPerWarp && (uint64_t)ppw * nwarps < n) ppw <<= 1;
  return ppw;
}

// The tail's photon shading (and closest hit) as out-of-line calls (1) or
// inline (0).  A tail path alternates between traversal and shading, and the
// inline kernel's largest stall is instruction fetch ("no instruction"); the
// calls did not help: mixed materials 3.65 ms per iteration with the shading
// out of line, 3.57 with both, 3.55-3.57 inline.
#ifndef FR_TAIL_SHADE_NOINLINE
#define FR_TAIL_SHADE_NOINLINE 0
#endif
#ifndef FR_TAIL_TRACE_NOINLINE
#define FR_TAIL_TRACE_NOINLINE 0
#endif
template <bool kEndDegenerate>
__device__ __noinline__ bool photon_bounce_call(const SceneGPU& sc, const IterParams& it, const PhotonSlots& ph, int i,
                                                PhotonState& s, const Hit& h) {
  return photon_shade<kEndDegenerate>(sc, it, ph, i, s, h) && photon_top(s);
}
template <bool kWT>
__device__ __noinline__ bool trace_closest_call(const SceneGPU& sc, V3 o, V3 d, Hit& h, int* err) {
  return trace_closest<kWT>(sc, o, d, kRayOffset, h, err);
}

template <bool kEndDegenerate, bool kWT>
__global__ void __launch_bounds__(128) k_pw_tail(SceneGPU sc, IterParams it, PhotonSlots ph, PathWave w,
                                                 uint32_t* counts, int rounds, int* err) {
  const int round = tail_round(w, rounds);
  const uint32_t n = *(volatile uint32_t*)(w.qcount + round);
  const uint32_t* q = w.queue[round & 1];
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t ppw = tail_paths_per_warp(n, nwarps);
  if (lane >= ppw) return;
  for (uint32_t j = warp * ppw + lane; j < n; j += nwarps * ppw) {
    const int i = (int)q[j];
    PhotonState s;
    load_state(w, i, s);
    while (true) {
      Hit h;
#if FR_TAIL_TRACE_NOINLINE
      if (!trace_closest_call<kWT>(sc, s.o, s.d, h, err)) break;
#else
      if (!trace_closest<kWT>(sc, s.o, s.d, kRayOffset, h, err)) break;
#endif
#if FR_TAIL_SHADE_NOINLINE
      if (!photon_bounce_call<kEndDegenerate>(sc, it, ph, i, s, h)) break;
#else
      if (!photon_shade<kEndDegenerate>(sc, it, ph, i, s, h) || !photon_top(s)) break;
#endif
    }
    photon_finish(it, ph, counts, i, s.k);
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
  const uint32_t n = counts[i];
  for (uint32_t k = 0; k < n; ++k) {
    const float4 p = ph.pos[slot_index(ph, i, (int)k)];
    atomicAdd(g.cell_count + cell_hash(cell_of(p.x, ox, inv), cell_of(p.y, oy, inv), cell_of(p.z, oz, inv), mask), 1u);
  }
}

// Each photon's bucket is hashed again from its position (the same float
// operations as k_photon_count) and its place in the bucket taken by counting
// the bucket's count down, which leaves the counts zero; the gather reads only
// cell_start.  (The order within a bucket follows the atomics, as the count's
// ranks would.)  Per-slot bucket and rank arrays, 128 bytes apart per path,
// cost a DRAM line per 4-byte read.
__global__ void __launch_bounds__(256) k_photon_scatter(PhotonSlots ph, const uint32_t* counts, int paths,
                                                        int stride, PhotonGrid g, const GridInfo* gi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= paths) return;
  const float ox = gi->origin[0], oy = gi->origin[1], oz = gi->origin[2], inv = gi->inv_cell;
  const uint32_t mask = g.table - 1u;
  const uint32_t n = counts[i];
  for (uint32_t k = 0; k < n; ++k) {
    const size_t s = slot_index(ph, i, (int)k);
    const float4 p = ph.pos[s];
    const uint32_t h = cell_hash(cell_of(p.x, ox, inv), cell_of(p.y, oy, inv), cell_of(p.z, oz, inv), mask);
    const uint32_t dst = g.cell_start[h] + atomicSub(g.cell_count + h, 1u) - 1u;
    g.pos[dst] = p;
    g.flux[dst] = ph.flux[s];
    float4 d = ph.dir[s];
    d.w = __uint_as_float((uint32_t)i * (uint32_t)stride + k);  // the photon's id
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

// tau <- (tau + phi) * a / b (SPPM.cpp:445), tau in FP64.  The ratio a / b is a
// float-float (within 2^-46 of a / b; an FP64 divide is about ten FP64
// instructions on GB300), then one FP64 add and multiply.
__device__ __forceinline__ double tau_update(double tau, float phi, float a, float b) {
  const xf::ff q = xf::div_f(xf::ff{a, 0.0f}, b);
  return (tau + (double)phi) * ((double)q.h + (double)q.l);
}

// The N/R update factors of SPPM.cpp:444-449, a = N + alpha M and b = N + M,
// and the new N.  The reference keeps N as an int, so N += M * alpha
// truncates (SPPM.h:119, SPPM.cpp:447); with kFlagFloatPhotonCount the same
// four bytes hold N as a float and nothing is truncated.
__device__ __forceinline__ void photon_count_update(int32_t n_bits, int M, float alpha, bool float_n, float& a,
                                                    float& b, int32_t& n_new) {
  if (float_n) {
    const float N = __int_as_float(n_bits);
    a = N + alpha * (float)M;
    b = N + (float)M;
    n_new = __float_as_int(N + (float)M * alpha);
  } else {
    const int N = n_bits;
    a = (float)N + alpha * (float)M;
    b = (float)(N + M);
    n_new = (int)((float)N + (float)M * alpha);
  }
}

// applyHitPointInfo (SPPM.cpp:395-451) with one group of G lanes per hitpoint
// of the hitpoint list (32 / G hitpoints per warp at a time: a hitpoint's
// work is a chain of dependent loads, so several in flight per warp hide
// it).  The group's lanes take one overlapping cell each, scan the cells'
// photon counts, and then share out the candidates of all cells, G at a time,
// so every lane tests and (if inside the ball) shades its own photon.
// Per-lane Kahan FP32 sums are added in a fixed butterfly order; the N/tau/R
// update follows with tau in FP64.
#ifndef FR_GATHER_GROUP
#define FR_GATHER_GROUP 16
#endif
constexpr int kGatherGroup = FR_GATHER_GROUP;

// kImportance: also add each photon's contribution to its path's importance
// (the guide's training signal); the plain gather keeps its registers.
template <bool kImportance>
__global__ void __launch_bounds__(256) k_gather(SceneGPU sc, IterParams it, HitpointBuf hp, PhotonGrid g,
                                               const GridInfo* gip, PixelState st, int32_t* dbg_m, float4* dbg_phi,
                                               unsigned long long* importance) {
  constexpr int G = kGatherGroup;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned gl = lane & (G - 1);                        // lane within the group
  const unsigned gmask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u) << (lane & ~(unsigned)(G - 1)));
  const uint32_t n = *(volatile const uint32_t*)hp.list_count;
  const uint32_t ngroups = (gridDim.x * blockDim.x) / G;
  const GridInfo gi = *gip;
  const float inv = gi.inv_cell;
  const uint32_t mask = g.table - 1u;
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) / G; w < n; w += ngroups) {
    const uint32_t i = hp.list[w];
    const float4 hp0 = hp.pos[i], hn = hp.nrm[i], ho = hp.out[i], hw = hp.wgt[i];
    const V3 x = v3(hp0.x, hp0.y, hp0.z), nrm = v3(hn.x, hn.y, hn.z), out = v3(ho.x, ho.y, ho.z);
    const MaterialGPU& mat = sc.mats[__float_as_int(ho.w)];
    const int type = mat.type;
    const float R = st.r[i];
    const V3 bmin = x - R * v3(1.f, 1.f, 1.f);
    const V3 bmax = x + R * v3(1.f, 1.f, 1.f);
    const float R2 = R * R;
    const int x0 = cell_of(bmin.x, gi.origin[0], inv), nx = cell_of(bmax.x, gi.origin[0], inv) - x0 + 1;
    const int y0 = cell_of(bmin.y, gi.origin[1], inv), ny = cell_of(bmax.y, gi.origin[1], inv) - y0 + 1;
    const int z0 = cell_of(bmin.z, gi.origin[2], inv), nz = cell_of(bmax.z, gi.origin[2], inv) - z0 + 1;
    const int ncell = nx * ny * nz;
    int M = 0;
    float sx = 0.f, sy = 0.f, sz = 0.f, kx = 0.f, ky = 0.f, kz = 0.f;
    for (int c0 = 0; c0 < ncell; c0 += G) {
      const int c = c0 + (int)gl;
      int cx = 0, cy = 0, cz = 0;
      uint32_t cb = 0, cn = 0;
      if (c < ncell) {
        const int q = c / nx;
        cx = x0 + (c - q * nx);
        cy = y0 + q % ny;
        cz = z0 + q / ny;
        const uint32_t h = cell_hash(cx, cy, cz, mask);
        cb = __ldg(g.cell_start + h);
        cn = __ldg(g.cell_start + h + 1) - cb;
      }
      uint32_t incl = cn;
#pragma unroll
      for (int o = 1; o < G; o <<= 1) {
        const uint32_t t = __shfl_up_sync(gmask, incl, o, G);
        if ((int)gl >= o) incl += t;
      }
      const uint32_t total = __shfl_sync(gmask, incl, G - 1, G);
      for (uint32_t t0 = 0; t0 < total; t0 += G) {
        const uint32_t k = t0 + gl;
        // Source lane: the first whose inclusive count exceeds k.
        int src = 0;
#pragma unroll
        for (int step = G / 2; step; step >>= 1) {
          const uint32_t v = __shfl_sync(gmask, incl, src + step - 1, G);
          if (v <= k) src += step;
        }
        const uint32_t sb = __shfl_sync(gmask, cb, src, G);
        const uint32_t se = __shfl_sync(gmask, incl, src, G) - __shfl_sync(gmask, cn, src, G);
        const int scx = __shfl_sync(gmask, cx, src, G);
        const int scy = __shfl_sync(gmask, cy, src, G);
        const int scz = __shfl_sync(gmask, cz, src, G);
        if (k >= total) continue;
        const uint32_t j = sb + (k - se);
        const float4 p4 = __ldg(g.pos + j);
        // Query box (kdtree.h:78-88, SPPM.cpp:424-428), ball (SPPM.cpp:432),
        // and the photon's own cell only (hash collisions share buckets).
        if (cell_of(p4.x, gi.origin[0], inv) != scx || cell_of(p4.y, gi.origin[1], inv) != scy ||
            cell_of(p4.z, gi.origin[2], inv) != scz)
          continue;
        if (bmin.x > p4.x || bmax.x < p4.x || bmin.y > p4.y || bmax.y < p4.y || bmin.z > p4.z || bmax.z < p4.z)
          continue;
        if (!(norm2(v3(p4.x, p4.y, p4.z) - x) < R2)) continue;
        const float4 f4 = __ldg(g.flux + j);
        const float4 d4 = __ldg(g.dir + j);
        const V3 indir = v3(d4.x, d4.y, d4.z);
        const float Ii = p4.w;
        const float Io = near1(p4.w) ? mat.index : 1.0f;
        const V3 nn = dot(indir, nrm) < 0.0f ? nrm : -nrm;
        const FParam p{indir, out, nn, Ii, Io, hn.w, mat.extinction, mat.reflectance};
        const float brdf = surface_brdf(type, p);
        const V3 add = v3(hw.x, hw.y, hw.z) * brdf * v3(f4.x, f4.y, f4.z) / f4.w;
        if (kImportance) {  // fixed point: the sum is the same in any order
          unsigned long long hi, lo;
          importance_split(add.x + add.y + add.z, &hi, &lo);
          unsigned long long* ip = importance + 2 * (size_t)(__float_as_uint(d4.w) >> 5);
          if (hi) atomicAdd(ip, hi);
          if (lo) atomicAdd(ip + 1, lo);
        }
        float y, t;
        y = add.x - kx; t = sx + y; kx = (t - sx) - y; sx = t;
        y = add.y - ky; t = sy + y; ky = (t - sy) - y; sy = t;
        y = add.z - kz; t = sz + y; kz = (t - sz) - y; sz = t;
        ++M;
      }
    }
    float vx = sx - kx, vy = sy - ky, vz = sz - kz;
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
      M += __shfl_xor_sync(gmask, M, o, G);
      vx += __shfl_xor_sync(gmask, vx, o, G);
      vy += __shfl_xor_sync(gmask, vy, o, G);
      vz += __shfl_xor_sync(gmask, vz, o, G);
    }
    vx = __shfl_sync(gmask, vx, 0, G);
    vy = __shfl_sync(gmask, vy, 0, G);
    vz = __shfl_sync(gmask, vz, 0, G);
    if (gl == 0 && dbg_m) {
      dbg_m[i] = M;
      dbg_phi[i] = make_float4(vx, vy, vz, 0.f);
    }
    if (M > 0 && gl < 3) {
      // N/tau/R update (SPPM.cpp:444-449); group lane c updates tau component c.
      float a, b;
      int32_t n_new;
      photon_count_update(st.n[i], M, it.alpha, (it.flags & kFlagFloatPhotonCount) != 0u, a, b, n_new);
      double* tau = st.tau + 3 * (size_t)i + gl;
      const float v = gl == 0 ? vx : (gl == 1 ? vy : vz);
      *tau = tau_update(*tau, v, a, b);
      if (gl == 0) {
        st.r[i] = R * sqrtf(a / b);
        st.n[i] = n_new;
        st.g[i] += 1;
      }
    }
  }
}

// The N/tau/R update alone (SPPM.cpp:444-449) from given per-pixel photon
// counts m and flux sums phi; the same arithmetic as the gather's update.
__global__ void k_update(PixelState st, const int32_t* m, const float4* phi, int pixels, float alpha,
                         bool float_n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= pixels) return;
  const int M = m[i];
  if (M <= 0) return;
  float a, b;
  int32_t n_new;
  photon_count_update(st.n[i], M, alpha, float_n, a, b, n_new);
  const float4 v = phi[i];
  double* tau = st.tau + 3 * (size_t)i;
  tau[0] = tau_update(tau[0], v.x, a, b);
  tau[1] = tau_update(tau[1], v.y, a, b);
  tau[2] = tau_update(tau[2], v.z, a, b);
  st.r[i] = st.r[i] * sqrtf(a / b);
  st.n[i] = n_new;
  st.g[i] += 1;
}

// ExportPNG (TextureUtility.cpp:52-65): pixel (i, j) of the exported image is
// the render target sampled by LinearSampler::Sample (TextureSampler.h:61-79)
// at u = i / W, v = j / H, each channel stored as max(0, min(255,
// int(c * 255))).  A float outside int's range converts as on the reference's
// x86 build (to INT_MIN, so 0 after the clamp); so does NaN.
__device__ __forceinline__ F4 image_texel(const float4* img, int idx) {
  const float4 v = img[idx];
  return F4{v.x, v.y, v.z, v.w};
}

__device__ __forceinline__ uint32_t quantize_255(float c) {
  const float s = c * 255.0f;
  const int q = (!(s == s) || fabsf(s) >= 2147483648.0f) ? INT_MIN : (int)s;
  return (uint32_t)max(0, min(255, q));
}

__global__ void k_export_rgba8(const float4* img, int W, int H, uint32_t* out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= W * H) return;
  const int i = idx % W, j = idx / W;
  const float u = (float)i / (float)W, v = (float)j / (float)H;
  const int iu = (int)((float)W * u), iv = (int)((float)H * v);
  const int x1 = abs(iu) % W, y1 = abs(iv) % H;
  const int x2 = min(W - 1, x1 + 1), y2 = min(H - 1, y1 + 1);
  const F4 t00 = image_texel(img, x1 + y1 * W), t10 = image_texel(img, x2 + y1 * W);
  const F4 t01 = image_texel(img, x1 + y2 * W), t11 = image_texel(img, x2 + y2 * W);
  const float w = fabsf(u * (float)W) - (float)abs(iu);
  const float h = fabsf(v * (float)H) - (float)abs(iv);
  const F4 up = lerp4(t00, 1.0f - w, t10, w);
  const F4 down = lerp4(t01, 1.0f - w, t11, w);
  const F4 c = lerp4(up, 1.0f - h, down, h);
  out[idx] = quantize_255(c.x) | quantize_255(c.y) << 8 | quantize_255(c.z) << 16 | quantize_255(c.w) << 24;
}

// ---------------------------------------------------------------- resolve
// reconstructImageFromSharedPoints (SPPM.cpp:473-493): normalisation in FP64,
// gamma 1/1.2 in FP32 as the reference applies it.
// standard = 0: the reference's estimate, which scales the photons emitted by
// the pixel's share of iterations that gathered photons (NumGather); 1: the
// standard SPPM estimate tau / (pi R^2 * all photons emitted).
__global__ void k_resolve(PixelState st, int pixels, double photons_total, double iterations, int standard,
                          float4* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= pixels) return;
  const double R = (double)st.r[i];
  const double share = standard ? 1.0 : ((double)st.g[i] + 1e-4) / (1e-4 + iterations);
  const double denom = (photons_total * share) * (double)kPI * R * R;
  const double* tau = st.tau + 3 * (size_t)i;
  // Direct (environment) light over its count (SPPM.cpp:485), zero without one.
  const float4 dl = st.dl[i];
  const float dn = (float)__float_as_int(dl.w) + 0.0001f;
  const float lr = dl.x / dn + (float)(tau[0] / denom), lg = dl.y / dn + (float)(tau[1] / denom),
              lb = dl.z / dn + (float)(tau[2] / denom);
  const float gm = 1.0f / 1.2f;
  out[i] = make_float4(powf(lr, gm), powf(lg, gm), powf(lb, gm), 1.0f);
}

// ------------------------------------------------------------ parity kernels
template <bool kWT>
__global__ void k_trace_closest(SceneGPU sc, const float* rays, int n, int32_t* facet, float* tuv, int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* r = rays + 7 * (size_t)i;
  Hit h;
  if (trace_closest<kWT>(sc, v3(r[0], r[1], r[2]), v3(r[3], r[4], r[5]), kRayOffset, h, err)) {
    facet[i] = h.facet;
    tuv[3 * i] = h.t; tuv[3 * i + 1] = h.u; tuv[3 * i + 2] = h.v;
  } else {
    facet[i] = -1;
    tuv[3 * i] = FLT_MAX; tuv[3 * i + 1] = 0.f; tuv[3 * i + 2] = 0.f;
  }
}

// rays: N x 8 {org, dir, minT, maxT}
template <bool kWT>
__global__ void k_trace_any(SceneGPU sc, const float* rays, int n, int32_t* hit, int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* r = rays + 8 * (size_t)i;
  hit[i] = trace_any<kWT>(sc, v3(r[0], r[1], r[2]), v3(r[3], r[4], r[5]), r[6], r[7], err) ? 1 : 0;
}

// hp: xyz position, w radius.  A ball query_ball_ok refuses gets the count
// -1 and sets kErrQuery in *err (when err is given).
__global__ void k_radius_count(const float4* hp, int nh, PhotonGrid g, const GridInfo* gip, int32_t* m,
                               uint32_t* pairs, uint32_t cap, uint32_t* pair_count, int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nh) return;
  const GridInfo gi = *gip;
  const float4 h = hp[i];
  if (!query_ball_ok(h.x, h.y, h.z, h.w, gi.origin, gi.inv_cell)) {
    m[i] = -1;
    if (err) atomicOr(err, kErrQuery);
    return;
  }
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

void launch_next_step(uint32_t* step, cudaStream_t s) { k_next_step<<<1, 1, 0, s>>>(step); }

int pw_tail_blocks_per_sm() {
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_pw_tail<false, false>, 128, 0);
  return b;
}

void launch_ew_start(const CameraGPU& cam, const IterParams& it, PathWave w, cudaStream_t s) {
  k_ew_start<<<blocks_for((size_t)it.width * it.height, 128), 128, 0, s>>>(cam, it, w);
}

void launch_wave_trace(const SceneGPU& sc, PathWave w, int round, int grid, bool coherent, int* err, cudaStream_t s) {
  const unsigned g = (unsigned)std::max(1, grid);
  if (coherent) {
    if (sc.watertight) k_wave_trace_static<true><<<g, 128, 0, s>>>(sc, w, round, err);
    else k_wave_trace_static<false><<<g, 128, 0, s>>>(sc, w, round, err);
  } else {
    if (sc.watertight) k_wave_trace<true><<<g, 128, 0, s>>>(sc, w, round, err);
    else k_wave_trace<false><<<g, 128, 0, s>>>(sc, w, round, err);
  }
}

// Sets the condition of the graph IF node holding wavefront round `round`:
// the round runs when it has at least w.min_live paths (the kernels' own
// round_skipped rule).  Counts the rounds it lets run.
__global__ void k_round_gate(cudaGraphConditionalHandle h, PathWave w, int round, uint32_t* rounds_run) {
  const bool run = !round_skipped(w, round);
  if (run) *rounds_run += 1u;
  cudaGraphSetConditional(h, run ? 1u : 0u);
}

void launch_round_gate(cudaGraphConditionalHandle h, const PathWave& w, int round, uint32_t* rounds_run,
                       cudaStream_t s) {
  k_round_gate<<<1, 1, 0, s>>>(h, w, round, rounds_run);
}

void launch_wave_sort(const SceneGPU& sc, PathWave w, int round, int grid, cudaStream_t s) {
  k_wave_sort<<<std::max(1, grid), 256, 0, s>>>(sc, w, round);
}

void launch_ew_shade(const SceneGPU& sc, const IterParams& it, const float* rr_eye, PathWave w, HitpointBuf hp,
                     PixelState st, GridInfo* gi, int round, int grid, cudaStream_t s) {
  if (it.flags & kFlagEndDegenerate)
    k_ew_shade<true><<<std::max(1, grid), 128, 0, s>>>(sc, it, rr_eye[0], rr_eye[1], w, hp, st, gi, round);
  else
    k_ew_shade<false><<<std::max(1, grid), 128, 0, s>>>(sc, it, rr_eye[0], rr_eye[1], w, hp, st, gi, round);
}

void launch_ew_tail(const SceneGPU& sc, const IterParams& it, const float* rr_eye, PathWave w, HitpointBuf hp,
                    PixelState st, GridInfo* gi, int round, int grid, int* err, cudaStream_t s) {
  const unsigned g = (unsigned)std::max(1, grid);
  const bool end = (it.flags & kFlagEndDegenerate) != 0;
  if (sc.watertight) {
    if (end) k_ew_tail<true, true><<<g, 128, 0, s>>>(sc, it, rr_eye[0], rr_eye[1], w, hp, st, gi, round, err);
    else k_ew_tail<false, true><<<g, 128, 0, s>>>(sc, it, rr_eye[0], rr_eye[1], w, hp, st, gi, round, err);
  } else {
    if (end) k_ew_tail<true, false><<<g, 128, 0, s>>>(sc, it, rr_eye[0], rr_eye[1], w, hp, st, gi, round, err);
    else k_ew_tail<false, false><<<g, 128, 0, s>>>(sc, it, rr_eye[0], rr_eye[1], w, hp, st, gi, round, err);
  }
}

void launch_pw_emit(const SceneGPU& sc, const IterParams& it, PhotonSlots ph, PathWave w, uint32_t* counts,
                    cudaStream_t s) {
  k_pw_emit<<<blocks_for(it.photons, 128), 128, 0, s>>>(sc, it, ph, w, counts);
}

void launch_pw_shade(const SceneGPU& sc, const IterParams& it, PhotonSlots ph, PathWave w, uint32_t* counts,
                     int round, int grid, cudaStream_t s) {
  if (it.flags & kFlagEndDegenerate)
    k_pw_shade<true><<<std::max(1, grid), 128, 0, s>>>(sc, it, ph, w, counts, round);
  else
    k_pw_shade<false><<<std::max(1, grid), 128, 0, s>>>(sc, it, ph, w, counts, round);
}

void launch_pw_tail(const SceneGPU& sc, const IterParams& it, PhotonSlots ph, PathWave w, uint32_t* counts,
                    int round, int grid, int* err, cudaStream_t s) {
  const unsigned g = (unsigned)std::max(1, grid);
  const bool end = (it.flags & kFlagEndDegenerate) != 0;
  if (sc.watertight) {
    if (end) k_pw_tail<true, true><<<g, 128, 0, s>>>(sc, it, ph, w, counts, round, err);
    else k_pw_tail<false, true><<<g, 128, 0, s>>>(sc, it, ph, w, counts, round, err);
  } else {
    if (end) k_pw_tail<true, false><<<g, 128, 0, s>>>(sc, it, ph, w, counts, round, err);
    else k_pw_tail<false, false><<<g, 128, 0, s>>>(sc, it, ph, w, counts, round, err);
  }
}

int photon_pass_blocks_per_sm() {
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_wave_trace<false>, 128, 0);
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
                           const GridInfo* gi, cudaStream_t s) {
  k_photon_scatter<<<blocks_for(paths, 256), 256, 0, s>>>(ph, counts, paths, stride, g, gi);
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
                          PixelState st, int32_t* dbg_m, float4* dbg_phi, unsigned long long* importance,
                          int resident_blocks,
                          cudaStream_t s) {
  if (importance)
    k_gather<true><<<std::max(1, resident_blocks), 256, 0, s>>>(sc, it, hp, g, gi, st, dbg_m, dbg_phi, importance);
  else
    k_gather<false><<<std::max(1, resident_blocks), 256, 0, s>>>(sc, it, hp, g, gi, st, dbg_m, dbg_phi, importance);
}

void launch_pw_emit_guided(const SceneGPU& sc, const IterParams& it, PhotonSlots ph, PathWave w, uint32_t* counts,
                           const GuideGPU& g, cudaStream_t s) {
  k_pw_emit_guided<<<blocks_for(it.photons, 128), 128, kEmitSmem, s>>>(sc, it, ph, w, counts, g);
}

int gather_blocks_per_sm() {
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_gather<false>, 256, 0);
  return b;
}

void launch_update(PixelState st, const int32_t* m, const float4* phi, int pixels, float alpha, bool float_n,
                   cudaStream_t s) {
  k_update<<<blocks_for(pixels, 256), 256, 0, s>>>(st, m, phi, pixels, alpha, float_n);
}

void launch_export_rgba8(const float4* img, int width, int height, uint32_t* out, cudaStream_t s) {
  k_export_rgba8<<<blocks_for((size_t)width * height, 256), 256, 0, s>>>(img, width, height, out);
}

void launch_resolve(PixelState st, int pixels, double photons_total, double iterations, bool standard, float4* out,
                    cudaStream_t s) {
  k_resolve<<<blocks_for(pixels, 256), 256, 0, s>>>(st, pixels, photons_total, iterations, standard ? 1 : 0, out);
}

void launch_trace_closest(const SceneGPU& sc, const float* rays, int n, int32_t* facet, float* tuv, int* err,
                          cudaStream_t s) {
  if (sc.watertight) k_trace_closest<true><<<blocks_for(n, 128), 128, 0, s>>>(sc, rays, n, facet, tuv, err);
  else k_trace_closest<false><<<blocks_for(n, 128), 128, 0, s>>>(sc, rays, n, facet, tuv, err);
}

void launch_trace_any(const SceneGPU& sc, const float* rays, int n, int32_t* hit, int* err, cudaStream_t s) {
  if (sc.watertight) k_trace_any<true><<<blocks_for(n, 128), 128, 0, s>>>(sc, rays, n, hit, err);
  else k_trace_any<false><<<blocks_for(n, 128), 128, 0, s>>>(sc, rays, n, hit, err);
}

void launch_radius_count(const float4* hp, int nh, PhotonGrid g, const GridInfo* gi, int32_t* m, uint32_t* pairs,
                         uint32_t cap, uint32_t* pair_count, int* err, cudaStream_t s) {
  k_radius_count<<<blocks_for(nh, 128), 128, 0, s>>>(hp, nh, g, gi, m, pairs, cap, pair_count, err);
}

}  // namespace fr
