// Host side of the GPU SPPM renderer: scene upload, light tables, camera set-up,
// the iteration driver and the C-ABI declared in include/friendsrender.h.
//
// Everything the reference computes once per scene on the host (camera basis,
// light alias tables, textured-emission tables) is computed here with the same
// float/double expressions, so the kernels see the reference's exact values.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/friendsrender.h"
#include "fr_bvh.h"
#include "fr_guide.h"
#include "fr_ingest.h"
#include "fr_kernels.h"
#include "fr_layout.h"

using namespace fr;

namespace {

thread_local std::string g_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_error = buf;
  return code;
}

#define FR_CUDA(call)                                                                     \
  do {                                                                                    \
    const cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) return fail(FR_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// ------------------------------------------------------- host vector helpers
// Float arithmetic in the reference's PTUtility::Vec3 order (Vec.h:179-243).
struct H3 {
  float x, y, z;
};
inline H3 operator+(H3 a, H3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline H3 operator-(H3 a, H3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline H3 operator*(H3 a, H3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline H3 operator*(float s, H3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline H3 operator*(H3 a, float s) { return {s * a.x, s * a.y, s * a.z}; }
inline H3 operator/(H3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline float dot(H3 a, H3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline H3 cross(H3 a, H3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float norm2(H3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline float norm(H3 a) { return std::sqrt(norm2(a)); }
inline H3 normalized(H3 a) {
  const float d = norm(a);
  return {a.x / d, a.y / d, a.z / d};
}
inline H3 h3(const float* p) { return {p[0], p[1], p[2]}; }
inline void put(float* d, H3 v) { d[0] = v.x; d[1] = v.y; d[2] = v.z; }

// LinearSampler::Sample (TextureSampler.h:61-79) on the host, used to build
// the textured-emission tables.
struct HostTex {
  int w, h;
  const uint8_t* t;
  void fetch(int idx, float o[4]) const {
    for (int c = 0; c < 4; ++c) o[c] = t[4 * (size_t)idx + c] / 255.0f;
  }
  void bilinear(float u, float v, float out[4]) const {
    const int iu = (int)((float)w * u), iv = (int)((float)h * v);
    const int x1 = std::abs(iu) % w, y1 = std::abs(iv) % h;
    const int x2 = std::min(w - 1, x1 + 1), y2 = std::min(h - 1, y1 + 1);
    float t00[4], t10[4], t01[4], t11[4];
    fetch(x1 + y1 * w, t00); fetch(x2 + y1 * w, t10); fetch(x1 + y2 * w, t01); fetch(x2 + y2 * w, t11);
    const float fw = std::fabs(u * (float)w) - (float)std::abs(iu);
    const float fh = std::fabs(v * (float)h) - (float)std::abs(iv);
    for (int c = 0; c < 4; ++c) {
      const float up = t00[c] * (1.0f - fw) + t10[c] * fw;
      const float down = t01[c] * (1.0f - fw) + t11[c] * fw;
      out[c] = up * (1.0f - fh) + down * fh;
    }
  }
};

// QRandSequence::HaltonCore<B>::Sample (QRandSequence.h:10-25), including its
// digit count from double log2.
float halton(int n, int B) {
  float result = 0.0f;
  if (n <= 0) return result;
  const int keta = (int)(std::log2((double)n) / std::log2((double)B) + 1);
  for (int i = 0; i < keta; ++i) {
    result = (float)((double)result + (double)(n % B) * std::pow((double)B, (double)(-(i + 1))));
    n /= B;
  }
  return result;
}

// TableSampler<T>::Init (TableSampler.h:44-120): the reference's alias
// construction, step for step, so its bins (and so every light / emission
// sample) are the reference's.
struct AliasBin {
  float prob = 1.0f;
  int left = -1, right = -1;
};
std::vector<AliasBin> alias_table(const std::vector<float>& values, float* average) {
  const int N = (int)values.size();
  std::vector<AliasBin> table(N);
  float avg = 0.0f;
  for (int i = 0; i < N; ++i) avg += std::max(0.0f, values[i]);
  avg /= N;
  std::vector<std::pair<float, int>> bigger, smaller;
  for (int i = 0; i < N; ++i) {
    const float v = std::max(0.0f, values[i]);
    if (v >= avg) bigger.push_back({v / avg, i});
    else smaller.push_back({v / avg, i});
  }
  size_t ids = 0, idb = 0;
  for (int i = 0; i < N; ++i) {
    if (ids < smaller.size()) {
      table[i].left = smaller[ids].second;
      table[i].prob = smaller[ids].first;
      ++ids;
      if (idb < bigger.size()) {
        table[i].right = bigger[idb].second;
        bigger[idb].first -= (1.0f - table[i].prob);
        if (bigger[idb].first < 1.0f) smaller.push_back(bigger[idb++]);
      } else if (smaller.size() == ids) {
        table[i].right = -1;
        table[i].prob = 1.0f;
      } else {
        table[i].right = smaller[ids].second;
      }
    } else {
      table[i].left = bigger[idb].second;
      table[i].prob = 1.0f;
      bigger[idb].first -= 1.0f;
      if (bigger[idb].first < 1.0f) smaller.push_back(bigger[idb++]);
    }
  }
  *average = avg;
  return table;
}

float facet_area(H3 p0, H3 p1, H3 p2) { return 0.5f * norm(cross(p1 - p0, p2 - p0)); }  // Normal_Facet.h:45-47

// Exact-value tables of the sampling routines' double functions of one
// 24-bit draw u (see fr_bsdf.cuh), computed with this host's libm — the
// functions the reference calls — once per device and kept for the
// process's life (192 MB of device memory).
struct ExactTables {
  float2* sincos = nullptr;
  float* sqrt1m = nullptr;
};
std::mutex g_tables_mu;
ExactTables g_tables[64];

int exact_tables(int dev, ExactTables* out) {
  if (dev < 0 || dev >= 64) return fail(FR_ERR_INVALID, "device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_tables_mu);
  ExactTables& t = g_tables[dev];
  if (!t.sincos) {
    const uint32_t n = 1u << 24;
    std::vector<float2> sc(n);
    std::vector<float> sq(n);
    const unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned w = 0; w < nt; ++w)
      th.emplace_back([&, w]() {
        for (uint32_t u = w; u < n; u += nt) {
          const float uf = (float)u * (1.0f / 16777216.0f);
          const float ph = (uf * 2.0f) * kPI;  // u*2.0f*PI (Sampling.cpp:65), rounded once
          sc[u] = make_float2((float)std::cos((double)ph), (float)std::sin((double)ph));
          sq[u] = (float)std::sqrt(1.000000001 - (double)uf);  // Sampling.cpp:24
        }
      });
    for (auto& x : th) x.join();
    float2* d_sc = nullptr;
    float* d_sq = nullptr;
    if (cudaMalloc(&d_sc, sizeof(float2) * n) != cudaSuccess || cudaMalloc(&d_sq, sizeof(float) * n) != cudaSuccess) {
      cudaFree(d_sc);
      return fail(FR_ERR_OOM, "exact tables: cudaMalloc failed");
    }
    FR_CUDA(cudaMemcpy(d_sc, sc.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
    FR_CUDA(cudaMemcpy(d_sq, sq.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    t.sincos = d_sc;
    t.sqrt1m = d_sq;
  }
  *out = t;
  return FR_OK;
}

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

}  // namespace

// Shares (percent) of the resident grid given to the eye pass's round kernels
// and to the gather.  Both run on the pixel stream beside the photon pass, the
// iteration's critical path; their kernels fetch work until their queues are
// empty, so a block holds its SM slots until the end of the launch, and a
// smaller grid leaves the photon pass more of the GPU (the eye pass has
// slack).  Mixed materials, ms per iteration: eye pass at 50% 3.55-3.58, 40%
// 3.57, 65% 3.59, 100% 3.62-3.63, 33% 3.62; the gather (its waits are its own
// critical path) at 75% 3.55, 50% 3.65-3.66.
#ifndef FR_EYE_GRID_PCT
#define FR_EYE_GRID_PCT 50
#endif
#ifndef FR_GATHER_GRID_PCT
#define FR_GATHER_GRID_PCT 100
#endif

struct fr_ctx {
  cudaStream_t stream = nullptr;
  std::vector<DevBuf> bufs;
  size_t device_bytes = 0;
  SceneGPU sc{};
  CameraGPU cam{};
  int W = 0, H = 0, P = 0;
  float alpha = 0.9f, r0 = 0.015f, cell_scale = 2.0f;
  uint32_t flags = 0;
  float rr_eye[2] = {0.f, 0.f};
  int bvh_depth = 0;
  HitpointBuf hp{};
  PixelState st{};
  PhotonSlots ph{};
  uint32_t* counts = nullptr;
  PathWave wave{};               // photon-pass wavefront state
  PathWave eye_wave{};           // eye-pass wavefront state (the passes run concurrently)
  // Two streams.  `stream` runs the photon pass and the grid build; `side`,
  // the pixel stream, runs the eye pass, the gather (with the guide's
  // publish and sample selection) and fr_resolve_async's resolve.  Events
  // order them: fork_ev (main -> side), join_ev (side -> main).
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  // Guided contexts: the guide's training runs on train_stream after the
  // selection (sel_ev), beside the next iteration's passes; train_ev marks
  // it done (the next publish of its weights waits for it).
  cudaStream_t train_stream = nullptr;
  cudaEvent_t sel_ev = nullptr, train_ev = nullptr;
  int photon_blocks = 0;         // grid of the photon pass's wavefront round kernels
  int eye_blocks = 0;            // grid of the eye pass's wavefront round kernels
  int tail_blocks = 0;           // grid of the photon tail kernel
  // Device iteration counters (IterParams::step): [0] the photon pass's,
  // [1] the eye pass's; each pass advances its own, so the two passes of an
  // iteration read the same number however their kernels interleave.
  uint32_t* step_dev = nullptr;
  uint32_t step_base = 0;        // fr_seek: the counters run at step_base + iterations
  cudaStream_t body[kPhotonRounds] = {};  // capture the bodies of the graph's nested round nodes
  uint32_t* rounds_run = nullptr;  // gated photon rounds run so far (device)
  bool capturing = false;        // an iteration part is being captured into a graph
  // One graph per part of an iteration (kPart*), each replayed on its stream.
  cudaGraph_t part_graph[5] = {};
  cudaGraphExec_t part_exec[5] = {};
  int64_t part_launches[5] = {};  // kernels per replay of each part
  int gather_blocks = 0;         // grid of the gather (one 16-lane group per hitpoint)
  int sms = 0;                   // streaming multiprocessors of the device
  bool guided = false;           // learned photon-emission guide on
  GuideGPU guide{};
  PhotonGrid grid{};
  GridInfo* gi = nullptr;
  ScanTemp scan{};
  int* err = nullptr;
  int32_t* dbg_m = nullptr;
  float4* dbg_phi = nullptr;
  float4* image = nullptr;
  uint32_t* image8 = nullptr;    // exported RGBA8
  // fr_resolve_async: images {image, image_b} in turn, copied to the host on
  // copy_stream; ready[b] marks resolve b written, copied[b] its copy landed.
  float4* image_b = nullptr;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ready[2] = {}, copied[2] = {};
  uint64_t async_seq = 0;
  int64_t iterations = 0, photons_total = 0;
  int64_t launches = 0;  // kernels launched by fr_iterate so far
  // Stage profiler: events recorded on the stream around each stage.
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_marks;  // (stage, (start, stop))
  size_t ev_used = 0;

  template <typename T>
  int alloc(T** out, size_t count) {
    void* p = nullptr;
    const size_t bytes = std::max<size_t>(count * sizeof(T), 16);
    const cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) return fail(FR_ERR_OOM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    bufs.push_back({p, bytes});
    device_bytes += bytes;
    *out = static_cast<T*>(p);
    return FR_OK;
  }
  template <typename T>
  int upload(T** out, const T* src, size_t count) {
    int rc = alloc(out, count);
    if (rc) return rc;
    if (count) FR_CUDA(cudaMemcpyAsync(*out, src, count * sizeof(T), cudaMemcpyHostToDevice, stream));
    return FR_OK;
  }
  ~fr_ctx() {
    if (stream) cudaStreamSynchronize(stream);
    if (side) cudaStreamSynchronize(side);
    if (train_stream) cudaStreamSynchronize(train_stream);
    for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
    for (auto& b : bufs) cudaFree(b.p);
    if (copy_stream) cudaStreamSynchronize(copy_stream);
    for (cudaEvent_t e : {fork_ev, join_ev, sel_ev, train_ev})
      if (e) cudaEventDestroy(e);
    for (int k = 0; k < 2; ++k) {
      if (ready[k]) cudaEventDestroy(ready[k]);
      if (copied[k]) cudaEventDestroy(copied[k]);
    }
    if (copy_stream) cudaStreamDestroy(copy_stream);
    for (int k = 0; k < 5; ++k) {
      if (part_exec[k]) cudaGraphExecDestroy(part_exec[k]);
      if (part_graph[k]) cudaGraphDestroy(part_graph[k]);
    }
    if (side) cudaStreamDestroy(side);
    if (train_stream) cudaStreamDestroy(train_stream);
    for (cudaStream_t b : body)
      if (b) cudaStreamDestroy(b);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

int check_scene(const fr_scene_desc* s) {
  if (!s || s->num_facets <= 0 || !s->positions || !s->normals || !s->uvs || !s->material_ids)
    return fail(FR_ERR_INVALID, "scene: no facets or a NULL array");
  if (s->num_materials <= 0 || !s->materials) return fail(FR_ERR_INVALID, "scene: no materials");
  if (s->num_textures < 0 || (s->num_textures > 0 && !s->textures)) return fail(FR_ERR_INVALID, "scene: textures");
  for (int t = 0; t < s->num_textures; ++t)
    if (s->textures[t].width <= 0 || s->textures[t].height <= 0 || !s->textures[t].texels)
      return fail(FR_ERR_INVALID, "scene: texture %d is empty", t);
  for (int m = 0; m < s->num_materials; ++m) {
    const fr_material_desc& d = s->materials[m];
    if (d.type < 0 || d.type > 7) return fail(FR_ERR_INVALID, "material %d: type %d", m, d.type);
    const int tex[3] = {d.tex_albedo, d.tex_roughness, d.tex_bump};
    for (int k = 0; k < 3; ++k)
      if (tex[k] < -1 || tex[k] >= s->num_textures) return fail(FR_ERR_INVALID, "material %d: texture index", m);
  }
  for (int f = 0; f < s->num_facets; ++f)
    if (s->material_ids[f] < 0 || s->material_ids[f] >= s->num_materials)
      return fail(FR_ERR_INVALID, "facet %d: material id %d out of range", f, s->material_ids[f]);
  if (s->num_facets >= (1 << kLeafCountShift)) return fail(FR_ERR_INVALID, "scene: too many facets");
  return FR_OK;
}

// iCamera constructor (Camera.h:132-151) and the thin-lens lens size.
CameraGPU setup_camera(const fr_camera_desc& c) {
  CameraGPU g{};
  g.type = c.type;
  g.width = c.width;
  g.height = c.height;
  const H3 pos = h3(c.position), tgt = h3(c.target);
  const H3 dir = normalized(tgt - pos);
  const float fov = (kPI * c.fov_degrees) / 360.0f;
  const float pw = (float)(2.0 * (double)c.distance_to_lens * std::tan((double)fov) * (double)c.aspect);
  const float ph = (float)(2.0 * (double)c.distance_to_lens * std::tan((double)fov));
  H3 e1, e2;
  if ((double)dir.y > 0.99) {
    e1 = {1.f, 0.f, 0.f};
    e2 = {0.f, 0.f, 1.f};
  } else {
    e1 = normalized(cross(H3{0.f, 1.f, 0.f}, dir));
    e2 = normalized(cross(dir, e1));
  }
  put(g.pos, pos); put(g.dir, dir); put(g.e1, e1); put(g.e2, e2);
  g.plane_w = pw;
  g.plane_h = ph;
  g.lens_w = c.lens_width > 0.0f ? c.lens_width : pw;
  g.lens_h = c.lens_height > 0.0f ? c.lens_height : ph;
  g.F = c.focal_length;
  g.dist = c.distance_to_lens;
  return g;
}

// Scene::CreateScene light collection (Scene.cpp:145-154), CreateAreaLight
// (LightSampler.cpp:30-66) and CreateLightSampler (LightSampler.cpp:6-28).
void build_lights(const fr_scene_desc& s, std::vector<LightGPU>& lights, std::vector<EmitEntry>& emit) {
  std::vector<float> flux_norm;  // AreaLight::Evaluate = |_Flux| (LightSampler.cpp:113-115)
  for (int f = 0; f < s.num_facets; ++f) {
    const fr_material_desc& m = s.materials[s.material_ids[f]];
    const H3 rad = h3(m.emission);
    if (!(rad.x + rad.y + rad.z > 0.00001f)) continue;
    const float* P = s.positions + 9 * (size_t)f;
    const float* N = s.normals + 9 * (size_t)f;
    const float* U = s.uvs + 6 * (size_t)f;
    const H3 p0 = h3(P), p1 = h3(P + 3), p2 = h3(P + 6);
    const float area = facet_area(p0, p1, p2);
    LightGPU L{};
    put(L.p0, p0); put(L.p1, p1); put(L.p2, p2);
    put(L.normal, normalized(h3(N) + h3(N + 3) + h3(N + 6)));
    L.pdf_point = 2.0f / std::fabs(norm(cross(p1 - p0, p2 - p0)));  // Sampling.cpp:347
    H3 flux;
    if (m.tex_albedo >= 0) {
      const fr_texture_desc& td = s.textures[m.tex_albedo];
      const HostTex tex{td.width, td.height, td.texels};
      std::vector<H3> uvw(kEmitSamples), Ls(kEmitSamples);
      H3 total{0.f, 0.f, 0.f};
      for (int i = 0; i < kEmitSamples; ++i) {
        H3 w{(float)i / (float)kEmitSamples, halton(i, 2), halton(i, 3)};  // Hammersley (QRandSequence.h:27-36)
        if (w.y > w.x) { w.x *= 0.5f; w.y -= w.x; }
        else { w.y *= 0.5f; w.x -= w.y; }
        const float uvx = w.x * U[0] + w.y * U[2] + (1.0f - w.x - w.y) * U[4];
        const float uvy = w.x * U[1] + w.y * U[3] + (1.0f - w.x - w.y) * U[5];
        float c[4];
        tex.bilinear(uvx, uvy, c);
        H3 Lv = H3{c[0], c[1], c[2]} * rad;
        if (norm2(Lv) < 0.01f) Lv = {0.f, 0.f, 0.f};
        uvw[i] = w;
        Ls[i] = Lv;
        total = total + Lv;
      }
      if ((double)norm2(total) < 1e-6) {
        Ls[0] = (float)1e-6 * H3{1.f, 1.f, 1.f};
        uvw[0] = {0.f, 0.f, 0.f};
      } else {
        total = total * ((2.0f * kPI * area) / (float)kEmitSamples);
      }
      flux = total;
      std::vector<float> vals(kEmitSamples);
      for (int i = 0; i < kEmitSamples; ++i) vals[i] = norm(Ls[i]);
      float avg = 0.f;
      const std::vector<AliasBin> tab = alias_table(vals, &avg);
      L.textured = 1;
      L.emit_offset = (int32_t)emit.size();
      for (int i = 0; i < kEmitSamples; ++i) {
        EmitEntry e{};
        e.prob = tab[i].prob;
        e.left = tab[i].left;
        e.right = tab[i].right;
        put(e.uvw, uvw[i]);
        put(e.L, Ls[i]);
        const float gp = norm(Ls[i]) / avg / (float)kEmitSamples;  // TableSampler::GetPDF (TableSampler.h:122-124)
        e.pdf = (gp * kEmitSamples) / area;                        // LightSampler.cpp:73
        emit.push_back(e);
      }
    } else {
      flux = rad * 2.0f * kPI * area;                              // LightSampler.cpp:62
      put(L.radiance, flux / (2.0f * kPI * area));                 // LightSampler.cpp:78
    }
    flux_norm.push_back(norm(flux));
    lights.push_back(L);
  }
  const int NL = (int)lights.size();
  if (!NL) return;
  float avg = 0.f;
  const std::vector<AliasBin> tab = alias_table(flux_norm, &avg);
  for (int i = 0; i < NL; ++i) {
    lights[i].alias_prob = tab[i].prob;
    lights[i].alias_left = tab[i].left;
    lights[i].alias_right = tab[i].right;
    lights[i].pdf_light = flux_norm[i] / avg / (float)NL;  // GetAreaLightPDF (LightSampler.h:87)
  }
}

uint32_t next_pow2(uint64_t v) {
  uint64_t p = 1;
  while (p < v) p <<= 1;
  return (uint32_t)std::min<uint64_t>(p, 1u << 31);
}

// Records an event pair around one stage when profiling is on.
struct StageMark {
  fr_ctx* c;
  int stage;
  cudaStream_t s;
  cudaEvent_t stop = nullptr;
  StageMark(fr_ctx* ctx, int st, cudaStream_t stream) : c(ctx), stage(st), s(stream) {
    if (!c->profiling || c->ev_used + 2 > c->ev_pool.size()) return;
    cudaEvent_t start = c->ev_pool[c->ev_used++];
    stop = c->ev_pool[c->ev_used++];
    cudaEventRecord(start, s);
    c->ev_marks.push_back({stage, {start, stop}});
  }
  ~StageMark() {
    if (stop) cudaEventRecord(stop, s);
  }
};

// Per-iteration counters, one block per pass (each pass clears its own):
// the eye pass's round queues, the hitpoint list, its shade queues and trace
// fetch counters; then the photon pass's round queues, shade queues and
// trace fetch counters.
constexpr size_t kEyeCounters = (kWaveRounds + 2) + 1 + kWaveRounds * kShadeQueues + kWaveRounds;
constexpr size_t kPhotonCounters = (kWaveRounds + 2) + kWaveRounds * kShadeQueues + kWaveRounds;
constexpr size_t kCounters = kEyeCounters + kPhotonCounters;

// Photon rounds r, r+1, ... as nested conditional (IF) nodes of the graph
// being captured on stream s: k_round_gate sets the node's condition, and
// the body (captured on the stream of the next nesting level) holds the
// round's trace, sort and shade kernels and then the node of round r + 1.
// A skipped round so ends the chain: it costs the one gate launch.
int enqueue_gated_photon_rounds(fr_ctx* c, const IterParams& it, int r, cudaStream_t s, int grid, int sort_grid) {
  if (r >= kPhotonRounds) return FR_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  FR_CUDA(cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, nullptr, nullptr, nullptr));
  if (cs != cudaStreamCaptureStatusActive || !g) return fail(FR_ERR_CUDA, "gated round %d: stream not capturing", r);
  cudaGraphConditionalHandle h;
  FR_CUDA(cudaGraphConditionalHandleCreate(&h, g, 0u, cudaGraphCondAssignDefault));
  launch_round_gate(h, c->wave, r, c->rounds_run, s);
  c->launches += 1;  // the gate; fr_profile_read adds the rounds it lets run
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  FR_CUDA(cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &ndeps));
  cudaGraphNodeParams p{};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeIf;
  p.conditional.size = 1;
  cudaGraphNode_t node = nullptr;
  FR_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &p));
  FR_CUDA(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  cudaStream_t b = c->body[r - kPhotonGatedFrom];
  FR_CUDA(cudaStreamBeginCaptureToGraph(b, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal));
  launch_wave_trace(c->sc, c->wave, r, grid, false, c->err, b);
  launch_wave_sort(c->sc, c->wave, r, sort_grid, b);
  launch_pw_shade(c->sc, it, c->ph, c->wave, c->counts, r, grid, b);
  const int rc = enqueue_gated_photon_rounds(c, it, r + 1, b, grid, sort_grid);
  cudaGraph_t captured = nullptr;
  const cudaError_t e = cudaStreamEndCapture(b, &captured);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(FR_ERR_CUDA, "gated round %d: %s", r, cudaGetErrorString(e));
  return FR_OK;
}

// The parts of an iteration and the stream each runs on.
enum { kPartPhoton = 0, kPartEye = 1, kPartGrid = 2, kPartGather = 3, kPartTrain = 4 };

IterParams iter_params(const fr_ctx* c, uint32_t* step) {
  IterParams it{};
  it.step = step;
  it.photons = c->P;
  it.width = c->W;
  it.height = c->H;
  it.alpha = c->alpha;
  it.flags = c->flags;
  return it;
}

// Photon pass (main stream): the photon pass's iteration counter, its
// counters, emission, the wavefront rounds (the late ones as conditional
// graph nodes while capturing) and the tail.
int enqueue_photon_pass(fr_ctx* c, cudaStream_t s) {
  const IterParams it = iter_params(c, c->step_dev);
  launch_next_step(c->step_dev, s);
  FR_CUDA(cudaMemsetAsync(c->wave.qcount, 0, sizeof(uint32_t) * kPhotonCounters, s));
  StageMark m(c, FR_STAGE_PHOTON, s);
  const int grid = c->photon_blocks;
  const int sort_grid = (int)std::min<size_t>(((size_t)c->P + 255) / 256, 4 * (size_t)grid);
  if (c->guided)
    launch_pw_emit_guided(c->sc, it, c->ph, c->wave, c->counts, c->guide, s);
  else
    launch_pw_emit(c->sc, it, c->ph, c->wave, c->counts, s);
  for (int r = 0; r < kPhotonRounds; ++r) {
    if (c->capturing && r == kPhotonGatedFrom) {
      const int rc = enqueue_gated_photon_rounds(c, it, r, s, grid, sort_grid);
      if (rc) return rc;
      break;
    }
    {
      StageMark t(c, FR_STAGE_PHOTON_TRACE, s);
      launch_wave_trace(c->sc, c->wave, r, grid, false, c->err, s);
    }
    launch_wave_sort(c->sc, c->wave, r, sort_grid, s);
    launch_pw_shade(c->sc, it, c->ph, c->wave, c->counts, r, grid, s);
    c->launches += 3;
  }
  launch_pw_tail(c->sc, it, c->ph, c->wave, c->counts, kPhotonRounds, c->tail_blocks, c->err, s);
  c->launches += 3;  // counter, emission, tail
  FR_CUDA(cudaGetLastError());
  return FR_OK;
}

// Eye pass (pixel stream): the eye pass's iteration counter, its counters
// and the hitpoint list, then the wavefront rounds and the tail.  It writes
// the hitpoints the gather reads, so it follows the previous gather.
int enqueue_eye_pass(fr_ctx* c, cudaStream_t e) {
  const IterParams it = iter_params(c, c->step_dev + 1);
  launch_next_step(c->step_dev + 1, e);
  FR_CUDA(cudaMemsetAsync(c->eye_wave.qcount, 0, sizeof(uint32_t) * kEyeCounters, e));
  StageMark m(c, FR_STAGE_EYE, e);
  const int grid = c->eye_blocks;
  const int sort_grid = (int)std::min<size_t>(((size_t)c->W * c->H + 255) / 256, 4 * (size_t)grid);
  if (c->sc.env) FR_CUDA(cudaMemsetAsync(c->hp.dl, 0, sizeof(float4) * (size_t)c->W * c->H, e));
  launch_ew_start(c->cam, it, c->eye_wave, e);
  for (int r = 0; r < kEyeRounds; ++r) {
    {
      StageMark t(c, FR_STAGE_EYE_TRACE, e);
      launch_wave_trace(c->sc, c->eye_wave, r, grid, r == 0, c->err, e);
    }
    launch_wave_sort(c->sc, c->eye_wave, r, sort_grid, e);
    launch_ew_shade(c->sc, it, c->rr_eye, c->eye_wave, c->hp, c->st, c->gi, r, grid, e);
  }
  launch_ew_tail(c->sc, it, c->rr_eye, c->eye_wave, c->hp, c->st, c->gi, kEyeRounds, grid, c->err, e);
  c->launches += 3 + 3 * kEyeRounds;  // counter, start, rounds, tail
  FR_CUDA(cudaGetLastError());
  return FR_OK;
}

// Photon grid (main stream): cell size from this iteration's hitpoint radii,
// then count, scan and scatter of the stored photons into the grid's own
// sorted copy, which is all the gather reads of them.
int enqueue_grid(fr_ctx* c, cudaStream_t s) {
  StageMark m(c, FR_STAGE_GRID, s);
  launch_grid_setup(c->gi, c->sc, c->cell_scale, c->r0, s);
  FR_CUDA(cudaMemsetAsync(c->grid.cell_count, 0, sizeof(uint32_t) * (size_t)c->grid.table, s));
  launch_photon_count(c->ph, c->counts, c->P, kPhotonSlots, c->grid, c->gi, s);
  c->launches += launch_scan(c->grid.cell_count, c->grid.cell_start, c->grid.table + 1, c->scan, s);
  launch_photon_scatter(c->ph, c->counts, c->P, kPhotonSlots, c->grid, c->gi, s);
  c->launches += 3;
  FR_CUDA(cudaGetLastError());
  return FR_OK;
}

// Gather with the N/tau/R update (pixel stream).  Guided: then the training's
// weights (from the previous iteration's training) become the emission's,
// and this iteration's samples are selected; the training itself is the
// next part.
int enqueue_gather(fr_ctx* c, cudaStream_t e) {
  const IterParams it = iter_params(c, c->step_dev + 1);
  {
    StageMark m(c, FR_STAGE_GATHER, e);
    FR_CUDA(cudaMemsetAsync(c->dbg_m, 0, sizeof(int32_t) * (size_t)c->W * c->H, e));
    FR_CUDA(cudaMemsetAsync(c->dbg_phi, 0, sizeof(float4) * (size_t)c->W * c->H, e));
    launch_gather_update(c->sc, it, c->hp, c->grid, c->gi, c->st, c->dbg_m, c->dbg_phi,
                         c->guided ? c->guide.importance : nullptr, c->gather_blocks, e);
    c->launches += 1;
  }
  if (c->guided) {
    if (launch_guide_publish(c->guide, e)) return fail(FR_ERR_CUDA, "guide: weight copy failed");
    c->launches += launch_guide_select_batch(c->guide, c->P, e);
  }
  FR_CUDA(cudaGetLastError());
  return FR_OK;
}

// The guide's training on the selected samples: per Adam step, gradients,
// Adam with the weight tiles, step bookkeeping.
int enqueue_train(fr_ctx* c, cudaStream_t t) {
  c->launches += launch_guide_steps(c->guide, t);
  FR_CUDA(cudaGetLastError());
  return FR_OK;
}

int enqueue_part(fr_ctx* c, int part, cudaStream_t s) {
  switch (part) {
    case kPartPhoton: return enqueue_photon_pass(c, s);
    case kPartEye: return enqueue_eye_pass(c, s);
    case kPartGrid: return enqueue_grid(c, s);
    case kPartGather: return enqueue_gather(c, s);
    default: return enqueue_train(c, s);
  }
}

// One part on stream s: a replay of its graph (captured on first use), or
// direct launches while the stage profiler records events or while a batch
// graph is being captured.
int run_part(fr_ctx* c, int part, cudaStream_t s, bool graphs) {
  if (!graphs) return enqueue_part(c, part, s);
  if (!c->part_exec[part]) {
    const int64_t before = c->launches;
    FR_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    c->capturing = true;
    const int rc = enqueue_part(c, part, s);
    c->capturing = false;
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(s, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ec != cudaSuccess) return fail(FR_ERR_CUDA, "iteration capture (part %d): %s", part, cudaGetErrorString(ec));
    c->part_graph[part] = g;
    FR_CUDA(cudaGraphInstantiate(&c->part_exec[part], g, 0));
    c->part_launches[part] = c->launches - before;
    c->launches = before;
  }
  FR_CUDA(cudaGraphLaunch(c->part_exec[part], s));
  c->launches += c->part_launches[part];
  return FR_OK;
}

// The pixel stream waits for the main stream's work so far, or the reverse.
int side_after_main(fr_ctx* c) {
  FR_CUDA(cudaEventRecord(c->fork_ev, c->stream));
  FR_CUDA(cudaStreamWaitEvent(c->side, c->fork_ev, 0));
  return FR_OK;
}
int main_after_side(fr_ctx* c) {
  FR_CUDA(cudaEventRecord(c->join_ev, c->side));
  FR_CUDA(cudaStreamWaitEvent(c->stream, c->join_ev, 0));
  return FR_OK;
}
// The main stream waits for all of the context's work: the pixel stream and
// the guide's training.
int join_streams(fr_ctx* c) {
  const int rc = main_after_side(c);
  if (rc || !c->guided) return rc;
  FR_CUDA(cudaStreamWaitEvent(c->stream, c->train_ev, 0));
  return FR_OK;
}

// One iteration on the context's streams:
//   main:  photon pass ........ wait(eye) grid
//   pixel: eye pass ---------^             wait(grid) gather [publish, selection]
//   train (guided):                                                  wait(selection) training
// The gather is left running on the pixel stream: the next iteration's
// photon pass starts as soon as this grid is built (it overwrites only the
// photon slots, which the grid has copied), and its eye pass follows the
// gather on the pixel stream (it rewrites the hitpoints the gather reads).
// Guided: the next emission clears the importance this gather accumulates
// and rewrites the inputs and directions of the paths, so the main stream
// waits for the selection, which has copied the samples; the emission
// samples the weights published before the selection (the training of the
// iteration before), so the training runs beside the next iteration, and the
// next publish waits for it.  In a batch graph's capture the training runs
// on the pixel stream instead (the capture may not wait on events recorded
// outside it); the weights each emission samples are the same.  Every call
// that reads or writes the per-pixel state or the guide from the main stream
// first makes it wait for the other streams (join_streams).
int issue_iteration(fr_ctx* c, bool graphs) {
  const bool batch = c->capturing;
  const bool train_apart = c->guided && !batch;
  int rc = side_after_main(c);  // calls that wrote state on the main stream since the last iteration
  if (!rc && train_apart) FR_CUDA(cudaStreamWaitEvent(c->stream, c->sel_ev, 0));
  if (!rc) rc = run_part(c, kPartPhoton, c->stream, graphs);
  if (!rc) rc = run_part(c, kPartEye, c->side, graphs);
  if (!rc) rc = main_after_side(c);
  if (!rc) rc = run_part(c, kPartGrid, c->stream, graphs);
  if (!rc) rc = side_after_main(c);
  if (!rc && train_apart) FR_CUDA(cudaStreamWaitEvent(c->side, c->train_ev, 0));
  if (!rc) rc = run_part(c, kPartGather, c->side, graphs);
  if (!rc && c->guided) {
    if (train_apart) {
      FR_CUDA(cudaEventRecord(c->sel_ev, c->side));
      FR_CUDA(cudaStreamWaitEvent(c->train_stream, c->sel_ev, 0));
      rc = run_part(c, kPartTrain, c->train_stream, graphs);
      if (!rc) FR_CUDA(cudaEventRecord(c->train_ev, c->train_stream));
    } else {
      rc = run_part(c, kPartTrain, c->side, graphs);
      if (!rc) rc = main_after_side(c);
    }
  }
  return rc;
}

// One iteration: replays of the part graphs, or (while the stage
// profiler records events) direct launches.
int run_iteration(fr_ctx* c) {
  const int rc = issue_iteration(c, !c->profiling);
  if (rc) return rc;
  ++c->iterations;
  c->photons_total += c->P;
  return FR_OK;
}

int check_device_error(fr_ctx* c) {
  int e = 0;
  FR_CUDA(cudaMemcpyAsync(&e, c->err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  FR_CUDA(cudaStreamSynchronize(c->stream));
  if (e & kErrStack) return fail(FR_ERR_DEVICE, "BVH traversal stack overflow (depth %d)", c->bvh_depth);
  if (e & kErrGuide) return fail(FR_ERR_DEVICE, "photon guide: a tensor-core wait gave up");
  if (e & kErrQuery) return fail(FR_ERR_INVALID, "radius query: a ball was refused (radius not finite, or more "
                                                 "than %d cells along an axis)", kMaxQuerySpan);
  if (e) return fail(FR_ERR_DEVICE, "device error word %d", e);
  return FR_OK;
}

}  // namespace

int fr::set_last_error(int code, const std::string& message) {
  g_error = message;
  return code;
}

extern "C" {

const char* fr_last_error(void) { return g_error.c_str(); }

int fr_create(const fr_scene_desc* scene, const fr_camera_desc* camera, const fr_sppm_params* params, fr_ctx** out) {
  g_error.clear();
  if (!out) return fail(FR_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int rc = check_scene(scene);
  if (rc) return rc;
  if (!camera || camera->width <= 0 || camera->height <= 0 || (camera->type != 0 && camera->type != 1))
    return fail(FR_ERR_INVALID, "camera: bad type or size");
  if (!params || params->photons_per_iteration <= 0) return fail(FR_ERR_INVALID, "params: photons_per_iteration");
  if (!(params->initial_radius > 0.0f)) return fail(FR_ERR_INVALID, "params: initial_radius");
  if ((int64_t)camera->width * camera->height > (1 << 30)) return fail(FR_ERR_INVALID, "camera: too many pixels");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(FR_ERR_CUDA, "no CUDA device");

  fr_ctx* c = new fr_ctx();
  auto bail = [&](int code) {
    delete c;
    return code;
  };
  // The photon pass (main stream) is the iteration's critical path; the eye
  // pass (side stream) runs at a lower priority and fills the SMs the photon
  // pass leaves idle.
  int prio_low = 0, prio_high = 0;
  cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
  if (cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, prio_high) != cudaSuccess ||
      cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, prio_low) != cudaSuccess ||
      cudaStreamCreateWithPriority(&c->train_stream, cudaStreamNonBlocking, prio_low) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->sel_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->train_ev, cudaEventDisableTiming) != cudaSuccess)
    return bail(fail(FR_ERR_CUDA, "cudaStreamCreate/cudaEventCreate failed"));
  for (cudaStream_t& b : c->body)
    if (cudaStreamCreateWithFlags(&b, cudaStreamNonBlocking) != cudaSuccess)
      return bail(fail(FR_ERR_CUDA, "cudaStreamCreate failed"));
  if (cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(FR_ERR_CUDA, "cudaStreamCreate failed"));
  for (int k = 0; k < 2; ++k)
    if (cudaEventCreateWithFlags(&c->ready[k], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->copied[k], cudaEventDisableTiming) != cudaSuccess)
      return bail(fail(FR_ERR_CUDA, "cudaEventCreate failed"));
  c->W = camera->width;
  c->H = camera->height;
  c->P = params->photons_per_iteration;
  c->alpha = params->alpha;
  c->r0 = params->initial_radius;
  c->flags = params->flags;
  c->cell_scale = params->grid_cell_scale > 0.0f ? params->grid_cell_scale : 2.0f;
  c->rr_eye[0] = (float)std::exp((double)(4 - 5));  // getHitpointInfo RR (SPPM.cpp:117)
  c->rr_eye[1] = (float)std::exp((double)(4 - 6));
  c->cam = setup_camera(*camera);
  upload_byte_lut(c->stream);
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return bail(fail(FR_ERR_CUDA, "device query failed"));
  ExactTables tabs;
  if ((rc = exact_tables(dev, &tabs))) return bail(rc);
  upload_tables(tabs.sincos, tabs.sqrt1m, c->stream);
  c->photon_blocks = std::max(1, photon_pass_blocks_per_sm()) * sms;
  c->eye_blocks = std::max(1, c->photon_blocks * FR_EYE_GRID_PCT / 100);
  c->tail_blocks = std::max(1, pw_tail_blocks_per_sm()) * sms;
  c->gather_blocks = std::max(1, std::max(1, gather_blocks_per_sm()) * sms * FR_GATHER_GRID_PCT / 100);
  c->sms = sms;

  // ---- geometry
  const int T = scene->num_facets;
  float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
  for (size_t i = 0; i < (size_t)T * 3; ++i)
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], scene->positions[3 * i + a]);
      hi[a] = std::max(hi[a], scene->positions[3 * i + a]);
    }
  const float diag = std::sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) + (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                               (hi[2] - lo[2]) * (hi[2] - lo[2]));
  BVHResult bvh;
  if (params->bvh_builder == FR_BVH_DEVICE_LBVH) {
    const char* msg = "";
    if (build_bvh8_lbvh(scene->positions, T, lo, hi, 1e-5f * diag + 1e-7f, bvh, &msg))
      return bail(fail(FR_ERR_CUDA, "device BVH build: %s", msg));
  } else if (params->bvh_builder == FR_BVH_HOST_SAH) {
    bvh = build_bvh8(scene->positions, T, 1e-5f * diag + 1e-7f);
  } else {
    return bail(fail(FR_ERR_INVALID, "params: bvh_builder %d", params->bvh_builder));
  }
  c->bvh_depth = bvh.depth;
  if (bvh.depth * 7 + 1 > kTraversalStackEntries) return bail(fail(FR_ERR_INVALID, "BVH depth %d exceeds the traversal stack", bvh.depth));
  std::vector<TriGPU> tris(T);
  for (int k = 0; k < T; ++k) {
    const int f = bvh.tri_order[k];
    const float* P = scene->positions + 9 * (size_t)f;
    TriGPU& t = tris[k];
    for (int a = 0; a < 3; ++a) {
      t.v0[a] = P[a];
      t.e1[a] = P[3 + a] - P[a];
      t.e2[a] = P[6 + a] - P[a];
    }
    int32_t fid = f;
    std::memcpy(&t.v0[3], &fid, 4);
    t.e1[3] = 0.f;
    t.e2[3] = 0.f;
  }
  std::vector<FacetShade> shade(T);
  for (int f = 0; f < T; ++f) {
    FacetShade& s = shade[f];
    const float* N = scene->normals + 9 * (size_t)f;
    const float* U = scene->uvs + 6 * (size_t)f;
    for (int a = 0; a < 3; ++a) { s.n0[a] = N[a]; s.n1[a] = N[3 + a]; s.n2[a] = N[6 + a]; }
    s.uv0[0] = U[0]; s.uv0[1] = U[1]; s.uv1[0] = U[2]; s.uv1[1] = U[3]; s.uv2[0] = U[4]; s.uv2[1] = U[5];
    s.attr = scene->material_ids[f];
  }
  std::vector<MaterialGPU> mats(scene->num_materials);
  for (int m = 0; m < scene->num_materials; ++m) {
    const fr_material_desc& d = scene->materials[m];
    MaterialGPU& g = mats[m];
    g.type = d.type;
    g.flags = (d.sppm_surface ? kMatSPPM : 0) | (d.opaque ? kMatOpaque : 0);
    g.tex_albedo = d.tex_albedo;
    g.tex_rough = d.tex_roughness;
    g.tex_bump = d.tex_bump;
    for (int a = 0; a < 3; ++a) { g.albedo[a] = d.albedo[a]; g.radiance[a] = d.emission[a]; }
    g.index = d.index;
    g.roughness = d.roughness;
    g.extinction = d.extinction;
    g.reflectance = d.reflectance;
  }
  std::vector<LightGPU> lights;
  std::vector<EmitEntry> emit;
  build_lights(*scene, lights, emit);
  if (lights.empty()) return bail(fail(FR_ERR_INVALID, "scene: no emissive facets"));

  BVHNodeW* d_nodes;
  TriGPU* d_tris;
  FacetShade* d_shade;
  MaterialGPU* d_mats;
  LightGPU* d_lights;
  EmitEntry* d_emit;
  if ((rc = c->upload(&d_nodes, bvh.nodes.data(), bvh.nodes.size())) ||
      (rc = c->upload(&d_tris, tris.data(), tris.size())) || (rc = c->upload(&d_shade, shade.data(), shade.size())) ||
      (rc = c->upload(&d_mats, mats.data(), mats.size())) ||
      (rc = c->upload(&d_lights, lights.data(), lights.size())) ||
      (rc = c->upload(&d_emit, emit.data(), emit.size())))
    return bail(rc);
  std::vector<TextureGPU> texs(scene->num_textures);
  for (int t = 0; t < scene->num_textures; ++t) {
    const fr_texture_desc& td = scene->textures[t];
    uint32_t* d_tex;
    const size_t n = (size_t)td.width * td.height;
    if ((rc = c->alloc(&d_tex, n))) return bail(rc);
    if (cudaMemcpyAsync(d_tex, td.texels, n * 4, cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
      return bail(fail(FR_ERR_CUDA, "texture upload"));
    texs[t] = TextureGPU{d_tex, td.width, td.height, 0, 0};
  }
  TextureGPU* d_texs;
  if ((rc = c->upload(&d_texs, texs.data(), texs.size()))) return bail(rc);
  // Environment map: texels c = byte / 255.0f (TextureUtility.cpp:28)
  // converted as LightSampler.cpp:24 does, 0.4 * (c^2, c^2, c^2, 0) (the
  // double literal meets Vec4's operator*(float, Vec4)).
  float4* d_env = nullptr;
  int32_t env_w = 0, env_h = 0;
  if (const fr_texture_desc* e = scene->environment) {
    if (e->width <= 0 || e->height <= 0 || !e->texels) return bail(fail(FR_ERR_INVALID, "scene: bad environment map"));
    env_w = e->width;
    env_h = e->height;
    std::vector<float4> env((size_t)env_w * env_h);
    const uint8_t* px = static_cast<const uint8_t*>(e->texels);
    for (size_t k = 0; k < env.size(); ++k) {
      float v[4];
      for (int ch = 0; ch < 4; ++ch) {
        const float cv = ch < 3 ? px[4 * k + ch] / 255.0f : 0.0f;
        v[ch] = 0.4f * (cv * cv);
      }
      env[k] = make_float4(v[0], v[1], v[2], v[3]);
    }
    if ((rc = c->upload(&d_env, env.data(), env.size()))) return bail(rc);
  }
  // Watertight mode: the exact v1, v2 of every triangle in leaf order (the
  // test must see the vertices a neighbouring triangle shares, not v0 + e1).
  float4* d_v12 = nullptr;
  if (params->flags & kFlagWatertight) {
    std::vector<float4> v12(2 * (size_t)T);
    for (int k = 0; k < T; ++k) {
      const float* P = scene->positions + 9 * (size_t)bvh.tri_order[k];
      v12[2 * (size_t)k] = make_float4(P[3], P[4], P[5], 0.0f);
      v12[2 * (size_t)k + 1] = make_float4(P[6], P[7], P[8], 0.0f);
    }
    if ((rc = c->upload(&d_v12, v12.data(), v12.size()))) return bail(rc);
  }
  c->sc = SceneGPU{d_nodes, d_tris, d_shade, d_mats, d_texs, d_lights, d_emit,
                   (int32_t)bvh.nodes.size(), T, T, (int32_t)lights.size(),
                   {lo[0], lo[1], lo[2]}, {hi[0], hi[1], hi[2]}, reinterpret_cast<const float*>(d_env), env_w, env_h,
                   reinterpret_cast<const float*>(d_v12), d_v12 ? 1 : 0, 0};

  // ---- per-iteration buffers (all allocated here; iterations allocate nothing)
  const size_t npix = (size_t)c->W * c->H;
  const size_t nslots = (size_t)c->P * kPhotonSlots;
  const size_t wave_n = (size_t)c->P;
  c->ph.paths = (uint32_t)c->P;  // slot stride of the slot-major photon slots
  if ((rc = c->alloc(&c->hp.pos, npix)) || (rc = c->alloc(&c->hp.nrm, npix)) || (rc = c->alloc(&c->hp.out, npix)) ||
      (rc = c->alloc(&c->hp.wgt, npix)) || (rc = c->alloc(&c->st.tau, 3 * npix)) || (rc = c->alloc(&c->st.n, npix)) ||
      (rc = c->alloc(&c->st.r, npix)) || (rc = c->alloc(&c->st.g, npix)) || (rc = c->alloc(&c->st.dl, npix)) ||
      (rc = c->alloc(&c->hp.dl, npix)) || (rc = c->alloc(&c->ph.pos, nslots)) ||
      (rc = c->alloc(&c->ph.flux, nslots)) || (rc = c->alloc(&c->ph.dir, nslots)) ||
      (rc = c->alloc(&c->counts, (size_t)c->P)) || (rc = c->alloc(&c->wave.a, wave_n)) ||
      (rc = c->alloc(&c->wave.b, wave_n)) || (rc = c->alloc(&c->wave.c, wave_n)) ||
      (rc = c->alloc(&c->wave.d, wave_n)) || (rc = c->alloc(&c->wave.hit, wave_n)) ||
      (rc = c->alloc(&c->wave.queue[0], wave_n)) || (rc = c->alloc(&c->wave.queue[1], wave_n)) ||
      (rc = c->alloc(&c->eye_wave.a, npix)) || (rc = c->alloc(&c->eye_wave.b, npix)) ||
      (rc = c->alloc(&c->eye_wave.c, npix)) || (rc = c->alloc(&c->eye_wave.d, npix)) ||
      (rc = c->alloc(&c->eye_wave.hit, npix)) || (rc = c->alloc(&c->eye_wave.queue[0], npix)) ||
      (rc = c->alloc(&c->eye_wave.queue[1], npix)) ||
      (rc = c->alloc(&c->wave.qcount, kCounters)) || (rc = c->alloc(&c->hp.list, npix)) ||
      (rc = c->alloc(&c->wave.mq, (size_t)kShadeQueues * wave_n)) ||
      (rc = c->alloc(&c->eye_wave.mq, (size_t)kShadeQueues * npix)) ||
      (rc = c->alloc(&c->gi, 1)) || (rc = c->alloc(&c->step_dev, 2)) || (rc = c->alloc(&c->rounds_run, 1)) ||
      (rc = c->alloc(&c->err, 1)) ||
      (rc = c->alloc(&c->dbg_m, npix)) || (rc = c->alloc(&c->dbg_phi, npix)) || (rc = c->alloc(&c->image, npix)) ||
      (rc = c->alloc(&c->image_b, npix)) || (rc = c->alloc(&c->image8, npix)))
    return bail(rc);
  // Counters, one contiguous block per pass (each pass clears its own):
  // eye rounds, the hitpoint list, eye shade queues, eye trace fetches; then
  // photon rounds, photon shade queues, photon trace fetches.
  c->eye_wave.qcount = c->wave.qcount;
  c->hp.list_count = c->eye_wave.qcount + (kWaveRounds + 2);
  c->eye_wave.mcount = c->hp.list_count + 1;
  c->eye_wave.tfetch = c->eye_wave.mcount + kWaveRounds * kShadeQueues;
  c->wave.qcount = c->eye_wave.qcount + kEyeCounters;
  c->wave.mcount = c->wave.qcount + (kWaveRounds + 2);
  c->wave.tfetch = c->wave.mcount + kWaveRounds * kShadeQueues;
  static_assert(kEyeCounters == (kWaveRounds + 2) + 1 + kWaveRounds * kShadeQueues + kWaveRounds, "eye block");
  c->eye_wave.cap = (uint32_t)npix;
  c->wave.cap = (uint32_t)wave_n;
  c->eye_wave.min_live = kEyeTailMin;
  c->wave.min_live = kPhotonTailMin;
  // Photon grid: about two buckets per photon path (paths store ~1.2 photons
  // on the mixed-materials scene).
// Buckets of the photon grid per photon path (rounded up to a power of two):
// 2 clears and scans a table half the size of 4 for a few more shared
// buckets (mixed materials: grid build 0.257 vs 0.272 ms, gather 0.368 vs
// 0.378 ms; 1 made the gather slower).
#ifndef FR_GRID_BUCKETS_PER_PATH
#define FR_GRID_BUCKETS_PER_PATH 2
#endif
  c->grid.table = next_pow2(std::max<uint64_t>((uint64_t)c->P * FR_GRID_BUCKETS_PER_PATH, 1u << 16));
  const size_t cap = nslots;
  if ((rc = c->alloc(&c->grid.pos, cap)) || (rc = c->alloc(&c->grid.flux, cap)) || (rc = c->alloc(&c->grid.dir, cap)) ||
      (rc = c->alloc(&c->grid.cell_count, (size_t)c->grid.table + 1)) ||
      (rc = c->alloc(&c->grid.cell_start, (size_t)c->grid.table + 1)))
    return bail(rc);
  const uint32_t words = scan_temp_words(c->grid.table + 1, c->scan);
  uint32_t* sw;
  if ((rc = c->alloc(&sw, words))) return bail(rc);
  for (int l = 0; l < c->scan.levels; ++l) {
    c->scan.level[l] = sw;
    sw += c->scan.level_n[l] + 1;
  }
  // ---- photon-emission guide
  if (params->guide) {
    GuideGPU& g = c->guide;
    g.plain_fraction = params->guide_plain_fraction > 0.0f ? std::min(1.0f, params->guide_plain_fraction) : 0.2f;
    g.batch_cap = std::min(c->P, params->guide_batch > 0 ? params->guide_batch : 16384);
    g.lr = params->guide_learning_rate > 0.0f ? params->guide_learning_rate : 0.005f;
    g.steps = params->guide_steps > 0 ? std::min(params->guide_steps, 64) : 16;
    g.train_ctas = std::max(1, c->sms);
    if ((rc = c->alloc(&g.params, kGuideParams)) || (rc = c->alloc(&g.grad, kGuideParams)) ||
        (rc = c->alloc(&g.adam_m, kGuideParams)) || (rc = c->alloc(&g.adam_v, kGuideParams)) ||
        (rc = c->alloc(&g.tiles, kTileBytes)) || (rc = c->alloc(&g.emit_params, kGuideParams)) ||
        (rc = c->alloc(&g.emit_tiles, kTileBytes)) || (rc = c->alloc(&g.feat, (size_t)c->P)) ||
        (rc = c->alloc(&g.dir, (size_t)c->P)) || (rc = c->alloc(&g.importance, 2 * (size_t)c->P)) ||
        (rc = c->alloc(&g.batch, (size_t)g.batch_cap)) || (rc = c->alloc(&g.batch_w, (size_t)g.batch_cap)) ||
        (rc = c->alloc(&g.batch_feat, (size_t)g.batch_cap)) || (rc = c->alloc(&g.batch_dir, (size_t)g.batch_cap)) ||
        (rc = c->alloc(&g.batch_count, 1)) || (rc = c->alloc(&g.select_part, (size_t)guide_select_blocks(c->P))) ||
        (rc = c->alloc(&g.grad_part, (size_t)g.train_ctas * kGuideParams)) ||
        (rc = c->alloc(&g.wsum_part, (size_t)g.train_ctas)) || (rc = c->alloc(&g.weight_sum, 1)) ||
        (rc = c->alloc(&g.adam_step, 1)))
      return bail(rc);
    g.err = c->err;
    if (guide_configure()) return bail(fail(FR_ERR_CUDA, "guide: shared-memory opt-in failed"));
    const std::vector<float> p0 = guide_initial_params(params->guide_seed);
    FR_CUDA(cudaMemcpyAsync(g.params, p0.data(), sizeof(float) * kGuideParams, cudaMemcpyHostToDevice, c->stream));
    for (float* z : {g.grad, g.adam_m, g.adam_v})
      FR_CUDA(cudaMemsetAsync(z, 0, sizeof(float) * kGuideParams, c->stream));
    FR_CUDA(cudaMemsetAsync(g.batch_count, 0, 4, c->stream));
    FR_CUDA(cudaMemsetAsync(g.weight_sum, 0, 4, c->stream));
    FR_CUDA(cudaMemsetAsync(g.adam_step, 0, 4, c->stream));
    FR_CUDA(cudaMemsetAsync(g.importance, 0, 2 * sizeof(unsigned long long) * (size_t)c->P, c->stream));
    launch_guide_prepare(g, c->stream);
    if (launch_guide_publish(g, c->stream)) return bail(fail(FR_ERR_CUDA, "guide: weight copy failed"));
    c->guided = true;
  }

  // Initial state: initializeSharedPoints (SPPM.cpp:356-373) and empty photon slots.
  std::vector<float> r(npix, c->r0);
  if (cudaMemcpyAsync(c->st.r, r.data(), npix * 4, cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
    return bail(fail(FR_ERR_CUDA, "state upload"));
  cudaMemsetAsync(c->st.tau, 0, 3 * npix * sizeof(double), c->stream);
  cudaMemsetAsync(c->st.n, 0, npix * 4, c->stream);
  cudaMemsetAsync(c->st.g, 0, npix * 4, c->stream);
  cudaMemsetAsync(c->st.dl, 0, npix * sizeof(float4), c->stream);
  cudaMemsetAsync(c->hp.dl, 0, npix * sizeof(float4), c->stream);
  cudaMemsetAsync(c->ph.dir, 0, nslots * sizeof(float4), c->stream);
  cudaMemsetAsync(c->ph.pos, 0, nslots * sizeof(float4), c->stream);
  cudaMemsetAsync(c->ph.flux, 0, nslots * sizeof(float4), c->stream);
  cudaMemsetAsync(c->gi, 0, sizeof(GridInfo), c->stream);
  cudaMemsetAsync(c->step_dev, 0, 2 * sizeof(uint32_t), c->stream);
  cudaMemsetAsync(c->rounds_run, 0, sizeof(uint32_t), c->stream);
  cudaMemsetAsync(c->err, 0, sizeof(int), c->stream);
  cudaMemsetAsync(c->hp.pos, 0, npix * sizeof(float4), c->stream);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess)
    return bail(fail(FR_ERR_CUDA, "initialisation failed"));
  *out = c;
  return FR_OK;
}

int fr_iterate(fr_ctx* c, int n) {
  if (!c || n < 0) return fail(FR_ERR_INVALID, "fr_iterate: bad arguments");
  for (int k = 0; k < n; ++k) {
    const int rc = run_iteration(c);
    if (rc) return rc;
  }
  return FR_OK;
}

int fr_iterate_batch(fr_ctx* const* ctxs, int count, int n) {
  if (!ctxs || count < 0 || n < 0) return fail(FR_ERR_INVALID, "fr_iterate_batch: bad arguments");
  for (int j = 0; j < count; ++j)
    if (!ctxs[j]) return fail(FR_ERR_INVALID, "fr_iterate_batch: context %d is NULL", j);
  // Iteration k of every context before iteration k + 1 of any: each context
  // replays its graph on its own streams, so the scenes' kernels share the
  // GPU and the small ones fill what the large ones leave idle.
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < count; ++j) {
      const int rc = run_iteration(ctxs[j]);
      if (rc) return rc;
    }
  return FR_OK;
}

struct fr_batch {
  std::vector<fr_ctx*> ctxs;
  std::vector<int64_t> launches;  // per context: kernels of one iteration
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr;
  std::vector<cudaEvent_t> ready;  // per context: its stream's prior work
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~fr_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (cudaEvent_t e : ready) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    if (done) cudaEventDestroy(done);
    if (stream) cudaStreamDestroy(stream);
  }
};

// One capture on the batch's stream: a fork event joins every context's main
// stream (and through issue_iteration its pixel stream and the streams of the
// conditional photon rounds), each context enqueues one iteration ending
// with its pixel stream joined back, and the batch stream joins them all.
int fr_batch_create(fr_ctx* const* ctxs, int count, fr_batch** out) {
  if (!ctxs || count < 1 || !out) return fail(FR_ERR_INVALID, "fr_batch_create: bad arguments");
  *out = nullptr;
  for (int j = 0; j < count; ++j) {
    if (!ctxs[j]) return fail(FR_ERR_INVALID, "fr_batch_create: context %d is NULL", j);
    if (ctxs[j]->profiling) return fail(FR_ERR_INVALID, "fr_batch_create: context %d has the stage profiler on", j);
  }
  std::unique_ptr<fr_batch> b(new fr_batch());
  b->ctxs.assign(ctxs, ctxs + count);
  FR_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  FR_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
  FR_CUDA(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
  b->ready.resize(count);
  for (int j = 0; j < count; ++j) FR_CUDA(cudaEventCreateWithFlags(&b->ready[j], cudaEventDisableTiming));
  std::vector<cudaEvent_t> join(count);
  for (int j = 0; j < count; ++j) FR_CUDA(cudaEventCreateWithFlags(&join[j], cudaEventDisableTiming));
  auto drop_joins = [&]() {
    for (cudaEvent_t e : join) cudaEventDestroy(e);
  };
  FR_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  int rc = FR_OK;
  cudaEventRecord(b->fork, b->stream);
  for (int j = 0; j < count && !rc; ++j) {
    fr_ctx* c = ctxs[j];
    cudaStreamWaitEvent(c->stream, b->fork, 0);
    const int64_t before = c->launches;
    c->capturing = true;
    rc = issue_iteration(c, false);
    if (!rc) rc = main_after_side(c);  // the capture joins every stream it forked
    c->capturing = false;
    b->launches.push_back(c->launches - before);
    c->launches = before;
    cudaEventRecord(join[j], c->stream);
    cudaStreamWaitEvent(b->stream, join[j], 0);
  }
  cudaGraph_t g = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
  drop_joins();
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (ec != cudaSuccess) return fail(FR_ERR_CUDA, "batch capture: %s", cudaGetErrorString(ec));
  b->graph = g;
  FR_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
  *out = b.release();
  return FR_OK;
}

int fr_batch_iterate(fr_batch* b, int n) {
  if (!b || n < 0) return fail(FR_ERR_INVALID, "fr_batch_iterate: bad arguments");
  if (!n) return FR_OK;
  const size_t count = b->ctxs.size();
  for (size_t j = 0; j < count; ++j) {
    if (b->ctxs[j]->profiling) return fail(FR_ERR_INVALID, "fr_batch_iterate: context %zu has the stage profiler on", j);
    const int rc = join_streams(b->ctxs[j]);  // a gather or training still running from fr_iterate
    if (rc) return rc;
    FR_CUDA(cudaEventRecord(b->ready[j], b->ctxs[j]->stream));
    FR_CUDA(cudaStreamWaitEvent(b->stream, b->ready[j], 0));
  }
  for (int k = 0; k < n; ++k) FR_CUDA(cudaGraphLaunch(b->exec, b->stream));
  FR_CUDA(cudaEventRecord(b->done, b->stream));
  for (size_t j = 0; j < count; ++j) {
    fr_ctx* c = b->ctxs[j];
    FR_CUDA(cudaStreamWaitEvent(c->stream, b->done, 0));
    c->iterations += n;
    c->photons_total += (int64_t)c->P * n;
    c->launches += b->launches[j] * n;
  }
  return FR_OK;
}

void fr_batch_destroy(fr_batch* b) { delete b; }

namespace {
// Graph replay time of `iterations` iterations (ms); the graph is captured
// (and one iteration run) first.
int timed_iterations(fr_ctx* c, int iterations, float* ms) {
  int rc = run_iteration(c);
  if (rc) return rc;
  cudaEvent_t a = nullptr, b = nullptr;
  FR_CUDA(cudaEventCreate(&a));
  FR_CUDA(cudaEventCreate(&b));
  FR_CUDA(cudaEventRecord(a, c->stream));
  for (int k = 0; k < iterations && !rc; ++k) rc = run_iteration(c);
  if (!rc) rc = join_streams(c);  // the last gather and training
  FR_CUDA(cudaEventRecord(b, c->stream));
  FR_CUDA(cudaEventSynchronize(b));
  FR_CUDA(cudaEventElapsedTime(ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return rc ? rc : check_device_error(c);
}

void drop_graph(fr_ctx* c) {
  for (int k = 0; k < 5; ++k) {
    if (c->part_exec[k]) cudaGraphExecDestroy(c->part_exec[k]);
    if (c->part_graph[k]) cudaGraphDestroy(c->part_graph[k]);
    c->part_exec[k] = nullptr;
    c->part_graph[k] = nullptr;
  }
}
}  // namespace

int fr_autotune(fr_ctx* c, int iterations, uint32_t* photon_tail_min) {
  if (!c || iterations < 1) return fail(FR_ERR_INVALID, "fr_autotune: bad arguments");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  if (c->profiling) return fail(FR_ERR_INVALID, "fr_autotune: stage profiler on");
  static const uint32_t kCandidates[] = {4096u, 8192u, 16384u, 32768u, 65536u};
  uint32_t best = c->wave.min_live;
  float best_ms = 3.0e38f;
  for (uint32_t cand : kCandidates) {
    c->wave.min_live = cand;
    drop_graph(c);
    float ms = 0.0f;
    const int rc = timed_iterations(c, iterations, &ms);
    if (rc) return rc;
    if (ms < best_ms) {
      best_ms = ms;
      best = cand;
    }
  }
  c->wave.min_live = best;
  drop_graph(c);
  if (photon_tail_min) *photon_tail_min = best;
  return FR_OK;
}

int fr_synchronize(fr_ctx* c) {
  if (!c) return fail(FR_ERR_INVALID, "fr_synchronize: NULL context");
  const int rc = join_streams(c);
  if (rc) return rc;
  FR_CUDA(cudaStreamSynchronize(c->stream));
  FR_CUDA(cudaGetLastError());
  return check_device_error(c);
}

namespace {
int enqueue_resolve(fr_ctx* c, float4* out, cudaStream_t s) {
  launch_resolve(c->st, c->W * c->H, (double)c->photons_total, (double)c->iterations,
                 (c->flags & kFlagStandardResolve) != 0, out, s);
  FR_CUDA(cudaGetLastError());
  return FR_OK;
}
}  // namespace

int fr_resolve_dev(fr_ctx* c, float* rgba_dev) {
  if (!c || !rgba_dev) return fail(FR_ERR_INVALID, "fr_resolve_dev: bad arguments");
  const int rc = main_after_side(c);
  return rc ? rc : enqueue_resolve(c, reinterpret_cast<float4*>(rgba_dev), c->stream);
}

int fr_resolve_async(fr_ctx* c, float* rgba, uint64_t* ticket) {
  if (!c || !rgba) return fail(FR_ERR_INVALID, "fr_resolve_async: bad arguments");
  const int b = (int)(c->async_seq & 1u);
  float4* img = b ? c->image_b : c->image;
  // The resolve runs on the pixel stream after the last gather, so the next
  // iteration's photon pass does not wait for it.  The copy that last read
  // this image (two calls ago) must have landed before the resolve
  // overwrites it; a never-recorded event is no wait.
  int rc = side_after_main(c);
  if (rc) return rc;
  FR_CUDA(cudaStreamWaitEvent(c->side, c->copied[b], 0));
  rc = enqueue_resolve(c, img, c->side);
  if (rc) return rc;
  FR_CUDA(cudaEventRecord(c->ready[b], c->side));
  FR_CUDA(cudaStreamWaitEvent(c->copy_stream, c->ready[b], 0));
  FR_CUDA(cudaMemcpyAsync(rgba, img, sizeof(float4) * (size_t)c->W * c->H, cudaMemcpyDeviceToHost, c->copy_stream));
  FR_CUDA(cudaEventRecord(c->copied[b], c->copy_stream));
  if (ticket) *ticket = c->async_seq;
  ++c->async_seq;
  return FR_OK;
}

int fr_resolve_wait(fr_ctx* c, uint64_t ticket) {
  if (!c || ticket >= c->async_seq) return fail(FR_ERR_INVALID, "fr_resolve_wait: bad arguments");
  // The event of this ticket's buffer was recorded for this copy or a later
  // one on the same copy stream; either way, once it completes this copy has.
  // The device error word is left to fr_synchronize / fr_resolve: reading it
  // here would wait for the iteration now running.
  FR_CUDA(cudaEventSynchronize(c->copied[ticket & 1u]));
  return FR_OK;
}

int fr_resolve(fr_ctx* c, float* rgba) {
  if (!c || !rgba) return fail(FR_ERR_INVALID, "fr_resolve: bad arguments");
  FR_CUDA(cudaStreamWaitEvent(c->stream, c->copied[0], 0));  // an asynchronous copy of `image` in flight
  int rc = fr_resolve_dev(c, reinterpret_cast<float*>(c->image));
  if (rc) return rc;
  FR_CUDA(cudaMemcpyAsync(rgba, c->image, sizeof(float4) * (size_t)c->W * c->H, cudaMemcpyDeviceToHost, c->stream));
  return fr_synchronize(c);
}

int fr_resolve_rgba8(fr_ctx* c, uint8_t* rgba) {
  if (!c || !rgba) return fail(FR_ERR_INVALID, "fr_resolve_rgba8: bad arguments");
  FR_CUDA(cudaStreamWaitEvent(c->stream, c->copied[0], 0));
  int rc = fr_resolve_dev(c, reinterpret_cast<float*>(c->image));
  if (rc) return rc;
  launch_export_rgba8(c->image, c->W, c->H, c->image8, c->stream);
  FR_CUDA(cudaMemcpyAsync(rgba, c->image8, 4 * (size_t)c->W * c->H, cudaMemcpyDeviceToHost, c->stream));
  return fr_synchronize(c);
}

int fr_export_png(fr_ctx* c, const char* path) {
  if (!c || !path) return fail(FR_ERR_INVALID, "fr_export_png: bad arguments");
  std::vector<uint8_t> px(4 * (size_t)c->W * c->H);
  int rc = fr_resolve_rgba8(c, px.data());
  if (rc) return rc;
  if (fr_write_png(path, c->W, c->H, px.data()) != FR_OK) return fail(FR_ERR_INVALID, "fr_export_png: cannot write %s", path);
  return FR_OK;
}

int fr_get_stats(fr_ctx* c, fr_stats* o) {
  if (!c || !o) return fail(FR_ERR_INVALID, "fr_get_stats: bad arguments");
  o->iterations = c->iterations;
  o->photon_paths = c->photons_total;
  o->pixels = (int64_t)c->W * c->H;
  o->triangles = c->sc.num_tris;
  o->bvh_nodes = c->sc.num_nodes;
  o->photon_table = c->grid.table;
  o->device_bytes = (double)c->device_bytes;
  return FR_OK;
}

void* fr_stream(fr_ctx* c) {
  if (!c) return nullptr;
  join_streams(c);  // work the caller puts on the stream sees the last gather and training
  return (void*)c->stream;
}

void fr_destroy(fr_ctx* c) { delete c; }

int fr_profile_enable(fr_ctx* c, int32_t on, int32_t max_iterations) {
  if (!c) return fail(FR_ERR_INVALID, "fr_profile_enable: NULL context");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  FR_CUDA(cudaStreamSynchronize(c->stream));
  c->ev_marks.clear();
  c->ev_used = 0;
  c->profiling = on != 0;
  // Marks per iteration: the four stages and every trace round of both passes.
  const size_t need = on ? (size_t)std::max(1, max_iterations) * (4 + kEyeRounds + kPhotonRounds) * 2 : 0;
  while (c->ev_pool.size() < need) {
    cudaEvent_t e;
    FR_CUDA(cudaEventCreate(&e));
    c->ev_pool.push_back(e);
  }
  return FR_OK;
}

int fr_profile_read(fr_ctx* c, double* stage_ms, int64_t* stage_count, int64_t* launches) {
  if (!c) return fail(FR_ERR_INVALID, "fr_profile_read: NULL context");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  FR_CUDA(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < FR_STAGES; ++k) {
    if (stage_ms) stage_ms[k] = 0.0;
    if (stage_count) stage_count[k] = 0;
  }
  for (auto& m : c->ev_marks) {
    float ms = 0.f;
    FR_CUDA(cudaEventElapsedTime(&ms, m.second.first, m.second.second));
    if (stage_ms) stage_ms[m.first] += ms;
    if (stage_count) stage_count[m.first] += 1;
  }
  if (launches) {
    uint32_t gated = 0;  // photon rounds run inside the graph's conditional nodes: 3 kernels each
    FR_CUDA(cudaMemcpy(&gated, c->rounds_run, sizeof gated, cudaMemcpyDeviceToHost));
    *launches = c->launches + 3 * (int64_t)gated;
  }
  c->ev_marks.clear();
  c->ev_used = 0;
  return FR_OK;
}

int fr_trace_closest(fr_ctx* c, const float* rays, int32_t n, int32_t* facet, float* tuv) {
  if (!c || n < 0 || (n && (!rays || !facet || !tuv))) return fail(FR_ERR_INVALID, "fr_trace_closest: bad arguments");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  if (!n) return FR_OK;
  float *d_rays = nullptr, *d_tuv = nullptr;
  int32_t* d_facet = nullptr;
  FR_CUDA(cudaMalloc(&d_rays, sizeof(float) * 7 * (size_t)n));
  FR_CUDA(cudaMalloc(&d_tuv, sizeof(float) * 3 * (size_t)n));
  FR_CUDA(cudaMalloc(&d_facet, sizeof(int32_t) * (size_t)n));
  cudaMemcpyAsync(d_rays, rays, sizeof(float) * 7 * (size_t)n, cudaMemcpyHostToDevice, c->stream);
  launch_trace_closest(c->sc, d_rays, n, d_facet, d_tuv, c->err, c->stream);
  cudaMemcpyAsync(facet, d_facet, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(tuv, d_tuv, sizeof(float) * 3 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
  const int rc = fr_synchronize(c);
  cudaFree(d_rays); cudaFree(d_tuv); cudaFree(d_facet);
  return rc;
}

int fr_trace_any(fr_ctx* c, const float* rays, int32_t n, int32_t* hit) {
  if (!c || n < 0 || (n && (!rays || !hit))) return fail(FR_ERR_INVALID, "fr_trace_any: bad arguments");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  if (!n) return FR_OK;
  float* d_rays = nullptr;
  int32_t* d_hit = nullptr;
  FR_CUDA(cudaMalloc(&d_rays, sizeof(float) * 8 * (size_t)n));
  FR_CUDA(cudaMalloc(&d_hit, sizeof(int32_t) * (size_t)n));
  cudaMemcpyAsync(d_rays, rays, sizeof(float) * 8 * (size_t)n, cudaMemcpyHostToDevice, c->stream);
  launch_trace_any(c->sc, d_rays, n, d_hit, c->err, c->stream);
  cudaMemcpyAsync(hit, d_hit, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
  const int rc = fr_synchronize(c);
  cudaFree(d_rays); cudaFree(d_hit);
  return rc;
}

int fr_radius_query(fr_ctx* c, const float* hp, int32_t nh, const float* photons_xyz, int32_t np, float cell,
                    int32_t* counts, uint32_t* pairs, uint32_t pair_capacity, uint32_t* pair_count) {
  if (!c || nh < 0 || np < 0 || (nh && (!hp || !counts)) || (np && !photons_xyz) || !(cell > 0.0f) ||
      !(cell <= 3.0e38f) || (pairs && !pair_count))
    return fail(FR_ERR_INVALID, "fr_radius_query: bad arguments");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  if (!nh) return FR_OK;
  if (!np) {
    std::fill(counts, counts + nh, 0);
    if (pair_count) *pair_count = 0;
    return FR_OK;
  }
  // Flat photon list (one photon per "path", stride 1) through the same grid kernels.
  std::vector<float4> pos(std::max(np, 1)), zero(std::max(np, 1), make_float4(0.f, 0.f, 0.f, 0.f));
  float lo[3] = {1e30f, 1e30f, 1e30f};
  for (int i = 0; i < np; ++i) {
    pos[i] = make_float4(photons_xyz[3 * i], photons_xyz[3 * i + 1], photons_xyz[3 * i + 2], 1.0f);
    for (int a = 0; a < 3; ++a) lo[a] = std::min(lo[a], photons_xyz[3 * i + a]);
  }
  for (int i = 0; i < nh; ++i)
    for (int a = 0; a < 3; ++a) lo[a] = std::min(lo[a], hp[4 * i + a] - hp[4 * i + 3]);
  std::vector<uint32_t> ones(std::max(np, 1), 1u);
  PhotonSlots ph{};
  ph.paths = (uint32_t)np;  // one photon per "path": slot 0 of photon i is i
  PhotonGrid g{};
  g.table = next_pow2(std::max<uint64_t>((uint64_t)np * 2, 1024));
  GridInfo gi{};
  gi.cell = cell;
  gi.inv_cell = 1.0f / cell;
  for (int a = 0; a < 3; ++a) gi.origin[a] = lo[a] - cell;
  // The kernel refuses the same balls (count -1); refusing them here keeps
  // the device error word clear.
  for (int i = 0; i < nh; ++i)
    if (!query_ball_ok(hp[4 * i], hp[4 * i + 1], hp[4 * i + 2], hp[4 * i + 3], gi.origin, gi.inv_cell))
      return fail(FR_ERR_INVALID,
                  "fr_radius_query: hitpoint %d: radius %g is not finite or spans more than %d cells of %g along "
                  "an axis",
                  i, (double)hp[4 * i + 3], kMaxQuerySpan, (double)cell);
  ScanTemp st{};
  const uint32_t words = scan_temp_words(g.table + 1, st);
  std::vector<void*> tmp;
  bool alloc_ok = true;
  auto dalloc = [&](size_t bytes) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(bytes, 16)) != cudaSuccess) {
      alloc_ok = false;
      return (void*)nullptr;
    }
    tmp.push_back(p);
    return p;
  };
  const size_t npp = (size_t)std::max(np, 1);
  ph.pos = (float4*)dalloc(npp * 16); ph.flux = (float4*)dalloc(npp * 16); ph.dir = (float4*)dalloc(npp * 16);
  g.pos = (float4*)dalloc(npp * 16); g.flux = (float4*)dalloc(npp * 16); g.dir = (float4*)dalloc(npp * 16);
  g.cell_count = (uint32_t*)dalloc(4 * ((size_t)g.table + 1));
  g.cell_start = (uint32_t*)dalloc(4 * ((size_t)g.table + 1));
  uint32_t* d_ones = (uint32_t*)dalloc(4 * npp);
  uint32_t* sw = (uint32_t*)dalloc(4 * (size_t)words);
  GridInfo* d_gi = (GridInfo*)dalloc(sizeof(GridInfo));
  float4* d_hp = (float4*)dalloc(16 * (size_t)nh);
  int32_t* d_m = (int32_t*)dalloc(4 * (size_t)nh);
  uint32_t* d_pairs = pairs ? (uint32_t*)dalloc(8 * std::max<size_t>(pair_capacity, 1)) : nullptr;
  uint32_t* d_pc = (uint32_t*)dalloc(4);
  int rc = alloc_ok ? FR_OK : fail(FR_ERR_OOM, "fr_radius_query: cudaMalloc failed");
  if (!rc) {
    for (int l = 0; l < st.levels; ++l) {
      st.level[l] = sw;
      sw += st.level_n[l] + 1;
    }
    cudaStream_t s = c->stream;
    cudaMemcpyAsync(ph.pos, pos.data(), npp * 16, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ph.flux, zero.data(), npp * 16, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ph.dir, zero.data(), npp * 16, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_ones, ones.data(), npp * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_gi, &gi, sizeof(gi), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_hp, hp, 16 * (size_t)nh, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(g.cell_count, 0, 4 * ((size_t)g.table + 1), s);
    cudaMemsetAsync(d_pc, 0, 4, s);
    launch_photon_count(ph, d_ones, np, 1, g, d_gi, s);
    launch_scan(g.cell_count, g.cell_start, g.table + 1, st, s);
    launch_photon_scatter(ph, d_ones, np, 1, g, d_gi, s);
    launch_radius_count(d_hp, nh, g, d_gi, d_m, d_pairs, pair_capacity, d_pc, c->err, s);
    cudaMemcpyAsync(counts, d_m, 4 * (size_t)nh, cudaMemcpyDeviceToHost, s);
    if (pairs) {
      uint32_t total = 0;
      cudaMemcpyAsync(&total, d_pc, 4, cudaMemcpyDeviceToHost, s);
      cudaStreamSynchronize(s);
      *pair_count = total;
      const size_t take = std::min<uint32_t>(total, pair_capacity);
      if (take) cudaMemcpyAsync(pairs, d_pairs, 8 * take, cudaMemcpyDeviceToHost, s);
    }
    rc = fr_synchronize(c);
  }
  for (void* p : tmp) cudaFree(p);
  return rc;
}

int fr_radius_count_noalloc(const float* hp_dev, int32_t num_hitpoints, const float* photons_dev,
                            int32_t num_photons, float cell, int32_t* counts_dev, void* stream) {
  const char* msg = "";
  const int rc = radius_count_noalloc(hp_dev, num_hitpoints, photons_dev, num_photons, cell, counts_dev,
                                      static_cast<cudaStream_t>(stream), &msg);
  if (rc) return fail(rc, "%s", msg);
  return FR_OK;
}

int fr_check_tc_gemm(uint32_t seed, double* max_abs_err) {
  if (!max_abs_err) return fail(FR_ERR_INVALID, "fr_check_tc_gemm: NULL output");
  const char* msg = "";
  if (check_tc_gemm(seed, max_abs_err, &msg)) return fail(FR_ERR_CUDA, "fr_check_tc_gemm: %s", msg);
  return FR_OK;
}

int fr_check_exact_math(uint64_t samples, uint32_t seed, uint64_t* mismatches, uint64_t* fast_paths) {
  if (!mismatches || !fast_paths) return fail(FR_ERR_INVALID, "fr_check_exact_math: NULL output");
  const char* msg = "";
  if (check_exact_math(samples, seed, mismatches, fast_paths, &msg)) return fail(FR_ERR_CUDA, "fr_check_exact_math: %s", msg);
  return FR_OK;
}

static_assert(kWaveRounds <= FR_MAX_WAVE_ROUNDS, "round counters exceed FR_MAX_WAVE_ROUNDS");

int fr_read_wave_counts(fr_ctx* c, uint32_t* eye_counts, uint32_t* photon_counts, int32_t* eye_rounds,
                        int32_t* photon_rounds) {
  if (!c || !eye_counts || !photon_counts) return fail(FR_ERR_INVALID, "fr_read_wave_counts: bad arguments");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  FR_CUDA(cudaMemcpyAsync(eye_counts, c->eye_wave.qcount, sizeof(uint32_t) * (kEyeRounds + 1), cudaMemcpyDeviceToHost,
                          c->stream));
  FR_CUDA(cudaMemcpyAsync(photon_counts, c->wave.qcount, sizeof(uint32_t) * (kPhotonRounds + 1),
                          cudaMemcpyDeviceToHost, c->stream));
  if (eye_rounds) *eye_rounds = kEyeRounds;
  if (photon_rounds) *photon_rounds = kPhotonRounds;
  const int rc = fr_synchronize(c);
  if (rc) return rc;
  // Skipped rounds: their paths were run by the tail.
  const auto fold = [](uint32_t* q, int rounds, uint32_t min_live) {
    const int t = wave_tail_round(q, rounds, min_live);
    if (t == rounds) return;
    q[rounds] = q[t];
    for (int r = t; r < rounds; ++r) q[r] = 0;
  };
  fold(eye_counts, kEyeRounds, kEyeTailMin);
  fold(photon_counts, kPhotonRounds, c->wave.min_live);
  return FR_OK;
}

int fr_read_direct(fr_ctx* c, float* last3, float* sum3, int32_t* count) {
  if (!c) return fail(FR_ERR_INVALID, "fr_read_direct: NULL context");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  const size_t np = (size_t)c->W * c->H;
  std::vector<float4> a(last3 ? np : 0), b((sum3 || count) ? np : 0);
  if (last3) FR_CUDA(cudaMemcpyAsync(a.data(), c->hp.dl, 16 * np, cudaMemcpyDeviceToHost, c->stream));
  if (sum3 || count) FR_CUDA(cudaMemcpyAsync(b.data(), c->st.dl, 16 * np, cudaMemcpyDeviceToHost, c->stream));
  const int rc = fr_synchronize(c);
  if (rc) return rc;
  for (size_t i = 0; i < np; ++i) {
    if (last3) { last3[3 * i] = a[i].x; last3[3 * i + 1] = a[i].y; last3[3 * i + 2] = a[i].z; }
    if (sum3) { sum3[3 * i] = b[i].x; sum3[3 * i + 1] = b[i].y; sum3[3 * i + 2] = b[i].z; }
    if (count) { int32_t k; std::memcpy(&k, &b[i].w, 4); count[i] = k; }
  }
  return FR_OK;
}

int fr_read_hitpoints(fr_ctx* c, float* pos_type, float* nrm_rough, float* out_mat, float* wgt_facet) {
  if (!c) return fail(FR_ERR_INVALID, "fr_read_hitpoints: NULL context");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  const size_t bytes = sizeof(float4) * (size_t)c->W * c->H;
  if (pos_type) FR_CUDA(cudaMemcpyAsync(pos_type, c->hp.pos, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (nrm_rough) FR_CUDA(cudaMemcpyAsync(nrm_rough, c->hp.nrm, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (out_mat) FR_CUDA(cudaMemcpyAsync(out_mat, c->hp.out, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (wgt_facet) FR_CUDA(cudaMemcpyAsync(wgt_facet, c->hp.wgt, bytes, cudaMemcpyDeviceToHost, c->stream));
  return fr_synchronize(c);
}

int fr_read_photon_slots(fr_ctx* c, float* pos, float* flux, float* dir, uint32_t* counts) {
  if (!c) return fail(FR_ERR_INVALID, "fr_read_photon_slots: NULL context");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  // The device keeps the slots slot-major (slot k of path i at k * P + i);
  // the caller gets them path-major (i * kPhotonSlots + k), one slot's row
  // of P entries at a time.
  const size_t P = (size_t)c->P;
  std::vector<float4> row((pos || flux || dir) ? P : 0);
  for (auto [dst, src] : {std::pair<float*, float4*>{pos, c->ph.pos}, {flux, c->ph.flux}, {dir, c->ph.dir}}) {
    if (!dst) continue;
    float4* out = reinterpret_cast<float4*>(dst);
    for (size_t k = 0; k < (size_t)kPhotonSlots; ++k) {
      FR_CUDA(cudaMemcpyAsync(row.data(), src + k * P, sizeof(float4) * P, cudaMemcpyDeviceToHost, c->stream));
      FR_CUDA(cudaStreamSynchronize(c->stream));
      for (size_t i = 0; i < P; ++i) out[i * kPhotonSlots + k] = row[i];
    }
  }
  if (counts) FR_CUDA(cudaMemcpyAsync(counts, c->counts, 4 * (size_t)c->P, cudaMemcpyDeviceToHost, c->stream));
  return fr_synchronize(c);
}

int fr_read_gather(fr_ctx* c, int32_t* m, float* phi4) {
  if (!c) return fail(FR_ERR_INVALID, "fr_read_gather: NULL context");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  const size_t n = (size_t)c->W * c->H;
  if (m) FR_CUDA(cudaMemcpyAsync(m, c->dbg_m, 4 * n, cudaMemcpyDeviceToHost, c->stream));
  if (phi4) FR_CUDA(cudaMemcpyAsync(phi4, c->dbg_phi, 16 * n, cudaMemcpyDeviceToHost, c->stream));
  return fr_synchronize(c);
}

int fr_read_state(fr_ctx* c, double* tau, int32_t* n, float* r, int32_t* g) {
  if (!c) return fail(FR_ERR_INVALID, "fr_read_state: NULL context");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  const size_t np = (size_t)c->W * c->H;
  if (tau) FR_CUDA(cudaMemcpyAsync(tau, c->st.tau, 24 * np, cudaMemcpyDeviceToHost, c->stream));
  if (n) FR_CUDA(cudaMemcpyAsync(n, c->st.n, 4 * np, cudaMemcpyDeviceToHost, c->stream));
  if (r) FR_CUDA(cudaMemcpyAsync(r, c->st.r, 4 * np, cudaMemcpyDeviceToHost, c->stream));
  if (g) FR_CUDA(cudaMemcpyAsync(g, c->st.g, 4 * np, cudaMemcpyDeviceToHost, c->stream));
  return fr_synchronize(c);
}

int fr_update(fr_ctx* c, const int32_t* m, const float* phi) {
  if (!c || !m || !phi) return fail(FR_ERR_INVALID, "fr_update: bad arguments");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  const size_t np = (size_t)c->W * c->H;
  std::vector<float4> phi4(np);
  for (size_t i = 0; i < np; ++i) phi4[i] = make_float4(phi[3 * i], phi[3 * i + 1], phi[3 * i + 2], 0.0f);
  FR_CUDA(cudaMemcpyAsync(c->dbg_m, m, sizeof(int32_t) * np, cudaMemcpyHostToDevice, c->stream));
  FR_CUDA(cudaMemcpyAsync(c->dbg_phi, phi4.data(), sizeof(float4) * np, cudaMemcpyHostToDevice, c->stream));
  launch_update(c->st, c->dbg_m, c->dbg_phi, (int)np, c->alpha, (c->flags & kFlagFloatPhotonCount) != 0u, c->stream);
  return fr_synchronize(c);
}

int fr_update_dev(fr_ctx* c, const int32_t* m_dev, const float* phi4_dev) {
  if (!c || !m_dev || !phi4_dev) return fail(FR_ERR_INVALID, "fr_update_dev: bad arguments");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  if ((reinterpret_cast<uintptr_t>(phi4_dev) & 15u) != 0) return fail(FR_ERR_INVALID, "fr_update_dev: phi4 not 16-byte aligned");
  launch_update(c->st, m_dev, reinterpret_cast<const float4*>(phi4_dev), c->W * c->H, c->alpha,
                (c->flags & kFlagFloatPhotonCount) != 0u, c->stream);
  FR_CUDA(cudaGetLastError());
  return FR_OK;
}

// ------------------------------------------------------------ guide
int fr_guide_params(fr_ctx* c, float* params) {
  if (!c || !params || !c->guided) return fail(FR_ERR_INVALID, "fr_guide_params: no guide");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  FR_CUDA(cudaMemcpyAsync(params, c->guide.params, sizeof(float) * kGuideParams, cudaMemcpyDeviceToHost, c->stream));
  return fr_synchronize(c);
}

int fr_guide_set_params(fr_ctx* c, const float* params) {
  if (!c || !params || !c->guided) return fail(FR_ERR_INVALID, "fr_guide_set_params: no guide");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  FR_CUDA(cudaMemcpyAsync(c->guide.params, params, sizeof(float) * kGuideParams, cudaMemcpyHostToDevice, c->stream));
  launch_guide_prepare(c->guide, c->stream);
  if (launch_guide_publish(c->guide, c->stream)) return fail(FR_ERR_CUDA, "guide: weight copy failed");
  return fr_synchronize(c);
}

int fr_read_guide_importance(fr_ctx* c, float* importance) {
  if (!c || !importance || !c->guided) return fail(FR_ERR_INVALID, "fr_read_guide_importance: no guide");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  std::vector<unsigned long long> fx(2 * (size_t)c->P);
  FR_CUDA(cudaMemcpyAsync(fx.data(), c->guide.importance, sizeof(unsigned long long) * fx.size(),
                          cudaMemcpyDeviceToHost, c->stream));
  const int rc = fr_synchronize(c);
  if (rc) return rc;
  for (size_t i = 0; i < (size_t)c->P; ++i) importance[i] = importance_value(fx[2 * i], fx[2 * i + 1]);
  return FR_OK;
}

int fr_guide_gradient(fr_ctx* c, int32_t n, const float* samples, float* grad, float* weight_sum) {
  if (!c || !c->guided || n < 0 || n > c->P || n > c->guide.batch_cap || (n && !samples) || !grad || !weight_sum)
    return fail(FR_ERR_INVALID, "fr_guide_gradient: bad arguments");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  const GuideGPU& g = c->guide;
  std::vector<float4> f(n), d(n);
  std::vector<unsigned long long> imp(2 * (size_t)c->P, 0ull);
  for (int j = 0; j < n; ++j) {
    const float* x = samples + 9 * (size_t)j;
    f[j] = make_float4(x[0], x[1], x[2], x[3]);
    d[j] = make_float4(x[4], x[5], x[6], x[7]);
    importance_split(x[8], &imp[2 * (size_t)j], &imp[2 * (size_t)j + 1]);
  }
  FR_CUDA(cudaStreamSynchronize(c->stream));
  if (n) {
    FR_CUDA(cudaMemcpyAsync(g.feat, f.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, c->stream));
    FR_CUDA(cudaMemcpyAsync(g.dir, d.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, c->stream));
  }
  FR_CUDA(cudaMemcpyAsync(g.importance, imp.data(), sizeof(unsigned long long) * imp.size(), cudaMemcpyHostToDevice,
                          c->stream));
  FR_CUDA(cudaMemsetAsync(g.grad, 0, sizeof(float) * kGuideParams, c->stream));
  FR_CUDA(cudaMemsetAsync(g.weight_sum, 0, 4, c->stream));
  FR_CUDA(cudaMemsetAsync(g.batch_count, 0, 4, c->stream));
  launch_guide_gradients(g, c->P, c->stream);
  FR_CUDA(cudaMemcpyAsync(grad, g.grad, sizeof(float) * kGuideParams, cudaMemcpyDeviceToHost, c->stream));
  FR_CUDA(cudaMemcpyAsync(weight_sum, g.weight_sum, 4, cudaMemcpyDeviceToHost, c->stream));
  int rc = fr_synchronize(c);
  FR_CUDA(cudaMemsetAsync(g.grad, 0, sizeof(float) * kGuideParams, c->stream));
  FR_CUDA(cudaMemsetAsync(g.weight_sum, 0, 4, c->stream));
  FR_CUDA(cudaMemsetAsync(g.batch_count, 0, 4, c->stream));
  FR_CUDA(cudaMemsetAsync(g.importance, 0, 2 * sizeof(unsigned long long) * c->P, c->stream));
  const int rc2 = fr_synchronize(c);
  return rc ? rc : rc2;
}

// ------------------------------------------------------------ checkpoint
// State between iterations: the iteration count and photon total (they key
// the random streams and the resolve), the per-pixel state and the photon
// slots (a slot stored in an earlier iteration can join a later iteration's
// photon set, SPPM.cpp:672).  Layout: a fixed header, then tau, N, R,
// NumGather, direct light with its count, slot positions, fluxes and
// directions, each as on the device.
namespace {
struct StateHeader {
  char magic[8];  // "FRSPPMS2" (photon slots slot-major)
  int32_t width, height, photons, flags;
  float alpha, initial_radius;
  int32_t triangles;
  uint32_t step_base;  // fr_seek's first step (0 without it)
  int64_t iterations, photons_total;
};
static_assert(sizeof(StateHeader) == 56, "checkpoint header is 56 bytes");
constexpr char kStateMagic[8] = {'F', 'R', 'S', 'P', 'P', 'M', 'S', '2'};

struct StatePart {
  void* dev;
  size_t bytes;
};

std::vector<StatePart> state_parts(fr_ctx* c) {
  const size_t np = (size_t)c->W * c->H, ns = (size_t)c->P * kPhotonSlots;
  std::vector<StatePart> parts = {{c->st.tau, 24 * np},  {c->st.n, 4 * np},     {c->st.r, 4 * np},
                                  {c->st.g, 4 * np},     {c->st.dl, 16 * np},   {c->ph.pos, 16 * ns},
                                  {c->ph.flux, 16 * ns},
                                  {c->ph.dir, 16 * ns}};
  if (c->guided) {  // the guide's network and optimizer state
    parts.push_back({c->guide.params, 4 * (size_t)kGuideParams});
    parts.push_back({c->guide.adam_m, 4 * (size_t)kGuideParams});
    parts.push_back({c->guide.adam_v, 4 * (size_t)kGuideParams});
    parts.push_back({c->guide.adam_step, 4});
    parts.push_back({c->guide.emit_params, 4 * (size_t)kGuideParams});  // the weights the next emission samples
  }
  return parts;
}

size_t state_bytes(fr_ctx* c) {
  size_t n = sizeof(StateHeader);
  for (const StatePart& p : state_parts(c)) n += p.bytes;
  return n;
}
}  // namespace

int fr_save_state(fr_ctx* c, void* buf, size_t* size) {
  if (!c || !size) return fail(FR_ERR_INVALID, "fr_save_state: bad arguments");
  const size_t need = state_bytes(c);
  if (!buf) {
    *size = need;
    return FR_OK;
  }
  if (*size < need) return fail(FR_ERR_INVALID, "fr_save_state: buffer of %zu bytes, %zu needed", *size, need);
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  StateHeader h{};
  std::memcpy(h.magic, kStateMagic, 8);
  h.width = c->W;
  h.height = c->H;
  h.photons = c->P;
  h.flags = (int32_t)c->flags;
  h.alpha = c->alpha;
  h.initial_radius = c->r0;
  h.triangles = c->sc.num_tris;
  h.step_base = c->step_base;
  h.iterations = c->iterations;
  h.photons_total = c->photons_total;
  std::memcpy(buf, &h, sizeof h);
  char* p = static_cast<char*>(buf) + sizeof h;
  for (const StatePart& part : state_parts(c)) {
    FR_CUDA(cudaMemcpyAsync(p, part.dev, part.bytes, cudaMemcpyDeviceToHost, c->stream));
    p += part.bytes;
  }
  *size = need;
  return fr_synchronize(c);
}

int fr_load_state(fr_ctx* c, const void* buf, size_t size) {
  if (!c || !buf) return fail(FR_ERR_INVALID, "fr_load_state: bad arguments");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  if (size < sizeof(StateHeader)) return fail(FR_ERR_INVALID, "fr_load_state: %zu bytes, no header", size);
  StateHeader h;
  std::memcpy(&h, buf, sizeof h);
  if (std::memcmp(h.magic, kStateMagic, 8) != 0) return fail(FR_ERR_INVALID, "fr_load_state: not a checkpoint");
  if (h.width != c->W || h.height != c->H || h.photons != c->P || h.flags != (int32_t)c->flags ||
      h.alpha != c->alpha || h.initial_radius != c->r0 || h.triangles != c->sc.num_tris)
    return fail(FR_ERR_INVALID, "fr_load_state: checkpoint of another configuration (%dx%d, %d paths)", h.width,
                h.height, h.photons);
  if (h.iterations < 0 || h.photons_total < 0) return fail(FR_ERR_INVALID, "fr_load_state: bad counters");
  if (size != state_bytes(c)) return fail(FR_ERR_INVALID, "fr_load_state: %zu bytes, %zu expected", size, state_bytes(c));
  FR_CUDA(cudaStreamSynchronize(c->stream));
  const char* p = static_cast<const char*>(buf) + sizeof h;
  for (const StatePart& part : state_parts(c)) {
    FR_CUDA(cudaMemcpyAsync(part.dev, p, part.bytes, cudaMemcpyHostToDevice, c->stream));
    p += part.bytes;
  }
  const uint32_t step = h.step_base + (uint32_t)h.iterations, steps[2] = {step, step};
  FR_CUDA(cudaMemcpyAsync(c->step_dev, steps, sizeof steps, cudaMemcpyHostToDevice, c->stream));
  if (c->guided) {  // both networks' BF16 tiles from their FP32 weights
    launch_guide_prepare(c->guide, c->stream);
    GuideGPU e = c->guide;
    e.params = e.emit_params;
    e.tiles = e.emit_tiles;
    launch_guide_prepare(e, c->stream);
  }
  FR_CUDA(cudaStreamSynchronize(c->stream));
  c->step_base = h.step_base;
  c->iterations = h.iterations;
  c->photons_total = h.photons_total;
  return FR_OK;
}

int fr_seek(fr_ctx* c, uint32_t first_step) {
  if (!c) return fail(FR_ERR_INVALID, "fr_seek: bad arguments");
  { const int jrc = join_streams(c); if (jrc) return jrc; }
  if (c->iterations != 0) return fail(FR_ERR_INVALID, "fr_seek: %lld iterations already run", (long long)c->iterations);
  FR_CUDA(cudaStreamSynchronize(c->stream));
  const uint32_t steps[2] = {first_step, first_step};
  FR_CUDA(cudaMemcpyAsync(c->step_dev, steps, sizeof steps, cudaMemcpyHostToDevice, c->stream));
  FR_CUDA(cudaStreamSynchronize(c->stream));
  c->step_base = first_step;
  return FR_OK;
}

}  // extern "C"
