// Oracle harness (test infrastructure only): drives the reference's own SPPM
// code, compiled from its sources with the overlay headers in ./overlay, and
// dumps its per-iteration state as .npy files.  Used to make the golden
// fixtures under tests/golden/ and to pin the CPU restatement in oracle/port.
//
//   frref <scene_dir> facets <out_dir>
//   frref <scene_dir> trace  <rays.bin> <out_dir>
//   frref <scene_dir> any    <rays.bin> <out_dir>
//   frref <scene_dir> render <photons_per_iter> <iterations> <out_dir>
//   frref <dir> texture <image_file> <out_dir>
//   frref <scene_dir> count <rays.bin> <out_dir>
//
// <scene_dir> holds meshData/scene.obj (+ .mtl, textures), materials.txt and
// camera.txt as written by frsppm.objio.
//
// The render mode follows RenderImage_FixRenderTime (SPPM/SPPM/SPPM.cpp:719-858)
// with a fixed iteration count and a fixed photon count: per iteration s = 1..n
// it resets slot 0 of every photon path and every hitpoint (SPPM.cpp:771-779),
// calls createPhotonMap(.., s) (SPPM.cpp:798), compacts the photon slots up to
// the first invalid one and builds the kd-tree (SPPM.cpp:809-833), calls
// createHitpoints(.., s) (SPPM.cpp:836) and applyHitPointInfo (SPPM.cpp:841);
// at the end reconstructImageFromSharedPoints (SPPM.cpp:857).

#include <omp.h>
#include <algorithm>
#include <array>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <fstream>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <sstream>
#include <string>
#include <thread>
#include <type_traits>
#include <utility>
#include <vector>
#include <unistd.h>

// The render driver's per-iteration members are private; the harness needs
// them to run a fixed number of iterations (the public drivers are either
// broken or wall-clock driven, SPPM.cpp:682-717,783-795).  Access control does
// not change layout or linkage.
#define private public
#include "Camera.h"
#include "SPPM.h"
#include "Scene.h"
#include "TextureUtility.h"
#include "stb_image.hpp"
#undef private

using namespace PTUtility;
using SPPMR = Render::StochasticProgressivePhotonMapping;

// The three timing members sit in the class's implicit-private section, which
// the #define above does not reach; an explicit instantiation may name them
// (access is not checked there), which yields their member pointers.
template <typename Tag, typename Tag::type M>
struct MemberAccess { friend typename Tag::type member_ptr(Tag) { return M; } };
struct StartTimeTag { typedef long int SPPMR::*type; friend type member_ptr(StartTimeTag); };
struct EndTimeTag { typedef long int SPPMR::*type; friend type member_ptr(EndTimeTag); };
struct CurTimeTag { typedef long int SPPMR::*type; friend type member_ptr(CurTimeTag); };
template struct MemberAccess<StartTimeTag, &SPPMR::m_RenderStartTime>;
template struct MemberAccess<EndTimeTag, &SPPMR::m_RenderEndTime>;
template struct MemberAccess<CurTimeTag, &SPPMR::m_CurrentTime>;

namespace {

// ---------------------------------------------------------------- npy output
void write_npy(const std::string& path, const char* descr, const std::vector<size_t>& shape,
               const void* data, size_t bytes) {
  std::string hdr = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': (";
  for (size_t i = 0; i < shape.size(); ++i) hdr += std::to_string(shape[i]) + (shape.size() == 1 || i + 1 < shape.size() ? ", " : "");
  hdr += "), }";
  size_t total = 10 + hdr.size() + 1;
  size_t pad = (64 - total % 64) % 64;
  hdr.append(pad, ' ');
  hdr += '\n';
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { std::perror(path.c_str()); std::exit(2); }
  const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
  std::fwrite(magic, 1, 8, f);
  uint16_t hl = (uint16_t)hdr.size();
  std::fwrite(&hl, 2, 1, f);
  std::fwrite(hdr.data(), 1, hdr.size(), f);
  if (bytes) std::fwrite(data, 1, bytes, f);
  std::fclose(f);
}
void npy_f32(const std::string& p, const std::vector<float>& v, std::vector<size_t> shape) {
  write_npy(p, "<f4", shape, v.data(), v.size() * 4);
}
void npy_i32(const std::string& p, const std::vector<int32_t>& v, std::vector<size_t> shape) {
  write_npy(p, "<i4", shape, v.data(), v.size() * 4);
}
void push3(std::vector<float>& v, const Vec3& a) { v.push_back(a[0]); v.push_back(a[1]); v.push_back(a[2]); }

// ---------------------------------------------------------- material plug-in
struct MatRow { int type, sppm, opaque; float index, roughness, extinction, reflectance; };

// The reference's material extension point (SceneMaterial.h:13-16), filled
// from materials.txt the way main.cpp:14-114 fills it in code.
class TableMaterials : public SceneMaterialManager {
 public:
  std::map<std::string, MatRow> rows;
  Material::Surface* SetParamtoAttribute_p(Attribute* at, const std::string& name) const override {
    auto it = rows.find(name);
    if (it == rows.end()) {
      // Not in the table: what the reference's default manager does
      // (SceneMaterial.h:13-16).
      at->m_Surface = new Material::DiffuseSurface();
      return at->m_Surface;
    }
    const MatRow& r = it->second;
    Material::Surface* s = nullptr;
    switch (r.type) {
      case 0: s = new Material::DiffuseSurface(); break;
      case 1: s = new Material::MetalSurface(); at->m_SurfaceParam.IfDeltaSurface = true; break;
      case 2: s = new Material::Roughconductor(); break;
      case 3: s = new Material::GGXGlass(); break;
      // The demo's further surfaces (main.cpp:14-114).
      case 4: s = new Material::BiMetalSurface(); at->m_SurfaceParam.IfDeltaSurface = true; break;
      case 5: s = new Material::GlassSurface(); break;
      case 6: s = new Material::GlossTransmitSurface(); break;
      case 7: s = new Material::DiffuseTransmitSurface(); break;
      default: std::fprintf(stderr, "bad material type\n"); std::exit(2);
    }
    at->m_Surface = s;
    at->m_SurfaceParam.isSPPMSurface = r.sppm != 0;
    at->m_SurfaceParam.IfOpeque = r.opaque != 0;
    at->m_SurfaceParam.Index = r.index;
    at->m_SurfaceParam.Roughness = r.roughness;
    at->m_SurfaceParam.Extinction = r.extinction;
    at->m_SurfaceParam.Reflectance = r.reflectance;
    return s;
  }
};

// Camera sampler plug-in (CameraSampler.h:11-17): three draws from the
// pixel's own generator, which createHitpoints builds right before it asks
// the camera for a ray (SPPM.cpp:334,344).
class PixelStreamSampler : public iCameraSsmpler {
 public:
  PixelStreamSampler() : iCameraSsmpler(0, 1) {}
  Vec3 Sample(int) override {
    RandomMT* mt = RandomMT::LatestOnThisThread();
    const float a = (float)mt->genrand64_real1();
    const float b = (float)mt->genrand64_real1();
    const float c = (float)mt->genrand64_real1();
    return Vec3(a, b, c);
  }
};

struct CamSpec { int type, W, H; float pos[3], tgt[3], fov, focal, dist, aspect, lens; };

// The reference's closest-hit traversal, N_BVH8::findClosestElement
// (bvh8.h:568-641), with its loop kept step for step and two counters
// added: V, the internal nodes whose eight child boxes are tested
// (Intersect_AABB8_RAY), and X, the leaves whose triangle is tested.  The
// traversal work of a ray on the reference's tree is 168 V + 40 X FP32
// operations (21 per slab test of one child, about 40 per Moller-Trumbore
// test, Intersect.cpp:67-89, 515-553).
template <class B>
float count_closest(const B& b, const Primitive::Ray& ray, int32_t& V, int32_t& X) {
  using NodeT = typename std::decay<decltype(b.m_NodeArray[0])>::type;
  std::deque<unsigned int> stack;
  stack.push_back(0u);
  float best = ray.m_MaxT;
  int num_box = 0;
  V = X = 0;
  while (stack.size() > 0 && num_box < (int)b.m_NumNodes) {
    const unsigned int id = *(stack.end() - 1);
    const NodeT& node = b.m_NodeArray[id];
    stack.pop_back();
    num_box++;
    if (node.isLeaf()) {
      if (node.m_children[0] != NodeT::InvalidID) {
        ++X;
        Isc::IntersectInfo info;
        if (Isc::Intersect(b.m_ElementArray[node.m_children[0]].second, ray, info))
          if (best >= info.t && info.t > ray.m_MinT) best = info.t;
      }
      continue;
    }
    ++V;
    std::array<float, 8> hd;
    if (!Isc::Intersect_AABB8_RAY(node.m_childAABBs, ray, hd)) continue;
    std::array<std::pair<unsigned int, float>, 8> res;
    const bool of = ray.m_Dir[node.getAxis(0)] > 0, of0 = ray.m_Dir[node.getAxis(1)] > 0;
    const bool of00 = ray.m_Dir[node.getAxis(3)] > 0;
    res[of * 4 + of0 * 2 + of00] = {0u, hd[0]};
    res[of * 4 + of0 * 2 + !of00] = {1u, hd[1]};
    res[of * 4 + !of0 * 2 + of00] = {2u, hd[2]};
    res[of * 4 + !of0 * 2 + !of00] = {3u, hd[3]};
    res[!of * 4 + of0 * 2 + of00] = {4u, hd[4]};
    res[!of * 4 + of0 * 2 + !of00] = {5u, hd[5]};
    res[!of * 4 + !of0 * 2 + of00] = {6u, hd[6]};
    res[!of * 4 + !of0 * 2 + !of00] = {7u, hd[7]};
    for (int i = 0; i < 8; ++i)
      if (res[i].second < best) stack.push_back(node.m_children[res[i].first]);
  }
  return best;
}

CamSpec read_camera(const std::string& path) {
  CamSpec c{};
  std::ifstream f(path);
  f >> c.type >> c.W >> c.H >> c.pos[0] >> c.pos[1] >> c.pos[2] >> c.tgt[0] >> c.tgt[1] >> c.tgt[2] >> c.fov >> c.focal >> c.dist >> c.aspect >> c.lens;
  if (!f) { std::fprintf(stderr, "bad camera file\n"); std::exit(2); }
  return c;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) { std::fprintf(stderr, "usage: frref <scene_dir> facets|trace|render ...\n"); return 2; }
  const std::string mode = argv[2];
  std::string out_dir;
  if (chdir(argv[1]) != 0) { std::perror("chdir"); return 2; }

  if (mode == "texture") {
    // TextureUtility::LoadTextureFromFile (TextureUtility.cpp:12-35) on one
    // image, and the channel count stbi_load reports for it.
    if (argc < 5) return 2;
    Texture2D tex;
    if (!TextureUtility::LoadTextureFromFile(tex, argv[3])) { std::fprintf(stderr, "load failed\n"); return 3; }
    int X = 0, Y = 0, C = 0;
    unsigned char* raw = stbi_load(argv[3], &X, &Y, &C, 0);
    if (raw) stbi_image_free(raw);
    const size_t W = tex.GetWidth(), H = tex.GetHeight();
    std::vector<float> texels(W * H * 4);
    for (size_t i = 0; i < W * H; ++i)
      for (int c = 0; c < 4; ++c) texels[i * 4 + c] = tex.GetRawData()[i][c];
    npy_f32(std::string(argv[4]) + "/texels.npy", texels, {H, W, 4});
    npy_i32(std::string(argv[4]) + "/channels.npy", std::vector<int32_t>{C}, {1});
    return 0;
  }

  TableMaterials mats;
  {
    std::ifstream f("materials.txt");
    std::string name; MatRow r;
    while (f >> name >> r.type >> r.sppm >> r.opaque >> r.index >> r.roughness >> r.extinction >> r.reflectance) mats.rows[name] = r;
  }
  const CamSpec cs = read_camera("camera.txt");

  // Keep the reference's progress printing out of the dumps' stdout.
  std::FILE* devnull = std::freopen("/dev/null", "w", stdout);
  (void)devnull;

  // An environment map, when the scene has one (meshData/ibl.png), goes to
  // CreateScene as the IBL texture (main.cpp:132-143).
  Texture2D ibl;
  const bool has_ibl = access("meshData/ibl.png", R_OK) == 0;
  if (has_ibl && !TextureUtility::LoadTextureFromFile(ibl, "meshData//ibl.png")) { std::fprintf(stderr, "IBL load failed\n"); return 2; }
  Scene scene;
  if (!scene.CreateScene("meshData//scene.obj", &mats, has_ibl ? &ibl : nullptr)) { std::fprintf(stderr, "CreateScene failed\n"); return 2; }

  // Rebuild the scene BVH with the reference's single-threaded Build2
  // (bvh8.h:44-76): Build3, which CreateScene uses (Scene.cpp:210-211), calls
  // createChildNodes on all 64 depth-2 nodes (bvh8.h:181-187) even when one
  // holds a single triangle; that node is then a leaf whose child slot holds
  // a triangle index, which the call writes through as a node index
  // (bvh8.h:284-289), corrupting the tree.  Build2 runs the same SAH split
  // code through the recursion that guards that case.  The triangle list is
  // the one CreateScene builds (Scene.cpp:234).
  if (std::getenv("FRREF_BUILD3") == nullptr) {
    std::vector<Primitive::Triangle_ID> tris(scene.m_Facets.size());
    for (size_t f = 0; f < scene.m_Facets.size(); ++f) tris[f] = Primitive::Triangle_ID(scene.m_Facets[f]._Pos, (int)f);
    scene.m_Aobject.reset(new aObject::N_BVH<Primitive::Triangle_ID, Primitive::Ray, 8>);
    scene.m_Aobject->Build2(tris);
  }

  PixelStreamSampler sampler;
  std::unique_ptr<iCamera> camera;
  if (cs.type == 0) {
    camera.reset(new PinholeCamera(cs.W, cs.H, Vec3(cs.pos[0], cs.pos[1], cs.pos[2]), Vec3(cs.tgt[0], cs.tgt[1], cs.tgt[2]), cs.fov, cs.focal, cs.dist, cs.aspect, &sampler));
  } else {
    camera.reset(new ThinLensCamera(cs.W, cs.H, Vec3(cs.pos[0], cs.pos[1], cs.pos[2]), Vec3(cs.tgt[0], cs.tgt[1], cs.tgt[2]), cs.fov, cs.focal, cs.dist, cs.aspect, &sampler, nullptr));
    if (cs.lens > 0.0f) { camera->_LensWidth = cs.lens; camera->_LensHeight = cs.lens; }
  }

  if (mode == "facets") {
    out_dir = argv[3];
    const size_t T = scene.m_Facets.size();
    std::vector<float> pos, nrm, uv; std::vector<int32_t> attr;
    for (const auto& f : scene.m_Facets) {
      for (int k = 0; k < 3; ++k) { push3(pos, f._Pos[k]); push3(nrm, f._Normal[k]); uv.push_back(f._UV[k][0]); uv.push_back(f._UV[k][1]); }
      attr.push_back(f._AttributeID);
    }
    npy_f32(out_dir + "/facet_pos.npy", pos, {T, 3, 3});
    npy_f32(out_dir + "/facet_nrm.npy", nrm, {T, 3, 3});
    npy_f32(out_dir + "/facet_uv.npy", uv, {T, 3, 2});
    npy_i32(out_dir + "/facet_attr.npy", attr, {T});
    // Attributes as CreateScene left them (Scene.cpp:60-77): Kd, Ke, the
    // surface parameters (index, roughness, extinction, reflectance, SPPM
    // surface, opaque) and the texture file names bound to albedo, roughness
    // and normal map.
    {
      std::vector<float> kd, ke, par;
      std::ofstream names(out_dir + "/attr_textures.txt");
      for (const auto& kv : scene.m_Attributes.m_AttributeTable) {
        const Attribute* at = kv.second.get();
        const auto& sp = at->m_SurfaceParam;
        push3(kd, sp.Albedo);
        push3(ke, sp.Radiance);
        for (float x : {sp.Index, sp.Roughness, sp.Extinction, sp.Reflectance, (float)sp.isSPPMSurface, (float)sp.IfOpeque})
          par.push_back(x);
        names << kv.first << '\t' << at->m_AlbedoTextureFileName << '\t' << at->m_RoughnessTextureFileName << '\t'
              << at->m_BumpMapTextureFileName << '\n';
      }
      npy_f32(out_dir + "/attr_albedo.npy", kd, {kd.size() / 3, 3});
      npy_f32(out_dir + "/attr_radiance.npy", ke, {ke.size() / 3, 3});
      npy_f32(out_dir + "/attr_params.npy", par, {par.size() / 6, 6});
    }
    // Area lights and their alias tables (LightSampler.cpp:6-66, TableSampler.h:44-120).
    const LightSampler* ls = scene.GetLightManager();
    const int NL = ls->GetNumAreaLights();
    std::vector<float> lflux, lpdf; std::vector<int32_t> lfacet, ltex;
    std::vector<float> tab_p; std::vector<int32_t> tab_l, tab_r;
    for (int i = 0; i < NL; ++i) {
      const auto& L = ls->GetAreaLightsData()[i];
      push3(lflux, L._Flux); lfacet.push_back(L._Facet._FacetID); ltex.push_back(L._Textured);
      lpdf.push_back(ls->GetAreaLightPDF(L));
    }
    for (int i = 0; i < NL; ++i) {
      const auto& b = ls->m_AreaLights.m_Table[i];
      tab_p.push_back(b.probLeftSample); tab_l.push_back(b.ID_Left); tab_r.push_back(b.ID_Right);
    }
    npy_f32(out_dir + "/light_flux.npy", lflux, {(size_t)NL, 3});
    npy_f32(out_dir + "/light_pdf.npy", lpdf, {(size_t)NL});
    npy_i32(out_dir + "/light_facet.npy", lfacet, {(size_t)NL});
    npy_i32(out_dir + "/light_textured.npy", ltex, {(size_t)NL});
    npy_f32(out_dir + "/light_alias_p.npy", tab_p, {(size_t)NL});
    npy_i32(out_dir + "/light_alias_l.npy", tab_l, {(size_t)NL});
    npy_i32(out_dir + "/light_alias_r.npy", tab_r, {(size_t)NL});
    // Per-light 1000-point emission tables of textured lights (LightSampler.cpp:30-66).
    std::vector<float> ep, euvw, eL, epdf; std::vector<int32_t> el, er;
    for (int i = 0; i < NL; ++i) {
      const auto& L = ls->GetAreaLightsData()[i];
      if (!L._Textured) continue;
      for (int k = 0; k < 1000; ++k) {
        const auto& b = L.m_Table.m_Table[k];
        ep.push_back(b.probLeftSample); el.push_back(b.ID_Left); er.push_back(b.ID_Right);
        push3(euvw, L.m_Table.m_Data[k].UV); push3(eL, L.m_Table.m_Data[k].L);
        epdf.push_back(L.m_Table.GetPDF(L.m_Table.m_Data[k]));
      }
    }
    const size_t NE = ep.size();
    npy_f32(out_dir + "/emit_alias_p.npy", ep, {NE});
    npy_i32(out_dir + "/emit_alias_l.npy", el, {NE});
    npy_i32(out_dir + "/emit_alias_r.npy", er, {NE});
    npy_f32(out_dir + "/emit_uvw.npy", euvw, {NE, 3});
    npy_f32(out_dir + "/emit_L.npy", eL, {NE, 3});
    npy_f32(out_dir + "/emit_pdf.npy", epdf, {NE});
    // Camera basis (Camera.h:132-151).
    std::vector<float> cam;
    push3(cam, camera->_CameraPos); push3(cam, camera->_CameraDir); push3(cam, camera->_e1); push3(cam, camera->_e2);
    cam.push_back(camera->_Fov); cam.push_back(camera->_PlaneWidth); cam.push_back(camera->_PlaneHeight);
    cam.push_back(camera->_LensWidth); cam.push_back(camera->_LensHeight); cam.push_back(camera->_F); cam.push_back(camera->_DistanceToLens);
    npy_f32(out_dir + "/camera.npy", cam, {cam.size()});
    return 0;
  }

  if (mode == "count") {
    // rays.bin as for "trace"; out: visits.npy, N x 2 int32 (V, X), and
    // best_t.npy, the closest t (FLT_MAX for a miss) as a check on the loop.
    const std::string rays_path = argv[3];
    out_dir = argv[4];
    std::ifstream f(rays_path, std::ios::binary | std::ios::ate);
    const size_t bytes = (size_t)f.tellg();
    f.seekg(0);
    std::vector<float> rays(bytes / 4);
    f.read(reinterpret_cast<char*>(rays.data()), bytes);
    const size_t N = rays.size() / 7;
    std::vector<int32_t> vx(N * 2);
    std::vector<float> best_t(N);
    const auto& bvh = *scene.m_Aobject;
#pragma omp parallel for schedule(dynamic, 64)
    for (long i = 0; i < (long)N; ++i) {
      const float* r = &rays[i * 7];
      Primitive::Ray ray(Vec3(r[0], r[1], r[2]), Vec3(r[3], r[4], r[5]), r[6], Primitive::Ray::RAY_OFFSET, FLT_MAX);
      best_t[i] = count_closest(bvh, ray, vx[i * 2], vx[i * 2 + 1]);
    }
    npy_i32(out_dir + "/visits.npy", vx, {N, 2});
    npy_f32(out_dir + "/best_t.npy", best_t, {N});
    return 0;
  }

  if (mode == "trace") {
    // rays.bin: N x 7 float32 {org xyz, dir xyz, index}; directions used as given
    // (Ray 5-argument constructor, Primitive.h:48-49: MinT = RAY_OFFSET, MaxT = FLT_MAX).
    const std::string rays_path = argv[3];
    out_dir = argv[4];
    std::ifstream f(rays_path, std::ios::binary | std::ios::ate);
    const size_t bytes = (size_t)f.tellg();
    f.seekg(0);
    std::vector<float> rays(bytes / 4);
    f.read(reinterpret_cast<char*>(rays.data()), bytes);
    const size_t N = rays.size() / 7;
    std::vector<int32_t> facet(N);
    std::vector<float> tuv(N * 3);
#pragma omp parallel for schedule(dynamic, 64)
    for (long i = 0; i < (long)N; ++i) {
      const float* r = &rays[i * 7];
      Primitive::Ray ray(Vec3(r[0], r[1], r[2]), Vec3(r[3], r[4], r[5]), r[6], Primitive::Ray::RAY_OFFSET, FLT_MAX);
      iScene::IntersectionResult res;
      if (scene.GetOneFacetFromRay(ray, res)) {
        facet[i] = res._Facet->_FacetID;
        tuv[i * 3] = res._t; tuv[i * 3 + 1] = res._u; tuv[i * 3 + 2] = res._v;
      } else {
        facet[i] = -1;
        tuv[i * 3] = FLT_MAX;
      }
    }
    npy_i32(out_dir + "/hit_facet.npy", facet, {N});
    npy_f32(out_dir + "/hit_tuv.npy", tuv, {N, 3});
    return 0;
  }

  if (mode == "any") {
    // rays.bin: N x 8 float32 {org xyz, dir xyz, min_t, max_t} -> findAnyElement
    // from the root (bvh8.h:643-707, AnyHit bvh8.h:767-769).
    const std::string rays_path = argv[3];
    out_dir = argv[4];
    std::ifstream f(rays_path, std::ios::binary | std::ios::ate);
    const size_t bytes = (size_t)f.tellg();
    f.seekg(0);
    std::vector<float> rays(bytes / 4);
    f.read(reinterpret_cast<char*>(rays.data()), bytes);
    const size_t N = rays.size() / 8;
    std::vector<int32_t> hit(N);
#pragma omp parallel for schedule(dynamic, 64)
    for (long i = 0; i < (long)N; ++i) {
      const float* r = &rays[i * 8];
      Primitive::Ray ray(Vec3(r[0], r[1], r[2]), Vec3(r[3], r[4], r[5]), 1.0f, r[6], r[7]);
      hit[i] = scene.m_Aobject->AnyHit(ray) ? 1 : 0;
    }
    npy_i32(out_dir + "/any_hit.npy", hit, {N});
    return 0;
  }

  if (mode != "render" || argc < 6) { std::fprintf(stderr, "bad mode\n"); return 2; }
  const int P = std::atoi(argv[3]);
  const int iters = std::atoi(argv[4]);
  out_dir = argv[5];
  const int W = cs.W, H = cs.H;

  SPPMR render;
  render.*member_ptr(StartTimeTag()) = 0;
  render.*member_ptr(CurTimeTag()) = 0;
  render.*member_ptr(EndTimeTag()) = (long int)1 << 40;

  std::vector<SPPMR::SharedHitPoint> sharedPoints;
  render.initializeSharedPoints(sharedPoints, W, H);
  std::vector<std::deque<SPPMR::Photon>> photons(P, std::deque<SPPMR::Photon>(32));
  std::vector<SPPMR::HitPoint> hitPoints(W * H);
  long long total_photon = 0;
  std::vector<double> t_photon, t_tree, t_eye, t_gather;

  for (int s = 1; s <= iters; ++s) {
    for (int i = 0; i < P; ++i) photons[i][0] = SPPMR::Photon();
    for (int i = 0; i < W * H; ++i) hitPoints[i] = SPPMR::HitPoint();

    double t0 = omp_get_wtime();
    const int n = render.createPhotonMap(photons, scene, *camera, P, s);
    double t1 = omp_get_wtime();
    total_photon += n;

    std::vector<SPPMR::Photon> photon;
    std::vector<int32_t> ph_path, ph_slot;
    for (int i = 0; i < P; ++i) {
      const auto& pdq = photons[i];
      for (int k = 0; k < (int)pdq.size(); ++k) {
        if (pdq[k].Valid) { photon.push_back(pdq[k]); ph_path.push_back(i); ph_slot.push_back(k); }
        else break;
      }
    }
    tgraph::kdtree<SPPMR::Photon> tree;
    if (!photon.empty()) tree.CreateTree(photon);
    double t2 = omp_get_wtime();

    render.createHitpoints(hitPoints, scene, s, *camera, W, H);
    double t3 = omp_get_wtime();

    // Per-hitpoint photon count and flux sum, with the query and filter of
    // applyHitPointInfo (SPPM.cpp:424-443), evaluated before the update.
    std::vector<int32_t> gM(W * H, 0);
    std::vector<float> gPhi(W * H * 3, 0.0f);
#pragma omp parallel for schedule(dynamic, 16)
    for (int v = 0; v < W * H; ++v) {
      const auto& i = hitPoints[v];
      if (i.Type != SPPMR::HitPoint::HIT) continue;
      const auto& s_ = sharedPoints[v];
      Vec3 bbMin(i.Position - s_.Radius * Vec3::Ones());
      Vec3 bbMax(i.Position + s_.Radius * Vec3::Ones());
      std::vector<SPPMR::Photon> ps;
      tree.GetElementsInsideBox(ps, bbMin, bbMax);
      Vec3 add(0, 0, 0); int m = 0;
      for (const auto& p : ps) {
        if ((p.Pos() - i.Position).norm2() < s_.Radius * s_.Radius) {
          const float Ii = p.Index;
          const float Io = SPPMR::near(p.Index, 1.0f) ? i.Gmt.param.Index : 1.0f;
          const Vec3 normal = p.InDir.dot(i.Gmt.Normal) < 0 ? i.Gmt.Normal : -i.Gmt.Normal;
          Material::FUNCTION_PARAM param(p.InDir, i.OutDir, normal, Ii, Io, i.Gmt.param.Roughness, i.Gmt.param.Extinction, i.Gmt.param.Reflectance);
          add += i.PixelWeight * i.Gmt.attribute->m_Surface->BRDF(param) * p.Flux / p.PDF;
          ++m;
        }
      }
      gM[v] = m; gPhi[v * 3] = add[0]; gPhi[v * 3 + 1] = add[1]; gPhi[v * 3 + 2] = add[2];
    }

    double t4 = omp_get_wtime();
    if (!photon.empty()) render.applyHitPointInfo(hitPoints, sharedPoints, tree, W, H);
    double t5 = omp_get_wtime();
    t_photon.push_back(t1 - t0); t_tree.push_back(t2 - t1); t_eye.push_back(t3 - t2); t_gather.push_back(t5 - t4);

    const std::string pre = out_dir + "/it" + std::to_string(s) + "_";
    const size_t HW = (size_t)W * H;
    std::vector<int32_t> hp_type(HW), hp_facet(HW);
    std::vector<float> hp_pos, hp_nrm, hp_out, hp_w, hp_rough, hp_dl;
    for (size_t v = 0; v < HW; ++v) {
      const auto& h = hitPoints[v];
      hp_type[v] = h.Type;
      hp_facet[v] = h.Type == SPPMR::HitPoint::HIT ? h.Facet._FacetID : -1;
      push3(hp_pos, h.Position); push3(hp_nrm, h.Gmt.Normal); push3(hp_out, h.OutDir); push3(hp_w, h.PixelWeight);
      push3(hp_dl, h.DirectLight);
      hp_rough.push_back(h.Gmt.param.Roughness);
    }
    npy_i32(pre + "hp_type.npy", hp_type, {HW});
    npy_i32(pre + "hp_facet.npy", hp_facet, {HW});
    npy_f32(pre + "hp_pos.npy", hp_pos, {HW, 3});
    npy_f32(pre + "hp_nrm.npy", hp_nrm, {HW, 3});
    npy_f32(pre + "hp_out.npy", hp_out, {HW, 3});
    npy_f32(pre + "hp_w.npy", hp_w, {HW, 3});
    npy_f32(pre + "hp_dl.npy", hp_dl, {HW, 3});
    npy_f32(pre + "hp_rough.npy", hp_rough, {HW});
    std::vector<float> ph;
    for (const auto& p : photon) {
      push3(ph, p.Position); push3(ph, p.Flux); push3(ph, p.InDir); ph.push_back(p.Index); ph.push_back(p.PDF);
    }
    npy_f32(pre + "ph.npy", ph, {photon.size(), 11});
    npy_i32(pre + "ph_path.npy", ph_path, {photon.size()});
    npy_i32(pre + "ph_slot.npy", ph_slot, {photon.size()});
    npy_i32(pre + "gather_m.npy", gM, {HW});
    npy_f32(pre + "gather_phi.npy", gPhi, {HW, 3});
    std::vector<float> sp_rad, sp_r, sp_dl; std::vector<int32_t> sp_n, sp_g, sp_ndl;
    for (const auto& sp : sharedPoints) {
      push3(sp_rad, sp.Radiance); sp_r.push_back(sp.Radius); sp_n.push_back(sp.NumPhoton); sp_g.push_back(sp.NumGather);
      push3(sp_dl, sp.DirectLight); sp_ndl.push_back(sp.NumDirectLight);
    }
    npy_f32(pre + "sp_dl.npy", sp_dl, {HW, 3});
    npy_i32(pre + "sp_ndl.npy", sp_ndl, {HW});
    npy_f32(pre + "sp_rad.npy", sp_rad, {HW, 3});
    npy_f32(pre + "sp_r.npy", sp_r, {HW});
    npy_i32(pre + "sp_n.npy", sp_n, {HW});
    npy_i32(pre + "sp_g.npy", sp_g, {HW});
  }

  Texture2D rt;
  rt.Init(W, H);
  render.reconstructImageFromSharedPoints(sharedPoints, rt, (int)total_photon, iters);
  std::vector<float> img;
  for (int i = 0; i < W * H; ++i) { const TColor c = rt.GetRawData()[i]; img.push_back(c[0]); img.push_back(c[1]); img.push_back(c[2]); img.push_back(c[3]); }
  npy_f32(out_dir + "/image.npy", img, {(size_t)W * H, 4});
  // The reference's own image output (main.cpp:161).
  TextureUtility::ExportPNG(rt, out_dir + "/image.png");
  std::vector<float> times;
  for (int s = 0; s < iters; ++s) { times.push_back(t_photon[s]); times.push_back(t_tree[s]); times.push_back(t_eye[s]); times.push_back(t_gather[s]); }
  npy_f32(out_dir + "/phase_seconds.npy", times, {(size_t)iters, 4});
  std::vector<int32_t> meta = {(int32_t)total_photon, iters, omp_get_max_threads()};
  npy_i32(out_dir + "/meta.npy", meta, {3});
  return 0;
}
