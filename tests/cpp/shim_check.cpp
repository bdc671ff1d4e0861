// The C++ mirror (include/friendsrender.hpp) on a hand-built scene: a box
// with a diffuse floor, a GGX-conductor back wall and a ceiling area light,
// seen by a pinhole camera.  RenderImage_FixStep must give the image the
// C-ABI calls give for the same iterations, and bad arguments must throw.
// The scene is also written as OBJ/MTL into <dir> and read back with
// fr::Scene::CreateScene and a SceneMaterialManager: the facets must be the
// hand-built ones and render the same image.
//
//   shim_check <dir>          everything (needs a GPU)
//   shim_check <dir> ingest   the OBJ round trip only (host code)
//
// Exit status 0 on success; prints the failing check otherwise.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "friendsrender.hpp"

namespace {

struct Box {
  std::vector<float> pos, nrm, uv;
  std::vector<int32_t> mat;
  void quad(const float a[3], const float b[3], const float c[3], const float d[3], const float n[3], int m) {
    const float* t[2][3] = {{a, b, c}, {a, c, d}};
    for (auto& tri : t) {
      for (const float* v : tri) {
        pos.insert(pos.end(), v, v + 3);
        nrm.insert(nrm.end(), n, n + 3);
        uv.push_back(0.5f);
        uv.push_back(0.5f);
      }
      mat.push_back(m);
    }
  }
};

int fail(const char* what) {
  std::printf("FAIL: %s\n", what);
  return 1;
}

const char* kNames[3] = {"floor", "wall", "light"};

// Writes the box as <dir>/box.obj and <dir>/box.mtl, one v/vt/vn per corner.
bool write_obj(const Box& b, const fr_material_desc* mats, const std::string& dir) {
  std::FILE* m = std::fopen((dir + "/box.mtl").c_str(), "w");
  std::FILE* o = std::fopen((dir + "/box.obj").c_str(), "w");
  if (!m || !o) return false;
  for (int k = 0; k < 3; ++k)
    std::fprintf(m, "newmtl %s\nKd %.9g %.9g %.9g\nKe %.9g %.9g %.9g\n\n", kNames[k], mats[k].albedo[0],
                 mats[k].albedo[1], mats[k].albedo[2], mats[k].emission[0], mats[k].emission[1], mats[k].emission[2]);
  std::fprintf(o, "mtllib box.mtl\n");
  for (size_t t = 0; t < b.mat.size(); ++t) {
    for (int c = 0; c < 3; ++c) {
      const float* p = &b.pos[(t * 3 + c) * 3];
      const float* n = &b.nrm[(t * 3 + c) * 3];
      const float* u = &b.uv[(t * 3 + c) * 2];
      std::fprintf(o, "v %.9g %.9g %.9g\nvt %.9g %.9g\nvn %.9g %.9g %.9g\n", p[0], p[1], p[2], u[0], u[1], n[0], n[1],
                   n[2]);
    }
    const int v = (int)t * 3 + 1;
    std::fprintf(o, "usemtl %s\nf %d/%d/%d %d/%d/%d %d/%d/%d\n", kNames[b.mat[t]], v, v, v, v + 1, v + 1, v + 1, v + 2,
                 v + 2, v + 2);
  }
  std::fclose(m);
  std::fclose(o);
  return true;
}

// The reference's way of giving materials their surfaces (main.cpp:14-114).
class BoxMaterials : public fr::SceneMaterialManager {
 public:
  explicit BoxMaterials(const fr_material_desc* mats) : mats_(mats) {}
  void SetParamtoAttribute(fr_material_desc& m, const std::string& name) const override {
    for (int k = 0; k < 3; ++k) {
      if (name != kNames[k]) continue;
      m.type = mats_[k].type;
      m.sppm_surface = mats_[k].sppm_surface;
      m.opaque = mats_[k].opaque;
      m.index = mats_[k].index;
      m.roughness = mats_[k].roughness;
      m.extinction = mats_[k].extinction;
      m.reflectance = mats_[k].reflectance;
      return;
    }
    throw std::runtime_error("unknown material " + name);
  }

 private:
  const fr_material_desc* mats_;
};

// Reads the box back and compares it with the hand-built arrays.
int check_ingest(const Box& b, const fr_material_desc* mats, const std::string& dir, fr::Scene& loaded) {
  if (!write_obj(b, mats, dir)) return fail("cannot write the OBJ files");
  BoxMaterials plugin(mats);
  const std::string asset_dir = dir + "/";
  if (!loaded.CreateScene((dir + "/box.obj").c_str(), &plugin, nullptr, asset_dir.c_str()))
    return fail("CreateScene failed");
  const fr_scene_desc& d = loaded.desc();
  if (d.num_facets != (int32_t)b.mat.size() || d.num_materials != 3 || d.num_textures != 0) return fail("counts");
  if (std::memcmp(d.positions, b.pos.data(), b.pos.size() * 4) || std::memcmp(d.normals, b.nrm.data(), b.nrm.size() * 4) ||
      std::memcmp(d.uvs, b.uv.data(), b.uv.size() * 4) || std::memcmp(d.material_ids, b.mat.data(), b.mat.size() * 4))
    return fail("loaded facets differ from the written ones");
  for (int k = 0; k < 3; ++k) {
    if (loaded.material_name(k) != kNames[k]) return fail("loaded material name differs");
    if (std::memcmp(&d.materials[k], &mats[k], sizeof(fr_material_desc)) != 0) {
      const fr_material_desc& m = d.materials[k];
      std::printf("material %d: type %d/%d sppm %d/%d opaque %d/%d tex %d %d %d idx %g/%g rough %g/%g ext %g/%g refl %g/%g\n", k,
                  m.type, mats[k].type, m.sppm_surface, mats[k].sppm_surface, m.opaque, mats[k].opaque, m.tex_albedo,
                  m.tex_roughness, m.tex_bump, m.index, mats[k].index, m.roughness, mats[k].roughness, m.extinction,
                  mats[k].extinction, m.reflectance, mats[k].reflectance);
      return fail("loaded material differs");
    }
  }
  fr::Scene missing;
  if (missing.CreateScene((dir + "/no_such.obj").c_str())) return fail("missing OBJ accepted");
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) return fail("usage: shim_check <dir> [ingest]");
  const std::string dir = argv[1];
  const bool ingest_only = argc > 2 && std::strcmp(argv[2], "ingest") == 0;
  Box b;
  const float f0[3] = {-1, 0, -1}, f1[3] = {1, 0, -1}, f2[3] = {1, 0, 1}, f3[3] = {-1, 0, 1}, up[3] = {0, 1, 0};
  const float w0[3] = {-1, 0, -1}, w1[3] = {-1, 2, -1}, w2[3] = {1, 2, -1}, w3[3] = {1, 0, -1}, fw[3] = {0, 0, 1};
  const float l0[3] = {-0.3f, 1.99f, -0.3f}, l1[3] = {-0.3f, 1.99f, 0.3f}, l2[3] = {0.3f, 1.99f, 0.3f},
              l3[3] = {0.3f, 1.99f, -0.3f}, dn[3] = {0, -1, 0};
  b.quad(f0, f3, f2, f1, up, 0);
  b.quad(w0, w3, w2, w1, fw, 1);
  b.quad(l0, l3, l2, l1, dn, 2);
  fr_material_desc mats[3] = {};
  mats[0].type = FR_MAT_DIFFUSE;
  mats[0].sppm_surface = 1;
  mats[0].opaque = 1;
  mats[1].type = FR_MAT_GGX_CONDUCTOR;
  mats[1].sppm_surface = 1;
  mats[1].opaque = 1;
  mats[1].roughness = 0.2f;
  mats[1].index = 1.5f;
  mats[1].extinction = 2.0f;
  mats[2].type = FR_MAT_DIFFUSE;
  mats[2].opaque = 1;
  for (auto& m : mats) m.tex_albedo = m.tex_roughness = m.tex_bump = -1;
  for (int c = 0; c < 3; ++c) {
    mats[0].albedo[c] = 0.75f;
    mats[1].albedo[c] = 0.9f;
    mats[2].albedo[c] = 1.0f;
    mats[2].emission[c] = 10.0f;
  }
  fr_scene_desc scene{(int32_t)b.mat.size(), b.pos.data(), b.nrm.data(), b.uv.data(), b.mat.data(), 3, mats, 0,
                      nullptr};
  fr::Scene loaded;
  if (const int rc = check_ingest(b, mats, dir, loaded)) return rc;
  if (ingest_only) {
    std::printf("ok\n");
    return 0;
  }
  fr_camera_desc cam{};
  cam.type = FR_CAMERA_PINHOLE;
  cam.width = 64;
  cam.height = 48;
  const float eye[3] = {0, 1, 3.5f}, at[3] = {0, 0.8f, 0};
  for (int c = 0; c < 3; ++c) {
    cam.position[c] = eye[c];
    cam.target[c] = at[c];
  }
  cam.fov_degrees = 40;
  cam.focal_length = 1;
  cam.distance_to_lens = 1;
  cam.aspect = 64.0f / 48.0f;

  const int photons = 20000, steps = 4;
  fr::StochasticProgressivePhotonMapping render(0.7f, 0.05f);
  fr::RenderTarget target;
  try {
    render.RenderImage_FixStep(target, scene, cam, photons * steps, steps);
  } catch (const std::exception& e) {
    std::printf("FAIL: RenderImage_FixStep threw: %s\n", e.what());
    return 1;
  }
  if (target.width != 64 || target.height != 48 || target.rgba.size() != 64u * 48u * 4u) return fail("target size");

  fr_sppm_params p{};
  p.photons_per_iteration = photons;
  p.alpha = 0.7f;
  p.initial_radius = 0.05f;
  fr_ctx* ctx = nullptr;
  if (fr_create(&scene, &cam, &p, &ctx) != FR_OK) return fail(fr_last_error());
  std::vector<float> img(target.rgba.size());
  if (fr_iterate(ctx, steps) != FR_OK || fr_resolve(ctx, img.data()) != FR_OK) return fail(fr_last_error());
  fr_destroy(ctx);

  double peak = 0, diff = 0;
  int lit = 0;
  for (size_t i = 0; i < img.size(); ++i) {
    if (!std::isfinite(target.rgba[i])) return fail("non-finite pixel");
    peak = std::fmax(peak, std::fabs(img[i]));
    diff = std::fmax(diff, std::fabs((double)img[i] - target.rgba[i]));
    if (i % 4 != 3 && target.rgba[i] > 0) ++lit;
  }
  if (lit < 64 * 48) return fail("image mostly black");
  if (diff > 1e-5 * peak) return fail("FixStep image differs from the C-ABI render");

  fr::RenderTarget from_obj;
  try {
    render.RenderImage_FixStep(from_obj, loaded, cam, photons * steps, steps);
  } catch (const std::exception& e) {
    std::printf("FAIL: RenderImage_FixStep on the loaded scene threw: %s\n", e.what());
    return 1;
  }
  // A grid cell's photons are summed in the order its atomic counter gave
  // them slots, so renders agree to float rounding, not bit for bit (as above).
  if (from_obj.rgba.size() != target.rgba.size()) return fail("OBJ render size");
  double odiff = 0;
  for (size_t i = 0; i < target.rgba.size(); ++i) odiff = std::fmax(odiff, std::fabs((double)from_obj.rgba[i] - target.rgba[i]));
  if (odiff > 1e-5 * peak) return fail("the scene read from OBJ renders differently");

  bool threw = false;
  try {
    render.RenderImage_FixStep(target, scene, cam, photons, 0);
  } catch (const std::invalid_argument&) {
    threw = true;
  }
  if (!threw) return fail("Step 0 accepted");
  threw = false;
  fr_camera_desc bad = cam;
  bad.width = 0;
  try {
    render.RenderImage_FixStep(target, scene, bad, photons, 1);
  } catch (const std::runtime_error&) {
    threw = true;
  }
  if (!threw) return fail("zero-width camera accepted");
  std::printf("ok\n");
  return 0;
}
