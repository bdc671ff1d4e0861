// C++ mirror of the reference's render-driver interface over the C-ABI.
//
// Render::StochasticProgressivePhotonMapping (SPPM/SPPM/SPPM.h:15-189) exposes
// RenderImage_FixStep and RenderImage_FixRenderTime (SPPM.h:184-185); this
// header keeps those names and argument meanings.  The reference's Scene and
// iCamera become the plain descriptors of friendsrender.h, the Texture2D
// render target a float RGBA buffer.  Errors throw std::runtime_error with
// the library's message (the reference's calls return void).
#pragma once
#include <chrono>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "friendsrender.h"

namespace fr {

// The material plug-in, SceneMaterialManager (SceneMaterial.h:9-33):
// SetParamtoAttribute is called once per MTL material with its name and the
// attribute's values (albedo Kd, emission Ke, SURFACE_PARAM() defaults); the
// base class keeps them, like the reference's default manager (a diffuse
// surface that is not an SPPM surface).  Exceptions fail the load.
class SceneMaterialManager {
 public:
  virtual ~SceneMaterialManager() = default;
  virtual void SetParamtoAttribute(fr_material_desc& material, const std::string& name) const {
    (void)material;
    (void)name;
  }
};

// Scene (Scene.h:55-93) as Scene::CreateScene (Scene.cpp:13-218) fills it,
// through fr_scene_load_obj: OBJ/MTL/PNG files read on the host.  The
// reference resolves MTL and texture names against "meshData//"; asset_dir
// (default that) is the prefix used here.
class Scene {
 public:
  Scene() = default;
  ~Scene() { fr_scene_free(scene_); }
  Scene(const Scene&) = delete;
  Scene& operator=(const Scene&) = delete;

  // Returns false and writes the reason to stderr on failure, as the
  // reference's CreateScene does.
  bool CreateScene(const char* obj_file, const SceneMaterialManager* materials = nullptr,
                   const char* ibl_file = nullptr, const char* asset_dir = nullptr) {
    fr_scene_free(scene_);
    scene_ = nullptr;
    const int rc = fr_scene_load_obj(obj_file, asset_dir, ibl_file, materials ? &Scene::plugin : nullptr,
                                     const_cast<SceneMaterialManager*>(materials), &scene_);
    if (rc != FR_OK) {
      std::fprintf(stderr, "%s\n", fr_last_error());
      return false;
    }
    return true;
  }
  bool loaded() const { return scene_ != nullptr; }
  const fr_scene_desc& desc() const {
    if (!scene_) throw std::logic_error("Scene: CreateScene has not succeeded");
    return *fr_scene_get_desc(scene_);
  }
  std::string material_name(int m) const {
    const char* n = scene_ ? fr_scene_material_name(scene_, m) : nullptr;
    return n ? n : "";
  }

 private:
  static int plugin(void* user, const char* name, fr_material_desc* material) {
    try {
      static_cast<const SceneMaterialManager*>(user)->SetParamtoAttribute(*material, name);
      return 0;
    } catch (...) {
      return 1;
    }
  }
  fr_scene* scene_ = nullptr;
};

struct RenderTarget {
  int width = 0, height = 0;
  std::vector<float> rgba;  // width * height * 4, pixel x + y * width
};

class StochasticProgressivePhotonMapping {
 public:
  explicit StochasticProgressivePhotonMapping(float alpha = 0.9f, float initial_radius = 0.015f)
      : alpha_(alpha), r0_(initial_radius) {}

  // RenderImage_FixStep (SPPM.cpp:682-717): Step iterations of NumPhotons/Step
  // photon paths each, then the image.  (The reference's version passes an
  // empty photon buffer; this is the fixed-iteration render it describes.)
  void RenderImage_FixStep(RenderTarget& target, const fr_scene_desc& scene, const fr_camera_desc& camera,
                           int NumPhotons, int Step) {
    if (Step <= 0) throw std::invalid_argument("RenderImage_FixStep: Step must be positive");
    fr_ctx* ctx = create(scene, camera, NumPhotons / Step);
    check(fr_iterate(ctx, Step), ctx);
    finish(target, camera, ctx);
  }

  void RenderImage_FixStep(RenderTarget& target, const Scene& scene, const fr_camera_desc& camera, int NumPhotons,
                           int Step) {
    RenderImage_FixStep(target, scene.desc(), camera, NumPhotons, Step);
  }

  // RenderImage_FixRenderTime (SPPM.cpp:719-858): iterations of
  // NumPhotonsPerStep paths until RenderTimeSecond has passed.
  void RenderImage_FixRenderTime(RenderTarget& target, const fr_scene_desc& scene, const fr_camera_desc& camera,
                                 int NumPhotonsPerStep, int RenderTimeSecond) {
    const auto end = std::chrono::steady_clock::now() + std::chrono::seconds(RenderTimeSecond);
    fr_ctx* ctx = create(scene, camera, NumPhotonsPerStep);
    do {
      check(fr_iterate(ctx, 1), ctx);
      check(fr_synchronize(ctx), ctx);
    } while (std::chrono::steady_clock::now() < end);
    finish(target, camera, ctx);
  }
  void RenderImage_FixRenderTime(RenderTarget& target, const Scene& scene, const fr_camera_desc& camera,
                                 int NumPhotonsPerStep, int RenderTimeSecond) {
    RenderImage_FixRenderTime(target, scene.desc(), camera, NumPhotonsPerStep, RenderTimeSecond);
  }

 private:
  float alpha_, r0_;

  fr_ctx* create(const fr_scene_desc& scene, const fr_camera_desc& camera, int photons) {
    fr_sppm_params p{};
    p.photons_per_iteration = photons;
    p.alpha = alpha_;
    p.initial_radius = r0_;
    fr_ctx* ctx = nullptr;
    if (fr_create(&scene, &camera, &p, &ctx) != FR_OK) throw std::runtime_error(fr_last_error());
    return ctx;
  }
  static void check(int rc, fr_ctx* ctx) {
    if (rc != FR_OK) {
      const std::string msg = fr_last_error();
      fr_destroy(ctx);
      throw std::runtime_error(msg);
    }
  }
  static void finish(RenderTarget& target, const fr_camera_desc& camera, fr_ctx* ctx) {
    target.width = camera.width;
    target.height = camera.height;
    target.rgba.resize((size_t)camera.width * camera.height * 4);
    check(fr_resolve(ctx, target.rgba.data()), ctx);
    fr_destroy(ctx);
  }
};

}  // namespace fr
