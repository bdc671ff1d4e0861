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
#include <stdexcept>
#include <string>
#include <vector>

#include "friendsrender.h"

namespace fr {

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
