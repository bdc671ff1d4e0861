// The C++ mirror (include/friendsrender.hpp) on a hand-built scene: a box
// with a diffuse floor, a GGX-conductor back wall and a ceiling area light,
// seen by a pinhole camera.  RenderImage_FixStep must give the image the
// C-ABI calls give for the same iterations, and bad arguments must throw.
// Exit status 0 on success; prints the failing check otherwise.
#include <cmath>
#include <cstdio>
#include <stdexcept>
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

}  // namespace

int main() {
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
