// Host check of query_ball_ok (csrc/fr_layout.h), the bound on a radius
// query's cell range that the grid kernels and fr_radius_query share.
// Prints "ok" when every case gives the expected answer.
#include <cmath>
#include <cstdio>
#include <limits>

#include "fr_layout.h"

int main() {
  using fr::query_ball_ok;
  const float o[3] = {0.0f, 0.0f, 0.0f};
  const float inf = std::numeric_limits<float>::infinity(), nan = std::numeric_limits<float>::quiet_NaN();
  struct Case {
    float x, y, z, R, inv;
    bool want;
    const char* what;
  } cases[] = {
      {0.5f, 0.5f, 0.5f, 0.05f, 50.0f, true, "ordinary ball"},
      {0.5f, 0.5f, 0.5f, 0.0f, 50.0f, true, "zero radius"},
      {0.5f, 0.5f, 0.5f, nan, 50.0f, false, "NaN radius"},
      {0.5f, 0.5f, 0.5f, inf, 50.0f, false, "infinite radius"},
      {0.5f, 0.5f, 0.5f, -0.01f, 50.0f, false, "negative radius"},
      {nan, 0.5f, 0.5f, 0.05f, 50.0f, false, "NaN position"},
      {0.5f, 0.5f, inf, 0.05f, 50.0f, false, "infinite position"},
      {0.0f, 0.0f, 0.0f, 1.26f, 50.0f, true, "126 cells"},
      {0.0f, 0.0f, 0.0f, 1.30f, 50.0f, false, "130 cells"},
      {0.0f, 0.0f, 0.0f, 1.0f, 1.0e6f, false, "two million cells"},
      {3.0e7f, 0.0f, 0.0f, 0.01f, 50.0f, false, "1.5e9 cells from the origin"},
      {-3.0e7f, 0.0f, 0.0f, 0.01f, 50.0f, false, "-1.5e9 cells from the origin"},
      {1.0e7f, 0.0f, 0.0f, 0.01f, 50.0f, true, "5e8 cells from the origin"},
  };
  int bad = 0;
  for (const Case& c : cases) {
    const bool got = query_ball_ok(c.x, c.y, c.z, c.R, o, c.inv);
    if (got != c.want) {
      std::printf("%s: got %d want %d\n", c.what, (int)got, (int)c.want);
      ++bad;
    }
  }
  // An accepted ball's cell range, computed as the kernels do, stays within
  // kMaxQuerySpan + 1 cells per axis and converts to int exactly.
  for (int k = 0; k < 100000; ++k) {
    const float x = -4.0f + 8.0f * (float)k / 100000.0f, R = 0.0001f * (float)(k % 3000), inv = 1.0f + (float)(k % 97);
    if (!query_ball_ok(x, x, x, R, o, inv)) continue;
    const float f0 = (x - R - o[0]) * inv, f1 = (x + R - o[0]) * inv;
    const double span = std::floor((double)f1) - std::floor((double)f0) + 1.0;
    if (span > fr::kMaxQuerySpan + 1 || span < 1.0) {
      std::printf("span %g at x %g R %g inv %g\n", span, (double)x, (double)R, (double)inv);
      ++bad;
    }
  }
  std::printf(bad ? "failed\n" : "ok\n");
  return bad ? 1 : 0;
}
