#pragma once
// Oracle overlay (test infrastructure only).  Replaces the reference's
// RandomMT (SPPM/SPPM/MT.h:7-43: std::mt19937 + uniform_real_distribution)
// with a counter-based Philox4x32-10 generator of the same interface, so the
// reference's CPU path and the GPU path draw identical numbers:
//
//   key     = { (uint32_t)Seed, 0x5350504D }
//   draw n  = Philox4x32-10(counter = {n / 4, 0, 0, 0}, key)[n % 4]
//   value   = (x >> 8) * 2^-24   (exact in float and double, in [0, 1))
//
// Philox4x32-10 follows Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers:
// As Easy as 1, 2, 3", SC'11.  The constructor also records the generator as
// the latest one built on the calling thread; the harness's camera sampler
// draws its three lens/jitter numbers from it (the reference's shared
// UniformSample generator, CameraSampler.h:19-29, is a data race across
// OpenMP threads).
#include <algorithm>
#include <cfloat>
#include <cstdint>
#include <float.h>
#include <random>
#include <time.h>

namespace fr_oracle_rng {

inline void philox4x32_10(const uint32_t in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

}  // namespace fr_oracle_rng

class RandomMT {
 private:
  RandomMT& operator=(const RandomMT&);
  RandomMT(const RandomMT&);

  uint32_t m_key[2];
  uint32_t m_draw;
  uint32_t m_block[4];
  double m_min, m_max;

  static RandomMT*& latest() {
    static thread_local RandomMT* p = nullptr;
    return p;
  }
  void init(int Seed, double mn, double mx) {
    m_key[0] = (uint32_t)Seed;
    m_key[1] = 0x5350504Du;
    m_draw = 0;
    m_min = mn;
    m_max = mx;
    latest() = this;
  }
  uint32_t next_u32() {
    const uint32_t lane = m_draw & 3u;
    if (lane == 0) {
      const uint32_t ctr[4] = {m_draw >> 2, 0u, 0u, 0u};
      fr_oracle_rng::philox4x32_10(ctr, m_key, m_block);
    }
    ++m_draw;
    return m_block[lane];
  }
  double unit() { return (double)((float)(next_u32() >> 8) * (1.0f / 16777216.0f)); }

 public:
  explicit RandomMT(int Seed, float min, float max) { init(Seed, min, max); }
  explicit RandomMT(int Seed) { init(Seed, 0.0, 1.0); }
  explicit RandomMT() { init(11101, 0.0, 1.0); }

  // [0,1]
  double genrand64_real1() { return m_min + (m_max - m_min) * unit(); }
  // [0,1)
  double genrand64_real2() { return std::min(genrand64_real1(), 1.0 - DBL_MIN); }
  // (0,1)
  double genrand64_real3() { return std::max(DBL_MIN, std::min(genrand64_real1(), 1.0 - DBL_MIN)); }

  uint32_t DrawCount() const { return m_draw; }
  static RandomMT* LatestOnThisThread() { return latest(); }
};
