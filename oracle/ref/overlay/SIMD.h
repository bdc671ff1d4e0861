#pragma once
// Oracle overlay (test infrastructure only).  Portable scalar replacement for
// the reference's AVX mSIMD::Double4 / mSIMD::Float8 (SPPM/SPPM/SIMD.h), with
// the std::array constructors that SPPM/SPPM/Primitive.h:208-252 relies on.
// Lane-wise IEEE arithmetic gives the same values as the AVX build; max/min
// follow _mm256_max_ps/_mm256_min_ps (second operand when unordered) and the
// comparisons follow _CMP_GT_OS/_CMP_LT_OS (false when unordered).
#include <array>
#include <cstddef>
#include <cstdint>
#include <iostream>

namespace mSIMD {

template <typename T, int N>
class LaneVec {
  T v[N];

 public:
  LaneVec() { for (int i = 0; i < N; ++i) v[i] = T(0); }
  LaneVec(T d) { for (int i = 0; i < N; ++i) v[i] = d; }
  LaneVec(const std::array<T, N>& a) { for (int i = 0; i < N; ++i) v[i] = a[i]; }

#define FR_LANE_OP(op)                                             \
  LaneVec operator op(const LaneVec& r) const {                    \
    LaneVec o;                                                     \
    for (int i = 0; i < N; ++i) o.v[i] = v[i] op r.v[i];           \
    return o;                                                      \
  }                                                                \
  LaneVec& operator op##=(const LaneVec& r) { return *this = *this op r; }
  FR_LANE_OP(+)
  FR_LANE_OP(-)
  FR_LANE_OP(*)
  FR_LANE_OP(/)
#undef FR_LANE_OP

  LaneVec operator-() const { return LaneVec(T(0)) - *this; }
  LaneVec operator+() const { return *this; }
  double operator[](size_t id) const { return v[id]; }

  uint32_t operator>(const LaneVec& r) const {
    uint32_t m = 0;
    for (int i = 0; i < N; ++i) m |= (v[i] > r.v[i] ? 1u : 0u) << i;
    return m;
  }
  uint32_t operator<(const LaneVec& r) const {
    uint32_t m = 0;
    for (int i = 0; i < N; ++i) m |= (v[i] < r.v[i] ? 1u : 0u) << i;
    return m;
  }
  static bool GetResult_i(uint32_t result, int i) { return result & (1u << i); }
  static LaneVec max(const LaneVec& a, const LaneVec& b) {
    LaneVec o;
    for (int i = 0; i < N; ++i) o.v[i] = a.v[i] > b.v[i] ? a.v[i] : b.v[i];
    return o;
  }
  static LaneVec min(const LaneVec& a, const LaneVec& b) {
    LaneVec o;
    for (int i = 0; i < N; ++i) o.v[i] = a.v[i] < b.v[i] ? a.v[i] : b.v[i];
    return o;
  }
};

class Double4 : public LaneVec<double, 4> {
 public:
  using LaneVec<double, 4>::LaneVec;
  Double4() : LaneVec<double, 4>() {}
  Double4(const LaneVec<double, 4>& b) : LaneVec<double, 4>(b) {}
  void PrintDouble4(std::ostream& ost) const {
    ost << (*this)[0] << " " << (*this)[1] << " " << (*this)[2] << " " << (*this)[3] << std::endl;
  }
};

class Float8 : public LaneVec<float, 8> {
 public:
  using LaneVec<float, 8>::LaneVec;
  Float8() : LaneVec<float, 8>() {}
  Float8(const LaneVec<float, 8>& b) : LaneVec<float, 8>(b) {}
  void PrintFloat8(std::ostream& ost) const {
    for (int i = 0; i < 8; ++i) ost << (*this)[i] << (i == 7 ? "\n" : " ");
  }
};

}  // namespace mSIMD
