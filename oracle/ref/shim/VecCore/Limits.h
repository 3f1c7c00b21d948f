// VecCore/Limits.h -- scalar stand-in (test infrastructure; see VecCore/VecCore).
// NumericLimits<T>::Max() is the largest finite value (VecGeom's kInfLength,
// VecGeom/base/Math.h:41); Min() the smallest positive normal value, which
// Vector3D::Normalized adds under its square root (VecGeom/base/Vector3D.h:288).
#ifndef VGREF_VECCORE_LIMITS_SHIM
#define VGREF_VECCORE_LIMITS_SHIM

#include <limits>

namespace vecCore {
template <typename T>
struct NumericLimits {
  static constexpr T Max() noexcept { return std::numeric_limits<T>::max(); }
  static constexpr T Min() noexcept { return std::numeric_limits<T>::min(); }
  static constexpr T Lowest() noexcept { return std::numeric_limits<T>::lowest(); }
  static constexpr T Highest() noexcept { return std::numeric_limits<T>::max(); }
  static constexpr T Epsilon() noexcept { return std::numeric_limits<T>::epsilon(); }
  static constexpr T Infinity() noexcept { return std::numeric_limits<T>::infinity(); }
};
} // namespace vecCore

#endif
