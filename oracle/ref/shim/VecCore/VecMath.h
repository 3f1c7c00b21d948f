// VecCore/VecMath.h -- scalar stand-in (test infrastructure; see VecCore/VecCore).
// Every function forwards to <cmath> on one scalar; Sign follows the sign bit.
#ifndef VGREF_VECCORE_VECMATH_SHIM
#define VGREF_VECCORE_VECMATH_SHIM

#include <cmath>

namespace vecCore {
namespace math {

template <typename T>
inline T Abs(T x)
{
  return std::abs(x);
}
template <typename T>
inline T Min(T a, T b)
{
  return a < b ? a : b;
}
template <typename T>
inline T Max(T a, T b)
{
  return a > b ? a : b;
}
template <typename T>
inline T Min(T a, T b, T c)
{
  return Min(a, Min(b, c));
}
template <typename T>
inline T Max(T a, T b, T c)
{
  return Max(a, Max(b, c));
}
template <typename T>
inline T CopySign(T x, T y)
{
  return std::copysign(x, y);
}
template <typename T>
inline T Sign(T x)
{
  return std::copysign(T(1), x);
}
template <typename T>
inline T Sqrt(T x)
{
  return std::sqrt(x);
}
template <typename T>
inline T Cbrt(T x)
{
  return std::cbrt(x);
}
template <typename T>
inline T Sin(T x)
{
  return std::sin(x);
}
template <typename T>
inline T Cos(T x)
{
  return std::cos(x);
}
template <typename T>
inline void SinCos(T x, T *s, T *c)
{
  *s = std::sin(x);
  *c = std::cos(x);
}
template <typename T>
inline T Tan(T x)
{
  return std::tan(x);
}
template <typename T>
inline T ASin(T x)
{
  return std::asin(x);
}
template <typename T>
inline T ACos(T x)
{
  return std::acos(x);
}
template <typename T>
inline T ATan(T x)
{
  return std::atan(x);
}
template <typename T>
inline T ATan2(T y, T x)
{
  return std::atan2(y, x);
}
template <typename T>
inline T Exp(T x)
{
  return std::exp(x);
}
template <typename T>
inline T Log(T x)
{
  return std::log(x);
}
template <typename T>
inline T Log2(T x)
{
  return std::log2(x);
}
template <typename T>
inline T Log10(T x)
{
  return std::log10(x);
}
template <typename T, typename U>
inline T Pow(T x, U y)
{
  return std::pow(x, y);
}
template <typename T>
inline T Floor(T x)
{
  return std::floor(x);
}
template <typename T>
inline T Ceil(T x)
{
  return std::ceil(x);
}
template <typename T>
inline T Round(T x)
{
  return std::round(x);
}
template <typename T>
inline T Trunc(T x)
{
  return std::trunc(x);
}
template <typename T>
inline bool IsInf(T x)
{
  return std::isinf(x);
}
template <typename T>
inline bool IsNaN(T x)
{
  return std::isnan(x);
}
template <typename T>
inline T Sinh(T x)
{
  return std::sinh(x);
}
template <typename T>
inline T Cosh(T x)
{
  return std::cosh(x);
}
template <typename T>
inline T Tanh(T x)
{
  return std::tanh(x);
}

} // namespace math
} // namespace vecCore

#endif
