// From-scratch stand-in for asl/Vec3.h (see defs.h).  Restated semantics:
//   dot a*b = (a.x*b.x + a.y*b.y) + a.z*b.z
//   length() = sqrt(x*x + y*y + z*z)
//   v / s divides each component by s; normalized() = v / length()
#ifndef ASL_SHIM_VEC3_H
#define ASL_SHIM_VEC3_H
#include "defs.h"
#include "Vec2.h"
namespace asl {
template <class T>
class Vec3_ {
 public:
  T x, y, z;
  Vec3_() {}
  Vec3_(T x_, T y_, T z_) : x(x_), y(y_), z(z_) {}
  template <class U> Vec3_<U> with() const { return Vec3_<U>((U)x, (U)y, (U)z); }
  Vec2_<T> xy() const { return Vec2_<T>(x, y); }
  Vec3_ operator+(const Vec3_& b) const { return Vec3_(x + b.x, y + b.y, z + b.z); }
  Vec3_ operator-(const Vec3_& b) const { return Vec3_(x - b.x, y - b.y, z - b.z); }
  Vec3_ operator-() const { return Vec3_(-x, -y, -z); }
  Vec3_ operator*(T s) const { return Vec3_(x * s, y * s, z * s); }
  Vec3_ operator/(T s) const { return Vec3_(x / s, y / s, z / s); }
  T operator*(const Vec3_& b) const { return x * b.x + y * b.y + z * b.z; }
  Vec3_ operator^(const Vec3_& b) const { return Vec3_(y * b.z - z * b.y, z * b.x - x * b.z, x * b.y - y * b.x); }
  Vec3_& operator+=(const Vec3_& b) { x += b.x; y += b.y; z += b.z; return *this; }
  Vec3_& operator-=(const Vec3_& b) { x -= b.x; y -= b.y; z -= b.z; return *this; }
  Vec3_& operator*=(T s) { x *= s; y *= s; z *= s; return *this; }
  bool operator==(const Vec3_& b) const { return x == b.x && y == b.y && z == b.z; }
  bool operator!=(const Vec3_& b) const { return !(*this == b); }
  T length() const { return sqrt(x * x + y * y + z * z); }
  T length2() const { return x * x + y * y + z * z; }
  Vec3_ normalized() const { return *this / length(); }
  static Vec3_ zeros() { return Vec3_(0, 0, 0); }
};
template <class T> inline Vec3_<T> operator*(T s, const Vec3_<T>& v) { return Vec3_<T>(s * v.x, s * v.y, s * v.z); }
template <class T> inline Vec3_<T> min(const Vec3_<T>& a, const Vec3_<T>& b) { return Vec3_<T>(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
template <class T> inline Vec3_<T> max(const Vec3_<T>& a, const Vec3_<T>& b) { return Vec3_<T>(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
typedef Vec3_<float> Vec3;
typedef Vec3_<double> Vec3d;
}  // namespace asl
#endif
