// From-scratch stand-in for asl/Vec2.h (see defs.h).  Restated semantics:
//   dot  a*b = a.x*b.x + a.y*b.y        (x term first)
//   cross a^b = a.x*b.y - a.y*b.x
//   perpend() = (-y, x)
#ifndef ASL_SHIM_VEC2_H
#define ASL_SHIM_VEC2_H
#include "defs.h"
namespace asl {
template <class T>
class Vec2_ {
 public:
  T x, y;
  Vec2_() {}
  Vec2_(T x_, T y_) : x(x_), y(y_) {}
  Vec2_ operator+(const Vec2_& b) const { return Vec2_(x + b.x, y + b.y); }
  Vec2_ operator-(const Vec2_& b) const { return Vec2_(x - b.x, y - b.y); }
  Vec2_ operator-() const { return Vec2_(-x, -y); }
  Vec2_ operator*(T s) const { return Vec2_(x * s, y * s); }
  Vec2_ operator/(T s) const { return Vec2_(x / s, y / s); }
  T operator*(const Vec2_& b) const { return x * b.x + y * b.y; }
  T operator^(const Vec2_& b) const { return x * b.y - y * b.x; }
  Vec2_& operator+=(const Vec2_& b) { x += b.x; y += b.y; return *this; }
  Vec2_& operator-=(const Vec2_& b) { x -= b.x; y -= b.y; return *this; }
  Vec2_ perpend() const { return Vec2_(-y, x); }
  T length() const { return sqrt(x * x + y * y); }
  Vec2_ normalized() const { T l = length(); return Vec2_(x / l, y / l); }
  static Vec2_ zeros() { return Vec2_(0, 0); }
};
template <class T> inline Vec2_<T> operator*(T s, const Vec2_<T>& v) { return Vec2_<T>(s * v.x, s * v.y); }
template <class T> inline Vec2_<T> min(const Vec2_<T>& a, const Vec2_<T>& b) { return Vec2_<T>(min(a.x, b.x), min(a.y, b.y)); }
template <class T> inline Vec2_<T> max(const Vec2_<T>& a, const Vec2_<T>& b) { return Vec2_<T>(max(a.x, b.x), max(a.y, b.y)); }
typedef Vec2_<float> Vec2;
typedef Vec2_<double> Vec2d;
}  // namespace asl
#endif
