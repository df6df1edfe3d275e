// From-scratch stand-in for asl/Matrix3.h (see defs.h): only the 2-D affine
// six-value constructor that Renderer.cpp instantiates (its value is unused).
#ifndef ASL_SHIM_MATRIX3_H
#define ASL_SHIM_MATRIX3_H
#include "defs.h"
#include "Vec2.h"
namespace asl {
template <class T>
class Matrix3_ {
 public:
  T a[3][3];
  Matrix3_(T m00, T m01, T m02, T m10, T m11, T m12) {
    a[0][0] = m00; a[0][1] = m01; a[0][2] = m02;
    a[1][0] = m10; a[1][1] = m11; a[1][2] = m12;
    a[2][0] = 0; a[2][1] = 0; a[2][2] = 1;
  }
};
typedef Matrix3_<float> Matrix3;
}  // namespace asl
#endif
