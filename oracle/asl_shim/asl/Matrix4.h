// From-scratch stand-in for asl/Matrix4.h (see defs.h).  Row-major 4x4,
// m(i,j) = row i, column j.  Restated semantics (left-to-right sums, no
// fused multiply-add):
//   (A*B)(i,j) = A(i,0)B(0,j) + A(i,1)B(1,j) + A(i,2)B(2,j) + A(i,3)B(3,j)
//   A*v  (Vec3) = affine: row_i . (x,y,z) + A(i,3), no w divide
//   A%v  (Vec3) = linear part only
//   inverse()   = adjugate / determinant via 2x2 complementary minors
#ifndef ASL_SHIM_MATRIX4_H
#define ASL_SHIM_MATRIX4_H
#include "defs.h"
#include "Vec3.h"
namespace asl {
template <class T>
class Matrix4_ {
 public:
  T a[4][4];
  Matrix4_() { *this = identity(); }
  Matrix4_(T m00, T m01, T m02, T m03, T m10, T m11, T m12, T m13,
           T m20, T m21, T m22, T m23, T m30 = 0, T m31 = 0, T m32 = 0, T m33 = 1) {
    a[0][0] = m00; a[0][1] = m01; a[0][2] = m02; a[0][3] = m03;
    a[1][0] = m10; a[1][1] = m11; a[1][2] = m12; a[1][3] = m13;
    a[2][0] = m20; a[2][1] = m21; a[2][2] = m22; a[2][3] = m23;
    a[3][0] = m30; a[3][1] = m31; a[3][2] = m32; a[3][3] = m33;
  }
  T& operator()(int i, int j) { return a[i][j]; }
  const T& operator()(int i, int j) const { return a[i][j]; }
  static Matrix4_ identity() { return Matrix4_(1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1); }
  static Matrix4_ translate(T x, T y, T z) { return Matrix4_(1, 0, 0, x, 0, 1, 0, y, 0, 0, 1, z, 0, 0, 0, 1); }
  static Matrix4_ translate(const Vec3_<T>& t) { return translate(t.x, t.y, t.z); }
  static Matrix4_ scale(T s) { return Matrix4_(s, 0, 0, 0, 0, s, 0, 0, 0, 0, s, 0, 0, 0, 0, 1); }
  static Matrix4_ scale(T x, T y, T z) { return Matrix4_(x, 0, 0, 0, 0, y, 0, 0, 0, 0, z, 0, 0, 0, 0, 1); }
  static Matrix4_ scale(const Vec3_<T>& s) { return scale(s.x, s.y, s.z); }
  // rotation by angle t about the axis a (normalized), right-handed
  static Matrix4_ rotate(const Vec3_<T>& a, T t) {
    Vec3_<T> u = a.normalized();
    T c = cos(t), s = sin(t), k = 1 - c;
    return Matrix4_(k * u.x * u.x + c, k * u.x * u.y - s * u.z, k * u.x * u.z + s * u.y, 0,
                    k * u.x * u.y + s * u.z, k * u.y * u.y + c, k * u.y * u.z - s * u.x, 0,
                    k * u.x * u.z - s * u.y, k * u.y * u.z + s * u.x, k * u.z * u.z + c, 0,
                    0, 0, 0, 1);
  }
  static Matrix4_ rotateX(T t) { T c = cos(t), s = sin(t); return Matrix4_(1, 0, 0, 0, 0, c, -s, 0, 0, s, c, 0, 0, 0, 0, 1); }
  static Matrix4_ rotateY(T t) { T c = cos(t), s = sin(t); return Matrix4_(c, 0, s, 0, 0, 1, 0, 0, -s, 0, c, 0, 0, 0, 0, 1); }
  static Matrix4_ rotateZ(T t) { T c = cos(t), s = sin(t); return Matrix4_(c, -s, 0, 0, s, c, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1); }
  Matrix4_ operator*(const Matrix4_& b) const {
    Matrix4_ r;
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++)
        r.a[i][j] = a[i][0] * b.a[0][j] + a[i][1] * b.a[1][j] + a[i][2] * b.a[2][j] + a[i][3] * b.a[3][j];
    return r;
  }
  Vec3_<T> operator*(const Vec3_<T>& p) const {
    return Vec3_<T>(a[0][0] * p.x + a[0][1] * p.y + a[0][2] * p.z + a[0][3],
                    a[1][0] * p.x + a[1][1] * p.y + a[1][2] * p.z + a[1][3],
                    a[2][0] * p.x + a[2][1] * p.y + a[2][2] * p.z + a[2][3]);
  }
  Vec3_<T> operator%(const Vec3_<T>& p) const {
    return Vec3_<T>(a[0][0] * p.x + a[0][1] * p.y + a[0][2] * p.z,
                    a[1][0] * p.x + a[1][1] * p.y + a[1][2] * p.z,
                    a[2][0] * p.x + a[2][1] * p.y + a[2][2] * p.z);
  }
  Matrix4_ t() const {
    Matrix4_ r;
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++) r.a[i][j] = a[j][i];
    return r;
  }
  Matrix4_ transposed() const { return t(); }
  Matrix4_ inverse() const {
    const T(&m)[4][4] = a;
    T s0 = m[0][0] * m[1][1] - m[1][0] * m[0][1];
    T s1 = m[0][0] * m[1][2] - m[1][0] * m[0][2];
    T s2 = m[0][0] * m[1][3] - m[1][0] * m[0][3];
    T s3 = m[0][1] * m[1][2] - m[1][1] * m[0][2];
    T s4 = m[0][1] * m[1][3] - m[1][1] * m[0][3];
    T s5 = m[0][2] * m[1][3] - m[1][2] * m[0][3];
    T c5 = m[2][2] * m[3][3] - m[3][2] * m[2][3];
    T c4 = m[2][1] * m[3][3] - m[3][1] * m[2][3];
    T c3 = m[2][1] * m[3][2] - m[3][1] * m[2][2];
    T c2 = m[2][0] * m[3][3] - m[3][0] * m[2][3];
    T c1 = m[2][0] * m[3][2] - m[3][0] * m[2][2];
    T c0 = m[2][0] * m[3][1] - m[3][0] * m[2][1];
    T det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    T id = 1 / det;
    Matrix4_ r;
    r.a[0][0] = (m[1][1] * c5 - m[1][2] * c4 + m[1][3] * c3) * id;
    r.a[0][1] = (-m[0][1] * c5 + m[0][2] * c4 - m[0][3] * c3) * id;
    r.a[0][2] = (m[3][1] * s5 - m[3][2] * s4 + m[3][3] * s3) * id;
    r.a[0][3] = (-m[2][1] * s5 + m[2][2] * s4 - m[2][3] * s3) * id;
    r.a[1][0] = (-m[1][0] * c5 + m[1][2] * c2 - m[1][3] * c1) * id;
    r.a[1][1] = (m[0][0] * c5 - m[0][2] * c2 + m[0][3] * c1) * id;
    r.a[1][2] = (-m[3][0] * s5 + m[3][2] * s2 - m[3][3] * s1) * id;
    r.a[1][3] = (m[2][0] * s5 - m[2][2] * s2 + m[2][3] * s1) * id;
    r.a[2][0] = (m[1][0] * c4 - m[1][1] * c2 + m[1][3] * c0) * id;
    r.a[2][1] = (-m[0][0] * c4 + m[0][1] * c2 - m[0][3] * c0) * id;
    r.a[2][2] = (m[3][0] * s4 - m[3][1] * s2 + m[3][3] * s0) * id;
    r.a[2][3] = (-m[2][0] * s4 + m[2][1] * s2 - m[2][3] * s0) * id;
    r.a[3][0] = (-m[1][0] * c3 + m[1][1] * c1 - m[1][2] * c0) * id;
    r.a[3][1] = (m[0][0] * c3 - m[0][1] * c1 + m[0][2] * c0) * id;
    r.a[3][2] = (-m[3][0] * s3 + m[3][1] * s1 - m[3][2] * s0) * id;
    r.a[3][3] = (m[2][0] * s3 - m[2][1] * s1 + m[2][2] * s0) * id;
    return r;
  }
};
typedef Matrix4_<float> Matrix4;
typedef Matrix4_<double> Matrix4d;
}  // namespace asl
#endif
