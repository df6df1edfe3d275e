// Host helpers of the C ABI: Matrix4 product and inverse, the projection
// builders of src/Renderer.cpp:40-83 and Scene::collectShapes
// (src/Scene.cpp:13-36).  Compiled with -ffp-contract=off so each float
// expression is evaluated as written (no fused multiply-add), matching the
// reference's host arithmetic on both x86-64 and aarch64.
#include <math.h>
#include <string.h>

#include <vector>

#include "host_math.h"

namespace mrg {

void mat4_mul(const float* a, const float* b, float* out) {
  float r[16];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++)
      r[4 * i + j] = a[4 * i + 0] * b[0 + j] + a[4 * i + 1] * b[4 + j] + a[4 * i + 2] * b[8 + j] +
                     a[4 * i + 3] * b[12 + j];
  memcpy(out, r, sizeof(r));
}

// Adjugate over 2x2 complementary minors, divided by the determinant.
void mat4_inverse(const float* m, float* out) {
  auto M = [m](int i, int j) { return m[4 * i + j]; };
  float s0 = M(0, 0) * M(1, 1) - M(1, 0) * M(0, 1);
  float s1 = M(0, 0) * M(1, 2) - M(1, 0) * M(0, 2);
  float s2 = M(0, 0) * M(1, 3) - M(1, 0) * M(0, 3);
  float s3 = M(0, 1) * M(1, 2) - M(1, 1) * M(0, 2);
  float s4 = M(0, 1) * M(1, 3) - M(1, 1) * M(0, 3);
  float s5 = M(0, 2) * M(1, 3) - M(1, 2) * M(0, 3);
  float c5 = M(2, 2) * M(3, 3) - M(3, 2) * M(2, 3);
  float c4 = M(2, 1) * M(3, 3) - M(3, 1) * M(2, 3);
  float c3 = M(2, 1) * M(3, 2) - M(3, 1) * M(2, 2);
  float c2 = M(2, 0) * M(3, 3) - M(3, 0) * M(2, 3);
  float c1 = M(2, 0) * M(3, 2) - M(3, 0) * M(2, 2);
  float c0 = M(2, 0) * M(3, 1) - M(3, 0) * M(2, 1);
  float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
  float id = 1 / det;
  float r[16];
  r[0] = (M(1, 1) * c5 - M(1, 2) * c4 + M(1, 3) * c3) * id;
  r[1] = (-M(0, 1) * c5 + M(0, 2) * c4 - M(0, 3) * c3) * id;
  r[2] = (M(3, 1) * s5 - M(3, 2) * s4 + M(3, 3) * s3) * id;
  r[3] = (-M(2, 1) * s5 + M(2, 2) * s4 - M(2, 3) * s3) * id;
  r[4] = (-M(1, 0) * c5 + M(1, 2) * c2 - M(1, 3) * c1) * id;
  r[5] = (M(0, 0) * c5 - M(0, 2) * c2 + M(0, 3) * c1) * id;
  r[6] = (-M(3, 0) * s5 + M(3, 2) * s2 - M(3, 3) * s1) * id;
  r[7] = (M(2, 0) * s5 - M(2, 2) * s2 + M(2, 3) * s1) * id;
  r[8] = (M(1, 0) * c4 - M(1, 1) * c2 + M(1, 3) * c0) * id;
  r[9] = (-M(0, 0) * c4 + M(0, 1) * c2 - M(0, 3) * c0) * id;
  r[10] = (M(3, 0) * s4 - M(3, 1) * s2 + M(3, 3) * s0) * id;
  r[11] = (-M(2, 0) * s4 + M(2, 1) * s2 - M(2, 3) * s0) * id;
  r[12] = (-M(1, 0) * c3 + M(1, 1) * c1 - M(1, 2) * c0) * id;
  r[13] = (M(0, 0) * c3 - M(0, 1) * c1 + M(0, 2) * c0) * id;
  r[14] = (-M(3, 0) * s3 + M(3, 1) * s1 - M(3, 2) * s0) * id;
  r[15] = (M(2, 0) * s3 - M(2, 1) * s1 + M(2, 2) * s0) * id;
  memcpy(out, r, sizeof(r));
}

void mat4_transpose(const float* a, float* out) {
  float r[16];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) r[4 * i + j] = a[4 * j + i];
  memcpy(out, r, sizeof(r));
}

void affine(const float* m, const float* p, float* out) {
  float x = p[0], y = p[1], z = p[2];
  out[0] = m[0] * x + m[1] * y + m[2] * z + m[3];
  out[1] = m[4] * x + m[5] * y + m[6] * z + m[7];
  out[2] = m[8] * x + m[9] * y + m[10] * z + m[11];
}

void normalized(const float* v, float* out) {
  float l = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  out[0] = v[0] / l;
  out[1] = v[1] / l;
  out[2] = v[2] / l;
}

static void set16(float* o, const float (&m)[16]) { memcpy(o, m, sizeof(m)); }

}  // namespace mrg

using namespace mrg;

extern "C" {

MR_API void mr_mat4_mul(const float* a, const float* b, float* out) { mat4_mul(a, b, out); }
MR_API void mr_mat4_inverse(const float* a, float* out) { mat4_inverse(a, out); }

// src/Renderer.cpp:40-47
MR_API void mr_projection_ortho(float l, float r, float b, float t, float n, float f, float* out) {
  float m[16] = {2 / (r - l), 0, 0, -(r + l) / (r - l),
                 0, 2 / (t - b), 0, -(t + b) / (t - b),
                 0, 0, -2 / (f - n), -(f + n) / (f - n),
                 0, 0, 0, 1};
  set16(out, m);
}

// src/Renderer.cpp:49-56
MR_API void mr_projection_perspective(float l, float r, float b, float t, float n, float f,
                                      float* out) {
  float m[16] = {2 * n / (r - l), 0, (r + l) / (r - l), 0,
                 0, 2 * n / (t - b), (t + b) / (t - b), 0,
                 0, 0, -(f + n) / (f - n), -2 * f * n / (f - n),
                 0, 0, -1, 0};
  set16(out, m);
}

// src/Renderer.cpp:68-72
MR_API void mr_projection_frustum(float fov, float aspect, float n, float f, float* out) {
  float t = tanf(fov / 2);
  mr_projection_perspective(-n * t * aspect, n * t * aspect, -n * t, n * t, n, f, out);
}

// src/Renderer.cpp:74-78
MR_API void mr_projection_frustum_h(float fov, float aspect, float n, float f, float* out) {
  float t = tanf(fov / 2);
  mr_projection_perspective(-n * t, n * t, -n * t / aspect, n * t / aspect, n, f, out);
}

// src/Renderer.cpp:80-83
MR_API void mr_projection_ortho_fov(float fov, float aspect, float n, float f, float* out) {
  mr_projection_ortho(-fov * aspect / 2, fov * aspect / 2, -fov / 2, fov / 2, n, f, out);
}

// src/Renderer.cpp:58-66
MR_API void mr_projection_cv(const float* K, float w, float h, float n, float f, float* out) {
  float m[16] = {K[0] * 2 / w, K[1] * 2 / w, -2 * K[2] / w + 1, 0,
                 K[4] * 2 / h, K[5] * 2 / h, 2 * K[6] / h - 1, 0,
                 0, 0, -(f + n) / (f - n), -2 * f * n / (f - n),
                 0, 0, -1, 0};
  set16(out, m);
}

// Scene::collectShapes / TriMesh::collectShapes, src/Scene.cpp:13-36.
MR_API int mr_collect_shapes(const mr_node* nodes, int32_t n_nodes, mr_renderable* out, int32_t cap,
                             int32_t* n_out) {
  static const float I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  // Material defaults, src/Scene.cpp:65-71.
  static const mr_material def = {{0.7f, 0.7f, 0.9f}, {0.8f, 0.8f, 0.8f}, {0, 0, 0}, 12.0f, -1};
  if (!nodes || !n_out || n_nodes <= 0 || nodes[0].parent != -1 || cap < 0) return MR_E_INVALID;
  std::vector<float> world((size_t)16 * n_nodes);
  int32_t n = 0;
  for (int32_t i = 0; i < n_nodes; i++) {
    const float* parent = I;
    if (i > 0) {
      if (nodes[i].parent < 0 || nodes[i].parent >= i) return MR_E_INVALID;
      parent = &world[(size_t)16 * nodes[i].parent];
    }
    mat4_mul(parent, nodes[i].transform, &world[(size_t)16 * i]);
    if (nodes[i].mesh >= 0) {
      if (n < cap && out) {
        out[n].mesh = nodes[i].mesh;
        out[n].flags = 0;
        memcpy(out[n].transform, &world[(size_t)16 * i], sizeof(float) * 16);
        out[n].material = nodes[i].has_material ? nodes[i].material : def;
      }
      n++;
    }
  }
  *n_out = n;
  return MR_OK;
}

}  // extern "C"
