// Host-side Matrix4/Vec3 arithmetic shared by the C ABI (no device code).
#pragma once
#include "../../include/minirender_gpu.h"

namespace mrg {
void mat4_mul(const float* a, const float* b, float* out);
void mat4_inverse(const float* a, float* out);
void mat4_transpose(const float* a, float* out);
void affine(const float* m, const float* p, float* out);
void normalized(const float* v, float* out);
}  // namespace mrg
