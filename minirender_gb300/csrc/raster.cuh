// Exact-order FP32 device helpers of the GB300 rasterisation path.
// Compiled with -fmad=false, -prec-div=true, -prec-sqrt=true, -ftz=false:
// every float expression below is one IEEE binary32 operation per operator,
// in source order, which is what makes the coverage, depth and winner per
// pixel equal to minirender's CPU Renderer (src/Renderer.cpp:163-309) bit
// for bit.
#pragma once
#include "layout.h"

namespace mrg {

struct V3 { float x, y, z; };
struct V2 { float x, y; };
struct Vtx { V3 pos, nrm; V2 uv; };

__device__ __forceinline__ V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ V2 v2(float x, float y) { V2 r; r.x = x; r.y = y; return r; }
__device__ __forceinline__ V3 add3(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 sub3(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 ks3(float k, V3 v) { return v3(k * v.x, k * v.y, k * v.z); }
__device__ __forceinline__ float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len3(V3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
__device__ __forceinline__ V3 normalized3(V3 a) { float l = len3(a); return v3(a.x / l, a.y / l, a.z / l); }
__device__ __forceinline__ V2 add2(V2 a, V2 b) { return v2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ V2 ks2(float k, V2 v) { return v2(k * v.x, k * v.y); }
__device__ __forceinline__ float minr(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float maxr(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float clampr(float x, float lo, float hi) { return (x < lo) ? lo : ((x > hi) ? hi : x); }

// 1/x correctly rounded (IEEE round-to-nearest reciprocal): the same value
// as the division 1.0f/x, at the cost of a reciprocal.  Also -1/x == -(1/x)
// exactly, since IEEE division rounds the magnitude independently of signs.
__device__ __forceinline__ float rcp(float x) { return __frcp_rn(x); }

// Matrix4 * Vec3 with the affine rows of a row-major matrix.
__device__ __forceinline__ V3 affine(const float* m, V3 p) {
  return v3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3],
            m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
            m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
}

// Order-preserving map of a non-NaN float to u32 (-0 and +0 map alike,
// because the reference's strict z < depth treats them as equal).
__device__ __forceinline__ uint32_t depth_key(float z) {
  uint32_t b = __float_as_uint(z);
  if ((b << 1) == 0) b = 0;
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

}  // namespace mrg
