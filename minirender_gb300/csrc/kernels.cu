// GB300 (sm_103a) kernels of the rasterisation path.
//
// One frame per call (launch_frame):
//   k_clear        vis[] = VIS_EMPTY                 (Renderer::clear, src/Renderer.cpp:113-119)
//   k_vertex       per-vertex view transform + projection to pixel space and
//                  per-normal transform, once per frame (the PREMULT loops,
//                  src/Renderer.cpp:344-348, plus htransform :13-20 and the
//                  pixel mapping :193-197, which depend on the vertex only)
//   k_setup        triangle assembly + near clip + triangle setup + cull;
//                  small triangles rasterised by the warp that set them up,
//                  one (triangle, row) per lane; large ones appended to a
//                  warp-compacted record list with their row blocks
//                                                   (src/Renderer.cpp:121-269, 351-379)
//   k_raster_large one warp per row block of a large sub-triangle (the setup
//                  kernel lists the blocks), each row walked across the whole
//                  bounding box with 64-bit atomicMin (src/Renderer.cpp:238-269)
//   k_resolve      deferred pass: re-derives the winning sub-triangle's
//                  barycentrics exactly, shades once per visible pixel and
//                  writes RGB8/depth/ids            (src/Renderer.cpp:271-305, src/io.cpp:358-362)
// Many frames per call (launch_batch):
//   k_vertex (when vertices are shared), a clear of the batch's visibility
//   words (when small triangles are rasterised in the setup), then
//   k_setup_batch (sub-triangles with a bounding box of at most small_max
//   pixels rasterised into their scene's visibility words, larger ones
//   become records counted into the scene's tiles), then k_batch: one
//   cooperative, persistent launch -- scan, scatter, and a dynamically
//   scheduled loop over all tiles of all scenes that rasterises each tile's
//   records into shared memory (seeded with the small triangles' words),
//   captures the winners' edge values and resolves + shades its pixels in
//   place.  The PRE template flag is false for triangle soups: no vertex
//   pass, kernels transform corners themselves.
// Also: k_validate (index checks at upload), k_range (getRangeImage,
// src/Renderer.cpp:388-415).
//
// Exactness: every float operation follows the reference's order; the edge
// functions are advanced column by column from the bounding-box edge exactly
// as the reference loop does (the running sums have no closed form), so every
// rasteriser and the resolve replay that chain.  Values the vertex pass stores
// are the same expressions the reference evaluates per triangle corner.
// Kernels templated on PRE read the vertex-pass buffers; without them
// (allocation-free entry point) vertices are transformed per triangle.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>
#include <utility>

#include "raster.cuh"

namespace cg = cooperative_groups;

namespace mrg {

// ------------------------------------------------------------------ helpers
// Programmatic dependent launch (sm_90+): a kernel launched with programmatic
// stream serialisation may be scheduled while its predecessor is finishing;
// pdl_wait() blocks until the predecessor grid has completed and its writes
// are visible (a no-op for a kernel launched the ordinary way); pdl_trigger()
// lets the successor's blocks start launching.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;"); }
// 8-byte global-to-shared copy that bypasses registers (cp.async); the
// thread's copies are complete after cp_async_wait_all().
__device__ __forceinline__ void cp_async8(void* smem_dst, const void* gsrc) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ int find_base(const uint32_t* base, int lo, int hi, uint32_t g) {
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (base[mid] <= g) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ V3 ld3(const float* p, int i) {
  return v3(__ldg(p + 3 * i), __ldg(p + 3 * i + 1), __ldg(p + 3 * i + 2));
}
__device__ __forceinline__ V2 ld2(const float* p, int i) {
  return v2(__ldg(p + 2 * i), __ldg(p + 2 * i + 1));
}

// htransform, src/Renderer.cpp:13-20
__device__ __forceinline__ V3 htransform(const float* m, V3 p) {
  float iw = rcp(m[12] * p.x + m[13] * p.y + m[14] * p.z + m[15]);
  return v3((m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3]) * iw,
            (m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7]) * iw,
            (m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]) * iw);
}

// Pixel coordinates and depth term of one corner, src/Renderer.cpp:186-197, 223-224.
__device__ __forceinline__ void project(const View& V, V3 v, float& px, float& py, float& zt) {
  V3 ndc = htransform(V.P, v);
  px = (1 + ndc.x) * (V.w / 2);
  py = (1 - ndc.y) * (V.h / 2);
  zt = V.persp ? -rcp(v.z) : ndc.z;
}

// clip(), src/Renderer.cpp:121-129
template <bool ATTR>
__device__ __forceinline__ Vtx clip_vtx(float z, const Vtx& a, const Vtx& b) {
  float k = (fabsf(b.pos.z - a.pos.z) < 1e-6f) ? 0.5f : (z - a.pos.z) / (b.pos.z - a.pos.z);
  float k1 = 1 - k;
  Vtx v;
  v.pos = add3(ks3(k, b.pos), ks3(k1, a.pos));
  if (ATTR) {
    v.nrm = add3(ks3(k, b.nrm), ks3(k1, a.nrm));
    v.uv = add2(ks2(k, b.uv), ks2(k1, a.uv));
  }
  return v;
}

// clipTriangle, src/Renderer.cpp:131-161, for a triangle with at least one
// corner in front of the near plane.  Returns 0, 1 or 2 sub-triangles.
template <bool ATTR>
__device__ __forceinline__ int clip_tri(float zn, Vtx (&v)[3], Vtx (&sub)[2][3]) {
  if (v[0].pos.z > zn && v[1].pos.z > zn && v[2].pos.z > zn) return 0;
  // rotate until v[0] has the largest z (at most two turns for any input)
  for (int it = 0; it < 3 && (v[0].pos.z < v[1].pos.z || v[0].pos.z < v[2].pos.z); it++) {
    Vtx t0 = v[0]; v[0] = v[2]; v[2] = v[1]; v[1] = t0;
  }
  if (v[1].pos.z > zn) {
    sub[0][0] = clip_vtx<ATTR>(zn, v[0], v[2]);
    sub[0][1] = clip_vtx<ATTR>(zn, v[1], v[2]);
    sub[0][2] = v[2];
    return 1;
  }
  if (v[2].pos.z > zn) {
    sub[0][0] = clip_vtx<ATTR>(zn, v[0], v[1]);
    sub[0][1] = v[1];
    sub[0][2] = clip_vtx<ATTR>(zn, v[1], v[2]);
    return 1;
  }
  Vtx v01 = clip_vtx<ATTR>(zn, v[0], v[1]);
  Vtx v02 = clip_vtx<ATTR>(zn, v[0], v[2]);
  sub[0][0] = v01; sub[0][1] = v[1]; sub[0][2] = v[2];
  sub[1][0] = v01; sub[1][1] = v[2]; sub[1][2] = v02;
  return 2;
}

// Sub-triangle s (0 or 1) of clipTriangle's output for a triangle that
// crosses the near plane and has that sub-triangle, computed in place in v:
// the same operations as clip_tri, without materialising both halves.
template <bool ATTR>
__device__ __forceinline__ void clip_pick(float zn, Vtx (&v)[3], int s) {
  for (int it = 0; it < 3 && (v[0].pos.z < v[1].pos.z || v[0].pos.z < v[2].pos.z); it++) {
    Vtx t0 = v[0]; v[0] = v[2]; v[2] = v[1]; v[1] = t0;
  }
  if (v[1].pos.z > zn) {
    const Vtx a = clip_vtx<ATTR>(zn, v[0], v[2]);
    v[1] = clip_vtx<ATTR>(zn, v[1], v[2]);
    v[0] = a;
    return;
  }
  if (v[2].pos.z > zn) {
    const Vtx a = clip_vtx<ATTR>(zn, v[0], v[1]);
    v[2] = clip_vtx<ATTR>(zn, v[1], v[2]);
    v[0] = a;
    return;
  }
  const Vtx v01 = clip_vtx<ATTR>(zn, v[0], v[1]);
  if (s) {  // (v01, v2, v02)
    const Vtx v02 = clip_vtx<ATTR>(zn, v[0], v[2]);
    v[1] = v[2];
    v[2] = v02;
  }
  v[0] = v01;
}

// View-space corners of triangle t (paintMesh, src/Renderer.cpp:344-379).
template <bool PRE, bool ATTR>
__device__ __forceinline__ void corners(const Geo& G, const DevRenderable& R, int t, const int (&ip)[3],
                                        Vtx (&v)[3]) {
  const DevMesh& M = R.mesh;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    if (PRE) {
      float4 a = G.va[R.vert_base + ip[c]];
      float2 b = G.vb[R.vert_base + ip[c]];
      v[c].pos = v3(b.x, b.y, a.w);
    } else {
      v[c].pos = affine(R.mv, ld3(M.pos, ip[c]));
    }
    if (ATTR) {
      // normalsI / texcoordsI shared with the indices: reuse the corner's index
      // (PRE only: without the vertex pass the extra live registers spill,
      // and the shared words are L1-hot anyway)
      const int in = (PRE && M.nidx == M.idx) ? ip[c] : __ldg(M.nidx + 3 * t + c);
      if (PRE) {
        float4 n = G.vn[R.nrm_base + in];
        v[c].nrm = v3(n.x, n.y, n.z);
      } else {
        v[c].nrm = affine(R.nm, ld3(M.nrm, in));
      }
      v[c].uv = M.has_uv ? ld2(M.uv, (PRE && M.tidx == M.idx) ? ip[c] : __ldg(M.tidx + 3 * t + c)) : v2(0, 0);
    }
  }
}

// Corner record of a triangle (32 words, 128 bytes; DevMesh::rec):
//   words 0-8   corner positions p0, p1, p2
//   word 15     layout flag: kRecPerFace or 0
// per-face layout (one normal index and one texcoord index for all three
// corners, as in a soup with face normals: everything in the first 64 bytes)
//   words 9-11  the normal, 12-13 the texcoord, 14 zero
// per-corner layout
//   words 9-11  n0, 12-14 n1, 16-18 n2, 19-24 uv0, uv1, uv2
// Texcoords are zero for meshes without them.
constexpr uint32_t kRecPerFace = 1u;

// The view-space corners with attributes of triangle t from its corner
// record: the same values corners<false, true> gathers (src/Renderer.cpp:
// 344-348, 356-373).  A per-face record needs its first 64 bytes only.
__device__ __forceinline__ void corners_rec(const DevRenderable& R, int t, Vtx (&v)[3]) {
  const float4* r = R.mesh.rec + (size_t)8 * t;
  const float4 q0 = __ldg(r), q1 = __ldg(r + 1), q2 = __ldg(r + 2), q3 = __ldg(r + 3);
  v[0].pos = affine(R.mv, v3(q0.x, q0.y, q0.z));
  v[1].pos = affine(R.mv, v3(q0.w, q1.x, q1.y));
  v[2].pos = affine(R.mv, v3(q1.z, q1.w, q2.x));
  const V3 n0 = v3(q2.y, q2.z, q2.w);
  if (__float_as_uint(q3.w) == kRecPerFace) {
    const V3 n = affine(R.nm, n0);
    const V2 uv = R.mesh.has_uv ? v2(q3.x, q3.y) : v2(0, 0);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      v[c].nrm = n;
      v[c].uv = uv;
    }
  } else {
    const float4 q4 = __ldg(r + 4), q5 = __ldg(r + 5), q6 = __ldg(r + 6);
    v[0].nrm = affine(R.nm, n0);
    v[1].nrm = affine(R.nm, v3(q3.x, q3.y, q3.z));
    v[2].nrm = affine(R.nm, v3(q4.x, q4.y, q4.z));
    if (R.mesh.has_uv) {
      v[0].uv = v2(q4.w, q5.x);
      v[1].uv = v2(q5.y, q5.z);
      v[2].uv = v2(q5.w, q6.x);
    } else {
      v[0].uv = v[1].uv = v[2].uv = v2(0, 0);
    }
  }
}

struct Setup {
  V2 p0, p2, n1, n2;
  float z[3];
  int x0, y0, x1, y1;
};

// paintTriangle setup from projected corners, src/Renderer.cpp:198-224.
// False = nothing to draw (off screen or culled).
__device__ __forceinline__ bool setup_from(const View& V, const V2 (&p)[3], const float (&zt)[3], Setup& S) {
  V2 pmin = v2(1e30f, 1e30f), pmax = v2(-1e30f, -1e30f);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    pmin = v2(minr(pmin.x, p[i].x), minr(pmin.y, p[i].y));
    pmax = v2(maxr(pmax.x, p[i].x), maxr(pmax.y, p[i].y));
  }
  if (pmax.x < 0 || pmax.y < 0 || pmin.x > V.w || pmin.y > V.h) return false;
  float d0x = p[0].x - p[1].x, d0y = p[0].y - p[1].y;
  float d2x = p[2].x - p[1].x, d2y = p[2].y - p[1].y;
  float a = d0x * d2y - d0y * d2x;
  if (a <= 0) return false;  // back-face cull, :207-210
  float i2a = (a == 0) ? 0.0f : -rcp(a);
  float ex = p[0].x - p[2].x, ey = p[0].y - p[2].y;
  S.n1 = v2(-ey * i2a, ex * i2a);
  ex = p[1].x - p[0].x;
  ey = p[1].y - p[0].y;
  S.n2 = v2(-ey * i2a, ex * i2a);
  pmin.x = clampr(pmin.x, 0.f, V.w - 1);
  pmax.x = clampr(pmax.x, 0.f, V.w - 1);
  pmin.y = clampr(pmin.y, 0.f, V.h - 1);
  pmax.y = clampr(pmax.y, 0.f, V.h - 1);
  S.x0 = (int)floorf(pmin.x);
  S.y0 = (int)floorf(pmin.y);
  S.x1 = (int)floorf(pmax.x);
  S.y1 = (int)floorf(pmax.y);
  S.p0 = p[0];
  S.p2 = p[2];
  S.z[0] = zt[0];
  S.z[1] = zt[1];
  S.z[2] = zt[2];
  return true;
}

// Setup of a sub-triangle given by view-space corners (the clipped path).
__device__ __forceinline__ bool setup_view(const View& V, const Vtx (&s)[3], Setup& S) {
  V2 p[3];
  float zt[3];
#pragma unroll
  for (int i = 0; i < 3; i++) project(V, s[i].pos, p[i].x, p[i].y, zt[i]);
  return setup_from(V, p, zt, S);
}

// Edge functions at the start of row y (pixel centre x0+0.5), :240-242.
__device__ __forceinline__ void row_start(const Setup& S, int y, float& e1, float& e2) {
  float yf = (float)y + 0.5f;
  float ptx = (float)S.x0 + 0.5f;
  float qx = ptx - S.p2.x, qy = yf - S.p2.y;
  e1 = S.n1.x * qx + S.n1.y * qy;
  qx = ptx - S.p0.x;
  qy = yf - S.p0.y;
  e2 = S.n2.x * qx + S.n2.y * qy;
}

// Depth of a covered fragment and its perspective-corrected weights, :247-261.
__device__ __forceinline__ float frag_depth(const Setup& S, bool persp, float e1, float e2,
                                            float& k0, float& k1, float& k2) {
  k0 = 1.f - e1 - e2;
  k1 = e1;
  k2 = e2;
  if (persp) {
    float z = rcp(k0 * S.z[0] + k1 * S.z[1] + k2 * S.z[2]);
    k0 *= S.z[0] * z;
    k1 *= S.z[1] * z;
    k2 *= S.z[2] * z;
    return z;
  }
  return k0 * S.z[0] + k1 * S.z[1] + k2 * S.z[2] + 0.0f * 1.0f;
}

__device__ __forceinline__ bool covered(float e1, float e2) {
  return !(e1 < 0 || e2 < 0 || 1 - e1 - e2 < 0);
}

// Walks columns xs..xe of row y (replaying the running sums from x0) and
// calls emit(x, packed, e1, e2) for every fragment that would pass z < 1e11f
// (e1, e2: the running edge values at column x).
template <typename Emit>
__device__ __forceinline__ void walk_row(const Setup& S, bool persp, uint32_t id, int y, int xs,
                                         int xe, Emit emit) {
  float e1, e2;
  row_start(S, y, e1, e2);
  const float d1 = S.n1.x, d2 = S.n2.x;
  for (int x = S.x0; x < xs; x++) {
    e1 += d1;
    e2 += d2;
  }
  for (int x = xs; x <= xe; x++) {
    if (covered(e1, e2)) {
      float k0, k1, k2;
      float z = frag_depth(S, persp, e1, e2, k0, k1, k2);
      if (z < 1e11f) emit(x, ((unsigned long long)depth_key(z) << 32) | id, e1, e2);
    }
    e1 += d1;
    e2 += d2;
  }
}

// Per-block statistics: warps add into shared counters, one global atomic per
// counter and block (a single global address updated by every warp would
// serialise in L2).  Every thread of the block must call block_flush.
struct BlockCounters {
  unsigned v[3];
};
__device__ __forceinline__ void block_count(BlockCounters& bc, int k, unsigned v) {
  unsigned s = __reduce_add_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(&bc.v[k], s);
}
__device__ __forceinline__ void block_flush(BlockCounters& bc, unsigned long long* d0, unsigned long long* d1,
                                            unsigned long long* d2) {
  __syncthreads();
  if (threadIdx.x == 0) {
    if (bc.v[0]) atomicAdd(d0, (unsigned long long)bc.v[0]);
    if (bc.v[1] && d1) atomicAdd(d1, (unsigned long long)bc.v[1]);
    if (bc.v[2]) atomicAdd(d2, (unsigned long long)bc.v[2]);
  }
}

__device__ __forceinline__ BigRec to_rec(const Setup& S, uint32_t id) {
  BigRec B;
  B.p0x = S.p0.x; B.p0y = S.p0.y; B.p2x = S.p2.x; B.p2y = S.p2.y;
  B.n1x = S.n1.x; B.n1y = S.n1.y; B.n2x = S.n2.x; B.n2y = S.n2.y;
  B.z0 = S.z[0]; B.z1 = S.z[1]; B.z2 = S.z[2];
  B.id = id;
  B.x0 = S.x0; B.y0 = S.y0; B.x1 = S.x1; B.y1 = S.y1;
  return B;
}

__device__ __forceinline__ Setup rec_setup(const BigRec& B) {
  Setup S;
  S.p0 = v2(B.p0x, B.p0y); S.p2 = v2(B.p2x, B.p2y);
  S.n1 = v2(B.n1x, B.n1y); S.n2 = v2(B.n2x, B.n2y);
  S.z[0] = B.z0; S.z[1] = B.z1; S.z[2] = B.z2;
  S.x0 = B.x0; S.y0 = B.y0; S.x1 = B.x1; S.y1 = B.y1;
  return S;
}

// Assembly, near clip and setup of global triangle g (paintMesh + the first
// half of paintTriangle).  Fills up to two setups in draw order; kind[s] = 1
// for a sub-triangle with pixels to test.  Returns false for a triangle whose
// indices failed the upload check.
template <bool PRE>
__device__ __forceinline__ bool setup_triangle(const View& V, const Geo& G, const DevRenderable& R,
                                               uint32_t g, Setup (&S)[2], int (&kind)[2],
                                               unsigned& n_clipped) {
  const int t = (int)(g - R.tri_base);
  if ((R.mesh.bad[t >> 5] >> (t & 31)) & 1u) return false;
  int ip[3];
#pragma unroll
  for (int c = 0; c < 3; c++) ip[c] = __ldg(R.mesh.idx + 3 * t + c);
  // no_clip (paintTriangle(..., world=false)): never clipped, so the near
  // test compares against +inf
  const float zn = R.no_clip ? __int_as_float(0x7f800000) : V.znear;
  if (PRE) {
    float4 a[3];
#pragma unroll
    for (int c = 0; c < 3; c++) a[c] = G.va[R.vert_base + ip[c]];
    if (!(a[0].w > zn || a[1].w > zn || a[2].w > zn)) {
      V2 p[3] = {v2(a[0].x, a[0].y), v2(a[1].x, a[1].y), v2(a[2].x, a[2].y)};
      float zt[3] = {a[0].z, a[1].z, a[2].z};
      if (setup_from(V, p, zt, S[0])) kind[0] = 1;
      return true;
    }
  }
  Vtx v[3], sub[2][3];
  corners<PRE, false>(G, R, t, ip, v);
  int n;
  if (!(v[0].pos.z > zn || v[1].pos.z > zn || v[2].pos.z > zn)) {
    sub[0][0] = v[0]; sub[0][1] = v[1]; sub[0][2] = v[2];
    n = 1;
  } else {
    n = clip_tri<false>(zn, v, sub);
    n_clipped += n > 0;
  }
  for (int s = 0; s < n; s++)
    if (setup_view(V, sub[s], S[s])) kind[s] = 1;
  return true;
}

// The sub-triangle `id` won by a pixel: its renderable, vertex indices and
// view-space corners with attributes (the clipped sub-triangle when the
// triangle crosses the near plane), src/Renderer.cpp:334-379, 131-161.
// Renderables of the pixel's frame are rs_lo..rs_hi-1.
// s_tb, when given, holds tri_base[rs_lo .. rs_hi) in shared memory.
template <bool PRE>
__device__ __forceinline__ const DevRenderable* winner_tri(const View& V, const Geo& G, int rs_lo, int rs_hi,
                                                         uint32_t id, int (&ip)[3], Vtx (&vc)[3],
                                                         bool& clipped, const uint32_t* s_tb = nullptr) {
  const uint32_t g = id >> 1;
  const int s = (int)(id & 1u);
  const int k = s_tb ? rs_lo + find_base(s_tb, 0, rs_hi - rs_lo, g) : find_base(G.tri_base, rs_lo, rs_hi, g);
  const DevRenderable* R = &G.rs[k];
  const int t = (int)(g - R->tri_base);
  if (!PRE && R->mesh.rec) {
    corners_rec(*R, t, vc);  // (ip is not used without the vertex pass)
  } else {
#pragma unroll
    for (int c = 0; c < 3; c++) ip[c] = __ldg(R->mesh.idx + 3 * t + c);
    corners<PRE, true>(G, *R, t, ip, vc);
  }
  const float zn = R->no_clip ? __int_as_float(0x7f800000) : V.znear;
  clipped = vc[0].pos.z > zn || vc[1].pos.z > zn || vc[2].pos.z > zn;
  if (clipped) clip_pick<true>(zn, vc, s);  // sub-triangle s exists: it won this pixel
  return R;
}

// Texture and Blinn-Phong lighting of a fragment with perspective-corrected
// weights k0..k2 over the corners vc, src/Renderer.cpp:262-305 (FAST_LIGHT).
__device__ __forceinline__ void shade(const View& V, const DevRenderable& R, const Vtx (&vc)[3], float k0,
                                      float k1, float k2, const float* s_dec, V3& value, V3& normal_out) {
  V3 color = v3(R.diffuse[0], R.diffuse[1], R.diffuse[2]);
  if (R.has_tex) {
    V2 uv = add2(add2(ks2(k0, vc[0].uv), ks2(k1, vc[1].uv)), ks2(k2, vc[2].uv));
    int ti = (int)((uv.y - floorf(uv.y)) * (float)R.tex_rows);
    int tj = (int)((uv.x - floorf(uv.x)) * (float)R.tex_cols);
    ti = min(max(ti, 0), R.tex_rows - 1);
    tj = min(max(tj, 0), R.tex_cols - 1);
    size_t o = 3 * ((size_t)ti * R.tex_cols + tj);
    if (R.tex8)
      color = v3(s_dec[R.tex8[o]], s_dec[R.tex8[o + 1]], s_dec[R.tex8[o + 2]]);
    else
      color = v3(R.texf[o], R.texf[o + 1], R.texf[o + 2]);
  }
  value = v3(R.emissive[0], R.emissive[1], R.emissive[2]);
  if (R.lit) {
    V3 position = add3(add3(ks3(k0, vc[0].pos), ks3(k1, vc[1].pos)), ks3(k2, vc[2].pos));
    V3 LD = v3(V.lightdir[0], V.lightdir[1], V.lightdir[2]);
    V3 lightdir = R.point ? normalized3(sub3(LD, position)) : LD;
    V3 normal = add3(add3(ks3(k0, vc[0].nrm), ks3(k1, vc[1].nrm)), ks3(k2, vc[2].nrm));
    float sdiff = maxr(0.0f, dot3(normal, lightdir)) / len3(normal) + V.ambient;
    value = add3(value, ks3(sdiff, color));
    if (R.shininess != 0) {
      V3 viewDir = normalized3(position);
      V3 lv = sub3(lightdir, viewDir);
      float spec = powf(maxr(dot3(lv, normal), 0.0f) / (len3(lv) * len3(normal)), R.shininess);
      value = add3(value, ks3(spec, v3(R.specular[0], R.specular[1], R.specular[2])));
    }
    normal_out = normal;
  }
}

// The setup (src/Renderer.cpp:198-224) of the winning sub-triangle, the same
// values its raster used.
template <bool PRE>
__device__ __forceinline__ void winner_setup(const View& V, const Geo& G, const DevRenderable& R,
                                             const int (&ip)[3], const Vtx (&vc)[3], bool clipped, Setup& S) {
  if (PRE && !clipped) {
    V2 p[3];
    float zt[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      float4 a = G.va[R.vert_base + ip[c]];
      p[c] = v2(a.x, a.y);
      zt[c] = a.z;
    }
    setup_from(V, p, zt, S);
  } else {
    setup_view(V, vc, S);
  }
}

// The running edge values at pixel (x, y): row start, then column by column
// from the bounding-box edge (src/Renderer.cpp:240-243).
__device__ __forceinline__ void replay(const Setup& S, int x, int y, float& e1, float& e2) {
  row_start(S, y, e1, e2);
  for (int c = S.x0; c < x; c++) {
    e1 += S.n1.x;
    e2 += S.n2.x;
  }
}

// Shading of the pixel (x, y) whose visibility word is vw, src/Renderer.cpp:
// 247-305 (FAST_LIGHT): re-derives the winner's setup, replays its edge
// functions to column x, and evaluates texture and Blinn-Phong lighting.
// Renderables of the pixel's frame are rs_lo..rs_hi-1.
template <bool PRE>
__device__ __forceinline__ void resolve_pixel(const View& V, const Geo& G, int rs_lo, int rs_hi,
                                              unsigned long long vw, int x, int y, const float* s_dec,
                                              V3& value, float& depth, uint32_t& id, V3& normal_out) {
  normal_out = v3(0, 0, 1);
  if (vw == VIS_EMPTY) {
    value = v3(V.bg[0], V.bg[1], V.bg[2]);
    depth = 1e11f;
    id = MR_NO_TRIANGLE;
    return;
  }
  id = (uint32_t)vw;
  int ip[3];
  Vtx vc[3];
  bool clipped;
  const DevRenderable& R = *winner_tri<PRE>(V, G, rs_lo, rs_hi, id, ip, vc, clipped);
  Setup S;
  winner_setup<PRE>(V, G, R, ip, vc, clipped, S);
  float e1, e2;
  replay(S, x, y, e1, e2);
  float k0, k1, k2;
  depth = frag_depth(S, V.persp != 0, e1, e2, k0, k1, k2);
  shade(V, R, vc, k0, k1, k2, s_dec, value, normal_out);
}

// savePPM conversion, src/io.cpp:358-362.
__device__ __forceinline__ uint8_t to_byte(float v) { return (uint8_t)(int)clampr(v * 255.0f, 0.0f, 255.0f); }

// ------------------------------------------------------------------ kernels
// vis[0..n) = VIS_EMPTY; also zeroes z[0..nz) (a frame's counters and tile
// tables, so they need no separate memset before the frame).
// With src, also copies n16 16-byte units from src (mapped pinned host
// memory: the frame's staging block) to dst, so a frame never queues behind
// other streams' transfers on the copy engine.
__global__ void k_clear(unsigned long long* vis, size_t n, uint32_t* z0, uint32_t nz0, uint32_t* z1, uint32_t nz1,
                        const uint4* src, uint4* dst, uint32_t n16) {
  pdl_trigger();
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t k = i; k < n16; k += stride) dst[k] = src[k];
  for (size_t k = i; k < nz0; k += stride) z0[k] = 0;
  for (size_t k = i; k < nz1; k += stride) z1[k] = 0;
  for (; i < n; i += stride) vis[i] = VIS_EMPTY;
}

// Index check of a mesh upload (one bit per triangle), and for meshes with
// corner records the gather of each valid triangle's corner attributes.
__global__ void k_validate(DevMesh M, uint32_t* bad, float4* rec) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  bool b = false;
  int ip[3] = {0, 0, 0}, in[3] = {0, 0, 0}, it[3] = {0, 0, 0};
  if (t < M.n_tri) {
    for (int c = 0; c < 3; c++) {
      ip[c] = M.idx[3 * t + c];
      in[c] = M.nidx[3 * t + c];
      b |= ip[c] < 0 || ip[c] >= M.n_pos || in[c] < 0 || in[c] >= M.n_nrm;
      if (M.has_uv) {
        it[c] = M.tidx[3 * t + c];
        b |= it[c] < 0 || it[c] >= M.n_uv;
      }
    }
  }
  unsigned m = __ballot_sync(0xffffffffu, b);
  if ((threadIdx.x & 31) == 0 && (t >> 5) < ((M.n_tri + 31) >> 5)) bad[t >> 5] = m;
  if (rec && t < M.n_tri && !b) {
    // the layout of corners_rec
    float f[28];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      f[3 * c + 0] = M.pos[3 * ip[c] + 0];
      f[3 * c + 1] = M.pos[3 * ip[c] + 1];
      f[3 * c + 2] = M.pos[3 * ip[c] + 2];
    }
    const bool per_face = in[0] == in[1] && in[1] == in[2] && it[0] == it[1] && it[1] == it[2];
    float4* r = rec + (size_t)8 * t;
    if (per_face) {
      f[9] = M.nrm[3 * in[0] + 0];
      f[10] = M.nrm[3 * in[0] + 1];
      f[11] = M.nrm[3 * in[0] + 2];
      f[12] = M.has_uv ? M.uv[2 * it[0] + 0] : 0.f;
      f[13] = M.has_uv ? M.uv[2 * it[0] + 1] : 0.f;
      f[14] = 0.f;
      f[15] = __uint_as_float(kRecPerFace);
#pragma unroll
      for (int k = 0; k < 4; k++) r[k] = make_float4(f[4 * k], f[4 * k + 1], f[4 * k + 2], f[4 * k + 3]);
    } else {
      const int nw[3] = {9, 12, 16}, uw[3] = {19, 21, 23};
#pragma unroll
      for (int c = 0; c < 3; c++) {
        f[nw[c] + 0] = M.nrm[3 * in[c] + 0];
        f[nw[c] + 1] = M.nrm[3 * in[c] + 1];
        f[nw[c] + 2] = M.nrm[3 * in[c] + 2];
        f[uw[c] + 0] = M.has_uv ? M.uv[2 * it[c] + 0] : 0.f;
        f[uw[c] + 1] = M.has_uv ? M.uv[2 * it[c] + 1] : 0.f;
      }
      f[15] = 0.f;
      f[25] = f[26] = f[27] = 0.f;
#pragma unroll
      for (int k = 0; k < 7; k++) r[k] = make_float4(f[4 * k], f[4 * k + 1], f[4 * k + 2], f[4 * k + 3]);
    }
  }
}

// Vertex pass: threads [0, n_verts) transform and project positions,
// threads [n_verts, n_verts + n_nrms) transform normals.  The view of a
// vertex is scenes[R.scene].v for batches, V otherwise.
__global__ void __launch_bounds__(256) k_vertex(Geo G, View V, const SceneRec* scenes) {
  pdl_wait();
  pdl_trigger();
  uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < G.n_verts) {
    const DevRenderable& R = G.rs[find_base(G.vert_base, 0, G.n_renderables, g)];
    V3 v = affine(R.mv, ld3(R.mesh.pos, (int)(g - R.vert_base)));
    float px, py, zt;
    project(scenes ? scenes[R.scene].v : V, v, px, py, zt);
    G.va[g] = make_float4(px, py, zt, v.z);
    G.vb[g] = make_float2(v.x, v.y);
  } else if (g - G.n_verts < G.n_nrms) {
    uint32_t gn = g - G.n_verts;
    const DevRenderable& R = G.rs[find_base(G.nrm_base, 0, G.n_renderables, gn)];
    V3 n = affine(R.nm, ld3(R.mesh.nrm, (int)(gn - R.nrm_base)));
    G.vn[gn] = make_float4(n.x, n.y, n.z, 0.f);
  }
}

// Small-triangle records staged in shared memory for the warp's cooperative
// raster, in two layouts: SmallRec (80 bytes, 16-byte aligned, copied with
// vector accesses) and PackedRec (60 bytes: pixel coordinates in 16 bits, an
// odd word stride so lanes touching different records still hit different
// banks), which leaves more of the SM's L1 to a kernel that spills.
struct __align__(16) SmallRec {
  float p0x, p0y, p2x, p2y, n1x, n1y, n2x, n2y, z0, z1, z2;
  uint32_t id;
  int x0, y0, x1, rows;
  uint32_t tag;  // target frame (batches: scene)
};
struct PackedRec {
  float p0x, p0y, p2x, p2y, n1x, n1y, n2x, n2y, z0, z1, z2;
  uint32_t id;
  uint32_t tag;
  uint32_t lo;  // x0 | y0 << 16
  uint32_t hi;  // x1 | rows << 16
};
__device__ __forceinline__ void rec_put(SmallRec& q, const Setup& S, uint32_t id, uint32_t tag) {
  q.p0x = S.p0.x; q.p0y = S.p0.y; q.p2x = S.p2.x; q.p2y = S.p2.y;
  q.n1x = S.n1.x; q.n1y = S.n1.y; q.n2x = S.n2.x; q.n2y = S.n2.y;
  q.z0 = S.z[0]; q.z1 = S.z[1]; q.z2 = S.z[2];
  q.id = id;
  q.x0 = S.x0; q.y0 = S.y0; q.x1 = S.x1;
  q.rows = S.y1 - S.y0 + 1;
  q.tag = tag;
}
__device__ __forceinline__ void rec_put(PackedRec& q, const Setup& S, uint32_t id, uint32_t tag) {
  q.p0x = S.p0.x; q.p0y = S.p0.y; q.p2x = S.p2.x; q.p2y = S.p2.y;
  q.n1x = S.n1.x; q.n1y = S.n1.y; q.n2x = S.n2.x; q.n2y = S.n2.y;
  q.z0 = S.z[0]; q.z1 = S.z[1]; q.z2 = S.z[2];
  q.id = id;
  q.tag = tag;
  // frame coordinates and small boxes' row counts fit 16 bits (sides <= 65536)
  q.lo = (uint32_t)S.x0 | ((uint32_t)S.y0 << 16);
  q.hi = (uint32_t)S.x1 | ((uint32_t)(S.y1 - S.y0 + 1) << 16);
}
__device__ __forceinline__ int rec_rows(const SmallRec& q) { return q.rows; }
__device__ __forceinline__ int rec_rows(const PackedRec& q) { return (int)(q.hi >> 16); }
template <class Rec>
__device__ __forceinline__ Setup rec_get(const Rec& q) {
  Setup U;
  U.p0 = v2(q.p0x, q.p0y); U.p2 = v2(q.p2x, q.p2y);
  U.n1 = v2(q.n1x, q.n1y); U.n2 = v2(q.n2x, q.n2y);
  U.z[0] = q.z0; U.z[1] = q.z1; U.z[2] = q.z2;
  if constexpr (sizeof(Rec) == sizeof(PackedRec)) {
    U.x0 = (int)(q.lo & 0xffffu); U.y0 = (int)(q.lo >> 16); U.x1 = (int)(q.hi & 0xffffu);
  } else {
    U.x0 = q.x0; U.y0 = q.y0; U.x1 = q.x1;
  }
  return U;
}
constexpr int kStageRecs = 32;  // records staged per warp and round

constexpr int kSetupThreads = 256;
constexpr int kSetupWarps = kSetupThreads / 32;

// Where small triangles' fragments go: the frame's visibility buffer...
struct FrameTarget {
  unsigned long long* vis;
  int W;
  bool persp;
  __device__ unsigned long long* row(uint32_t, int y) const { return vis + (size_t)y * W; }
  __device__ bool perspective(uint32_t) const { return persp; }
};
// ...or, in a batch, the visibility buffer of the triangle's scene (tag).
struct BatchTarget {
  const SceneRec* scenes;
  __device__ unsigned long long* row(uint32_t sc, int y) const {
    return scenes[sc].vis + (size_t)y * scenes[sc].v.W;
  }
  __device__ bool perspective(uint32_t sc) const { return scenes[sc].v.persp != 0; }
};

// Raster of a sub-triangle whose bounding box spans at most 4x4 pixels by
// one thread (src/Renderer.cpp:238-269): the row and column loops have
// constant bounds and unroll, so the rows' independent edge evaluations
// interleave (each row still starts from its bounding-box edge and steps
// column by column).  row(y) gives the visibility words of row y.
template <typename RowFn>
__device__ __forceinline__ void raster_tiny(const Setup& Q, bool persp, uint32_t id, RowFn row_of) {
#pragma unroll
  for (int r = 0; r < 4; r++) {
    const int y = Q.y0 + r;
    if (y <= Q.y1) {
      unsigned long long* row = row_of(y);
      float e1, e2;
      row_start(Q, y, e1, e2);
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const int x = Q.x0 + c;
        if (x <= Q.x1 && covered(e1, e2)) {
          float k0, k1, k2;
          const float z = frag_depth(Q, persp, e1, e2, k0, k1, k2);
          if (z < 1e11f) atomicMin(row + x, ((unsigned long long)depth_key(z) << 32) | id);
        }
        e1 += Q.n1.x;
        e2 += Q.n2.x;
      }
    }
  }
}

// Raster of the warp's small sub-triangles (kind 1; ids[s] the id of
// sub-triangle s), whose frame is `tag`, with 64-bit atomicMin into the
// target (src/Renderer.cpp:
// 238-269).  When every one in the warp spans at most 4x4 pixels the lanes
// rasterise their own (the loops are short and nearly uniform); otherwise
// they are staged in shared memory and rasterised with one (triangle, row)
// per lane so every lane has work.  Called by all lanes of the warp.
template <class Target, class Rec>
__device__ __forceinline__ void raster_small(const Setup (&S)[2], const int (&kind)[2], const uint32_t (&ids)[2],
                                             uint32_t tag, const Target& T, Rec* s_rec, int* s_pre) {
  const unsigned lane = threadIdx.x & 31, lt = (1u << lane) - 1u;
  int span = 0;
#pragma unroll
  for (int s = 0; s < 2; s++)
    if (kind[s] == 1) span = max(span, max(S[s].x1 - S[s].x0, S[s].y1 - S[s].y0) + 1);
  if (__reduce_max_sync(0xffffffffu, (unsigned)span) <= 4u) {
#pragma unroll
    for (int s = 0; s < 2; s++)
      if (kind[s] == 1)
        raster_tiny(S[s], T.perspective(tag), ids[s], [&](int y) { return T.row(tag, y); });
    return;
  }
  // one round per sub-triangle slot (at most 32 records; slot 1 holds the
  // second half of near-clipped triangles only)
#pragma unroll
  for (int s = 0; s < 2; s++) {
    const unsigned m = __ballot_sync(0xffffffffu, kind[s] == 1);
    if (m == 0) continue;
    const int n = __popc(m);
    if (kind[s] == 1) rec_put(s_rec[__popc(m & lt)], S[s], ids[s], tag);
    __syncwarp();
    const int c = (int)lane < n ? rec_rows(s_rec[lane]) : 0;
    int inc = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, inc, o);
      if ((int)lane >= o) inc += u;
    }
    const int total = __shfl_sync(0xffffffffu, inc, 31);
    s_pre[lane] = inc - c;
    __syncwarp();
    for (int b = 0; b < total; b += 32) {
      const int k = b + (int)lane;
      if (k < total) {
        int lo = 0;  // the last record lo < n with s_pre[lo] <= k
#pragma unroll
        for (int step = 16; step; step >>= 1)
          if (lo + step < n && s_pre[lo + step] <= k) lo += step;
        const Rec& q = s_rec[lo];
        const Setup U = rec_get(q);
        const int y = U.y0 + (k - s_pre[lo]);
        const uint32_t tg = q.tag;
        unsigned long long* row = T.row(tg, y);
        walk_row(U, T.perspective(tg), q.id, y, U.x0, U.x1,
                 [&](int x, unsigned long long v, float, float) { atomicMin(row + x, v); });
      }
    }
    __syncwarp();  // s_rec / s_pre free for the warp's next use
  }
}

// Blocks per SM the register budget of k_setup must allow.  With the vertex
// pass the kernel waits on index -> vertex gathers and more resident warps
// hide that: 6 blocks (40 registers, some spilled to L1) with the packed
// staging records, which leave more L1 to the spills.  Without it (triangle
// soups) it is bound by instruction issue, spilling costs more than the
// extra warps hide, and the aligned records' vector copies are cheaper: 4
// blocks (64 registers).  Measured on 1080p and 4K frames.
template <bool PRE>
constexpr int kSetupMinBlocks = PRE ? 6 : 4;
template <bool PRE>
__global__ void __launch_bounds__(kSetupThreads, kSetupMinBlocks<PRE>) k_setup(FrameParams F) {
  pdl_wait();
  using Rec = std::conditional_t<PRE, PackedRec, SmallRec>;  // see kSetupMinBlocks
  __shared__ Rec s_rec[kSetupWarps][kStageRecs];
  __shared__ int s_pre[kSetupWarps][kStageRecs];
  __shared__ BlockCounters bc;
  if (threadIdx.x < 3) bc.v[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const bool persp = F.v.persp != 0;
  Setup S[2];
  int kind[2] = {0, 0};  // 0 none, 1 small, 2 big
  unsigned n_clipped = 0, n_raster = 0, n_small = 0;
  if (g < F.g.n_tris) {
    const DevRenderable& R = F.g.rs[find_base(F.g.tri_base, 0, F.g.n_renderables, g)];
    if (!setup_triangle<PRE>(F.v, F.g, R, g, S, kind, n_clipped)) {
      atomicOr(&F.counters->error_flags, 1u);
    } else {
#pragma unroll
      for (int s = 0; s < 2; s++)
        if (kind[s]) {
          n_raster++;
          long long bw = S[s].x1 - S[s].x0 + 1, bh = S[s].y1 - S[s].y0 + 1;
          if (bw * bh <= (long long)F.small_max) n_small++;
          else kind[s] = 2;
        }
    }
  }
  // large records: warp-level compaction, one atomic per warp and slot
#pragma unroll
  for (int s = 0; s < 2; s++) {
    unsigned m = __ballot_sync(0xffffffffu, kind[s] == 2);
    if (m == 0) continue;
    unsigned base = 0;
    if (lane == 0) base = atomicAdd(&F.counters->rec_count, (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    unsigned n_items = 0, slot = 0;
    if (kind[s] == 2) {
      slot = base + __popc(m & lt);
      if (slot < F.rec_cap) {
        F.recs[slot] = to_rec(S[s], 2u * g + (uint32_t)s);
        n_items = (unsigned)(S[s].y1 - S[s].y0 + kLargeRows) / kLargeRows;
      } else {
        kind[s] = 1;  // no record left (a fixed record store): rasterised below
      }
    }
    // its row blocks: one range per warp, each lane's at its exclusive prefix
    unsigned inc = n_items;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned u = __shfl_up_sync(0xffffffffu, inc, o);
      if ((int)lane >= o) inc += u;
    }
    const unsigned total = __shfl_sync(0xffffffffu, inc, 31);
    unsigned ibase = 0;
    if (lane == 0 && total) ibase = atomicAdd(&F.counters->item_count, total);
    ibase = __shfl_sync(0xffffffffu, ibase, 0) + inc - n_items;
    // blocks past the end of the list: the record's remaining rows go to the
    // spill list (at most one entry per record, so it cannot overflow)
    for (unsigned k = 0; k < n_items; k++) {
      const uint32_t row = (uint32_t)(S[s].y0 + (int)k * kLargeRows);
      if (ibase + k < F.item_cap) {
        F.items[ibase + k] = LargeItem{slot, row};
      } else {
        F.spill[atomicAdd(&F.counters->spill_count, 1u)] = LargeItem{slot, row};
        break;
      }
    }
  }
  const uint32_t ids[2] = {2u * g, 2u * g + 1u};
  raster_small(S, kind, ids, 0u, FrameTarget{F.vis, F.v.W, persp}, s_rec[w], s_pre[w]);
  block_count(bc, 0, n_raster);
  block_count(bc, 1, n_small);
  block_count(bc, 2, n_clipped);
  block_flush(bc, &F.counters->rasterised, &F.counters->small_direct, &F.counters->clipped);
}

// Large sub-triangles, one warp per row block of kLargeRows rows of a record,
// one row per lane: each row is walked across the record's whole bounding
// box (no replay beyond the reference's own) with 64-bit atomicMin into
// vis[] (src/Renderer.cpp:238-269).  Then the spill list: one warp per
// record, its remaining rows kLargeRows at a time.  An ordinary launch: with
// no large record every warp leaves at once.
__device__ __forceinline__ void raster_rec_row(const FrameParams& F, bool persp, const BigRec& R, int y) {
  const Setup S = rec_setup(R);
  unsigned long long* row = F.vis + (size_t)y * F.v.W;
  walk_row(S, persp, R.id, y, S.x0, S.x1,
           [&](int x, unsigned long long v, float, float) { atomicMin(row + x, v); });
}

__global__ void __launch_bounds__(256) k_raster_large(FrameParams F) {
  pdl_wait();
  pdl_trigger();
  const uint32_t n = min(F.counters->item_count, F.item_cap);
  const uint32_t n_spill = F.counters->spill_count;
  const bool persp = F.v.persp != 0;
  const int lane = (int)(threadIdx.x & 31);
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  const uint32_t w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  for (uint32_t it = w0; it < n; it += nw) {
    const LargeItem item = F.items[it];
    const BigRec& R = F.recs[item.rec];
    const int y = (int)item.row + lane;
    if (y <= R.y1) raster_rec_row(F, persp, R, y);
  }
  for (uint32_t it = w0; it < n_spill; it += nw) {
    const LargeItem item = F.spill[it];
    const BigRec& R = F.recs[item.rec];
    for (int y = (int)item.row + lane; y <= R.y1; y += kLargeRows) raster_rec_row(F, persp, R, y);
  }
}

// Deferred resolve + shade: one thread per pixel, 256-thread blocks over
// 32x8-pixel tiles.
constexpr int kResolveTileW = 32, kResolveTileH = 8;
template <bool PRE>
__global__ void __launch_bounds__(256, 4) k_resolve(FrameParams F) {
  pdl_wait();
  // loadPPM's texel decode b/255.0f (src/io.cpp:410), one division per byte value
  __shared__ float s_dec[256];
  s_dec[threadIdx.x] = (float)threadIdx.x / 255.0f;
  __syncthreads();
  // 32x8-pixel block tiles, 16x2 per warp: neighbouring rows of a small
  // triangle are shaded by the same warp, so its corner data is fetched once
  const int tiles_x = (F.v.W + kResolveTileW - 1) / kResolveTileW;
  const int bx = blockIdx.x % tiles_x, by = blockIdx.x / tiles_x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int x = bx * kResolveTileW + (lane & 15) + 16 * (w & 1), y = by * kResolveTileH + (lane >> 4) + 2 * (w >> 1);
  if (x >= F.v.W || y >= F.v.H) return;
  const size_t px = (size_t)y * F.v.W + x;
  V3 value, normal;
  float depth;
  uint32_t id;
  resolve_pixel<PRE>(F.v, F.g, 0, F.g.n_renderables, F.vis[px], x, y, s_dec, value, depth, id, normal);
  if (F.rgb8) {
    F.rgb8[3 * px + 0] = to_byte(value.x);
    F.rgb8[3 * px + 1] = to_byte(value.y);
    F.rgb8[3 * px + 2] = to_byte(value.z);
  }
  if (F.depth) F.depth[px] = depth;
  if (F.ids) F.ids[px] = id;
  if (F.rgbf) {
    F.rgbf[3 * px + 0] = value.x;
    F.rgbf[3 * px + 1] = value.y;
    F.rgbf[3 * px + 2] = value.z;
  }
  if (F.normals) {
    F.normals[3 * px + 0] = normal.x;
    F.normals[3 * px + 1] = normal.y;
    F.normals[3 * px + 2] = normal.z;
  }
}

// ---------------------------------------------------------------- batches
// Setup of every triangle of every scene: each sub-triangle with pixels to
// test becomes a record (warp-compacted), counted into its scene's tiles.
// (the register budget and staging layout of k_setup, for the same reasons;
// on the 256-scene batch: 0.665 -> 0.453 ms)
template <bool PRE>
__global__ void __launch_bounds__(kSetupThreads, kSetupMinBlocks<PRE>) k_setup_batch(BatchParams B) {
  using Rec = std::conditional_t<PRE, PackedRec, SmallRec>;
  __shared__ Rec s_rec[kSetupWarps][kStageRecs];
  __shared__ int s_pre[kSetupWarps][kStageRecs];
  __shared__ BlockCounters bc;
  __shared__ unsigned s_fill, s_base;
  if (threadIdx.x < 3) bc.v[threadIdx.x] = 0;
  if (threadIdx.x == 0) s_fill = 0;
  __syncthreads();
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5, lt = (1u << lane) - 1u;
  Setup S[2];
  int kind[2] = {0, 0};  // 0 none, 1 small (rasterised here), 2 record
  unsigned n_clipped = 0, n_raster = 0, n_small = 0;
  uint32_t scene = 0;
  if (g < B.g.n_tris) {
    const DevRenderable& R = B.g.rs[find_base(B.g.tri_base, 0, B.g.n_renderables, g)];
    scene = R.scene;
    if (!setup_triangle<PRE>(B.scenes[scene].v, B.g, R, g, S, kind, n_clipped))
      atomicOr(&B.counters->error_flags, 1u);
#pragma unroll
    for (int s = 0; s < 2; s++)
      if (kind[s]) {
        n_raster++;
        long long bw = S[s].x1 - S[s].x0 + 1, bh = S[s].y1 - S[s].y0 + 1;
        if (bw * bh <= (long long)B.small_max) n_small++;
        else kind[s] = 2;
      }
  }
  // record slots: each warp reserves within the block, the block once globally
  unsigned m2[2], wbase = 0;
#pragma unroll
  for (int s = 0; s < 2; s++) m2[s] = __ballot_sync(0xffffffffu, kind[s] == 2);
  const unsigned wn = __popc(m2[0]) + __popc(m2[1]);
  if (lane == 0 && wn) wbase = atomicAdd(&s_fill, wn);
  wbase = __shfl_sync(0xffffffffu, wbase, 0);
  __syncthreads();
  if (threadIdx.x == 0) s_base = s_fill ? atomicAdd(&B.counters->rec_count, s_fill) : 0;
  __syncthreads();
  unsigned base = s_base + wbase;
#pragma unroll
  for (int s = 0; s < 2; s++) {
    const unsigned m = m2[s];
    if (m == 0) continue;
    if (kind[s] == 2) {
      unsigned slot = base + __popc(m & lt);
      if (slot < B.rec_cap) {
        B.recs[slot] = to_rec(S[s], 2u * g + (uint32_t)s);
        B.rec_scene[slot] = scene;
        const SceneRec& SR = B.scenes[scene];
        int tx0 = S[s].x0 / B.tile_w, tx1 = S[s].x1 / B.tile_w, ty0 = S[s].y0 / B.tile_h, ty1 = S[s].y1 / B.tile_h;
        for (int ty = ty0; ty <= ty1; ty++)
          for (int tx = tx0; tx <= tx1; tx++)
            atomicAdd(B.tile_count + SR.tile_base + ty * SR.tiles_x + tx, 1u);
      }
    }
    base += __popc(m);
  }
  const uint32_t ids[2] = {2u * g, 2u * g + 1u};
  if (B.small_max > 0) raster_small(S, kind, ids, scene, BatchTarget{B.scenes}, s_rec[w], s_pre[w]);
  block_count(bc, 0, n_raster);
  block_count(bc, 1, n_small);
  block_count(bc, 2, n_clipped);
  block_flush(bc, &B.counters->rasterised, &B.counters->small_direct, &B.counters->clipped);
}

// Renderables per scene whose triangle bases k_batch keeps in shared memory
// (larger scenes search the global table).
constexpr int kBatchTbMax = 256;

// Exclusive prefix sum of v over the threads of the block (blockDim.x a
// multiple of 32, at most 1024); tot = the block's sum.  Every thread of the
// block must call it; s_part holds 33 words.
__device__ __forceinline__ uint32_t block_scan(uint32_t v, uint32_t* s_part, uint32_t& tot) {
  const int lane = (int)(threadIdx.x & 31), w = (int)(threadIdx.x >> 5), nw = (int)(blockDim.x >> 5);
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  __syncthreads();  // s_part free from a previous call
  if (lane == 31) s_part[w] = inc;
  __syncthreads();
  if (w == 0) {
    const uint32_t p = lane < nw ? s_part[lane] : 0u;
    uint32_t pi = p;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, pi, o);
      if (lane >= o) pi += u;
    }
    if (lane < nw) s_part[lane] = pi - p;
    if (lane == 31) s_part[32] = pi;
  }
  __syncthreads();
  tot = s_part[32];
  return s_part[w] + inc - v;
}

// Stages the tile's records bins[c0 .. c0+cn) in shared memory with the
// exclusive prefix of the rows each covers inside the tile (px0..px1,
// py0..py1): s_off[cn] is the number of (record, row) items.  Block-wide.
__device__ __forceinline__ void stage_chunk(const BigRec* recs, const uint32_t* bins, uint32_t c0, uint32_t cn,
                                            int px0, int py0, int px1, int py1, BigRec* s_recs,
                                            uint32_t* s_off, int* s_run = nullptr) {
  __syncthreads();  // the previous pass over s_recs / s_off is done
  int run = 0;
  for (uint32_t i = threadIdx.x; i < cn; i += blockDim.x) {
    const BigRec r = recs[bins[c0 + i]];
    s_recs[i] = r;
    const int ys = max(r.y0, py0), ye = min(r.y1, py1);
    const bool hit = ys <= ye && max(r.x0, px0) <= min(r.x1, px1);
    s_off[i] = hit ? (uint32_t)(ye - ys + 1) : 0u;
    if (hit) run = max(run, min(r.x1, px1) - r.x0);
  }
  if (s_run && run) atomicMax(s_run, run);
  __syncthreads();
  if (threadIdx.x < 32) {  // one warp scans: each lane a contiguous run
    const int lane = (int)threadIdx.x;
    const uint32_t per = (cn + 31) / 32;
    const uint32_t b = min(cn, (uint32_t)lane * per), e = min(cn, b + per);
    uint32_t sum = 0;
    for (uint32_t i = b; i < e; i++) sum += s_off[i];
    uint32_t inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += u;
    }
    uint32_t run = inc - sum;
    for (uint32_t i = b; i < e; i++) {
      const uint32_t c = s_off[i];
      s_off[i] = run;
      run += c;
    }
    if (lane == 31) s_off[cn] = inc;
  }
  __syncthreads();
}

// The (record, row) items of a staged chunk, one per thread: CAPTURE=false
// merges the fragments into the shared visibility tile; CAPTURE=true (after
// every record of the tile has been merged) stores, for each pixel, the
// running edge values of the fragment that won it, so the resolve needs no
// replay.  A pixel's winning word is unique (it holds the sub-triangle id).
// Tiles whose records could make a pixel replay its winner's edge functions
// over more columns than this capture the winners' edge values (pass 2).
constexpr int kReplayMax = 256;

template <bool CAPTURE>
__device__ __forceinline__ void raster_items(const BigRec* s_recs, const uint32_t* s_off, uint32_t cn, int TW,
                                             int px0, int py0, int px1, int py1, bool persp,
                                             unsigned long long* svis, float2* s_e) {
  const uint32_t total = s_off[cn];
  for (uint32_t it = threadIdx.x; it < total; it += blockDim.x) {
    int lo = 0, hi = (int)cn;  // s_off[lo] <= it < s_off[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (s_off[mid] <= it) lo = mid; else hi = mid;
    }
    const BigRec& R = s_recs[lo];
    const int y = max(R.y0, py0) + (int)(it - s_off[lo]);
    const int xs = max(R.x0, px0), xe = min(R.x1, px1);
    const Setup S = rec_setup(R);
    if (CAPTURE) {
      // the fragment that won a pixel is the one whose id the pixel holds
      // (it was covered and passed the depth test in the first pass)
      float e1, e2;
      row_start(S, y, e1, e2);
      const float d1 = S.n1.x, d2 = S.n2.x;
      for (int x = S.x0; x < xs; x++) {
        e1 += d1;
        e2 += d2;
      }
      const uint32_t* row = reinterpret_cast<const uint32_t*>(svis + (y - py0) * TW);  // low words: ids
      for (int x = xs; x <= xe; x++) {
        if (row[2 * (x - px0)] == R.id) s_e[(y - py0) * TW + (x - px0)] = make_float2(e1, e2);
        e1 += d1;
        e2 += d2;
      }
    } else {
      walk_row(S, persp, R.id, y, xs, xe, [&](int x, unsigned long long v, float, float) {
        atomicMin(svis + (y - py0) * TW + (x - px0), v);
      });
    }
  }
}

// The batch's persistent kernel (cooperative launch, grid-wide barriers):
//   1. exclusive scan of the per-tile counts (per-block segments, then one
//      block scanning the block sums), 2. scatter record indices into tile
//      lists, 3. tiles of all scenes taken from a work counter: the tile's
//      visibility words start from the scene's small-triangle words; its
//      records are staged in shared memory `chunk` at a time and rasterised
//      (pass 1), walked again to capture each winner's edge values (pass 2),
//      then every pixel of the tile is resolved, shaded and written to its
//      scene's outputs.
// MINB: blocks of 256 threads per SM the register allocation must allow
// (2: up to 128 registers per thread, for 64-thread blocks; 4: up to 64, so
// that 128- and 256-thread blocks keep enough warps resident).  At 64
// registers the vertex-pass instance spills 216 bytes per thread; an 80-
// register instance (3 blocks) that spills 36 was measured slower on the
// 256-scene batch (fused stage 3.62 vs 3.37 ms), so the warps win.
template <int MINB, bool PRE>
__global__ void __launch_bounds__(256, MINB) k_batch(BatchParams B, uint32_t* block_sums) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int TW = B.tile_w, TH = B.tile_h, TP = TW * TH;
  unsigned long long* svis = (unsigned long long*)smem;
  float2* s_e = (float2*)(smem + (size_t)TP * sizeof(unsigned long long));
  BigRec* s_recs = (BigRec*)(smem + (size_t)TP * (sizeof(unsigned long long) + sizeof(float2)));
  uint32_t* s_off = (uint32_t*)(s_recs + B.chunk);  // chunk + 1 entries
  __shared__ float s_dec[256];
  __shared__ uint32_t s_part[33];
  __shared__ uint32_t s_tile;
  __shared__ int s_run;  // longest column replay a pixel of the tile could need
  __shared__ View s_view;
  __shared__ int s_meta[8];
  __shared__ uint32_t s_tb[kBatchTbMax];
  __shared__ int s_tb_scene;
  __shared__ uint8_t* s_out8;
  __shared__ float* s_outd;
  __shared__ uint32_t* s_outi;
  __shared__ const unsigned long long* s_invis;  // small triangles' visibility words of the scene
  cg::grid_group grid = cg::this_grid();
  const uint32_t nb = gridDim.x, nt = blockDim.x;
  for (uint32_t i = threadIdx.x; i < 256; i += nt) s_dec[i] = (float)i / 255.0f;
  if (threadIdx.x == 0) s_tb_scene = -1;
  // 1. scan: block b owns tiles [b*seg, (b+1)*seg)
  const uint32_t seg = (B.n_tiles + nb - 1) / nb;
  const uint32_t t0 = min(B.n_tiles, blockIdx.x * seg), t1 = min(B.n_tiles, t0 + seg);
  {
    uint32_t sum = 0;
    for (uint32_t i = t0 + threadIdx.x; i < t1; i += nt) sum += B.tile_count[i];
    uint32_t tot;
    block_scan(sum, s_part, tot);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
  }
  grid.sync();
  if (blockIdx.x == 0) {  // exclusive scan of the block sums, by the whole block
    uint32_t run = 0;
    for (uint32_t b0 = 0; b0 < nb; b0 += nt) {
      const uint32_t i = b0 + threadIdx.x;
      const uint32_t v = i < nb ? block_sums[i] : 0u;
      uint32_t tot;
      const uint32_t ex = block_scan(v, s_part, tot);
      if (i < nb) block_sums[i] = run + ex;
      run += tot;
    }
    if (threadIdx.x == 0) {
      B.tile_start[B.n_tiles] = run;
      B.counters->bin_needed = run;
      B.counters->bin_entries += run;
    }
  }
  grid.sync();
  {
    uint32_t run = block_sums[blockIdx.x];
    for (uint32_t b0 = t0; b0 < t1; b0 += nt) {
      const uint32_t i = b0 + threadIdx.x;
      const uint32_t v = i < t1 ? B.tile_count[i] : 0u;
      uint32_t tot;
      const uint32_t ex = block_scan(v, s_part, tot);
      if (i < t1) B.tile_start[i] = run + ex;
      run += tot;
    }
  }
  grid.sync();
  // 2. scatter
  const uint32_t nrec = min(B.counters->rec_count, B.rec_cap);
  for (uint32_t i = blockIdx.x * nt + threadIdx.x; i < nrec; i += nb * nt) {
    const BigRec& R = B.recs[i];
    const SceneRec& SR = B.scenes[B.rec_scene[i]];
    int tx0 = R.x0 / TW, tx1 = R.x1 / TW, ty0 = R.y0 / TH, ty1 = R.y1 / TH;
    for (int ty = ty0; ty <= ty1; ty++)
      for (int tx = tx0; tx <= tx1; tx++) {
        uint32_t t = SR.tile_base + ty * SR.tiles_x + tx;
        uint32_t pos = B.tile_start[t] + atomicAdd(B.tile_fill + t, 1u);
        if (pos < B.bin_cap) B.bins[pos] = i;
        else B.counters->bin_overflow = 1;
      }
  }
  grid.sync();
  // 3. tiles
  for (;;) {
    __syncthreads();
    if (threadIdx.x < 32) {  // warp 0 takes the next tile and loads its scene
      const int lane = (int)threadIdx.x;
      uint32_t t = 0;
      if (lane == 0) t = atomicAdd(&B.counters->work_next, 1u);
      t = __shfl_sync(0xffffffffu, t, 0);
      if (t < B.n_tiles) {
        // the scene: the last j with scene_tile_base[j] <= t (bases ascending)
        unsigned cnt = 0;
        for (int j = 1 + lane; j < B.n_scenes; j += 32) cnt += B.scene_tile_base[j] <= t;
        const int sc = (int)__reduce_add_sync(0xffffffffu, cnt);
        const SceneRec& SR = B.scenes[sc];
        const uint32_t* src = reinterpret_cast<const uint32_t*>(&SR.v);
        uint32_t* dst = reinterpret_cast<uint32_t*>(&s_view);
        for (int k = lane; k < (int)(sizeof(View) / 4); k += 32) dst[k] = src[k];
        if (lane == 0) {
          s_meta[0] = sc;
          s_meta[1] = (int)(t - SR.tile_base);
          s_meta[2] = SR.tiles_x;
          s_meta[3] = (int)SR.rs_begin;
          s_meta[4] = (int)SR.rs_end;
          s_meta[5] = (int)(2u * B.g.tri_base[SR.rs_begin]);  // ids are reported per scene
          // the tile's list (bins truncated at capacity on overflow)
          s_meta[6] = (int)min(B.tile_start[t], B.bin_cap);
          s_meta[7] = (int)min(B.tile_start[t + 1], B.bin_cap);
          s_out8 = SR.rgb8;
          s_outd = SR.depth;
          s_outi = SR.ids;
          s_invis = SR.vis;
        }
      }
      if (lane == 0) s_tile = t;
    }
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= B.n_tiles) break;
    const int n_rs = s_meta[4] - s_meta[3];
    const bool tb_shared = n_rs <= kBatchTbMax;
    if (tb_shared && s_tb_scene != s_meta[0]) {  // uniform: read after the barrier above
      for (int i = threadIdx.x; i < n_rs; i += nt) s_tb[i] = B.g.tri_base[s_meta[3] + i];
      __syncthreads();
      if (threadIdx.x == 0) s_tb_scene = s_meta[0];
    }
    const int lt = s_meta[1], tx = lt % s_meta[2], ty = lt / s_meta[2];
    const int px0 = tx * TW, py0 = ty * TH;
    const int px1 = min(px0 + TW, s_view.W) - 1, py1 = min(py0 + TH, s_view.H) - 1;
    // the tile starts from the small triangles' words (or empty), copied
    // with cp.async so all of a thread's loads are in flight at once (made
    // visible to the block by the barrier that opens pass 1)
    for (int i = threadIdx.x; i < TP; i += nt) {
      const int x = px0 + i % TW, y = py0 + i / TW;
      if (s_invis && x <= px1 && y <= py1) cp_async8(&svis[i], &s_invis[(size_t)y * s_view.W + x]);
      else svis[i] = VIS_EMPTY;
    }
    cp_async_wait_all();
    const uint32_t s = (uint32_t)s_meta[6], e = (uint32_t)s_meta[7];
    const bool persp = s_view.persp != 0;
    const uint32_t nck = (e - s + (uint32_t)B.chunk - 1) / (uint32_t)B.chunk;
    if (threadIdx.x == 0) s_run = 0;  // (ordered by stage_chunk's first barrier)
    for (uint32_t c = 0; c < nck; c++) {  // pass 1: depth test
      const uint32_t c0 = s + c * (uint32_t)B.chunk, cn = min((uint32_t)B.chunk, e - c0);
      stage_chunk(B.recs, B.bins, c0, cn, px0, py0, px1, py1, s_recs, s_off, &s_run);
      raster_items<false>(s_recs, s_off, cn, TW, px0, py0, px1, py1, persp, svis, s_e);
    }
    // pass 2, the winners' edge values, only where a replay from the
    // bounding-box edge could be long: otherwise the resolve replays (cheaper
    // than walking every record of the tile a second time)
    const bool captured = nck > 0 && s_run > kReplayMax;
    if (captured) {
      // captured edge values start as NaN (no fragment with a NaN edge value
      // is ever written: its depth is NaN and fails z < 1e11f); ordered
      // before the capture by the barrier that opens each pass-2 chunk
      for (int i = threadIdx.x; i < TP; i += nt) s_e[i] = make_float2(__int_as_float(0x7fc00000), 0.f);
      for (uint32_t c = 0; c < nck; c++) {
        const uint32_t c0 = s + c * (uint32_t)B.chunk, cn = min((uint32_t)B.chunk, e - c0);
        if (nck > 1) stage_chunk(B.recs, B.bins, c0, cn, px0, py0, px1, py1, s_recs, s_off);
        else __syncthreads();
        raster_items<true>(s_recs, s_off, cn, TW, px0, py0, px1, py1, persp, svis, s_e);
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < TP; i += nt) {
      const int x = px0 + i % TW, y = py0 + i / TW;
      if (x > px1 || y > py1) continue;
      const unsigned long long vw = svis[i];
      V3 value, normal;
      float depth;
      const uint32_t id = (uint32_t)vw;
      if (vw == VIS_EMPTY) {
        value = v3(s_view.bg[0], s_view.bg[1], s_view.bg[2]);
        depth = 1e11f;
      } else {
        int ip[3];
        Vtx vc[3];
        bool clipped;
        const DevRenderable& R = *winner_tri<PRE>(s_view, B.g, s_meta[3], s_meta[4], id, ip, vc, clipped,
                                                   tb_shared ? s_tb : nullptr);
        Setup S;
        float e1, e2;
        const float2 ee = captured ? s_e[i] : make_float2(__int_as_float(0x7fc00000), 0.f);
        winner_setup<PRE>(s_view, B.g, R, ip, vc, clipped, S);
        if (ee.x == ee.x) {  // won by a record of this tile: edge values captured
          e1 = ee.x;
          e2 = ee.y;
        } else {  // won by a small triangle rasterised in the setup kernel
          replay(S, x, y, e1, e2);
        }
        float k0, k1, k2;
        depth = frag_depth(S, persp, e1, e2, k0, k1, k2);
        shade(s_view, R, vc, k0, k1, k2, s_dec, value, normal);
      }
      const size_t px = (size_t)y * s_view.W + x;
      if (uint8_t* o8 = s_out8) {
        o8[3 * px + 0] = to_byte(value.x);
        o8[3 * px + 1] = to_byte(value.y);
        o8[3 * px + 2] = to_byte(value.z);
      }
      if (s_outd) s_outd[px] = depth;
      if (s_outi) s_outi[px] = vw == VIS_EMPTY ? MR_NO_TRIANGLE : id - (uint32_t)s_meta[5];
    }
  }
}

__global__ void k_range(int W, int H, const float* P, const float* depth, float* xyz) {
  size_t px = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (px >= (size_t)W * H) return;
  int i = (int)(px / W), j = (int)(px - (size_t)i * W);
  bool persp = P[15] == 0;
  float zfar = persp ? P[11] / (P[10] + 1) : (P[11] - 1) / P[10];
  float fardepth = persp ? zfar : 1.0f;
  float w = (float)W, h = (float)H;
  float d = depth[px];
  float* o = xyz + 3 * px;
  if (d > fardepth) {
    o[0] = 0; o[1] = 0; o[2] = 0;
  } else {
    float u = (j + 0.5f) / (w / 2) - 1;
    float v = -(i + 0.5f) / (h / 2) + 1;
    float z = -d;
    o[0] = -(u + P[2]) * z / P[0];
    o[1] = -(v + P[6]) * z / P[5];
    o[2] = z;
  }
}

// ------------------------------------------------------------ host launchers
static int grid_for(size_t n, int block) { return (int)((n + block - 1) / block); }

static int sm_count() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

cudaError_t launch_validate(const DevMesh& M, uint32_t* bad, cudaStream_t st) {
  if (M.n_tri <= 0) return cudaSuccess;
  k_validate<<<grid_for((size_t)M.n_tri, 256), 256, 0, st>>>(M, bad, const_cast<float4*>(M.rec));
  return cudaGetLastError();
}

// Ordinary launch allowed to overlap its predecessor's tail (the kernel calls
// pdl_wait() before touching anything the predecessor writes).
template <typename... Exp, typename... Act>
static cudaError_t launch_after(void (*k)(Exp...), int grid, int block, cudaStream_t st, Act&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, std::forward<Act>(args)...);
}

static cudaError_t launch_coop(const void* fn, int grid, int block, void** args, size_t smem, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelExC(&cfg, fn, args);
}

// Launch sequence of one frame.  With F.g.va set, the vertex pass runs first
// and the setup/resolve kernels read its buffers.  ev (optional, 6 events)
// brackets the stages: clear+vertex, setup, large-triangle raster, -, resolve.
cudaError_t launch_frame(const FrameParams& F, cudaStream_t st, cudaEvent_t* ev, cudaEvent_t staged) {
  size_t npx = (size_t)F.v.W * F.v.H;
  const bool pre = F.g.va != nullptr;
  if (ev) cudaEventRecord(ev[0], st);
  // The clear also brings vis[] into L2 (write-allocate), so the setup
  // kernel's atomics hit L2.
  const int cgrid = std::min(grid_for(npx, 256), sm_count() * 16);
  k_clear<<<cgrid, 256, 0, st>>>(
      F.vis, npx, reinterpret_cast<uint32_t*>(F.counters), (uint32_t)(sizeof(Counters) / 4), nullptr, 0,
      F.stage_src, F.stage_dst, F.stage_n16);
  if (staged) cudaEventRecord(staged, st);  // the staging block has been read
  // vertex pass, setup and resolve may be scheduled while their predecessor
  // finishes (they wait for it before reading its output)
  cudaError_t le = cudaSuccess;
  if (pre && (F.g.n_verts + F.g.n_nrms) > 0)
    le = launch_after(k_vertex, grid_for((size_t)F.g.n_verts + F.g.n_nrms, 256), 256, st, F.g, F.v,
                      (const SceneRec*)nullptr);
  if (le != cudaSuccess) return le;
  if (ev) cudaEventRecord(ev[1], st);
  if (F.g.n_tris) {
    le = launch_after(pre ? k_setup<true> : k_setup<false>, grid_for(F.g.n_tris, kSetupThreads), kSetupThreads, st, F);
    if (le != cudaSuccess) return le;
  }
  if (ev) cudaEventRecord(ev[2], st);
  le = launch_after(k_raster_large, sm_count() * 8, 256, st, F);
  if (le != cudaSuccess) return le;
  if (ev) cudaEventRecord(ev[3], st);
  if (ev) cudaEventRecord(ev[4], st);
  const int rgrid = ((F.v.W + kResolveTileW - 1) / kResolveTileW) * ((F.v.H + kResolveTileH - 1) / kResolveTileH);
  le = launch_after(pre ? k_resolve<true> : k_resolve<false>, rgrid, 256, st, F);
  if (le != cudaSuccess) return le;
  if (ev) cudaEventRecord(ev[5], st);
  return cudaGetLastError();
}

size_t batch_smem(int tile_w, int tile_h, int chunk) {
  // visibility words + captured edge values per pixel, staged records, row prefix
  return (size_t)tile_w * tile_h * (sizeof(unsigned long long) + sizeof(float2)) + (size_t)chunk * sizeof(BigRec) +
         (size_t)(chunk + 1) * sizeof(uint32_t);
}
static const void* batch_kernel(int threads, bool pre) {
  if (pre)
    return threads <= 64 ? (const void*)k_batch<2, true>
                         : (const void*)k_batch<4, true>;
  return threads <= 64 ? (const void*)k_batch<2, false>
                       : (const void*)k_batch<4, false>;
}
// Co-resident blocks of k_batch for the given shape (its cooperative grid).
int batch_grid(int tile_w, int tile_h, int chunk, int threads, bool pre) {
  int per = 0;
  size_t smem = batch_smem(tile_w, tile_h, chunk);
  const void* k = batch_kernel(threads, pre);
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, threads, smem);
  if (per <= 0) return 0;
  return sm_count() * per;
}
cudaError_t launch_batch(const BatchParams& B, int threads, int grid, uint32_t* block_sums, cudaStream_t st,
                         cudaEvent_t* ev) {
  const bool pre = B.g.va != nullptr;  // null: kernels transform corners themselves
  if (ev) cudaEventRecord(ev[0], st);
  if (pre && B.g.n_verts + B.g.n_nrms > 0) {
    View none = {};
    k_vertex<<<grid_for((size_t)B.g.n_verts + B.g.n_nrms, 256), 256, 0, st>>>(B.g, none, B.scenes);
  }
  if (B.small_max > 0 && B.n_px) {  // small triangles' visibility words of every scene
    const int cgrid = std::min(grid_for(B.n_px, 256), sm_count() * 16);
    k_clear<<<cgrid, 256, 0, st>>>(B.vis, B.n_px, nullptr, 0, nullptr, 0, nullptr, nullptr, 0);
  }
  if (ev) cudaEventRecord(ev[1], st);
  if (B.g.n_tris) {
    if (pre) k_setup_batch<true><<<grid_for(B.g.n_tris, kSetupThreads), kSetupThreads, 0, st>>>(B);
    else k_setup_batch<false><<<grid_for(B.g.n_tris, kSetupThreads), kSetupThreads, 0, st>>>(B);
  }
  if (ev) cudaEventRecord(ev[2], st);
  BatchParams Bc = B;
  void* args[] = {&Bc, &block_sums};
  cudaError_t e = launch_coop(batch_kernel(threads, pre), grid, threads, args, batch_smem(B.tile_w, B.tile_h, B.chunk),
                              st);
  if (ev) cudaEventRecord(ev[3], st);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t launch_range(int W, int H, const float* dP, const float* depth, float* xyz, cudaStream_t st) {
  size_t npx = (size_t)W * H;
  k_range<<<grid_for(npx, 256), 256, 0, st>>>(W, H, dP, depth, xyz);
  return cudaGetLastError();
}

}  // namespace mrg
