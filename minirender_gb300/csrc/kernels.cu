// GB300 (sm_103a) kernels of the one-frame-per-call rasterisation path.
//
//   k_clear        vis[] = VIS_EMPTY                 (Renderer::clear, src/Renderer.cpp:113-119)
//   k_validate     per-mesh bad-triangle bitmask     (index checks done once at upload)
//   k_vertex       per-vertex view transform + projection to pixel space and
//                  per-normal transform, once per frame (the PREMULT loops,
//                  src/Renderer.cpp:344-348, plus htransform :13-20 and the
//                  pixel mapping :193-197, which depend on the vertex only)
//   k_setup        triangle assembly + near clip + triangle setup + cull;
//                  small triangles rasterised by the warp that set them up,
//                  one (triangle, row) per lane; large ones appended to a
//                  warp-compacted record list       (src/Renderer.cpp:121-269, 351-379)
//   k_bin_tile     one cooperative launch: screen-tile binning of the large
//                  records (count, scan, scatter), then per-tile raster into a
//                  shared-memory visibility tile merged into vis[] with
//                  64-bit atomicMin                  (src/Renderer.cpp:238-269)
//   k_resolve      deferred pass: re-derives the winning sub-triangle's
//                  barycentrics exactly, shades once per visible pixel and
//                  writes RGB8/depth/ids            (src/Renderer.cpp:271-305, src/io.cpp:358-362)
//   k_range        getRangeImage                      (src/Renderer.cpp:388-415)
//
// Exactness: every float operation follows the reference's order; the
// edge functions are advanced column by column from the bounding-box edge
// exactly as the reference loop does (the running sums have no closed form),
// so both the rasterisers and the resolve pass replay that chain.  Values the
// vertex pass stores are the same expressions the reference evaluates per
// triangle corner, so storing them changes no bit.
//
// Kernels templated on PRE use the vertex-pass buffers when PRE is true and
// transform vertices per triangle otherwise (the allocation-free entry point
// has no room for per-vertex buffers).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "raster.cuh"

namespace cg = cooperative_groups;

namespace mrg {

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ int find_base(const uint32_t* base, int n, uint32_t g) {
  int lo = 0, hi = n;
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
__device__ __forceinline__ void project(const FrameParams& F, V3 v, float& px, float& py, float& zt) {
  V3 ndc = htransform(F.P, v);
  px = (1 + ndc.x) * (F.w / 2);
  py = (1 - ndc.y) * (F.h / 2);
  zt = F.persp ? -rcp(v.z) : ndc.z;
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

// View-space corners of triangle t (paintMesh, src/Renderer.cpp:344-379).
template <bool PRE, bool ATTR>
__device__ __forceinline__ void corners(const FrameParams& F, const DevRenderable& R, int t,
                                        const int (&ip)[3], Vtx (&v)[3]) {
  const DevMesh& M = R.mesh;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    if (PRE) {
      float4 a = F.va[R.vert_base + ip[c]];
      float2 b = F.vb[R.vert_base + ip[c]];
      v[c].pos = v3(b.x, b.y, a.w);
    } else {
      v[c].pos = affine(R.mv, ld3(M.pos, ip[c]));
    }
    if (ATTR) {
      int in = __ldg(M.nidx + 3 * t + c);
      if (PRE) {
        float4 n = F.vn[R.nrm_base + in];
        v[c].nrm = v3(n.x, n.y, n.z);
      } else {
        v[c].nrm = affine(R.nm, ld3(M.nrm, in));
      }
      v[c].uv = M.has_uv ? ld2(M.uv, __ldg(M.tidx + 3 * t + c)) : v2(0, 0);
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
__device__ __forceinline__ bool setup_from(const FrameParams& F, const V2 (&p)[3], const float (&zt)[3],
                                           Setup& S) {
  V2 pmin = v2(1e30f, 1e30f), pmax = v2(-1e30f, -1e30f);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    pmin = v2(minr(pmin.x, p[i].x), minr(pmin.y, p[i].y));
    pmax = v2(maxr(pmax.x, p[i].x), maxr(pmax.y, p[i].y));
  }
  if (pmax.x < 0 || pmax.y < 0 || pmin.x > F.w || pmin.y > F.h) return false;
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
  pmin.x = clampr(pmin.x, 0.f, F.w - 1);
  pmax.x = clampr(pmax.x, 0.f, F.w - 1);
  pmin.y = clampr(pmin.y, 0.f, F.h - 1);
  pmax.y = clampr(pmax.y, 0.f, F.h - 1);
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
__device__ __forceinline__ bool setup_view(const FrameParams& F, const Vtx (&s)[3], Setup& S) {
  V2 p[3];
  float zt[3];
#pragma unroll
  for (int i = 0; i < 3; i++) project(F, s[i].pos, p[i].x, p[i].y, zt[i]);
  return setup_from(F, p, zt, S);
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
// calls emit(x, packed) for every fragment that would pass z < 1e11f.
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
      if (z < 1e11f) emit(x, ((unsigned long long)depth_key(z) << 32) | id);
    }
    e1 += d1;
    e2 += d2;
  }
}

__device__ __forceinline__ void warp_add(unsigned long long* dst, unsigned v) {
  unsigned s = __reduce_add_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(dst, (unsigned long long)s);
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

// ------------------------------------------------------------------ kernels
__global__ void k_clear(unsigned long long* vis, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) vis[i] = VIS_EMPTY;
}

__global__ void k_validate(DevMesh M, uint32_t* bad) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  bool b = false;
  if (t < M.n_tri) {
    for (int c = 0; c < 3; c++) {
      int ip = M.idx[3 * t + c], in = M.nidx[3 * t + c];
      b |= ip < 0 || ip >= M.n_pos || in < 0 || in >= M.n_nrm;
      if (M.has_uv) {
        int it = M.tidx[3 * t + c];
        b |= it < 0 || it >= M.n_uv;
      }
    }
  }
  unsigned m = __ballot_sync(0xffffffffu, b);
  if ((threadIdx.x & 31) == 0 && (t >> 5) < ((M.n_tri + 31) >> 5)) bad[t >> 5] = m;
}

// Vertex pass: threads [0, n_verts) transform and project positions,
// threads [n_verts, n_verts + n_nrms) transform normals.
__global__ void __launch_bounds__(256) k_vertex(FrameParams F) {
  uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < F.n_verts) {
    int r = find_base(F.vert_base, F.n_renderables, g);
    const DevRenderable& R = F.rs[r];
    V3 v = affine(R.mv, ld3(R.mesh.pos, (int)(g - R.vert_base)));
    float px, py, zt;
    project(F, v, px, py, zt);
    F.va[g] = make_float4(px, py, zt, v.z);
    F.vb[g] = make_float2(v.x, v.y);
  } else if (g - F.n_verts < F.n_nrms) {
    uint32_t gn = g - F.n_verts;
    int r = find_base(F.nrm_base, F.n_renderables, gn);
    const DevRenderable& R = F.rs[r];
    V3 n = affine(R.nm, ld3(R.mesh.nrm, (int)(gn - R.nrm_base)));
    F.vn[gn] = make_float4(n.x, n.y, n.z, 0.f);
  }
}

// Small-triangle record staged in shared memory for the warp's cooperative raster.
struct __align__(16) SmallRec {
  float p0x, p0y, p2x, p2y, n1x, n1y, n2x, n2y, z0, z1, z2;
  uint32_t id;
  int x0, y0, x1, rows;
};

constexpr int kSetupThreads = 256;
constexpr int kSetupWarps = kSetupThreads / 32;

template <bool PRE>
__global__ void __launch_bounds__(kSetupThreads) k_setup(FrameParams F) {
  __shared__ SmallRec s_rec[kSetupWarps][64];
  __shared__ int s_pre[kSetupWarps][65];
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const bool persp = F.persp != 0;
  Setup S[2];
  int kind[2] = {0, 0};  // 0 none, 1 small, 2 big
  unsigned n_clipped = 0, n_raster = 0, n_small = 0;
  if (g < F.n_tris) {
    int r = find_base(F.tri_base, F.n_renderables, g);
    const DevRenderable& R = F.rs[r];
    const int t = (int)(g - R.tri_base);
    if ((R.mesh.bad[t >> 5] >> (t & 31)) & 1u) {
      atomicOr(&F.counters->error_flags, 1u);
    } else {
      int ip[3];
#pragma unroll
      for (int c = 0; c < 3; c++) ip[c] = __ldg(R.mesh.idx + 3 * t + c);
      const float zn = F.znear;
      int n = 0;
      if (PRE) {
        float4 a[3];
#pragma unroll
        for (int c = 0; c < 3; c++) a[c] = F.va[R.vert_base + ip[c]];
        if (!(a[0].w > zn || a[1].w > zn || a[2].w > zn)) {
          V2 p[3] = {v2(a[0].x, a[0].y), v2(a[1].x, a[1].y), v2(a[2].x, a[2].y)};
          float zt[3] = {a[0].z, a[1].z, a[2].z};
          if (setup_from(F, p, zt, S[0])) { kind[0] = 1; n_raster++; }
        } else {
          n = -1;  // clipped below
        }
      } else {
        n = -1;
      }
      if (n < 0) {
        Vtx v[3], sub[2][3];
        corners<PRE, false>(F, R, t, ip, v);
        bool any = v[0].pos.z > zn || v[1].pos.z > zn || v[2].pos.z > zn;
        if (!any) {
          sub[0][0] = v[0]; sub[0][1] = v[1]; sub[0][2] = v[2];
          n = 1;
        } else {
          n = clip_tri<false>(zn, v, sub);
          n_clipped += n > 0;
        }
        for (int s = 0; s < n; s++)
          if (setup_view(F, sub[s], S[s])) { kind[s] = 1; n_raster++; }
      }
#pragma unroll
      for (int s = 0; s < 2; s++)
        if (kind[s]) {
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
    if (kind[s] == 2) {
      unsigned slot = base + __popc(m & lt);
      if (slot < F.rec_cap) F.recs[slot] = to_rec(S[s], 2u * g + (uint32_t)s);
    }
  }
  // small records: stage in shared memory, then rasterise with one
  // (triangle, row) per lane so every lane has work
  int n = 0;
#pragma unroll
  for (int s = 0; s < 2; s++) {
    unsigned m = __ballot_sync(0xffffffffu, kind[s] == 1);
    if (kind[s] == 1) {
      SmallRec& q = s_rec[w][n + __popc(m & lt)];
      q.p0x = S[s].p0.x; q.p0y = S[s].p0.y; q.p2x = S[s].p2.x; q.p2y = S[s].p2.y;
      q.n1x = S[s].n1.x; q.n1y = S[s].n1.y; q.n2x = S[s].n2.x; q.n2y = S[s].n2.y;
      q.z0 = S[s].z[0]; q.z1 = S[s].z[1]; q.z2 = S[s].z[2];
      q.id = 2u * g + (uint32_t)s;
      q.x0 = S[s].x0; q.y0 = S[s].y0; q.x1 = S[s].x1;
      q.rows = S[s].y1 - S[s].y0 + 1;
    }
    n += __popc(m);
  }
  __syncwarp();
  if (n > 0) {
    int c0 = (int)lane < n ? s_rec[w][lane].rows : 0;
    int c1 = (int)lane + 32 < n ? s_rec[w][lane + 32].rows : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int u0 = __shfl_up_sync(0xffffffffu, c0, o), u1 = __shfl_up_sync(0xffffffffu, c1, o);
      if ((int)lane >= o) { c0 += u0; c1 += u1; }
    }
    int tot0 = __shfl_sync(0xffffffffu, c0, 31), tot1 = __shfl_sync(0xffffffffu, c1, 31);
    if (lane == 0) s_pre[w][0] = 0;
    s_pre[w][lane + 1] = c0;
    s_pre[w][lane + 33] = tot0 + c1;
    __syncwarp();
    const int total = tot0 + tot1;
    unsigned long long* vis = F.vis;
    const int W = F.W;
    for (int b = 0; b < total; b += 32) {
      int k = b + (int)lane;
      if (k < total) {
        int lo = 0, hi = n;
        while (hi - lo > 1) {
          int mid = (lo + hi) >> 1;
          if (s_pre[w][mid] <= k) lo = mid; else hi = mid;
        }
        const SmallRec& q = s_rec[w][lo];
        Setup T;
        T.p0 = v2(q.p0x, q.p0y); T.p2 = v2(q.p2x, q.p2y);
        T.n1 = v2(q.n1x, q.n1y); T.n2 = v2(q.n2x, q.n2y);
        T.z[0] = q.z0; T.z[1] = q.z1; T.z[2] = q.z2;
        T.x0 = q.x0; T.x1 = q.x1; T.y0 = q.y0;
        const int y = q.y0 + (k - s_pre[w][lo]);
        walk_row(T, persp, q.id, y, T.x0, T.x1, [&](int x, unsigned long long v) {
          atomicMin(vis + (size_t)y * W + x, v);
        });
      }
    }
  }
  warp_add(&F.counters->rasterised, n_raster);
  warp_add(&F.counters->small_direct, n_small);
  warp_add(&F.counters->clipped, n_clipped);
}

__device__ __forceinline__ void rec_tiles(const FrameParams& F, const BigRec& B, int& tx0, int& ty0,
                                          int& tx1, int& ty1) {
  tx0 = B.x0 / F.tile; tx1 = B.x1 / F.tile;
  ty0 = B.y0 / F.tile; ty1 = B.y1 / F.tile;
}

// Rasterises the binned (record, row) pairs of one tile into a shared-memory
// visibility tile, then merges it into vis[] with 64-bit atomicMin.  Called
// by every thread of the block.
__device__ __forceinline__ void tile_raster(const FrameParams& F, int tile, unsigned long long* svis) {
  const int TS = F.tile;
  uint32_t s = F.tile_start[tile], e = min(F.tile_start[tile + 1], F.bin_cap);
  if (s >= e) return;  // uniform across the block
  const int tx = tile % F.tiles_x, ty = tile / F.tiles_x;
  const int px0 = tx * TS, py0 = ty * TS;
  const int px1 = min(px0 + TS, F.W) - 1, py1 = min(py0 + TS, F.H) - 1;
  for (int i = threadIdx.x; i < TS * TS; i += blockDim.x) svis[i] = VIS_EMPTY;
  __syncthreads();
  const bool persp = F.persp != 0;
  const uint32_t work = (e - s) * (uint32_t)TS;
  for (uint32_t i = threadIdx.x; i < work; i += blockDim.x) {
    uint32_t ent = s + i / TS;
    int y = py0 + (int)(i % TS);
    BigRec B = F.recs[F.bins[ent]];
    if (y < B.y0 || y > B.y1 || y > py1) continue;
    int xs = max(B.x0, px0), xe = min(B.x1, px1);
    if (xs > xe) continue;
    Setup S = rec_setup(B);
    walk_row(S, persp, B.id, y, xs, xe, [&](int x, unsigned long long v) {
      atomicMin(svis + (y - py0) * TS + (x - px0), v);
    });
  }
  __syncthreads();
  for (int i = threadIdx.x; i < TS * TS; i += blockDim.x) {
    unsigned long long v = svis[i];
    if (v != VIS_EMPTY) {
      int x = px0 + i % TS, y = py0 + i / TS;
      atomicMin(F.vis + (size_t)y * F.W + x, v);
    }
  }
  __syncthreads();  // svis is reused by the block's next tile
}

constexpr int kBinThreads = 256;

// Screen-tile binning of the large records and their tile raster in one
// cooperative launch (all blocks co-resident; grid-wide barriers between the
// phases): count per tile -> exclusive scan -> scatter -> per-tile raster.
// With no large record every block returns at once, before any barrier.
__global__ void __launch_bounds__(kBinThreads) k_bin_tile(FrameParams F) {
  extern __shared__ unsigned long long svis[];
  __shared__ uint32_t part[kBinThreads];
  const uint32_t nrec = min(F.counters->rec_count, F.rec_cap);
  if (nrec == 0) return;
  cg::grid_group grid = cg::this_grid();
  const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  const int ntiles = F.tiles_x * F.tiles_y;
  for (uint32_t i = gt; i < nrec; i += gs) {  // 1. count
    BigRec B = F.recs[i];
    int tx0, ty0, tx1, ty1;
    rec_tiles(F, B, tx0, ty0, tx1, ty1);
    for (int ty = ty0; ty <= ty1; ty++)
      for (int tx = tx0; tx <= tx1; tx++) atomicAdd(F.tile_count + ty * F.tiles_x + tx, 1u);
  }
  grid.sync();
  if (blockIdx.x == 0) {  // 2. exclusive scan, one block
    int per = (ntiles + blockDim.x - 1) / blockDim.x;
    int b = threadIdx.x * per, e = min(ntiles, b + per);
    uint32_t sum = 0;
    for (int i = b; i < e; i++) sum += F.tile_count[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int off = 1; off < (int)blockDim.x; off <<= 1) {
      uint32_t v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0;
      __syncthreads();
      part[threadIdx.x] += v;
      __syncthreads();
    }
    uint32_t run = threadIdx.x ? part[threadIdx.x - 1] : 0;
    for (int i = b; i < e; i++) {
      F.tile_start[i] = run;
      run += F.tile_count[i];
    }
    if (threadIdx.x == blockDim.x - 1) {
      F.tile_start[ntiles] = part[blockDim.x - 1];
      F.counters->bin_needed = part[blockDim.x - 1];
      F.counters->bin_entries += part[blockDim.x - 1];
    }
  }
  grid.sync();
  for (uint32_t i = gt; i < nrec; i += gs) {  // 3. scatter
    BigRec B = F.recs[i];
    int tx0, ty0, tx1, ty1;
    rec_tiles(F, B, tx0, ty0, tx1, ty1);
    for (int ty = ty0; ty <= ty1; ty++)
      for (int tx = tx0; tx <= tx1; tx++) {
        int t = ty * F.tiles_x + tx;
        uint32_t pos = F.tile_start[t] + atomicAdd(F.tile_fill + t, 1u);
        if (pos < F.bin_cap) F.bins[pos] = i;
        else F.counters->bin_overflow = 1;
      }
  }
  grid.sync();
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) tile_raster(F, tile, svis);  // 4.
}

// Deferred resolve + shade: one thread per pixel.
template <bool PRE>
__global__ void __launch_bounds__(256) k_resolve(FrameParams F) {
  // loadPPM's texel decode b/255.0f (src/io.cpp:410), one division per byte value
  __shared__ float s_dec[256];
  s_dec[threadIdx.x] = (float)threadIdx.x / 255.0f;
  __syncthreads();
  size_t px = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t npx = (size_t)F.W * F.H;
  if (px >= npx) return;
  unsigned long long v = F.vis[px];
  V3 value;
  float depth;
  uint32_t id;
  V3 normal_out = v3(0, 0, 1);
  if (v == VIS_EMPTY) {
    value = v3(F.bg[0], F.bg[1], F.bg[2]);
    depth = 1e11f;
    id = MR_NO_TRIANGLE;
  } else {
    id = (uint32_t)v;
    const uint32_t g = id >> 1;
    const int s = (int)(id & 1u);
    const int r = find_base(F.tri_base, F.n_renderables, g);
    const DevRenderable& R = F.rs[r];
    const int t = (int)(g - R.tri_base);
    int ip[3];
#pragma unroll
    for (int c = 0; c < 3; c++) ip[c] = __ldg(R.mesh.idx + 3 * t + c);
    Vtx v3c[3];
    corners<PRE, true>(F, R, t, ip, v3c);
    Setup S;
    const float zn = F.znear;
    const bool clipped = v3c[0].pos.z > zn || v3c[1].pos.z > zn || v3c[2].pos.z > zn;
    if (clipped) {
      Vtx sub[2][3];
      clip_tri<true>(zn, v3c, sub);
      // select sub-triangle s into v3c (s is 0 or 1 and exists: it won a pixel)
#pragma unroll
      for (int c = 0; c < 3; c++) v3c[c] = s ? sub[1][c] : sub[0][c];
      setup_view(F, v3c, S);
    } else if (PRE) {
      V2 p[3];
      float zt[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        float4 a = F.va[R.vert_base + ip[c]];
        p[c] = v2(a.x, a.y);
        zt[c] = a.z;
      }
      setup_from(F, p, zt, S);
    } else {
      setup_view(F, v3c, S);
    }
    const int y = (int)(px / F.W), x = (int)(px - (size_t)y * F.W);
    float e1, e2;
    row_start(S, y, e1, e2);
    for (int c = S.x0; c < x; c++) {
      e1 += S.n1.x;
      e2 += S.n2.x;
    }
    float k0, k1, k2;
    depth = frag_depth(S, F.persp != 0, e1, e2, k0, k1, k2);
    // shading, src/Renderer.cpp:271-305 (FAST_LIGHT)
    V3 color = v3(R.diffuse[0], R.diffuse[1], R.diffuse[2]);
    if (R.has_tex) {
      V2 uv = add2(add2(ks2(k0, v3c[0].uv), ks2(k1, v3c[1].uv)), ks2(k2, v3c[2].uv));
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
    if (F.lighting) {
      V3 position = add3(add3(ks3(k0, v3c[0].pos), ks3(k1, v3c[1].pos)), ks3(k2, v3c[2].pos));
      V3 LD = v3(F.lightdir[0], F.lightdir[1], F.lightdir[2]);
      V3 lightdir = F.point ? normalized3(sub3(LD, position)) : LD;
      V3 normal = add3(add3(ks3(k0, v3c[0].nrm), ks3(k1, v3c[1].nrm)), ks3(k2, v3c[2].nrm));
      float sdiff = maxr(0.0f, dot3(normal, lightdir)) / len3(normal) + F.ambient;
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
  if (F.rgb8) {
    F.rgb8[3 * px + 0] = (uint8_t)(int)clampr(value.x * 255.0f, 0.0f, 255.0f);
    F.rgb8[3 * px + 1] = (uint8_t)(int)clampr(value.y * 255.0f, 0.0f, 255.0f);
    F.rgb8[3 * px + 2] = (uint8_t)(int)clampr(value.z * 255.0f, 0.0f, 255.0f);
  }
  if (F.depth) F.depth[px] = depth;
  if (F.ids) F.ids[px] = id;
  if (F.rgbf) {
    F.rgbf[3 * px + 0] = value.x;
    F.rgbf[3 * px + 1] = value.y;
    F.rgbf[3 * px + 2] = value.z;
  }
  if (F.normals) {
    F.normals[3 * px + 0] = normal_out.x;
    F.normals[3 * px + 1] = normal_out.y;
    F.normals[3 * px + 2] = normal_out.z;
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

cudaError_t launch_validate(const DevMesh& M, uint32_t* bad, cudaStream_t st) {
  if (M.n_tri <= 0) return cudaSuccess;
  k_validate<<<grid_for((size_t)M.n_tri, 256), 256, 0, st>>>(M, bad);
  return cudaGetLastError();
}

// Launch sequence of one frame.  With F.va set, the vertex pass runs first
// and the setup/resolve kernels read its buffers.  ev (optional, 6 events)
// brackets the stages: clear+vertex, setup, binning, tile raster, resolve.
cudaError_t launch_frame(const FrameParams& F, cudaStream_t st, cudaEvent_t* ev) {
  size_t npx = (size_t)F.W * F.H;
  const bool pre = F.va != nullptr;
  if (ev) cudaEventRecord(ev[0], st);
  // The clear also brings vis[] into L2 (write-allocate), so the setup
  // kernel's atomics hit L2.
  int cgrid = grid_for(npx, 256);
  k_clear<<<cgrid < 152 * 16 ? cgrid : 152 * 16, 256, 0, st>>>(F.vis, npx);
  if (pre && (F.n_verts + F.n_nrms) > 0)
    k_vertex<<<grid_for((size_t)F.n_verts + F.n_nrms, 256), 256, 0, st>>>(F);
  if (ev) cudaEventRecord(ev[1], st);
  if (F.n_tris) {
    if (pre) k_setup<true><<<grid_for(F.n_tris, kSetupThreads), kSetupThreads, 0, st>>>(F);
    else k_setup<false><<<grid_for(F.n_tris, kSetupThreads), kSetupThreads, 0, st>>>(F);
  }
  if (ev) cudaEventRecord(ev[2], st);
  {
    // one cooperative launch, as many blocks as are co-resident
    static int grid = 0;
    size_t smem = (size_t)32 * 32 * sizeof(unsigned long long);
    if (!grid) {
      int dev = 0, sms = 0, per = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_bin_tile, kBinThreads, smem);
      grid = sms * (per > 0 ? per : 1);
    }
    FrameParams Fc = F;
    void* args[] = {&Fc};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_bin_tile, grid, kBinThreads, args, smem, st);
    if (e != cudaSuccess) return e;
  }
  if (ev) cudaEventRecord(ev[3], st);
  if (ev) cudaEventRecord(ev[4], st);
  if (pre) k_resolve<true><<<grid_for(npx, 256), 256, 0, st>>>(F);
  else k_resolve<false><<<grid_for(npx, 256), 256, 0, st>>>(F);
  if (ev) cudaEventRecord(ev[5], st);
  return cudaGetLastError();
}

cudaError_t launch_range(int W, int H, const float* dP, const float* depth, float* xyz,
                         cudaStream_t st) {
  size_t npx = (size_t)W * H;
  k_range<<<grid_for(npx, 256), 256, 0, st>>>(W, H, dP, depth, xyz);
  return cudaGetLastError();
}

}  // namespace mrg
