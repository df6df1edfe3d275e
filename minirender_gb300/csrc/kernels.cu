// GB300 (sm_103a) kernels of the one-frame-per-call rasterisation path.
//
//   k_clear        vis[] = VIS_EMPTY                 (Renderer::clear, src/Renderer.cpp:113-119)
//   k_validate     per-mesh bad-triangle bitmask     (index checks done once at upload)
//   k_setup        assemble + vertex transform + near clip + triangle setup;
//                  small triangles rasterised in place, large ones appended
//                  to a warp-compacted record list   (src/Renderer.cpp:121-236, 344-379)
//   k_bin_count / k_scan / k_bin_scatter
//                  screen-tile binning of the large records
//   k_tile_raster  per-tile raster into a shared-memory visibility tile,
//                  merged into vis[] with 64-bit atomicMin (src/Renderer.cpp:238-269)
//   k_resolve      deferred pass: re-derives the winning sub-triangle's
//                  barycentrics exactly, shades once per visible pixel and
//                  writes RGB8/depth/ids            (src/Renderer.cpp:271-305, src/io.cpp:358-362)
//   k_range        getRangeImage                      (src/Renderer.cpp:388-415)
//
// Exactness: every float operation follows the reference's order; the
// edge functions are advanced column by column from the bounding-box edge
// exactly as the reference loop does (the running sums have no closed form),
// so both the rasterisers and the resolve pass replay that chain.
#include <cuda_runtime.h>

#include "raster.cuh"

namespace mrg {

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ int find_renderable(const FrameParams& F, uint32_t g) {
  int lo = 0, hi = F.n_renderables;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (F.tri_base[mid] <= g) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ V3 ld3(const float* p, int i) {
  return v3(__ldg(p + 3 * i), __ldg(p + 3 * i + 1), __ldg(p + 3 * i + 2));
}
__device__ __forceinline__ V2 ld2(const float* p, int i) {
  return v2(__ldg(p + 2 * i), __ldg(p + 2 * i + 1));
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

// Vertex assembly (paintMesh, src/Renderer.cpp:351-379) plus the near-plane
// test and clipTriangle (src/Renderer.cpp:131-177).  Returns the number of
// sub-triangles (0, 1 or 2) in draw order; ATTR also builds normals and UVs.
template <bool ATTR>
__device__ __forceinline__ int assemble(const FrameParams& F, const DevRenderable& R, int t,
                                        Vtx (&sub)[2][3], bool& clipped) {
  const DevMesh& M = R.mesh;
  Vtx v[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    int ip = __ldg(M.idx + 3 * t + c);
    v[c].pos = affine(R.mv, ld3(M.pos, ip));
    if (ATTR) {
      int in = __ldg(M.nidx + 3 * t + c);
      v[c].nrm = affine(R.nm, ld3(M.nrm, in));
      if (M.has_uv) v[c].uv = ld2(M.uv, __ldg(M.tidx + 3 * t + c));
      else v[c].uv = v2(0, 0);
    }
  }
  const float zn = F.znear;
  bool any = v[0].pos.z > zn || v[1].pos.z > zn || v[2].pos.z > zn;
  clipped = any;
  if (!any) {
    sub[0][0] = v[0]; sub[0][1] = v[1]; sub[0][2] = v[2];
    return 1;
  }
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

struct Setup {
  V2 p0, p2, n1, n2;
  float z[3];
  int x0, y0, x1, y1;
};

// htransform, src/Renderer.cpp:13-20
__device__ __forceinline__ V3 htransform(const float* m, V3 p) {
  float iw = 1 / (m[12] * p.x + m[13] * p.y + m[14] * p.z + m[15]);
  return v3((m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3]) * iw,
            (m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7]) * iw,
            (m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]) * iw);
}

// paintTriangle setup, src/Renderer.cpp:179-224.  False = nothing to draw.
__device__ __forceinline__ bool setup_tri(const FrameParams& F, const Vtx (&s)[3], Setup& S) {
  V3 ndc[3];
  V2 p[3];
#pragma unroll
  for (int i = 0; i < 3; i++) ndc[i] = htransform(F.P, s[i].pos);
  float hw = F.w / 2, hh = F.h / 2;
  V2 pmin = v2(1e30f, 1e30f), pmax = v2(-1e30f, -1e30f);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    p[i].x = (1 + ndc[i].x) * hw;
    p[i].y = (1 - ndc[i].y) * hh;
    pmin = v2(minr(pmin.x, p[i].x), minr(pmin.y, p[i].y));
    pmax = v2(maxr(pmax.x, p[i].x), maxr(pmax.y, p[i].y));
  }
  if (pmax.x < 0 || pmax.y < 0 || pmin.x > F.w || pmin.y > F.h) return false;
  float d0x = p[0].x - p[1].x, d0y = p[0].y - p[1].y;
  float d2x = p[2].x - p[1].x, d2y = p[2].y - p[1].y;
  float a = d0x * d2y - d0y * d2x;
  if (a <= 0) return false;  // back-face cull, :207-210
  float i2a = (a == 0) ? 0.0f : -1.0f / a;
  float ex = p[0].x - p[2].x, ey = p[0].y - p[2].y;
  S.n1 = v2(-ey * i2a, ex * i2a);
  ex = p[1].x - p[0].x; ey = p[1].y - p[0].y;
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
  if (F.persp) {
#pragma unroll
    for (int i = 0; i < 3; i++) S.z[i] = -1 / s[i].pos.z;
  } else {
#pragma unroll
    for (int i = 0; i < 3; i++) S.z[i] = ndc[i].z;
  }
  return true;
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
    float z = 1.f / (k0 * S.z[0] + k1 * S.z[1] + k2 * S.z[2]);
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

__global__ void __launch_bounds__(256) k_setup(FrameParams F) {
  uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  bool active = g < F.n_tris;
  const bool persp = F.persp != 0;
  BigRec rec[2];
  bool big[2] = {false, false};
  unsigned n_clipped = 0, n_raster = 0, n_small = 0;
  if (active) {
    int r = find_renderable(F, g);
    const DevRenderable& R = F.rs[r];
    int t = (int)(g - R.tri_base);
    bool bad = (R.mesh.bad[t >> 5] >> (t & 31)) & 1u;
    if (bad) {
      atomicOr(&F.counters->error_flags, 1u);
    } else {
      Vtx sub[2][3];
      bool clipped;
      int n = assemble<false>(F, R, t, sub, clipped);
      n_clipped += clipped && n > 0;
      for (int s = 0; s < n; s++) {
        Setup S;
        if (!setup_tri(F, sub[s], S)) continue;
        n_raster++;
        uint32_t id = 2u * g + (uint32_t)s;
        long long bw = S.x1 - S.x0 + 1, bh = S.y1 - S.y0 + 1;
        if (bw * bh <= (long long)F.small_max) {
          n_small++;
          unsigned long long* vis = F.vis;
          const int W = F.W;
          for (int y = S.y0; y <= S.y1; y++)
            walk_row(S, persp, id, y, S.x0, S.x1, [&](int x, unsigned long long v) {
              atomicMin(vis + (size_t)y * W + x, v);
            });
        } else {
          BigRec& B = rec[s];
          B.p0x = S.p0.x; B.p0y = S.p0.y; B.p2x = S.p2.x; B.p2y = S.p2.y;
          B.n1x = S.n1.x; B.n1y = S.n1.y; B.n2x = S.n2.x; B.n2y = S.n2.y;
          B.z0 = S.z[0]; B.z1 = S.z[1]; B.z2 = S.z[2];
          B.id = id;
          B.x0 = S.x0; B.y0 = S.y0; B.x1 = S.x1; B.y1 = S.y1;
          big[s] = true;
        }
      }
    }
  }
  // warp-level compaction of the large records: one atomic per warp and slot
  const unsigned lane = threadIdx.x & 31;
#pragma unroll
  for (int s = 0; s < 2; s++) {
    unsigned m = __ballot_sync(0xffffffffu, big[s]);
    if (m == 0) continue;
    unsigned base = 0;
    if (lane == 0) base = atomicAdd(&F.counters->rec_count, (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (big[s]) {
      unsigned slot = base + __popc(m & ((1u << lane) - 1u));
      if (slot < F.rec_cap) F.recs[slot] = rec[s];
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

__global__ void k_bin_count(FrameParams F) {
  uint32_t n = min(F.counters->rec_count, F.rec_cap);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    BigRec B = F.recs[i];
    int tx0, ty0, tx1, ty1;
    rec_tiles(F, B, tx0, ty0, tx1, ty1);
    for (int ty = ty0; ty <= ty1; ty++)
      for (int tx = tx0; tx <= tx1; tx++) atomicAdd(F.tile_count + ty * F.tiles_x + tx, 1u);
  }
}

// Exclusive scan of tile_count into tile_start[0..n], single block.
__global__ void __launch_bounds__(1024) k_scan(FrameParams F, int n) {
  __shared__ uint32_t part[1024];
  int per = (n + blockDim.x - 1) / blockDim.x;
  int b = threadIdx.x * per, e = min(n, b + per);
  uint32_t s = 0;
  for (int i = b; i < e; i++) s += F.tile_count[i];
  part[threadIdx.x] = s;
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
    F.tile_start[n] = part[blockDim.x - 1];
    F.counters->bin_needed = part[blockDim.x - 1];
    F.counters->bin_entries += part[blockDim.x - 1];
  }
}

__global__ void k_bin_scatter(FrameParams F) {
  uint32_t n = min(F.counters->rec_count, F.rec_cap);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
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
}

__device__ __forceinline__ Setup rec_setup(const BigRec& B) {
  Setup S;
  S.p0 = v2(B.p0x, B.p0y); S.p2 = v2(B.p2x, B.p2y);
  S.n1 = v2(B.n1x, B.n1y); S.n2 = v2(B.n2x, B.n2y);
  S.z[0] = B.z0; S.z[1] = B.z1; S.z[2] = B.z2;
  S.x0 = B.x0; S.y0 = B.y0; S.x1 = B.x1; S.y1 = B.y1;
  return S;
}

// One block per screen tile; threads take (record, row) pairs.
__global__ void __launch_bounds__(128) k_tile_raster(FrameParams F) {
  extern __shared__ unsigned long long svis[];
  const int tile = blockIdx.x;
  const int TS = F.tile;
  uint32_t s = F.tile_start[tile], e = F.tile_start[tile + 1];
  e = min(e, F.bin_cap);
  if (s >= e) return;
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
}

// Deferred resolve + shade: one thread per pixel.
__global__ void __launch_bounds__(256) k_resolve(FrameParams F) {
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
    uint32_t g = id >> 1;
    int s = (int)(id & 1u);
    int r = find_renderable(F, g);
    const DevRenderable& R = F.rs[r];
    int t = (int)(g - R.tri_base);
    Vtx sub[2][3];
    bool clipped;
    assemble<true>(F, R, t, sub, clipped);
    Setup S;
    setup_tri(F, sub[s], S);
    int y = (int)(px / F.W), x = (int)(px - (size_t)y * F.W);
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
      V2 uv = add2(add2(ks2(k0, sub[s][0].uv), ks2(k1, sub[s][1].uv)), ks2(k2, sub[s][2].uv));
      int ti = (int)((uv.y - floorf(uv.y)) * (float)R.tex_rows);
      int tj = (int)((uv.x - floorf(uv.x)) * (float)R.tex_cols);
      ti = min(max(ti, 0), R.tex_rows - 1);
      tj = min(max(tj, 0), R.tex_cols - 1);
      size_t o = 3 * ((size_t)ti * R.tex_cols + tj);
      if (R.tex8)
        color = v3((float)R.tex8[o] / 255.0f, (float)R.tex8[o + 1] / 255.0f, (float)R.tex8[o + 2] / 255.0f);
      else
        color = v3(R.texf[o], R.texf[o + 1], R.texf[o + 2]);
    }
    value = v3(R.emissive[0], R.emissive[1], R.emissive[2]);
    if (F.lighting) {
      V3 position = add3(add3(ks3(k0, sub[s][0].pos), ks3(k1, sub[s][1].pos)), ks3(k2, sub[s][2].pos));
      V3 LD = v3(F.lightdir[0], F.lightdir[1], F.lightdir[2]);
      V3 lightdir = F.point ? normalized3(sub3(LD, position)) : LD;
      V3 normal = add3(add3(ks3(k0, sub[s][0].nrm), ks3(k1, sub[s][1].nrm)), ks3(k2, sub[s][2].nrm));
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

cudaError_t launch_frame(const FrameParams& F, cudaStream_t st, cudaEvent_t* ev) {
  size_t npx = (size_t)F.W * F.H;
  int ntiles = F.tiles_x * F.tiles_y;
  if (ev) cudaEventRecord(ev[0], st);
  k_clear<<<grid_for(npx, 256) < 152 * 16 ? grid_for(npx, 256) : 152 * 16, 256, 0, st>>>(F.vis, npx);
  if (ev) cudaEventRecord(ev[1], st);
  if (F.n_tris) k_setup<<<grid_for(F.n_tris, 256), 256, 0, st>>>(F);
  if (ev) cudaEventRecord(ev[2], st);
  k_bin_count<<<152 * 4, 256, 0, st>>>(F);
  k_scan<<<1, 1024, 0, st>>>(F, ntiles);
  k_bin_scatter<<<152 * 4, 256, 0, st>>>(F);
  if (ev) cudaEventRecord(ev[3], st);
  k_tile_raster<<<ntiles, 128, (size_t)F.tile * F.tile * sizeof(unsigned long long), st>>>(F);
  if (ev) cudaEventRecord(ev[4], st);
  k_resolve<<<grid_for(npx, 256), 256, 0, st>>>(F);
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
