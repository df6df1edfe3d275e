// Data layout shared by the host side of the C ABI and the kernels: one
// resident mesh, one renderable, the view of one frame, the setup record of a
// rasterised sub-triangle, per-frame counters and the kernel parameter
// blocks.  Plain C++ (no device code), so host translation units can include it.
#pragma once
#include <stdint.h>
#include <vector_types.h>

#include "../../include/minirender_gpu.h"

namespace mrg {

// Packed visibility word: (order-preserving depth key << 32) | sub-triangle
// id.  A pixel nobody wrote keeps VIS_EMPTY, which is larger than any real
// fragment because real fragments need z < 1e11f (the clear value of the
// reference z-buffer, src/Renderer.cpp:116) and id < 0xFFFFFFFF.
static constexpr unsigned long long VIS_EMPTY = ~0ull;

// One resident mesh (TriMesh arrays, include/minirender/Scene.h:73-87).
struct DevMesh {
  const float* pos;   // n_pos x 3
  const float* nrm;   // n_nrm x 3
  const float* uv;    // n_uv x 2
  const int32_t* idx;   // 3 per triangle
  const int32_t* nidx;
  const int32_t* tidx;
  const uint32_t* bad;   // bit t set: triangle t has an index out of range
  // Soup-like meshes (3 * n_tri < 2 * n_pos): triangle t's corner positions,
  // normals and texcoords gathered at upload into rec[8t .. 8t+7] (128 B per
  // triangle; the first 64 B hold all of a triangle whose three corners share
  // one normal and one texcoord), so a pixel's winner is read from one record
  // instead of six scattered arrays.  Null otherwise.
  const float4* rec;
  int32_t n_pos, n_nrm, n_uv, n_tri;
  int32_t has_uv;       // texcoords and texcoordsI both non-empty
};

// Meshes that get corner records: those whose vertices are not shared
// (the per-vertex pass would not pay for them alone).
inline bool mesh_wants_records(long long n_tri, long long n_pos) { return n_tri > 0 && 3 * n_tri < 2 * n_pos; }
constexpr size_t kRecBytes = 128;

// One renderable: mesh, matrices and material.
struct DevRenderable {
  float mv[12];         // rows 0..2 of view * transform (src/Renderer.cpp:337)
  float nm[12];         // rows 0..2 of inverse(mv)^T (src/Renderer.cpp:338)
  DevMesh mesh;
  uint32_t tri_base;    // global index of the first triangle
  uint32_t vert_base;   // global index of the first vertex in the per-frame vertex buffers
  uint32_t nrm_base;    // global index of the first normal
  uint32_t scene;       // frame (scene) this renderable belongs to (batches)
  int32_t has_tex;      // texturing on and the material has a texture
  int32_t no_clip;      // MR_RS_NO_CLIP: no near-plane clipping
  int32_t lit;          // lighting on for its fragments (the frame's or its paint call's)
  int32_t point;        // point light for its fragments (the frame's or its paint call's)
  float diffuse[3], specular[3], emissive[3], shininess;
  const uint8_t* tex8;  // rows x cols x 3 bytes (decoded b/255), or
  const float* texf;    // rows x cols x 3 floats
  int32_t tex_rows, tex_cols;
};

// Renderer state of one frame that the kernels read (src/Renderer.cpp:311-326).
struct View {
  int W, H;
  float w, h;
  float P[16];
  int persp;
  float znear;
  float lightdir[3];  // placed as render() places it (src/Renderer.cpp:317-320)
  float ambient;
  float bg[3];
};

// Geometry of a launch: renderable table, base tables and the per-vertex
// buffers of the vertex pass (va null: kernels transform per triangle).
struct Geo {
  const DevRenderable* rs;
  const uint32_t* tri_base;   // n_renderables + 1 prefix of triangle counts
  const uint32_t* vert_base;  // n_renderables + 1 prefix of vertex counts
  const uint32_t* nrm_base;   // n_renderables + 1 prefix of normal counts
  int n_renderables;
  uint32_t n_tris, n_verts, n_nrms;
  float4* va;                 // (pixel x, pixel y, z term, view z) per vertex
  float2* vb;                 // (view x, view y) per vertex
  float4* vn;                 // view-space normal per normal
};

// Setup record of a rasterised sub-triangle (64 bytes).
struct __align__(16) BigRec {
  float p0x, p0y, p2x, p2y;   // pixel-space corners 0 and 2
  float n1x, n1y, n2x, n2y;   // edge-function gradients
  float z0, z1, z2;           // iz[] (perspective) or zz[] (orthographic)
  uint32_t id;                // 2 * global triangle + clip sub-triangle
  int32_t x0, y0, x1, y1;     // inclusive clamped pixel bounding box
};

struct Counters {
  unsigned long long triangles, clipped, rasterised, small_direct, binned, bin_entries;
  unsigned int error_flags;
  unsigned int rec_count;      // records written
  unsigned int bin_needed;     // total (tile, record) pairs requested
  unsigned int bin_overflow;
  unsigned int work_next;      // persistent-kernel work counter
  unsigned int item_count;     // large-triangle row blocks requested (single frames)
  unsigned int spill_count;    // records whose remaining rows did not fit the row-block list
  unsigned int pad;
};

// One-frame launch.
// Row block of a large sub-triangle: kLargeRows rows from `row` of record
// `rec`; in the spill list, every row from `row` to the record's last.
struct LargeItem {
  uint32_t rec, row;
};
constexpr int kLargeRows = 32;

struct FrameParams {
  View v;
  Geo g;
  int small_max;
  unsigned long long* vis;    // W*H
  BigRec* recs;               // large sub-triangles
  uint32_t rec_cap;
  LargeItem* items;           // their row blocks
  uint32_t item_cap;
  LargeItem* spill;           // rec_cap entries: records past the end of items[]
  const uint4* stage_src;     // the frame's staging block in mapped pinned host memory,
  uint4* stage_dst;           // fetched by the clear kernel (no copy-engine transfer)
  uint32_t stage_n16;         // its size in 16-byte units
  uint8_t* rgb8;
  float* depth;
  float* rgbf;
  uint32_t* ids;
  float* normals;
  Counters* counters;
};

// One scene of a batch: its view, tiles and output buffers.
struct SceneRec {
  View v;
  int tiles_x, tiles_y;
  uint32_t tile_base;         // first tile in the batch-wide tile index space
  uint32_t rs_begin, rs_end;  // renderables of this scene
  uint8_t* rgb8;
  float* depth;
  uint32_t* ids;
  unsigned long long* vis;    // visibility words of the small triangles (null: all binned)
};

// Batched launch: many scenes, one persistent fused bin-raster-shade kernel.
struct BatchParams {
  Geo g;
  const SceneRec* scenes;
  const uint32_t* scene_tile_base;  // n_scenes + 1 prefix of tile counts
  int n_scenes;
  uint32_t n_tiles;
  int tile_w, tile_h, chunk;        // tile width and height (pixels), records staged per pass
  int small_max;                    // bbox pixels up to which the setup kernel rasterises (0: none)
  unsigned long long* vis;          // all scenes' visibility words (small_max > 0)
  size_t n_px;                      // pixels of all scenes
  BigRec* recs;
  uint32_t rec_cap;
  uint32_t* rec_scene;              // scene of each record
  uint32_t* tile_count;             // n_tiles
  uint32_t* tile_start;             // n_tiles + 1
  uint32_t* tile_fill;              // n_tiles
  uint32_t* bins;
  uint32_t bin_cap;
  Counters* counters;
};

}  // namespace mrg
