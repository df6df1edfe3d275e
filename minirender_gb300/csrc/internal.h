// Internal declarations shared by the C-ABI translation units: the context,
// resident meshes/textures, device buffers, batch slots and error helpers.
#pragma once
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "host_math.h"
#include "layout.h"

namespace mrg {
cudaError_t launch_validate(const DevMesh& M, uint32_t* bad, cudaStream_t st);
cudaError_t launch_frame(const FrameParams& F, cudaStream_t st, cudaEvent_t* ev, cudaEvent_t staged = nullptr);
cudaError_t launch_range(int W, int H, const float* dP, const float* depth, float* xyz,
                         cudaStream_t st);
cudaError_t launch_batch(const BatchParams& B, int threads, int grid, uint32_t* block_sums, cudaStream_t st,
                         cudaEvent_t* ev);
int batch_grid(int tile_w, int tile_h, int chunk, int threads, bool pre);
// Tile shapes k_batch takes: power-of-two sides, 64..4096 pixels (whole warps).
inline bool batch_tile_ok(int tw, int th) {
  auto pow2 = [](int v) { return v > 0 && (v & (v - 1)) == 0; };
  return pow2(tw) && pow2(th) && tw >= 4 && tw <= 256 && th >= 2 && th <= 64 && tw * th >= 64 && tw * th <= 4096;
}
}  // namespace mrg

using namespace mrg;

namespace mrgi {

struct MeshRec {
  bool live = false;
  bool stream_ordered = false;  // allocated with cudaMallocAsync
  void* mem = nullptr;
  size_t bytes = 0;
  DevMesh d{};
  int32_t n_idx = 0;
  bool validate_pending = false;  // updated on the upload stream, indices not yet checked
};

struct TexRec {
  bool live = false;
  bool stream_ordered = false;
  void* mem = nullptr;
  size_t bytes = 0;
  bool rgb8 = false;
  int32_t rows = 0, cols = 0;
};

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t cap = 0;  // elements
  // Grows to at least 1.5x the old capacity: a stream of frames or batches
  // of varying sizes then reallocates O(log) times, not at every new
  // maximum (each cudaFree waits for the whole device).
  cudaError_t ensure(size_t n) {
    if (n <= cap && p) return cudaSuccess;
    const size_t grown = cap + cap / 2;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(std::max<size_t>(n, grown), 1);
    cudaError_t e = cudaMalloc(&p, want * sizeof(T));
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace mrgi

using namespace mrgi;

// One batch in flight: its tuning, device buffers, pinned staging, counters
// and (optionally) the CUDA graph of its launch sequence.  The context owns
// one for mr_render_batch; a render server owns several.
struct BatchSlot {
  int tile_w = 16, tile_h = 16, threads = 256, chunk = 64;
  int small_max = 64;  // bbox pixels up to which the setup kernel rasterises (0: every triangle binned)
  bool graphs = true;
  DevBuf<DevRenderable> rs;
  DevBuf<uint32_t> bases;
  DevBuf<SceneRec> scenes;
  DevBuf<uint32_t> stb;
  DevBuf<float4> va, vn;
  DevBuf<float2> vb;
  DevBuf<BigRec> recs;
  DevBuf<uint32_t> rec_scene, tiles, bins, block_sums;
  DevBuf<unsigned long long> vis;
  DevBuf<uint8_t> out8;
  DevBuf<float> outd;
  DevBuf<uint32_t> outi;
  DevRenderable* h_rs = nullptr;
  size_t h_rs_cap = 0;
  uint32_t* h_u32 = nullptr;  // bases (3(n+1)) then scene tile bases (S+1)
  size_t h_u32_cap = 0;
  SceneRec* h_scenes = nullptr;
  size_t h_scenes_cap = 0;
  Counters* d_cnt = nullptr;
  Counters* h_cnt = nullptr;
  BatchParams P{};
  int grid = 0;
  int n_scenes = 0, n_rs = 0;
  std::vector<int> W, H;
  std::vector<int32_t> rs_scene;  // scene of each renderable (staging)
  std::vector<size_t> px_off;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<uint64_t> key;
  cudaEvent_t done = nullptr;
  cudaEvent_t staged = nullptr;   // the batch's host staging has been copied
  bool have = false;
  cudaStream_t stream = nullptr;  // null: the context stream
  cudaEvent_t ev[8] = {};         // profiling events (slots other than the context's)
  bool profiling = false;
  void release();
};

// Host destinations of one frame's reads (null: not read).
struct ReadTargets {
  uint8_t* rgb8;
  float* depth;
  float* rgbf;
  uint32_t* ids;
  float* normals;
};

struct mr_ctx {
  int device = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  std::recursive_mutex mu;
  std::vector<MeshRec> meshes;
  std::vector<TexRec> textures;
  DevBuf<unsigned long long> vis;
  DevBuf<uint8_t> rgb8;
  DevBuf<float> depth, rgbf, normals, range;
  DevBuf<uint32_t> ids;
  DevBuf<BigRec> recs;
  DevBuf<LargeItem> items;     // large-triangle row blocks of the last frame
  DevBuf<LargeItem> spill;     // records whose rows did not fit items (one entry each)
  // Per-frame staging, one block on both sides (one copy per frame):
  // renderables (cap) | tri, vertex and normal base tables 3 x (cap+1) | projection
  DevBuf<unsigned char> stage;
  unsigned char* h_stage = nullptr;
  unsigned char* d_stage_src = nullptr;  // h_stage as the device sees it (mapped)
  size_t h_rs_cap = 0, stage_bytes = 0, off_bases = 0, off_P = 0;
  DevRenderable* h_rs = nullptr;
  uint32_t* h_tri_base = nullptr;
  float* h_P = nullptr;
  DevBuf<float4> va, vn;        // per-frame vertex-pass outputs
  DevBuf<float2> vb;
  Counters* d_cnt = nullptr;
  Counters* h_cnt = nullptr;
  cudaEvent_t ev[8] = {};
  cudaEvent_t staged = nullptr;
  cudaEvent_t read_done = nullptr;  // after the copies of the last mr_read_async
  cudaStream_t upload = nullptr;     // mesh / texture updates (null: the compute stream)
  cudaEvent_t compute_mark = nullptr, uploaded = nullptr;
  bool upload_waiting = false;       // the compute stream has not yet waited for `uploaded`
  bool profiling = false;
  int tile = 16;
  int small_max = 64;
  bool have_frame = false;
  bool pending = false;  // a frame was launched and not yet checked
  bool async_read = false;  // mr_read_async copies queued, not yet waited for
  FrameParams last{};
  mr_frame last_frame{};
  int outputs = 0;
  std::string err;

  BatchSlot b;
};

inline int fail(mr_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

inline int cuda_fail(mr_ctx* c, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return fail(c, MR_E_NOMEM, m);
  return fail(c, MR_E_CUDA, m);
}

#define CK(expr, what)                              \
  do {                                              \
    cudaError_t _e = (expr);                        \
    if (_e != cudaSuccess) return cuda_fail(c, _e, what); \
  } while (0)


extern "C" {  // internal (not exported): defined inside the C-ABI translation unit
// Why a mesh descriptor cannot be used (negative counts, an index count not a
// multiple of 3, normalsI / texcoordsI shorter than indices, a null array
// with a non-zero count), or null when it is well formed.  Checked before
// any device work by every entry point that takes a descriptor.
const char* mesh_desc_problem(const mr_mesh_desc* d);
// Batch stages shared by mr_render_batch and the render server.
int batch_stage(mr_ctx* c, BatchSlot& B, const mr_batch_scene* sc, int32_t n_scenes, const mr_renderable* rs,
                int32_t n_rs, int32_t outputs);
int batch_run(mr_ctx* c, BatchSlot& B, cudaStream_t st, bool profiling, cudaEvent_t* ev);
int batch_settle(mr_ctx* c, BatchSlot& B, cudaStream_t st);
// Resident meshes/textures; with `stream` the memory is stream-ordered
// (cudaMallocAsync / cudaFreeAsync) so no device-wide synchronisation occurs.
// stream != null: stream-ordered allocation (from `pool` when given).
// defer_check: the upload queues copies only; the index check runs at
// check_pending_mesh (the server calls it right before the batch that first
// reads the mesh, so its copies never wait behind kernels).
int mesh_create(mr_ctx* c, const mr_mesh_desc* d, cudaStream_t stream, int32_t* out, size_t* bytes,
                cudaMemPool_t pool = nullptr, bool defer_check = false);
// Launches the deferred index check of mesh h on st (no-op if none pending).
int check_pending_mesh(mr_ctx* c, int32_t h, cudaStream_t st, bool* launched);
int mesh_destroy(mr_ctx* c, int32_t h, cudaStream_t stream);
int texture_create(mr_ctx* c, const void* data, bool rgb8, int32_t rows, int32_t cols, cudaStream_t stream,
                   int32_t* out, cudaMemPool_t pool = nullptr);
int texture_destroy(mr_ctx* c, int32_t h, cudaStream_t stream);
}  // extern "C"
