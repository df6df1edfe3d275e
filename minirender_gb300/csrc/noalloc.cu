// mr_render_noalloc: one frame of one mesh with no device allocation.
//
// Some callers cannot allocate device memory: code hosted by a framework
// whose memory pool owns the whole device, or a real-time loop that cannot
// pay for cudaMalloc/cudaFree (cudaFree synchronises the device).  This entry
// point takes the caller's device inputs and outputs and keeps all of its
// working memory in g_scratch below, a file-scope device array the library
// reserves on every GPU it is loaded on, for the life of the process.
//
// g_scratch is a host-side stand-in in host code, not a device address: its
// device address is looked up once per device (cudaGetSymbolAddress, with
// that device current) on the first call there, and that address is what the
// kernels receive.  The address belongs to the device's primary context, so
// the device must not be reset (cudaDeviceReset) while the library is in use.
// Every call shares the array and inherits the previous call's contents, so
// the counters are cleared each call; the visibility buffer is cleared by the
// frame's own clear kernel and the index mask is rewritten by the validation
// kernel.  Large sub-triangles get records and row blocks in the array as in
// mr_render, up to kRecCap of them; any further ones are rasterised by the
// setup kernel itself.  Calls whose GPU work overlaps race on the array.
#include <cuda_runtime.h>
#include <string.h>

#include <mutex>

#include "internal.h"

namespace {

constexpr size_t al(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kVisOff = 0;
constexpr size_t kVisBytes = (size_t)MR_NOALLOC_MAX_PIXELS * sizeof(unsigned long long);
constexpr size_t kBadOff = al(kVisOff + kVisBytes);
constexpr size_t kBadBytes = ((size_t)MR_NOALLOC_MAX_TRIANGLES / 32 + 1) * sizeof(uint32_t);
constexpr size_t kCntOff = al(kBadOff + kBadBytes);
constexpr size_t kRsOff = al(kCntOff + sizeof(Counters));
constexpr size_t kBaseOff = al(kRsOff + sizeof(DevRenderable));
constexpr uint32_t kRecCap = 1u << 15;   // large sub-triangles with a record
constexpr uint32_t kItemCap = 1u << 16;  // their 32-row blocks (more: the spill list)
constexpr size_t kRecOff = al(kBaseOff + 2 * sizeof(uint32_t));
constexpr size_t kItemOff = al(kRecOff + (size_t)kRecCap * sizeof(BigRec));
constexpr size_t kSpillOff = al(kItemOff + (size_t)kItemCap * sizeof(LargeItem));
constexpr size_t kEnd = al(kSpillOff + (size_t)kRecCap * sizeof(LargeItem));  // one entry per record at most
static_assert(kEnd <= MR_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds MR_NOALLOC_SCRATCH_BYTES");

}  // namespace

static __device__ __align__(256) unsigned char g_scratch[MR_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_addr[kMaxDevices] = {};

// Device address of g_scratch on the current device (looked up once).
cudaError_t scratch_address(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return e;
    g_addr[dev] = (unsigned char*)p;
  }
  *out = g_addr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" MR_API int mr_render_noalloc(const mr_frame* f, const mr_mesh_desc* d, const float* transform,
                                        const mr_material* mat, const void* texture, int32_t tex_rows,
                                        int32_t tex_cols, int32_t tex_is_rgb8, uint8_t* rgb8, float* depth,
                                        uint32_t* tri_id, void* cuda_stream) {
  // every argument is checked before any device work: a null array with a
  // non-zero count would otherwise reach the kernels as address 0
  if (!f || !d || !transform || !mat) return MR_E_INVALID;
  if (f->width <= 0 || f->height <= 0) return MR_E_INVALID;
  if (mesh_desc_problem(d)) return MR_E_INVALID;
  if (f->width > MR_NOALLOC_MAX_SIDE || f->height > MR_NOALLOC_MAX_SIDE ||
      (int64_t)f->width * f->height > MR_NOALLOC_MAX_PIXELS)
    return MR_E_NOALLOC_LIMIT;
  if (d->n_indices / 3 > MR_NOALLOC_MAX_TRIANGLES) return MR_E_NOALLOC_LIMIT;
  const bool has_uv = d->n_texcoords > 0 && d->n_texcoordsI > 0;
  if (texture && (tex_rows <= 0 || tex_cols <= 0)) return MR_E_INVALID;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MR_E_NO_DEVICE;
  unsigned char* S = nullptr;
  if (scratch_address(dev, &S) != cudaSuccess) return MR_E_CUDA;
  cudaStream_t st = (cudaStream_t)cuda_stream;

  // The renderable record (paintMesh, src/Renderer.cpp:336-338).
  DevRenderable R;
  memset(&R, 0, sizeof(R));
  float mv[16], inv[16], nm[16];
  mat4_mul(f->view, transform, mv);
  mat4_inverse(mv, inv);
  mat4_transpose(inv, nm);
  memcpy(R.mv, mv, sizeof(R.mv));
  memcpy(R.nm, nm, sizeof(R.nm));
  DevMesh& M = R.mesh;
  M.pos = d->vertices;
  M.nrm = d->normals;
  M.uv = has_uv ? d->texcoords : nullptr;
  M.idx = d->indices;
  M.nidx = d->normalsI;
  M.tidx = has_uv ? d->texcoordsI : nullptr;
  M.bad = (const uint32_t*)(S + kBadOff);
  M.n_pos = d->n_vertices;
  M.n_nrm = d->n_normals;
  M.n_uv = has_uv ? d->n_texcoords : 0;
  M.n_tri = d->n_indices / 3;
  M.has_uv = has_uv;
  R.tri_base = 0;
  R.lit = f->lighting != 0;
  R.point = f->light_is_point != 0;
  memcpy(R.diffuse, mat->diffuse, sizeof(R.diffuse));
  memcpy(R.specular, mat->specular, sizeof(R.specular));
  memcpy(R.emissive, mat->emissive, sizeof(R.emissive));
  R.shininess = mat->shininess;
  if (f->texturing && texture) {
    R.has_tex = 1;
    R.tex_rows = tex_rows;
    R.tex_cols = tex_cols;
    if (tex_is_rgb8) R.tex8 = (const uint8_t*)texture;
    else R.texf = (const float*)texture;
  }
  const uint32_t base[2] = {0, (uint32_t)M.n_tri};

  const int W = f->width, H = f->height;
  FrameParams F;
  memset(&F, 0, sizeof(F));
  F.v.W = W;
  F.v.H = H;
  F.v.w = (float)W;
  F.v.h = (float)H;
  memcpy(F.v.P, f->projection, sizeof(F.v.P));
  // Renderer::render, src/Renderer.cpp:317-326.
  F.v.persp = f->projection[15] == 0;
  float zn = F.v.persp ? f->projection[11] / (f->projection[10] - 1) : (f->projection[11] + 1) / f->projection[10];
  F.v.znear = -zn;
  if (f->light_is_point) affine(f->view, f->light, F.v.lightdir);
  else normalized(f->light, F.v.lightdir);
  F.v.ambient = f->ambient;
  memcpy(F.v.bg, f->background, sizeof(F.v.bg));
  F.g.n_renderables = 1;
  F.g.n_tris = (uint32_t)M.n_tri;
  // Sub-triangles up to 64 pixels of bounding box are rasterised by the setup
  // kernel; larger ones take records and row blocks from the fixed store
  // (the spill list holds one entry per record, so it cannot overflow).
  F.small_max = 64;
  F.g.rs = (const DevRenderable*)(S + kRsOff);
  F.g.tri_base = (const uint32_t*)(S + kBaseOff);
  F.vis = (unsigned long long*)(S + kVisOff);
  F.recs = (BigRec*)(S + kRecOff);
  F.rec_cap = kRecCap;
  F.items = (LargeItem*)(S + kItemOff);
  F.item_cap = kItemCap;
  F.spill = (LargeItem*)(S + kSpillOff);
  F.rgb8 = rgb8;
  F.depth = depth;
  F.ids = tri_id;
  F.counters = (Counters*)(S + kCntOff);

  cudaError_t e = cudaMemcpyAsync(S + kRsOff, &R, sizeof(R), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S + kBaseOff, base, sizeof(base), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(S + kCntOff, 0, sizeof(Counters), st);
  if (e == cudaSuccess) e = launch_validate(M, (uint32_t*)(S + kBadOff), st);
  if (e == cudaSuccess) e = launch_frame(F, st, nullptr);
  Counters c;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&c, S + kCntOff, sizeof(c), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return MR_E_CUDA;
  return (c.error_flags & 1u) ? MR_E_BAD_INDEX : MR_OK;
}
