// C ABI of the GB300 rasterisation path (include/minirender_gpu.h): context,
// resident meshes/textures, per-frame staging and the launch sequence.
//
// Memory: the context owns every device buffer.  Meshes and textures are
// allocated once at upload; frame buffers grow to the largest frame seen and
// are then reused, so steady-state frames allocate nothing.  The one
// single-frame buffer whose size is data dependent -- the list of 32-row
// blocks of large triangles -- is checked on the device: blocks past its end
// go to a per-record spill list (which cannot overflow), and the list grows
// for later frames.  Batches keep a (tile, record) list; an overflow there is
// detected at the next synchronisation and the batch is re-run.
#include <unistd.h>

#include <condition_variable>
#include <functional>
#include <thread>

#include "internal.h"

namespace {

// Host worker threads for large staging loops, created on first use and
// kept (spawning threads per batch cost more than the work they split).
// One job at a time; the caller runs the first range itself.
class HostPool {
 public:
  static HostPool& get() {
    static HostPool pool;
    return pool;
  }
  // Runs fn(begin, end) over [0, n) in up to size() + 1 contiguous ranges.
  void run(size_t n, const std::function<void(size_t, size_t)>& fn) {
    std::lock_guard<std::mutex> one(job_mu_);
    // a forked child has none of the workers: it runs the job itself
    const size_t parts = getpid() == pid_ ? std::min(n, workers_.size() + 1) : 1;
    if (parts <= 1) {
      fn(0, n);
      return;
    }
    const size_t per = (n + parts - 1) / parts;
    {
      std::lock_guard<std::mutex> lk(mu_);
      fn_ = &fn;
      n_ = n;
      per_ = per;
      parts_ = parts;
      pending_ = parts - 1;
      gen_++;
    }
    cv_.notify_all();
    fn(0, std::min(n, per));
    std::unique_lock<std::mutex> lk(mu_);
    done_.wait(lk, [&] { return pending_ == 0; });
    fn_ = nullptr;
  }

 private:
  HostPool() : pid_(getpid()) {
    const unsigned hw = std::thread::hardware_concurrency();
    const unsigned nw = std::min(7u, hw > 1 ? hw - 1 : 0u);
    for (unsigned t = 0; t < nw; t++) workers_.emplace_back([this, t] { loop(t + 1); });
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& w : workers_) w.join();
  }
  void loop(size_t part) {
    uint64_t seen = 0;
    for (;;) {
      const std::function<void(size_t, size_t)>* fn;
      size_t b, e;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
        if (stop_) return;
        seen = gen_;
        if (part >= parts_) continue;  // fewer parts than workers this time
        fn = fn_;
        b = part * per_;
        e = std::min(n_, b + per_);
      }
      if (b < e) (*fn)(b, e);
      std::lock_guard<std::mutex> lk(mu_);
      if (--pending_ == 0) done_.notify_one();
    }
  }
  const pid_t pid_;
  std::vector<std::thread> workers_;
  std::mutex job_mu_, mu_;
  std::condition_variable cv_, done_;
  const std::function<void(size_t, size_t)>* fn_ = nullptr;
  size_t n_ = 0, per_ = 0, parts_ = 0, pending_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

// Runs fn(begin, end) over [0, n): on the calling thread below `min_split`
// items, else split over the host pool.
template <class Fn>
void parallel_ranges(size_t n, size_t min_split, Fn fn) {
  if (n < min_split) {
    fn(0, n);
    return;
  }
  const std::function<void(size_t, size_t)> f = fn;
  HostPool::get().run(n, f);
}

}  // namespace

extern "C" {

MR_API int mr_abi_version(void) { return MR_ABI_VERSION; }

MR_API const char* mr_status_string(int s) {
  switch (s) {
    case MR_OK: return "ok";
    case MR_E_INVALID: return "invalid argument";
    case MR_E_CUDA: return "CUDA error";
    case MR_E_NOMEM: return "out of device memory";
    case MR_E_HANDLE: return "unknown handle";
    case MR_E_BAD_INDEX: return "mesh index out of range";
    case MR_E_BUDGET: return "over device-memory budget";
    case MR_E_TIMEOUT: return "device wait timed out";
    case MR_E_NOT_READY: return "not ready";
    case MR_E_NO_DEVICE: return "no CUDA device";
    case MR_E_NOALLOC_LIMIT: return "request exceeds the fixed scratch of mr_render_noalloc";
    case MR_E_IO: return "file could not be read, written or parsed";
    default: return "unknown status";
  }
}

MR_API const char* mr_last_error(const mr_ctx* c) { return c ? c->err.c_str() : ""; }

MR_API int mr_create(int device, mr_ctx** out) {
  if (!out) return MR_E_INVALID;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    return MR_E_NO_DEVICE;
  }
  if (device < 0 || device >= n) return MR_E_INVALID;
  mr_ctx* c = new mr_ctx();
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_cnt, sizeof(Counters));
  if (e == cudaSuccess) e = cudaMallocHost(&c->h_cnt, sizeof(Counters));
  for (int i = 0; i < 8 && e == cudaSuccess; i++) e = cudaEventCreate(&c->ev[i]);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->staged, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->read_done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->compute_mark, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->uploaded, cudaEventDisableTiming);

  if (e != cudaSuccess) {
    delete c;
    return e == cudaErrorMemoryAllocation ? MR_E_NOMEM : MR_E_CUDA;
  }
  c->stream = c->own;
  *out = c;
  return MR_OK;
}

MR_API int mr_destroy(mr_ctx* c) {
  if (!c) return MR_E_INVALID;
  {
    std::lock_guard<std::recursive_mutex> g(c->mu);
    cudaSetDevice(c->device);
    if (c->upload_waiting) cudaEventSynchronize(c->uploaded);
    cudaStreamSynchronize(c->stream);
    for (auto& m : c->meshes)
      if (m.mem) cudaFree(m.mem);
    for (auto& t : c->textures)
      if (t.mem) cudaFree(t.mem);
    c->vis.release(); c->rgb8.release(); c->depth.release(); c->rgbf.release();
    c->normals.release(); c->range.release(); c->ids.release(); c->recs.release();
    c->items.release(); c->spill.release(); c->stage.release();
    c->va.release(); c->vb.release(); c->vn.release();
    if (c->h_stage) cudaFreeHost(c->h_stage);
    if (c->d_cnt) cudaFree(c->d_cnt);
    if (c->h_cnt) cudaFreeHost(c->h_cnt);
    for (auto& e : c->ev)
      if (e) cudaEventDestroy(e);
    if (c->staged) cudaEventDestroy(c->staged);
    if (c->read_done) cudaEventDestroy(c->read_done);
    if (c->compute_mark) cudaEventDestroy(c->compute_mark);
    if (c->uploaded) cudaEventDestroy(c->uploaded);
    c->b.release();
    if (c->own) cudaStreamDestroy(c->own);
  }
  delete c;
  return MR_OK;
}

// The compute stream waits (on the device) for the last update issued on the
// upload stream.
static int join_upload(mr_ctx* c) {
  if (!c->upload_waiting) return MR_OK;
  CK(cudaStreamWaitEvent(c->stream, c->uploaded, 0), "upload wait");
  c->upload_waiting = false;
  for (auto& m : c->meshes)
    if (m.live && m.validate_pending) {
      CK(launch_validate(m.d, (uint32_t*)m.d.bad, c->stream), "validate launch");
      m.validate_pending = false;
    }
  return MR_OK;
}

// Stream for a mesh or texture update: the upload stream, after everything
// queued so far on the compute stream (frames that read the old contents);
// without one, the compute stream itself.
static cudaStream_t begin_update(mr_ctx* c) {
  if (!c->upload) return c->stream;
  if (cudaEventRecord(c->compute_mark, c->stream) != cudaSuccess ||
      cudaStreamWaitEvent(c->upload, c->compute_mark, 0) != cudaSuccess)
    return nullptr;
  return c->upload;
}

static int end_update(mr_ctx* c) {
  if (!c->upload) return MR_OK;
  CK(cudaEventRecord(c->uploaded, c->upload), "upload event");
  c->upload_waiting = true;
  return MR_OK;
}

MR_API int mr_set_stream(mr_ctx* c, void* s) {
  if (!c) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  cudaSetDevice(c->device);
  int rc = join_upload(c);
  if (rc) return rc;
  c->stream = s ? (cudaStream_t)s : c->own;
  return MR_OK;
}

MR_API int mr_set_upload_stream(mr_ctx* c, void* s) {
  if (!c) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  cudaSetDevice(c->device);
  int rc = join_upload(c);
  if (rc) return rc;
  c->upload = (cudaStream_t)s;
  return MR_OK;
}

MR_API int mr_synchronize(mr_ctx* c) {
  if (!c) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  cudaSetDevice(c->device);
  int rc = join_upload(c);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  return MR_OK;
}

MR_API int mr_set_tuning(mr_ctx* c, int tile, int small_max) {
  if (!c) return MR_E_INVALID;
  if (tile != 8 && tile != 16 && tile != 32) return fail(c, MR_E_INVALID, "tile must be 8, 16 or 32");
  if (small_max < 0 || small_max > 4096) return fail(c, MR_E_INVALID, "small_max out of range");
  std::lock_guard<std::recursive_mutex> g(c->mu);
  c->tile = tile;
  c->small_max = small_max;
  return MR_OK;
}

MR_API int mr_set_profiling(mr_ctx* c, int on) {
  if (!c) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  c->profiling = on != 0;
  return MR_OK;
}

static constexpr int32_t kRenderableFlags =
    MR_RS_MODELVIEW | MR_RS_NO_CLIP | MR_RS_OWN_STATE | MR_RS_LIGHTING | MR_RS_TEXTURING | MR_RS_POINT_LIGHT;

// The switches paintTriangle reads for a renderable's fragments
// (src/Renderer.cpp:264-289): its own (MR_RS_OWN_STATE) or the frame's.
// Sets R.lit and R.point; returns whether texturing is on.
static bool switches(int32_t flags, const mr_frame& f, DevRenderable& R) {
  const bool own = (flags & MR_RS_OWN_STATE) != 0;
  R.lit = own ? (flags & MR_RS_LIGHTING) != 0 : f.lighting != 0;
  R.point = own ? (flags & MR_RS_POINT_LIGHT) != 0 : f.light_is_point != 0;
  return own ? (flags & MR_RS_TEXTURING) != 0 : f.texturing != 0;
}

// Copies the mesh arrays on st and checks the indices there, or -- when st
// is the upload stream (or the caller defers the check), which carries
// copies only so the next transfer never waits for SMs -- later, before the
// first launch that reads the mesh (join_upload, check_pending_meshes).
static int copy_mesh(mr_ctx* c, MeshRec& m, const mr_mesh_desc* d, cudaStream_t st, bool defer_check = false) {
  DevMesh& M = m.d;
  char* base = (char*)m.mem;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* p = base + off;
    off += align256(bytes);
    return (void*)p;
  };
  M.pos = (const float*)take((size_t)12 * d->n_vertices);
  M.nrm = (const float*)take((size_t)12 * d->n_normals);
  M.uv = (const float*)take((size_t)8 * (M.has_uv ? d->n_texcoords : 0));
  // normalsI / texcoordsI given as the very array of indices (the usual case:
  // one index per corner for every attribute) share its device copy; the
  // kernels then reuse the corner's vertex index
  const bool n_alias = d->normalsI == d->indices, t_alias = M.has_uv && d->texcoordsI == d->indices;
  M.idx = (const int32_t*)take((size_t)4 * d->n_indices);
  M.nidx = n_alias ? M.idx : (const int32_t*)take((size_t)4 * d->n_indices);
  M.tidx = t_alias ? M.idx : (const int32_t*)take((size_t)4 * (M.has_uv ? d->n_indices : 0));
  M.bad = (const uint32_t*)take((size_t)4 * ((M.n_tri + 31) / 32 + 1));
  M.rec = mesh_wants_records(M.n_tri, M.n_pos) ? (const float4*)take(kRecBytes * (size_t)M.n_tri) : nullptr;
  if (d->n_vertices) CK(cudaMemcpyAsync((void*)M.pos, d->vertices, (size_t)12 * d->n_vertices, cudaMemcpyHostToDevice, st), "mesh copy");
  if (d->n_normals) CK(cudaMemcpyAsync((void*)M.nrm, d->normals, (size_t)12 * d->n_normals, cudaMemcpyHostToDevice, st), "mesh copy");
  if (M.has_uv) CK(cudaMemcpyAsync((void*)M.uv, d->texcoords, (size_t)8 * d->n_texcoords, cudaMemcpyHostToDevice, st), "mesh copy");
  if (d->n_indices) {
    CK(cudaMemcpyAsync((void*)M.idx, d->indices, (size_t)4 * d->n_indices, cudaMemcpyHostToDevice, st), "mesh copy");
    if (!n_alias)
      CK(cudaMemcpyAsync((void*)M.nidx, d->normalsI, (size_t)4 * d->n_indices, cudaMemcpyHostToDevice, st), "mesh copy");
    if (M.has_uv && !t_alias)
      CK(cudaMemcpyAsync((void*)M.tidx, d->texcoordsI, (size_t)4 * d->n_indices, cudaMemcpyHostToDevice, st), "mesh copy");
  }
  if (defer_check || (c->upload && st == c->upload)) m.validate_pending = true;
  else CK(launch_validate(M, (uint32_t*)M.bad, st), "validate launch");
  return MR_OK;
}

const char* mesh_desc_problem(const mr_mesh_desc* d) {
  if (!d) return "null mesh descriptor";
  if (d->n_vertices < 0 || d->n_normals < 0 || d->n_texcoords < 0 || d->n_indices < 0 ||
      d->n_normalsI < 0 || d->n_texcoordsI < 0)
    return "negative count";
  if (d->n_indices % 3) return "index count is not a multiple of 3";
  if (d->n_normalsI < d->n_indices) return "normalsI shorter than indices";
  bool has_uv = d->n_texcoords > 0 && d->n_texcoordsI > 0;
  if (has_uv && d->n_texcoordsI < d->n_indices) return "texcoordsI shorter than indices";
  if ((d->n_vertices && !d->vertices) || (d->n_normals && !d->normals) ||
      (has_uv && (!d->texcoords || !d->texcoordsI)) || (d->n_indices && (!d->indices || !d->normalsI)))
    return "null array with non-zero count";
  return nullptr;
}

static int check_desc(mr_ctx* c, const mr_mesh_desc* d) {
  const char* why = mesh_desc_problem(d);
  return why ? fail(c, MR_E_INVALID, why) : MR_OK;
}

static size_t mesh_bytes(const mr_mesh_desc* d, bool has_uv) {
  int ntri = d->n_indices / 3;
  const bool n_alias = d->normalsI == d->indices, t_alias = has_uv && d->texcoordsI == d->indices;
  return align256((size_t)12 * d->n_vertices) + align256((size_t)12 * d->n_normals) +
         align256((size_t)8 * (has_uv ? d->n_texcoords : 0)) + align256((size_t)4 * d->n_indices) +
         (n_alias ? 0 : align256((size_t)4 * d->n_indices)) +
         (t_alias ? 0 : align256((size_t)4 * (has_uv ? d->n_indices : 0))) +
         align256((size_t)4 * ((ntri + 31) / 32 + 1)) +
         (mesh_wants_records(ntri, d->n_vertices) ? align256(kRecBytes * (size_t)ntri) : 0);
}

int mesh_create(mr_ctx* c, const mr_mesh_desc* d, cudaStream_t stream, int32_t* out, size_t* bytes,
                cudaMemPool_t pool, bool defer_check) {
  int rc = check_desc(c, d);
  if (rc) return rc;
  MeshRec m;
  m.live = true;
  m.n_idx = d->n_indices;
  m.d.has_uv = d->n_texcoords > 0 && d->n_texcoordsI > 0;
  m.d.n_pos = d->n_vertices;
  m.d.n_nrm = d->n_normals;
  m.d.n_uv = m.d.has_uv ? d->n_texcoords : 0;
  m.d.n_tri = d->n_indices / 3;
  m.bytes = mesh_bytes(d, m.d.has_uv);
  m.stream_ordered = stream != nullptr;
  cudaStream_t st = stream ? stream : c->stream;
  if (stream)
    CK(pool ? cudaMallocFromPoolAsync(&m.mem, m.bytes, pool, stream) : cudaMallocAsync(&m.mem, m.bytes, stream),
       "mesh allocation");
  else CK(cudaMalloc(&m.mem, m.bytes), "mesh allocation");
  rc = copy_mesh(c, m, d, st, defer_check);
  if (rc) {
    if (stream) cudaFreeAsync(m.mem, stream);
    else cudaFree(m.mem);
    return rc;
  }
  int32_t h = -1;
  for (size_t i = 0; i < c->meshes.size(); i++)
    if (!c->meshes[i].live) { h = (int32_t)i; break; }
  if (h < 0) {
    h = (int32_t)c->meshes.size();
    c->meshes.push_back(m);
  } else {
    c->meshes[h] = m;
  }
  *out = h;
  if (bytes) *bytes = m.bytes;
  return MR_OK;
}

int check_pending_mesh(mr_ctx* c, int32_t h, cudaStream_t st, bool* launched) {
  if (launched) *launched = false;
  if (h < 0 || h >= (int32_t)c->meshes.size() || !c->meshes[h].live) return fail(c, MR_E_HANDLE, "unknown mesh");
  MeshRec& m = c->meshes[h];
  if (!m.validate_pending) return MR_OK;
  CK(launch_validate(m.d, (uint32_t*)m.d.bad, st), "validate launch");
  m.validate_pending = false;
  if (launched) *launched = true;
  return MR_OK;
}

int mesh_destroy(mr_ctx* c, int32_t h, cudaStream_t stream) {
  if (h < 0 || h >= (int32_t)c->meshes.size() || !c->meshes[h].live) return fail(c, MR_E_HANDLE, "unknown mesh");
  MeshRec& m = c->meshes[h];
  if (stream) {
    CK(cudaFreeAsync(m.mem, stream), "mesh free");
  } else {
    join_upload(c);
    cudaStreamSynchronize(c->stream);
    if (m.stream_ordered) cudaDeviceSynchronize();
    cudaFree(m.mem);
  }
  m = MeshRec();
  return MR_OK;
}

MR_API int mr_mesh_upload(mr_ctx* c, const mr_mesh_desc* d, int32_t* out) {
  if (!c || !out) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  cudaSetDevice(c->device);
  return mesh_create(c, d, nullptr, out, nullptr);
}

MR_API int mr_mesh_update(mr_ctx* c, int32_t h, const mr_mesh_desc* d) {
  if (!c) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  if (h < 0 || h >= (int32_t)c->meshes.size() || !c->meshes[h].live) return fail(c, MR_E_HANDLE, "unknown mesh");
  int rc = check_desc(c, d);
  if (rc) return rc;
  MeshRec& m = c->meshes[h];
  bool has_uv = d->n_texcoords > 0 && d->n_texcoordsI > 0;
  if (d->n_vertices != m.d.n_pos || d->n_normals != m.d.n_nrm || d->n_indices != m.n_idx ||
      has_uv != (m.d.has_uv != 0) || (has_uv && d->n_texcoords != m.d.n_uv))
    return fail(c, MR_E_INVALID, "mr_mesh_update needs the same element counts");
  if ((d->normalsI == d->indices) != (m.d.nidx == m.d.idx) ||
      (has_uv && (d->texcoordsI == d->indices) != (m.d.tidx == m.d.idx)))
    return fail(c, MR_E_INVALID, "mr_mesh_update needs normalsI / texcoordsI shared with indices as at upload");
  cudaSetDevice(c->device);
  cudaStream_t st = begin_update(c);
  if (!st) return fail(c, MR_E_CUDA, "upload stream ordering failed");
  rc = copy_mesh(c, m, d, st);
  if (rc) return rc;
  return end_update(c);
}

MR_API int mr_mesh_free(mr_ctx* c, int32_t h) {
  if (!c) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  cudaSetDevice(c->device);
  return mesh_destroy(c, h, nullptr);
}

int texture_create(mr_ctx* c, const void* data, bool rgb8, int32_t rows, int32_t cols, cudaStream_t stream,
                   int32_t* out, cudaMemPool_t pool) {
  if (!out || !data || rows <= 0 || cols <= 0) return fail(c, MR_E_INVALID, "bad texture");
  TexRec t;
  t.live = true;
  t.rgb8 = rgb8;
  t.rows = rows;
  t.cols = cols;
  t.bytes = (size_t)rows * cols * (rgb8 ? 3 : 12);
  t.stream_ordered = stream != nullptr;
  cudaStream_t st = stream ? stream : c->stream;
  if (stream)
    CK(pool ? cudaMallocFromPoolAsync(&t.mem, t.bytes, pool, stream) : cudaMallocAsync(&t.mem, t.bytes, stream),
       "texture allocation");
  else CK(cudaMalloc(&t.mem, t.bytes), "texture allocation");
  cudaError_t e = cudaMemcpyAsync(t.mem, data, t.bytes, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) {
    if (stream) cudaFreeAsync(t.mem, stream);
    else cudaFree(t.mem);
    return cuda_fail(c, e, "texture copy");
  }
  int32_t h = -1;
  for (size_t i = 0; i < c->textures.size(); i++)
    if (!c->textures[i].live) { h = (int32_t)i; break; }
  if (h < 0) {
    h = (int32_t)c->textures.size();
    c->textures.push_back(t);
  } else {
    c->textures[h] = t;
  }
  *out = h;
  return MR_OK;
}

int texture_destroy(mr_ctx* c, int32_t h, cudaStream_t stream) {
  if (h < 0 || h >= (int32_t)c->textures.size() || !c->textures[h].live) return fail(c, MR_E_HANDLE, "unknown texture");
  TexRec& t = c->textures[h];
  if (stream) {
    CK(cudaFreeAsync(t.mem, stream), "texture free");
  } else {
    join_upload(c);
    cudaStreamSynchronize(c->stream);
    if (t.stream_ordered) cudaDeviceSynchronize();
    cudaFree(t.mem);
  }
  t = TexRec();
  return MR_OK;
}

static int tex_upload(mr_ctx* c, const void* data, size_t bytes, bool rgb8, int32_t rows, int32_t cols,
                      int32_t* out) {
  (void)bytes;
  if (!c) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  cudaSetDevice(c->device);
  return texture_create(c, data, rgb8, rows, cols, nullptr, out);
}

MR_API int mr_texture_upload_rgb8(mr_ctx* c, const uint8_t* rgb, int32_t rows, int32_t cols, int32_t* out) {
  return tex_upload(c, rgb, (size_t)3 * rows * cols, true, rows, cols, out);
}

MR_API int mr_texture_upload_f32(mr_ctx* c, const float* rgb, int32_t rows, int32_t cols, int32_t* out) {
  return tex_upload(c, rgb, (size_t)12 * rows * cols, false, rows, cols, out);
}

MR_API int mr_texture_update(mr_ctx* c, int32_t h, const void* texels) {
  if (!c || !texels) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  if (h < 0 || h >= (int32_t)c->textures.size() || !c->textures[h].live) return fail(c, MR_E_HANDLE, "unknown texture");
  const TexRec& t = c->textures[h];
  size_t bytes = (size_t)t.rows * t.cols * (t.rgb8 ? 3 : 12);
  cudaSetDevice(c->device);
  cudaStream_t st = begin_update(c);
  if (!st) return fail(c, MR_E_CUDA, "upload stream ordering failed");
  CK(cudaMemcpyAsync(t.mem, texels, bytes, cudaMemcpyHostToDevice, st), "texture copy");
  return end_update(c);
}

MR_API int mr_texture_free(mr_ctx* c, int32_t h) {
  if (!c) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  cudaSetDevice(c->device);
  return texture_destroy(c, h, nullptr);
}

static int settle(mr_ctx* c);

// Launches the kernels of c->last after resetting the per-frame counters.
static int launch_last(mr_ctx* c) {
  FrameParams& F = c->last;
  cudaStream_t st = c->stream;
  // (the clear kernel also zeroes the counters and the tile tables)
  CK(launch_frame(F, st, c->profiling ? c->ev : nullptr, c->staged), "frame launch");
  return MR_OK;
}

MR_API int mr_render(mr_ctx* c, const mr_frame* f, const mr_renderable* rs, int32_t n, int32_t outputs) {
  if (!c) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  if (!f || (n > 0 && !rs) || n < 0) return fail(c, MR_E_INVALID, "null frame or renderables");
  if (f->width <= 0 || f->height <= 0 || (int64_t)f->width * f->height > (int64_t)1 << 28 ||
      f->width > (1 << 16) || f->height > (1 << 16))
    return fail(c, MR_E_INVALID, "frame size out of range");
  cudaSetDevice(c->device);
  if (c->async_read) {  // the last frame's reads complete before it is replaced
    int rc = settle(c);
    if (rc && rc != MR_E_BAD_INDEX) return rc;
  }
  {
    int rc = join_upload(c);
    if (rc) return rc;
  }
  // Per-renderable matrices and materials, Renderer::paintMesh (src/Renderer.cpp:336-338).
  uint64_t total = 0;
  for (int32_t i = 0; i < n; i++) {
    int32_t h = rs[i].mesh;
    if (h < 0 || h >= (int32_t)c->meshes.size() || !c->meshes[h].live)
      return fail(c, MR_E_HANDLE, "renderable refers to an unknown mesh");
    int32_t t = rs[i].material.texture;
    if (t >= 0 && (t >= (int32_t)c->textures.size() || !c->textures[t].live))
      return fail(c, MR_E_HANDLE, "material refers to an unknown texture");
    if (rs[i].flags & ~kRenderableFlags) return fail(c, MR_E_INVALID, "unknown renderable flags");
    total += (uint64_t)c->meshes[h].d.n_tri;
  }
  if (total >= ((uint64_t)1 << 31)) return fail(c, MR_E_INVALID, "more than 2^31-1 triangles in one frame");
  size_t nrs = (size_t)std::max(n, 1);
  if (c->h_rs_cap < nrs) {
    CK(cudaEventSynchronize(c->staged), "staging wait");
    if (c->h_stage) cudaFreeHost(c->h_stage);
    c->h_stage = nullptr;
    c->h_rs = nullptr;
    c->h_tri_base = nullptr;
    c->h_P = nullptr;
    c->h_rs_cap = 0;
    c->off_bases = align256(sizeof(DevRenderable) * nrs);
    c->off_P = c->off_bases + align256(sizeof(uint32_t) * 3 * (nrs + 1));
    c->stage_bytes = (c->off_P + sizeof(float) * 16 + 15) & ~(size_t)15;
    CK(cudaMallocHost(&c->h_stage, c->stage_bytes), "pinned staging");
    CK(cudaHostGetDevicePointer((void**)&c->d_stage_src, c->h_stage, 0), "mapped staging");
    CK(c->stage.ensure(c->stage_bytes), "staging buffer");
    c->h_rs = (DevRenderable*)c->h_stage;
    c->h_tri_base = (uint32_t*)(c->h_stage + c->off_bases);
    c->h_P = (float*)(c->h_stage + c->off_P);
    c->h_rs_cap = nrs;
  } else {
    CK(cudaEventSynchronize(c->staged), "staging wait");
  }
  uint32_t base = 0;
  uint64_t vbase = 0, nbase = 0;
  uint32_t* h_vbase = c->h_tri_base + (n + 1);
  uint32_t* h_nbase = c->h_tri_base + 2 * (n + 1);
  for (int32_t i = 0; i < n; i++) {
    const MeshRec& m = c->meshes[rs[i].mesh];
    DevRenderable& R = c->h_rs[i];
    float mv[16], inv[16], nm[16];
    if (rs[i].flags & MR_RS_MODELVIEW) memcpy(mv, rs[i].transform, sizeof(mv));
    else mat4_mul(f->view, rs[i].transform, mv);
    mat4_inverse(mv, inv);
    mat4_transpose(inv, nm);
    memcpy(R.mv, mv, sizeof(R.mv));
    memcpy(R.nm, nm, sizeof(R.nm));
    R.mesh = m.d;
    R.no_clip = (rs[i].flags & MR_RS_NO_CLIP) ? 1 : 0;
    const bool texturing = switches(rs[i].flags, *f, R);
    R.tri_base = base;
    c->h_tri_base[i] = base;
    base += (uint32_t)m.d.n_tri;
    R.vert_base = (uint32_t)vbase;
    R.nrm_base = (uint32_t)nbase;
    h_vbase[i] = (uint32_t)vbase;
    h_nbase[i] = (uint32_t)nbase;
    vbase += (uint64_t)m.d.n_pos;
    nbase += (uint64_t)m.d.n_nrm;
    if (vbase >= ((uint64_t)1 << 32) || nbase >= ((uint64_t)1 << 32))
      return fail(c, MR_E_INVALID, "more than 2^32-1 vertices or normals in one frame");
    const mr_material& M = rs[i].material;
    memcpy(R.diffuse, M.diffuse, sizeof(R.diffuse));
    memcpy(R.specular, M.specular, sizeof(R.specular));
    memcpy(R.emissive, M.emissive, sizeof(R.emissive));
    R.shininess = M.shininess;
    R.has_tex = 0;
    R.tex8 = nullptr;
    R.texf = nullptr;
    R.tex_rows = R.tex_cols = 0;
    if (texturing && M.texture >= 0) {
      const TexRec& T = c->textures[M.texture];
      R.has_tex = 1;
      R.tex_rows = T.rows;
      R.tex_cols = T.cols;
      if (T.rgb8) R.tex8 = (const uint8_t*)T.mem;
      else R.texf = (const float*)T.mem;
    }
  }
  c->h_tri_base[n] = base;
  h_vbase[n] = (uint32_t)vbase;
  h_nbase[n] = (uint32_t)nbase;

  const int W = f->width, H = f->height;
  const size_t npx = (size_t)W * H;
  CK(c->vis.ensure(npx), "vis buffer");
  if (outputs & MR_OUT_RGB8) CK(c->rgb8.ensure(3 * npx), "rgb8 buffer");
  if (outputs & MR_OUT_DEPTH) CK(c->depth.ensure(npx), "depth buffer");
  if (outputs & MR_OUT_RGB_F32) CK(c->rgbf.ensure(3 * npx), "rgb buffer");
  if (outputs & MR_OUT_TRI_ID) CK(c->ids.ensure(npx), "id buffer");
  if (f->save_normals) CK(c->normals.ensure(3 * npx), "normals buffer");
  CK(c->recs.ensure((size_t)2 * total), "record buffer");
  CK(c->spill.ensure((size_t)2 * total), "spill buffer");
  if (c->items.cap < ((size_t)1 << 18)) CK(c->items.ensure((size_t)1 << 18), "row-block buffer");
  // The per-vertex pass pays off when vertices are shared (each one used by
  // two or more triangle corners on average); for triangle soups every
  // corner is its own vertex and the kernels transform corners themselves.
  const bool vertex_pass = 3 * (uint64_t)total >= 2 * (uint64_t)vbase;
  if (vertex_pass) {
    CK(c->va.ensure(vbase), "vertex buffer");
    CK(c->vb.ensure(vbase), "vertex buffer");
    CK(c->vn.ensure(nbase), "normal buffer");
  }
  memcpy(c->h_P, f->projection, sizeof(float) * 16);

  FrameParams& F = c->last;
  memset(&F, 0, sizeof(F));
  // the clear kernel fetches the staging block from mapped pinned memory
  F.stage_src = (const uint4*)c->d_stage_src;
  F.stage_dst = (uint4*)c->stage.p;
  F.stage_n16 = (uint32_t)(c->stage_bytes / 16);
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
  F.g.n_renderables = n;
  F.g.n_tris = (uint32_t)total;
  F.small_max = c->small_max;
  const uint32_t* d_bases = (const uint32_t*)(c->stage.p + c->off_bases);
  F.g.rs = (const DevRenderable*)c->stage.p;
  F.g.tri_base = d_bases;
  F.g.vert_base = d_bases + (n + 1);
  F.g.nrm_base = d_bases + 2 * (n + 1);
  F.g.n_verts = (uint32_t)vbase;
  F.g.n_nrms = (uint32_t)nbase;
  F.g.va = vertex_pass ? c->va.p : nullptr;  // null: kernels transform per corner
  F.g.vb = vertex_pass ? c->vb.p : nullptr;
  F.g.vn = vertex_pass ? c->vn.p : nullptr;
  F.vis = c->vis.p;
  F.recs = c->recs.p;
  F.rec_cap = (uint32_t)std::min<size_t>(c->recs.cap, 0xFFFFFFFFu);
  F.items = c->items.p;
  F.item_cap = (uint32_t)std::min<size_t>(c->items.cap, 0xFFFFFFFFu);
  F.spill = c->spill.p;
  F.rgb8 = (outputs & MR_OUT_RGB8) ? c->rgb8.p : nullptr;
  F.depth = (outputs & MR_OUT_DEPTH) ? c->depth.p : nullptr;
  F.rgbf = (outputs & MR_OUT_RGB_F32) ? c->rgbf.p : nullptr;
  F.ids = (outputs & MR_OUT_TRI_ID) ? c->ids.p : nullptr;
  F.normals = f->save_normals ? c->normals.p : nullptr;
  F.counters = c->d_cnt;
  c->last_frame = *f;
  c->outputs = outputs;
  c->have_frame = true;
  c->pending = true;
  return launch_last(c);
}

// Queues the device-to-host copies of the last frame's outputs (null
// pointers are skipped) on the context's stream.
static int queue_reads(mr_ctx* c, const ReadTargets& r) {
  size_t npx = (size_t)c->last.v.W * c->last.v.H;
  cudaStream_t st = c->stream;
  if (r.rgb8) CK(cudaMemcpyAsync(r.rgb8, c->last.rgb8, 3 * npx, cudaMemcpyDeviceToHost, st), "rgb8 read");
  if (r.depth) CK(cudaMemcpyAsync(r.depth, c->last.depth, 4 * npx, cudaMemcpyDeviceToHost, st), "depth read");
  if (r.rgbf) CK(cudaMemcpyAsync(r.rgbf, c->last.rgbf, 12 * npx, cudaMemcpyDeviceToHost, st), "rgb read");
  if (r.ids) CK(cudaMemcpyAsync(r.ids, c->last.ids, 4 * npx, cudaMemcpyDeviceToHost, st), "id read");
  if (r.normals) CK(cudaMemcpyAsync(r.normals, c->last.normals, 12 * npx, cudaMemcpyDeviceToHost, st), "normals read");
  return MR_OK;
}

// Waits for the last frame and reads its counters.  An outstanding
// mr_read_async completes here: its counter copy was queued behind the frame
// and its output copies before the read_done event (work queued on the
// stream after them, such as the next frame's mesh upload, is not waited
// for).  A frame whose row blocks overflowed the list was still rasterised
// completely (through the spill list); the list grows for the next frames.
static int settle(mr_ctx* c) {
  if (!c->have_frame) return fail(c, MR_E_INVALID, "no frame rendered yet");
  if (c->async_read) {
    CK(cudaEventSynchronize(c->read_done), "read wait");
    c->async_read = false;
  } else {
    CK(cudaMemcpyAsync(c->h_cnt, c->d_cnt, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream), "counter read");
    CK(cudaStreamSynchronize(c->stream), "frame wait");
  }
  c->pending = false;
  const Counters& k = *c->h_cnt;
  if (k.item_count > c->last.item_cap) {
    size_t want = (size_t)k.item_count + k.item_count / 4 + 1024;
    CK(c->items.ensure(want), "row-block buffer");
  }
  return (k.error_flags & 1u) ? fail(c, MR_E_BAD_INDEX, "a mesh index was out of range; those triangles were skipped") : MR_OK;
}

static int check_reads(mr_ctx* c, const ReadTargets& r) {
  if (!c->have_frame) return fail(c, MR_E_INVALID, "no frame rendered yet");
  if (r.rgb8 && !c->last.rgb8) return fail(c, MR_E_INVALID, "rgb8 was not requested for this frame");
  if (r.depth && !c->last.depth) return fail(c, MR_E_INVALID, "depth was not requested for this frame");
  if (r.rgbf && !c->last.rgbf) return fail(c, MR_E_INVALID, "float image was not requested for this frame");
  if (r.ids && !c->last.ids) return fail(c, MR_E_INVALID, "ids were not requested for this frame");
  if (r.normals && !c->last.normals) return fail(c, MR_E_INVALID, "normals were not requested for this frame");
  return MR_OK;
}

MR_API int mr_read(mr_ctx* c, uint8_t* rgb8, float* depth, float* rgb_f32, uint32_t* tri_id, float* normals) {
  if (!c) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  cudaSetDevice(c->device);
  const ReadTargets r{rgb8, depth, rgb_f32, tri_id, normals};
  int rc = check_reads(c, r);
  if (rc) return rc;
  rc = settle(c);
  if (rc && rc != MR_E_BAD_INDEX) return rc;
  int q = queue_reads(c, r);
  if (q) return q;
  CK(cudaStreamSynchronize(c->stream), "read wait");
  return rc;
}

MR_API int mr_read_async(mr_ctx* c, uint8_t* rgb8, float* depth, float* rgb_f32, uint32_t* tri_id, float* normals) {
  if (!c) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  cudaSetDevice(c->device);
  const ReadTargets r{rgb8, depth, rgb_f32, tri_id, normals};
  int rc = check_reads(c, r);
  if (rc) return rc;
  if (c->async_read) {  // an earlier read of this frame still outstanding
    rc = settle(c);
    if (rc && rc != MR_E_BAD_INDEX) return rc;
  }
  if (c->pending)
    CK(cudaMemcpyAsync(c->h_cnt, c->d_cnt, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream), "counter read");
  int q = queue_reads(c, r);
  if (q) return q;
  CK(cudaEventRecord(c->read_done, c->stream), "read event");
  c->async_read = true;
  return MR_OK;
}

MR_API int mr_wait(mr_ctx* c) {
  if (!c) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  cudaSetDevice(c->device);
  if (c->have_frame && (c->pending || c->async_read)) return settle(c);
  CK(cudaStreamSynchronize(c->stream), "wait");
  return MR_OK;
}

MR_API int mr_get_outputs(mr_ctx* c, mr_outputs* o) {
  if (!c || !o) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  if (!c->have_frame) return fail(c, MR_E_INVALID, "no frame rendered yet");
  o->width = c->last.v.W;
  o->height = c->last.v.H;
  o->rgb8 = c->last.rgb8;
  o->depth = c->last.depth;
  o->rgb_f32 = c->last.rgbf;
  o->tri_id = c->last.ids;
  o->normals = c->last.normals;
  return MR_OK;
}

MR_API int mr_get_stats(mr_ctx* c, mr_stats* s) {
  if (!c || !s) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  cudaSetDevice(c->device);
  int rc = settle(c);
  if (rc && rc != MR_E_BAD_INDEX) return rc;
  memset(s, 0, sizeof(*s));
  const Counters& k = *c->h_cnt;
  s->triangles = c->last.g.n_tris;
  s->clipped = (int64_t)k.clipped;
  s->rasterised = (int64_t)k.rasterised;
  s->small_direct = (int64_t)k.small_direct;
  s->binned = (int64_t)k.rec_count;
  s->bin_entries = (int64_t)k.item_count;
  s->error_flags = k.error_flags;
  if (c->profiling) {
    s->n_stages = 5;
    for (int i = 0; i < 5; i++) cudaEventElapsedTime(&s->stage_ms[i], c->ev[i], c->ev[i + 1]);
  }
  return rc;
}

MR_API int mr_read_range_image(mr_ctx* c, float* xyz) {
  if (!c || !xyz) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  cudaSetDevice(c->device);
  int rc = settle(c);
  if (rc && rc != MR_E_BAD_INDEX) return rc;
  if (!c->last.depth) return fail(c, MR_E_INVALID, "depth was not requested for this frame");
  size_t npx = (size_t)c->last.v.W * c->last.v.H;
  CK(c->range.ensure(3 * npx), "range buffer");
  CK(launch_range(c->last.v.W, c->last.v.H, (const float*)(c->stage.p + c->off_P), c->last.depth, c->range.p,
                  c->stream), "range launch");
  CK(cudaMemcpyAsync(xyz, c->range.p, 12 * npx, cudaMemcpyDeviceToHost, c->stream), "range read");
  CK(cudaStreamSynchronize(c->stream), "range wait");
  return rc;
}

// ------------------------------------------------------------------ batches
// View of a frame as Renderer::render() prepares it (src/Renderer.cpp:317-326).
static void make_view(const mr_frame* f, View& V) {
  memset(&V, 0, sizeof(V));
  V.W = f->width;
  V.H = f->height;
  V.w = (float)f->width;
  V.h = (float)f->height;
  memcpy(V.P, f->projection, sizeof(V.P));
  V.persp = f->projection[15] == 0;
  float zn = V.persp ? f->projection[11] / (f->projection[10] - 1) : (f->projection[11] + 1) / f->projection[10];
  V.znear = -zn;
  if (f->light_is_point) affine(f->view, f->light, V.lightdir);
  else normalized(f->light, V.lightdir);
  V.ambient = f->ambient;
  memcpy(V.bg, f->background, sizeof(V.bg));
}

extern "C++" {
template <typename T>
static cudaError_t pinned(T*& p, size_t& cap, size_t n) {
  if (n <= cap && p) return cudaSuccess;
  if (p) cudaFreeHost(p);
  p = nullptr;
  cap = 0;
  cudaError_t e = cudaMallocHost(&p, sizeof(T) * std::max<size_t>(n, 1));
  if (e == cudaSuccess) cap = std::max<size_t>(n, 1);
  return e;
}
}  // extern "C++"

MR_API int mr_set_batch_tiling(mr_ctx* c, int tile_w, int tile_h, int threads, int chunk) {
  if (!c) return MR_E_INVALID;
  if (!batch_tile_ok(tile_w, tile_h))
    return fail(c, MR_E_INVALID, "tile sides must be powers of two, 4..256 x 2..64, 64..4096 pixels");
  if (threads != 64 && threads != 128 && threads != 256) return fail(c, MR_E_INVALID, "threads must be 64, 128 or 256");
  if (chunk < 16 || chunk > 256) return fail(c, MR_E_INVALID, "chunk must be in 16..256");
  std::lock_guard<std::recursive_mutex> g(c->mu);
  c->b.tile_w = tile_w;
  c->b.tile_h = tile_h;
  c->b.threads = threads;
  c->b.chunk = chunk;
  return MR_OK;
}

MR_API int mr_set_batch_small_max(mr_ctx* c, int small_max) {
  if (!c) return MR_E_INVALID;
  if (small_max < 0 || small_max > 4096) return fail(c, MR_E_INVALID, "small_max must be in 0..4096");
  std::lock_guard<std::recursive_mutex> g(c->mu);
  c->b.small_max = small_max;
  return MR_OK;
}

MR_API int mr_set_batch_tuning(mr_ctx* c, int tile, int threads, int chunk) {
  if (!c) return MR_E_INVALID;
  if (tile != 8 && tile != 16 && tile != 32) return fail(c, MR_E_INVALID, "tile must be 8, 16 or 32");
  return mr_set_batch_tiling(c, tile, tile, threads, chunk);
}

MR_API int mr_set_batch_graphs(mr_ctx* c, int graphs) {
  if (!c) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  c->b.graphs = graphs != 0;
  return MR_OK;
}

// Enqueues the batch of slot B (staging already filled) on stream st.
static int enqueue_batch(mr_ctx* c, BatchSlot& B, cudaStream_t st, cudaEvent_t* ev) {
  const int n = B.n_rs, S = B.n_scenes;
  CK(cudaMemcpyAsync(B.rs.p, B.h_rs, sizeof(DevRenderable) * n, cudaMemcpyHostToDevice, st), "renderable upload");
  CK(cudaMemcpyAsync(B.bases.p, B.h_u32, sizeof(uint32_t) * (3 * (n + 1) + S + 1), cudaMemcpyHostToDevice, st),
     "base upload");
  CK(cudaMemcpyAsync(B.scenes.p, B.h_scenes, sizeof(SceneRec) * S, cudaMemcpyHostToDevice, st), "scene upload");
  // the host staging may be refilled once these copies are done (inside a
  // graph capture this becomes an external event-record node, which the
  // host can wait for after each launch of the graph)
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(st, &cap), "capture status");
  if (cap == cudaStreamCaptureStatusActive)
    CK(cudaEventRecordWithFlags(B.staged, st, cudaEventRecordExternal), "staging event");
  else
    CK(cudaEventRecord(B.staged, st), "staging event");
  CK(cudaMemsetAsync(B.d_cnt, 0, sizeof(Counters), st), "counter reset");
  CK(cudaMemsetAsync(B.tiles.p, 0, sizeof(uint32_t) * (3 * (size_t)B.P.n_tiles + 1), st), "tile reset");
  CK(launch_batch(B.P, B.threads, B.grid, B.block_sums.p, st, ev), "batch launch");
  return MR_OK;
}

// Runs the staged batch of slot B on st; with profiling, ev[6]/ev[7] bracket
// the whole batch and (outside graphs) ev[0..3] its stages.
int batch_run(mr_ctx* c, BatchSlot& B, cudaStream_t st, bool profiling, cudaEvent_t* ev) {
  std::vector<uint64_t> key = {(uint64_t)B.n_scenes, (uint64_t)B.n_rs, B.P.g.n_tris, B.P.g.n_verts, B.P.g.n_nrms,
                               (uint64_t)B.tile_w, (uint64_t)B.tile_h, (uint64_t)B.threads, (uint64_t)B.chunk,
                               (uint64_t)B.grid, (uint64_t)B.P.small_max, (uint64_t)(uintptr_t)B.P.vis,
                               (uint64_t)profiling, (uint64_t)(uintptr_t)st,
                               (uint64_t)(uintptr_t)B.h_rs, (uint64_t)(uintptr_t)B.h_u32,
                               (uint64_t)(uintptr_t)B.h_scenes, (uint64_t)(uintptr_t)B.rs.p,
                               (uint64_t)(uintptr_t)B.bases.p, (uint64_t)(uintptr_t)B.scenes.p,
                               (uint64_t)(uintptr_t)B.va.p, (uint64_t)(uintptr_t)B.vn.p, (uint64_t)(uintptr_t)B.vb.p,
                               (uint64_t)(uintptr_t)B.recs.p, (uint64_t)B.P.rec_cap, (uint64_t)(uintptr_t)B.bins.p,
                               (uint64_t)B.P.bin_cap, (uint64_t)(uintptr_t)B.tiles.p, B.P.n_tiles};
  for (int s = 0; s < B.n_scenes; s++) {
    key.push_back(((uint64_t)B.W[s] << 32) | (uint64_t)B.H[s]);
    key.push_back((uint64_t)(uintptr_t)B.h_scenes[s].rgb8 ^ ((uint64_t)(uintptr_t)B.h_scenes[s].depth << 1) ^
                  ((uint64_t)(uintptr_t)B.h_scenes[s].ids << 2));
  }
  if (!B.graphs) {
    if (profiling) CK(cudaEventRecord(ev[6], st), "profiling event");
    int rc = enqueue_batch(c, B, st, profiling ? ev : nullptr);
    if (profiling) CK(cudaEventRecord(ev[7], st), "profiling event");
    return rc;
  }
  if (!B.exec || key != B.key) {
    if (B.exec) cudaGraphExecDestroy(B.exec);
    if (B.graph) cudaGraphDestroy(B.graph);
    B.exec = nullptr;
    B.graph = nullptr;
    B.key.clear();
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
    // stage events only outside graphs (inside a capture they would become graph nodes)
    int rc = enqueue_batch(c, B, st, nullptr);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    CK(e, "end capture");
    B.graph = g;
    CK(cudaGraphInstantiate(&B.exec, g, 0), "graph instantiate");
    B.key = key;
  }
  if (profiling) CK(cudaEventRecord(ev[6], st), "profiling event");
  CK(cudaGraphLaunch(B.exec, st), "graph launch");
  if (profiling) CK(cudaEventRecord(ev[7], st), "profiling event");
  return MR_OK;
}

void BatchSlot::release() {
  rs.release(); bases.release(); scenes.release(); stb.release(); va.release(); vn.release();
  vb.release(); recs.release(); rec_scene.release(); tiles.release(); bins.release();
  block_sums.release(); out8.release(); outd.release(); outi.release(); vis.release();
  if (h_rs) cudaFreeHost(h_rs);
  if (h_u32) cudaFreeHost(h_u32);
  if (h_scenes) cudaFreeHost(h_scenes);
  if (d_cnt) cudaFree(d_cnt);
  if (h_cnt) cudaFreeHost(h_cnt);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (done) cudaEventDestroy(done);
  if (staged) cudaEventDestroy(staged);
  for (auto& e : ev)
    if (e) cudaEventDestroy(e);
  h_rs = nullptr; h_u32 = nullptr; h_scenes = nullptr; d_cnt = nullptr; h_cnt = nullptr;
  exec = nullptr; graph = nullptr; done = nullptr; staged = nullptr;
  for (auto& e : ev) e = nullptr;
}

// Validates a batch and fills slot B's staging, buffers and launch parameters.
int batch_stage(mr_ctx* c, BatchSlot& B, const mr_batch_scene* sc, int32_t n_scenes, const mr_renderable* rs,
                int32_t n_rs, int32_t outputs) {
  if (!sc || n_scenes <= 0 || n_rs < 0 || (n_rs > 0 && !rs)) return fail(c, MR_E_INVALID, "bad batch");
  if (!B.d_cnt) CK(cudaMalloc(&B.d_cnt, sizeof(Counters)), "batch counters");
  if (!B.h_cnt) CK(cudaMallocHost(&B.h_cnt, sizeof(Counters)), "batch counters");
  if (!B.done) CK(cudaEventCreateWithFlags(&B.done, cudaEventDisableTiming), "batch event");
  if (!B.staged) CK(cudaEventCreateWithFlags(&B.staged, cudaEventDisableTiming), "batch event");
  uint64_t tris = 0, verts = 0, nrms = 0, pixels = 0, tiles = 0;
  const int TW = B.tile_w, TH = B.tile_h;
  for (int32_t s = 0; s < n_scenes; s++) {
    const mr_frame* f = &sc[s].frame;
    if (f->width <= 0 || f->height <= 0 || f->width > (1 << 16) || f->height > (1 << 16))
      return fail(c, MR_E_INVALID, "scene frame size out of range");
    if (sc[s].first_renderable < 0 || sc[s].n_renderables < 0 ||
        (int64_t)sc[s].first_renderable + sc[s].n_renderables > n_rs ||
        (s > 0 && sc[s].first_renderable != sc[s - 1].first_renderable + sc[s - 1].n_renderables) ||
        (s == 0 && sc[s].first_renderable != 0))
      return fail(c, MR_E_INVALID, "scene renderable ranges must tile the renderable array in order");
    pixels += (uint64_t)f->width * f->height;
    tiles += (uint64_t)((f->width + TW - 1) / TW) * ((f->height + TH - 1) / TH);
  }
  if (sc[n_scenes - 1].first_renderable + sc[n_scenes - 1].n_renderables != n_rs)
    return fail(c, MR_E_INVALID, "scene renderable ranges must cover every renderable");
  for (int32_t i = 0; i < n_rs; i++) {
    int32_t h = rs[i].mesh;
    if (h < 0 || h >= (int32_t)c->meshes.size() || !c->meshes[h].live)
      return fail(c, MR_E_HANDLE, "renderable refers to an unknown mesh");
    int32_t t = rs[i].material.texture;
    if (t >= 0 && (t >= (int32_t)c->textures.size() || !c->textures[t].live))
      return fail(c, MR_E_HANDLE, "material refers to an unknown texture");
    if (rs[i].flags & ~kRenderableFlags) return fail(c, MR_E_INVALID, "unknown renderable flags");
    tris += (uint64_t)c->meshes[h].d.n_tri;
    verts += (uint64_t)c->meshes[h].d.n_pos;
    nrms += (uint64_t)c->meshes[h].d.n_nrm;
  }
  if (tris >= ((uint64_t)1 << 31) || verts >= ((uint64_t)1 << 32) || nrms >= ((uint64_t)1 << 32) ||
      tiles >= ((uint64_t)1 << 31))
    return fail(c, MR_E_INVALID, "batch too large for 32-bit indices");
  // staging (wait until the previous batch of this slot has copied it; its
  // kernels may still run, so the host stages while the device renders)
  CK(cudaEventSynchronize(B.staged), "staging wait");
  CK(pinned(B.h_rs, B.h_rs_cap, (size_t)n_rs), "pinned staging");
  CK(pinned(B.h_u32, B.h_u32_cap, (size_t)3 * (n_rs + 1) + n_scenes + 1), "pinned staging");
  CK(pinned(B.h_scenes, B.h_scenes_cap, (size_t)n_scenes), "pinned staging");
  uint32_t* tb = B.h_u32;
  uint32_t* vbase = tb + (n_rs + 1);
  uint32_t* nbase = tb + 2 * (n_rs + 1);
  uint32_t* stb = tb + 3 * (n_rs + 1);
  B.rs_scene.resize((size_t)n_rs);
  B.W.assign(n_scenes, 0);
  B.H.assign(n_scenes, 0);
  B.px_off.assign(n_scenes + 1, 0);
  for (int32_t s = 0; s < n_scenes; s++) {
    B.W[s] = sc[s].frame.width;
    B.H[s] = sc[s].frame.height;
    B.px_off[s + 1] = B.px_off[s] + (size_t)B.W[s] * B.H[s];
  }
  if (outputs & MR_OUT_RGB8) CK(B.out8.ensure(3 * pixels), "batch rgb8");
  if (outputs & MR_OUT_DEPTH) CK(B.outd.ensure(pixels), "batch depth");
  if (outputs & MR_OUT_TRI_ID) CK(B.outi.ensure(pixels), "batch ids");
  CK(B.rs.ensure((size_t)n_rs), "batch renderables");
  CK(B.bases.ensure((size_t)3 * (n_rs + 1) + n_scenes + 1), "batch bases");
  CK(B.scenes.ensure((size_t)n_scenes), "batch scenes");
  // per-vertex pass only when vertices are shared (see mr_render)
  const bool vertex_pass = 3 * tris >= 2 * verts;
  if (vertex_pass) {
    CK(B.va.ensure(verts), "batch vertex buffer");
    CK(B.vb.ensure(verts), "batch vertex buffer");
    CK(B.vn.ensure(nrms), "batch normal buffer");
  }
  CK(B.recs.ensure(2 * tris), "batch records");
  CK(B.rec_scene.ensure(2 * tris), "batch records");
  CK(B.tiles.ensure(3 * tiles + 1), "batch tiles");
  if (B.small_max > 0) CK(B.vis.ensure(pixels), "batch visibility");
  if (B.bins.cap < std::max<size_t>((size_t)1 << 20, 2 * tris))
    CK(B.bins.ensure(std::max<size_t>((size_t)1 << 20, 2 * tris)), "batch bins");
  int grid = batch_grid(TW, TH, B.chunk, B.threads, vertex_pass);
  if (grid <= 0) return fail(c, MR_E_INVALID, "batch tuning does not fit on the device");
  CK(B.block_sums.ensure((size_t)grid + 1), "batch scan");
  uint32_t tri = 0, vb = 0, nb = 0, tile_base = 0;
  for (int32_t s = 0; s < n_scenes; s++) {
    const mr_frame* f = &sc[s].frame;
    SceneRec& SR = B.h_scenes[s];
    memset(&SR, 0, sizeof(SR));
    make_view(f, SR.v);
    SR.tiles_x = (f->width + TW - 1) / TW;
    SR.tiles_y = (f->height + TH - 1) / TH;
    SR.tile_base = tile_base;
    stb[s] = tile_base;
    tile_base += (uint32_t)(SR.tiles_x * SR.tiles_y);
    SR.rs_begin = (uint32_t)sc[s].first_renderable;
    SR.rs_end = (uint32_t)(sc[s].first_renderable + sc[s].n_renderables);
    SR.rgb8 = (outputs & MR_OUT_RGB8) ? B.out8.p + 3 * B.px_off[s] : nullptr;
    SR.depth = (outputs & MR_OUT_DEPTH) ? B.outd.p + B.px_off[s] : nullptr;
    SR.ids = (outputs & MR_OUT_TRI_ID) ? B.outi.p + B.px_off[s] : nullptr;
    SR.vis = B.small_max > 0 ? B.vis.p + B.px_off[s] : nullptr;
    for (int32_t i = sc[s].first_renderable; i < sc[s].first_renderable + sc[s].n_renderables; i++) {
      const MeshRec& m = c->meshes[rs[i].mesh];
      B.rs_scene[i] = s;
      tb[i] = tri;
      vbase[i] = vb;
      nbase[i] = nb;
      tri += (uint32_t)m.d.n_tri;
      vb += (uint32_t)m.d.n_pos;
      nb += (uint32_t)m.d.n_nrm;
    }
  }
  // per-renderable matrices and materials (Renderer::paintMesh,
  // src/Renderer.cpp:336-338), split over host threads for large batches
  parallel_ranges((size_t)n_rs, 2048, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; i++) {
      const int32_t s = B.rs_scene[i];
      const mr_frame* f = &sc[s].frame;
      const MeshRec& m = c->meshes[rs[i].mesh];
      DevRenderable& R = B.h_rs[i];
      memset(&R, 0, sizeof(R));
      float mv[16], inv[16], nm[16];
      if (rs[i].flags & MR_RS_MODELVIEW) memcpy(mv, rs[i].transform, sizeof(mv));
      else mat4_mul(f->view, rs[i].transform, mv);
      mat4_inverse(mv, inv);
      mat4_transpose(inv, nm);
      memcpy(R.mv, mv, sizeof(R.mv));
      memcpy(R.nm, nm, sizeof(R.nm));
      R.mesh = m.d;
      R.no_clip = (rs[i].flags & MR_RS_NO_CLIP) ? 1 : 0;
      const bool texturing = switches(rs[i].flags, *f, R);
      R.tri_base = tb[i];
      R.vert_base = vbase[i];
      R.nrm_base = nbase[i];
      R.scene = (uint32_t)s;
      const mr_material& M = rs[i].material;
      memcpy(R.diffuse, M.diffuse, sizeof(R.diffuse));
      memcpy(R.specular, M.specular, sizeof(R.specular));
      memcpy(R.emissive, M.emissive, sizeof(R.emissive));
      R.shininess = M.shininess;
      if (texturing && M.texture >= 0) {
        const TexRec& T = c->textures[M.texture];
        R.has_tex = 1;
        R.tex_rows = T.rows;
        R.tex_cols = T.cols;
        if (T.rgb8) R.tex8 = (const uint8_t*)T.mem;
        else R.texf = (const float*)T.mem;
      }
    }
  });
  tb[n_rs] = tri;
  vbase[n_rs] = vb;
  nbase[n_rs] = nb;
  stb[n_scenes] = tile_base;
  BatchParams& P = B.P;
  memset(&P, 0, sizeof(P));
  P.g.rs = B.rs.p;
  P.g.tri_base = B.bases.p;
  P.g.vert_base = B.bases.p + (n_rs + 1);
  P.g.nrm_base = B.bases.p + 2 * (n_rs + 1);
  P.g.n_renderables = n_rs;
  P.g.n_tris = tri;
  P.g.n_verts = vb;
  P.g.n_nrms = nb;
  P.g.va = vertex_pass ? B.va.p : nullptr;
  P.g.vb = vertex_pass ? B.vb.p : nullptr;
  P.g.vn = vertex_pass ? B.vn.p : nullptr;
  P.scenes = B.scenes.p;
  P.scene_tile_base = B.bases.p + 3 * (n_rs + 1);
  P.n_scenes = n_scenes;
  P.n_tiles = tile_base;
  P.tile_w = TW;
  P.tile_h = TH;
  P.chunk = B.chunk;
  P.small_max = B.small_max;
  P.vis = B.small_max > 0 ? B.vis.p : nullptr;
  P.n_px = (size_t)pixels;
  P.recs = B.recs.p;
  P.rec_cap = (uint32_t)std::min<size_t>(B.recs.cap, 0xFFFFFFFFu);
  P.rec_scene = B.rec_scene.p;
  P.tile_count = B.tiles.p;
  P.tile_fill = B.tiles.p + tile_base;
  P.tile_start = B.tiles.p + 2 * (size_t)tile_base;
  P.bins = B.bins.p;
  P.bin_cap = (uint32_t)std::min<size_t>(B.bins.cap, 0xFFFFFFFFu);
  P.counters = B.d_cnt;
  B.grid = grid;
  B.n_scenes = n_scenes;
  B.n_rs = n_rs;
  return MR_OK;
}

MR_API int mr_render_batch(mr_ctx* c, const mr_batch_scene* sc, int32_t n_scenes, const mr_renderable* rs,
                           int32_t n_rs, int32_t outputs) {
  if (!c) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  cudaSetDevice(c->device);
  BatchSlot& B = c->b;
  int rc = join_upload(c);
  if (rc) return rc;
  rc = batch_stage(c, B, sc, n_scenes, rs, n_rs, outputs);
  if (rc) return rc;
  rc = batch_run(c, B, c->stream, c->profiling, c->ev);
  if (rc) return rc;
  CK(cudaEventRecord(B.done, c->stream), "batch event");
  B.have = true;
  return MR_OK;
}

// Waits for the last batch of slot B; re-runs it while the bin list overflowed.
int batch_settle(mr_ctx* c, BatchSlot& B, cudaStream_t st) {
  if (!B.have) return fail(c, MR_E_INVALID, "no batch rendered yet");
  for (int attempt = 0; attempt < 8; attempt++) {
    CK(cudaMemcpyAsync(B.h_cnt, B.d_cnt, sizeof(Counters), cudaMemcpyDeviceToHost, st), "counter read");
    CK(cudaStreamSynchronize(st), "batch wait");
    if (!B.h_cnt->bin_overflow)
      return (B.h_cnt->error_flags & 1u) ? fail(c, MR_E_BAD_INDEX, "a mesh index was out of range; those triangles were skipped") : MR_OK;
    size_t want = (size_t)B.h_cnt->bin_needed + B.h_cnt->bin_needed / 4 + 1024;
    CK(B.bins.ensure(want), "batch bins");
    B.P.bins = B.bins.p;
    B.P.bin_cap = (uint32_t)std::min<size_t>(B.bins.cap, 0xFFFFFFFFu);
    int rc = batch_run(c, B, st, false, nullptr);
    if (rc) return rc;
  }
  return fail(c, MR_E_NOMEM, "row-block list kept overflowing");
}

MR_API int mr_read_batch(mr_ctx* c, int32_t s, uint8_t* rgb8, float* depth, uint32_t* ids) {
  if (!c) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  cudaSetDevice(c->device);
  int rc = batch_settle(c, c->b, c->stream);
  if (rc && rc != MR_E_BAD_INDEX) return rc;
  auto& B = c->b;
  if (s < 0 || s >= B.n_scenes) return fail(c, MR_E_INVALID, "scene index out of range");
  size_t npx = (size_t)B.W[s] * B.H[s];
  const SceneRec& SR = B.h_scenes[s];
  cudaStream_t st = c->stream;
  if (rgb8) {
    if (!SR.rgb8) return fail(c, MR_E_INVALID, "rgb8 was not requested for this batch");
    CK(cudaMemcpyAsync(rgb8, SR.rgb8, 3 * npx, cudaMemcpyDeviceToHost, st), "rgb8 read");
  }
  if (depth) {
    if (!SR.depth) return fail(c, MR_E_INVALID, "depth was not requested for this batch");
    CK(cudaMemcpyAsync(depth, SR.depth, 4 * npx, cudaMemcpyDeviceToHost, st), "depth read");
  }
  if (ids) {
    if (!SR.ids) return fail(c, MR_E_INVALID, "ids were not requested for this batch");
    CK(cudaMemcpyAsync(ids, SR.ids, 4 * npx, cudaMemcpyDeviceToHost, st), "id read");
  }
  CK(cudaStreamSynchronize(st), "read wait");
  return rc;
}

MR_API int mr_get_batch_outputs(mr_ctx* c, int32_t s, mr_outputs* o) {
  if (!c || !o) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  auto& B = c->b;
  if (!B.have || s < 0 || s >= B.n_scenes) return fail(c, MR_E_INVALID, "no such scene in the last batch");
  memset(o, 0, sizeof(*o));
  o->width = B.W[s];
  o->height = B.H[s];
  o->rgb8 = B.h_scenes[s].rgb8;
  o->depth = B.h_scenes[s].depth;
  o->tri_id = B.h_scenes[s].ids;
  return MR_OK;
}

MR_API int mr_get_batch_stats(mr_ctx* c, mr_stats* s) {
  if (!c || !s) return MR_E_INVALID;
  std::lock_guard<std::recursive_mutex> g(c->mu);
  cudaSetDevice(c->device);
  int rc = batch_settle(c, c->b, c->stream);
  if (rc && rc != MR_E_BAD_INDEX) return rc;
  memset(s, 0, sizeof(*s));
  const Counters& k = *c->b.h_cnt;
  s->triangles = c->b.P.g.n_tris;
  s->clipped = (int64_t)k.clipped;
  s->rasterised = (int64_t)k.rasterised;
  s->binned = (int64_t)k.rec_count;
  s->bin_entries = (int64_t)k.bin_needed;
  s->error_flags = k.error_flags;
  if (c->profiling) {
    // stage_ms[0..2]: vertex pass, setup, fused kernel (launches without a
    // graph only); stage_ms[3]: the whole batch on the device
    s->n_stages = 4;
    if (!c->b.graphs)
      for (int i = 0; i < 3; i++) cudaEventElapsedTime(&s->stage_ms[i], c->ev[i], c->ev[i + 1]);
    cudaEventElapsedTime(&s->stage_ms[3], c->ev[6], c->ev[7]);
  }
  return rc;
}

}  // extern "C"
