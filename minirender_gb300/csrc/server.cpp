// Render server: continuous batching of independent frame requests.
//
// Client threads submit requests (mr_server_submit) into a FIFO queue.  One
// worker thread owns `slots` batch slots, each with its own CUDA stream and
// buffers.  Whenever a slot is free it admits requests from the head of the
// queue while the device-memory budget allows (resident meshes and textures
// plus the estimated footprint of every request in flight), uploads meshes
// and textures that are not resident yet (stream-ordered allocation on the
// slot's stream), stages the batch, launches it and queues the copies of each
// request's outputs to its host buffers -- then returns to the queue while
// the batch runs.  A new mesh's copies are queued without a kernel between
// them; its index check runs right before the batch that first reads it.
// While every slot is busy, the meshes and textures of the next queued
// requests are uploaded ahead on a stream of their own.  Finished slots are
// detected with non-blocking event queries; their requests are marked done
// with their latency.  The server lock is not held during CUDA calls.
//
// Meshes and textures stay resident in an LRU cache keyed by the caller's
// ids; an entry no queued or running request refers to is evicted when the
// budget needs room, with a stream-ordered free (no device-wide sync).
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>
#include <unordered_map>

#include "internal.h"

namespace {

double now_us() {
  return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
  uint64_t ticket = 0;
  mr_request req{};
  size_t cost = 0;      // footprint while queued/running
  size_t scene_px = 0;
  double t_submit = 0, t_launch = 0, t_done = 0;
  int status = 1;       // 1 queued, 2 running, 0 done
  int result = MR_OK;
  int batch_size = 0;
  uint64_t mesh_key = 0, tex_key = 0;
  bool mesh_ref = false, tex_ref = false;  // a reference taken by the upload-ahead stage
};

struct Cached {
  int32_t handle = -1;
  size_t bytes = 0;
  int refs = 0;
  uint64_t last_use = 0;
  cudaEvent_t ready = nullptr;  // recorded on the uploading stream after the upload
};

struct Slot {
  BatchSlot b;
  cudaStream_t stream = nullptr;
  std::vector<Request*> reqs;
  bool busy = false;
};

size_t mesh_footprint(const mr_mesh_desc& d) {
  const size_t nt = (size_t)(d.n_indices / 3);
  return (size_t)12 * d.n_vertices + (size_t)12 * d.n_normals + (size_t)8 * d.n_texcoords +
         (size_t)12 * d.n_indices + nt / 8 + 4096 +
         (mesh_wants_records((long long)nt, d.n_vertices) ? kRecBytes * nt : 0);
}

// Device bytes a request occupies while it runs: its outputs and the
// per-triangle, per-vertex, per-pixel (visibility words) and per-tile
// working buffers of a batch.
size_t request_footprint(const mr_request& r) {
  const size_t px = (size_t)r.frame.width * r.frame.height;
  const size_t nt = (size_t)(r.mesh.n_indices / 3);
  size_t out = 8 * px;
  if (r.outputs & MR_OUT_RGB8) out += 3 * px;
  if (r.outputs & MR_OUT_DEPTH) out += 4 * px;
  if (r.outputs & MR_OUT_TRI_ID) out += 4 * px;
  return out + nt * (2 * sizeof(BigRec) + 16) + (size_t)r.mesh.n_vertices * 24 +
         (size_t)r.mesh.n_normals * 16 + (px / 64 + 16) * 12 + sizeof(DevRenderable) + sizeof(SceneRec);
}

}  // namespace

struct mr_server {
  mr_ctx* c = nullptr;
  mr_server_opts o{};
  std::mutex m;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> queue;
  std::unordered_map<uint64_t, Request*> reqs;
  std::unordered_map<uint64_t, Cached> meshes, textures;
  size_t committed = 0, resident = 0;
  uint64_t use_clock = 0;
  std::vector<Slot*> slots;
  // Meshes and textures come from a pool of the server's own that keeps up
  // to the budget mapped between uses (the default pool would return freed
  // memory to the system at every synchronisation and map it again).
  cudaMemPool_t pool = nullptr;
  // uploads made ahead of a free slot for queued requests
  cudaStream_t upload = nullptr;
  std::thread worker;
  bool stop = false;
  uint64_t next_ticket = 1;
  // statistics since the last reset
  std::vector<double> lat;
  int64_t submitted = 0, completed = 0, rejected = 0, batches = 0, batched = 0;
  double t_first = 0, t_last = 0;

  void run();
  void upload_ahead(std::unique_lock<std::mutex>& lk);
  bool evict_for(size_t need, Slot* s);
  void launch(Slot* s, std::vector<Request*>& batch);
  void retire(Slot* s);
};

// Frees least-recently-used resident entries nobody refers to until `need`
// more bytes fit the budget.  Called with m held.
bool mr_server::evict_for(size_t need, Slot* s) {
  while (committed + need > o.budget_bytes) {
    std::unordered_map<uint64_t, Cached>* pool = nullptr;
    uint64_t key = 0, best = ~0ull;
    for (auto* p : {&meshes, &textures})
      for (auto& kv : *p)
        if (kv.second.refs == 0 && kv.second.last_use < best) {
          best = kv.second.last_use;
          key = kv.first;
          pool = p;
        }
    if (!pool) return false;
    Cached e = (*pool)[key];
    pool->erase(key);
    {
      std::lock_guard<std::recursive_mutex> g(c->mu);
      if (pool == &meshes) mesh_destroy(c, e.handle, s->stream);
      else texture_destroy(c, e.handle, s->stream);
      if (e.ready) cudaEventDestroy(e.ready);
    }
    committed -= e.bytes;
    resident -= e.bytes;
  }
  return true;
}

// Uploads what is missing, stages and launches the batch on the slot, and
// queues the output copies.  Called without m held (the worker owns slots).
void mr_server::launch(Slot* s, std::vector<Request*>& batch) {
  std::vector<mr_batch_scene> scenes(batch.size());
  std::vector<mr_renderable> rs(batch.size());
  int32_t outputs = 0;
  int rc = MR_OK;
  {
    std::lock_guard<std::recursive_mutex> g(c->mu);
    cudaSetDevice(c->device);
    for (size_t i = 0; i < batch.size(); i++) {
      Request* r = batch[i];
      int32_t mh, th = -1;
      cudaEvent_t mready, tready = nullptr;
      {
        std::lock_guard<std::mutex> lk(m);
        mh = meshes[r->mesh_key].handle;
        mready = meshes[r->mesh_key].ready;
        if (r->tex_key) {
          th = textures[r->tex_key].handle;
          tready = textures[r->tex_key].ready;
        }
      }
      // a mesh uploaded for this batch: its deferred index check, then its
      // ready event (other slots' batches wait on it); one uploaded for an
      // earlier batch may have run on another slot's stream
      // (a mesh uploaded ahead ran on the upload stream: wait for its copies
      // before its check; waiting on a never-recorded event is a no-op)
      if (mready) cudaStreamWaitEvent(s->stream, mready, 0);
      bool checked = false;
      if (check_pending_mesh(c, mh, s->stream, &checked) != MR_OK) rc = MR_E_CUDA;
      if (checked && mready && cudaEventRecord(mready, s->stream) != cudaSuccess) rc = MR_E_CUDA;
      if (tready) cudaStreamWaitEvent(s->stream, tready, 0);
      scenes[i].frame = r->req.frame;
      scenes[i].first_renderable = (int32_t)i;
      scenes[i].n_renderables = 1;
      rs[i].mesh = mh;
      rs[i].flags = 0;
      memcpy(rs[i].transform, r->req.transform, sizeof(rs[i].transform));
      rs[i].material = r->req.material;
      rs[i].material.texture = th;
      outputs |= r->req.outputs;
    }
    rc = batch_stage(c, s->b, scenes.data(), (int32_t)scenes.size(), rs.data(), (int32_t)rs.size(), outputs);
    if (rc == MR_OK) rc = batch_run(c, s->b, s->stream, false, nullptr);
    if (rc == MR_OK) {
      for (size_t i = 0; i < batch.size(); i++) {
        const mr_request& q = batch[i]->req;
        const SceneRec& SR = s->b.h_scenes[i];
        const size_t npx = (size_t)q.frame.width * q.frame.height;
        if (q.rgb8 && SR.rgb8) cudaMemcpyAsync(q.rgb8, SR.rgb8, 3 * npx, cudaMemcpyDeviceToHost, s->stream);
        if (q.depth && SR.depth) cudaMemcpyAsync(q.depth, SR.depth, 4 * npx, cudaMemcpyDeviceToHost, s->stream);
        if (q.tri_id && SR.ids) cudaMemcpyAsync(q.tri_id, SR.ids, 4 * npx, cudaMemcpyDeviceToHost, s->stream);
      }
      cudaMemcpyAsync(s->b.h_cnt, s->b.d_cnt, sizeof(Counters), cudaMemcpyDeviceToHost, s->stream);
      if (cudaEventRecord(s->b.done, s->stream) != cudaSuccess) rc = MR_E_CUDA;
      s->b.have = true;
    }
  }
  std::lock_guard<std::mutex> lk(m);
  const double t = now_us();
  for (auto* r : batch) {
    r->t_launch = t;
    r->batch_size = (int)batch.size();
    r->status = 2;
  }
  s->reqs = batch;
  s->busy = true;
  batches++;
  batched += (int64_t)batch.size();
  if (rc != MR_OK) {
    for (auto* r : batch) r->result = rc;
    cudaEventRecord(s->b.done, s->stream);
  }
}

// Completes a slot whose event has fired.  Called with m held.
void mr_server::retire(Slot* s) {
  int rc = MR_OK;
  if (s->b.h_cnt && s->b.h_cnt->bin_overflow) {
    // rare: the batch's bin list overflowed -- re-run it at the right size
    std::lock_guard<std::recursive_mutex> g(c->mu);
    rc = batch_settle(c, s->b, s->stream);
    if (rc == MR_OK || rc == MR_E_BAD_INDEX) {
      for (size_t i = 0; i < s->reqs.size(); i++) {
        const mr_request& q = s->reqs[i]->req;
        const SceneRec& SR = s->b.h_scenes[i];
        const size_t npx = (size_t)q.frame.width * q.frame.height;
        if (q.rgb8 && SR.rgb8) cudaMemcpyAsync(q.rgb8, SR.rgb8, 3 * npx, cudaMemcpyDeviceToHost, s->stream);
        if (q.depth && SR.depth) cudaMemcpyAsync(q.depth, SR.depth, 4 * npx, cudaMemcpyDeviceToHost, s->stream);
        if (q.tri_id && SR.ids) cudaMemcpyAsync(q.tri_id, SR.ids, 4 * npx, cudaMemcpyDeviceToHost, s->stream);
      }
      cudaStreamSynchronize(s->stream);
    }
  } else if (s->b.h_cnt && (s->b.h_cnt->error_flags & 1u)) {
    rc = MR_E_BAD_INDEX;
  }
  const double t = now_us();
  for (auto* r : s->reqs) {
    if (r->result == MR_OK) r->result = rc;
    r->t_done = t;
    r->status = 0;
    committed -= r->cost;
    auto it = meshes.find(r->mesh_key);
    if (it != meshes.end()) it->second.refs--;
    if (r->tex_key) {
      auto jt = textures.find(r->tex_key);
      if (jt != textures.end()) jt->second.refs--;
    }
    lat.push_back(r->t_done - r->t_submit);
    completed++;
    t_last = t;
  }
  s->reqs.clear();
  s->busy = false;
  cv_done.notify_all();
}

// While every slot is busy: makes the meshes and textures of the next
// queued requests (up to two batches ahead, in queue order) resident on the
// upload stream, so the host link keeps working and a slot that frees finds
// them there.  Each upload holds a reference for its request (no eviction
// before use) and records `ready` after its copies; the index check runs
// with the batch (launch).  Never evicts: it stops at the budget.  Called
// with m held; releases it around the CUDA calls.
void mr_server::upload_ahead(std::unique_lock<std::mutex>& lk) {
  // by position: a submit may append while the lock is released (which
  // would invalidate deque iterators); only this thread removes entries
  for (size_t i = 0; i < queue.size() && i < (size_t)(2 * o.max_batch); i++) {
    Request* r = queue[i];
    const bool need_mesh = !r->mesh_ref && !meshes.count(r->mesh_key);
    const bool need_tex = r->tex_key && !r->tex_ref && !textures.count(r->tex_key);
    if (!need_mesh && !need_tex) continue;
    const size_t tex_bytes = (size_t)r->req.tex_rows * r->req.tex_cols * 3;
    const size_t extra = (need_mesh ? mesh_footprint(r->req.mesh) : 0) + (need_tex ? tex_bytes : 0);
    if (committed + extra > o.budget_bytes) break;
    Cached me, te;
    int rc = MR_OK;
    lk.unlock();
    {
      std::lock_guard<std::recursive_mutex> g(c->mu);
      if (need_mesh) {
        rc = mesh_create(c, &r->req.mesh, upload, &me.handle, &me.bytes, pool, true);
        if (rc == MR_OK && (cudaEventCreateWithFlags(&me.ready, cudaEventDisableTiming) != cudaSuccess ||
                            cudaEventRecord(me.ready, upload) != cudaSuccess))
          rc = MR_E_CUDA;
      }
      if (rc == MR_OK && need_tex) {
        te.bytes = tex_bytes;
        rc = texture_create(c, r->req.texture_rgb8, true, r->req.tex_rows, r->req.tex_cols, upload, &te.handle,
                            pool);
        if (rc == MR_OK && (cudaEventCreateWithFlags(&te.ready, cudaEventDisableTiming) != cudaSuccess ||
                            cudaEventRecord(te.ready, upload) != cudaSuccess))
          rc = MR_E_CUDA;
      }
    }
    lk.lock();
    if (rc != MR_OK) break;  // the slot's own upload path reports the error
    // (only this thread changes the maps and the queue's front, so
    // position i still holds r)
    if (need_mesh) {
      me.refs = 1;
      meshes[r->mesh_key] = me;
      committed += me.bytes;
      resident += me.bytes;
      r->mesh_ref = true;
    }
    if (need_tex) {
      te.refs = 1;
      textures[r->tex_key] = te;
      committed += te.bytes;
      resident += te.bytes;
      r->tex_ref = true;
    }
  }
}

void mr_server::run() {
  cudaSetDevice(c->device);
  std::unique_lock<std::mutex> lk(m);
  for (;;) {
    for (Slot* s : slots)
      if (s->busy && cudaEventQuery(s->b.done) == cudaSuccess) retire(s);
    bool any_busy = false;
    for (Slot* s : slots) any_busy |= s->busy;
    if (stop && queue.empty() && !any_busy) break;
    bool launched = false;
    for (Slot* s : slots) {
      if (s->busy || queue.empty()) continue;
      std::vector<Request*> batch;
      while (!queue.empty() && (int)batch.size() < o.max_batch) {
        Request* r = queue.front();
        // bytes to make resident for this request, on top of its own footprint
        size_t extra = 0;
        if (!meshes.count(r->mesh_key)) extra += mesh_footprint(r->req.mesh);
        if (r->tex_key && !textures.count(r->tex_key))
          extra += (size_t)r->req.tex_rows * r->req.tex_cols * 3;
        if (committed + r->cost + extra > o.budget_bytes && !evict_for(r->cost + extra, s)) break;
        queue.pop_front();
        committed += r->cost;
        // make the mesh / texture resident (upload is stream-ordered on this slot)
        // (the uploads' CUDA calls run without the server lock, so submit and
        // wait stay responsive; only this thread changes the resident maps)
        int rc = MR_OK;
        if (!meshes.count(r->mesh_key)) {
          Cached e;
          lk.unlock();
          {
            std::lock_guard<std::recursive_mutex> g(c->mu);
            // copies only: the index check runs right before this slot's
            // batch (launch), which also records `ready`
            rc = mesh_create(c, &r->req.mesh, s->stream, &e.handle, &e.bytes, pool, true);
            if (rc == MR_OK && cudaEventCreateWithFlags(&e.ready, cudaEventDisableTiming) != cudaSuccess)
              rc = MR_E_CUDA;
          }
          lk.lock();
          if (rc == MR_OK) {
            meshes[r->mesh_key] = e;
            committed += e.bytes;
            resident += e.bytes;
          }
        }
        if (rc == MR_OK && r->tex_key && !textures.count(r->tex_key)) {
          Cached e;
          e.bytes = (size_t)r->req.tex_rows * r->req.tex_cols * 3;
          lk.unlock();
          {
            std::lock_guard<std::recursive_mutex> g(c->mu);
            rc = texture_create(c, r->req.texture_rgb8, true, r->req.tex_rows, r->req.tex_cols, s->stream,
                                &e.handle, pool);
            if (rc == MR_OK && (cudaEventCreateWithFlags(&e.ready, cudaEventDisableTiming) != cudaSuccess ||
                                cudaEventRecord(e.ready, s->stream) != cudaSuccess))
              rc = MR_E_CUDA;
          }
          lk.lock();
          if (rc == MR_OK) {
            textures[r->tex_key] = e;
            committed += e.bytes;
            resident += e.bytes;
          }
        }
        if (rc != MR_OK) {
          committed -= r->cost;
          if (r->mesh_ref && meshes.count(r->mesh_key)) meshes[r->mesh_key].refs--;
          if (r->tex_ref && textures.count(r->tex_key)) textures[r->tex_key].refs--;
          r->result = rc;
          r->status = 0;
          r->t_done = now_us();
          completed++;
          cv_done.notify_all();
          continue;
        }
        // one reference per request (the upload-ahead stage may hold it already)
        if (!r->mesh_ref) meshes[r->mesh_key].refs++;
        meshes[r->mesh_key].last_use = ++use_clock;
        if (r->tex_key) {
          if (!r->tex_ref) textures[r->tex_key].refs++;
          textures[r->tex_key].last_use = use_clock;
        }
        batch.push_back(r);
      }
      if (batch.empty()) continue;
      lk.unlock();
      launch(s, batch);
      lk.lock();
      launched = true;
    }
    if (!launched) {
      upload_ahead(lk);
      cv_work.wait_for(lk, std::chrono::microseconds(50));
    }
  }
}

extern "C" {

MR_API int mr_server_create(mr_ctx* c, const mr_server_opts* o, mr_server** out) {
  if (!c || !o || !out || o->slots < 1 || o->max_batch < 1 || o->budget_bytes == 0) return MR_E_INVALID;
  const int tw = o->tile ? o->tile : 16, th = o->tile_h ? o->tile_h : tw;
  const int threads = o->threads ? o->threads : 64, chunk = o->chunk ? o->chunk : 64;
  const int small_max = o->small_max < 0 ? 64 : o->small_max;
  if (!batch_tile_ok(tw, th) || (threads != 64 && threads != 128 && threads != 256) || chunk < 16 || chunk > 256 ||
      small_max > 4096)
    return MR_E_INVALID;
  mr_server* s = new mr_server();
  s->c = c;
  s->o = *o;
  cudaSetDevice(c->device);
  {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = c->device;
    uint64_t keep = o->budget_bytes;
    if (cudaMemPoolCreate(&s->pool, &props) != cudaSuccess ||
        cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
      if (s->pool) cudaMemPoolDestroy(s->pool);
      delete s;
      return MR_E_CUDA;
    }
  }
  for (int i = 0; i < o->slots; i++) {
    Slot* sl = new Slot();
    sl->b.tile_w = tw;
    sl->b.tile_h = th;
    sl->b.threads = threads;
    sl->b.chunk = chunk;
    sl->b.small_max = small_max;
    sl->b.graphs = false;  // shapes change from batch to batch
    if (cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete sl;
      for (Slot* x : s->slots) {
        cudaStreamDestroy(x->stream);
        delete x;
      }
      cudaMemPoolDestroy(s->pool);
      delete s;
      return MR_E_CUDA;
    }
    s->slots.push_back(sl);
  }
  if (cudaStreamCreateWithFlags(&s->upload, cudaStreamNonBlocking) != cudaSuccess) {
    for (Slot* x : s->slots) {
      cudaStreamDestroy(x->stream);
      delete x;
    }
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
    return MR_E_CUDA;
  }
  // Grow the pool to the budget once (at most half the free device memory
  // beyond a 4 GiB margin).  Resident meshes are freed only when evicted, so
  // without this every upload made the pool map new memory: about 0.2 ms of
  // host time per allocation on GB300, most of the worker's time per upload.
  // Freed at once, the memory stays mapped in the pool (its release
  // threshold is the budget) and later allocations are carved from it.
  {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
      const size_t margin = (size_t)4 << 30;
      const size_t want = std::min<size_t>(o->budget_bytes, free_b > margin ? (free_b - margin) / 2 : 0);
      void* p = nullptr;
      if (want && cudaMallocFromPoolAsync(&p, want, s->pool, s->upload) == cudaSuccess) {
        cudaFreeAsync(p, s->upload);
        cudaStreamSynchronize(s->upload);
      }
    }
    cudaGetLastError();  // a pool that could not grow ahead grows on demand
  }
  s->worker = std::thread([s] { s->run(); });
  *out = s;
  return MR_OK;
}

MR_API int mr_server_submit(mr_server* s, const mr_request* q, uint64_t* ticket) {
  if (!s || !q || !ticket) return MR_E_INVALID;
  // the mesh descriptor is checked as every entry point checks it (negative
  // counts would otherwise reach the footprint arithmetic below)
  if (q->frame.width <= 0 || q->frame.height <= 0 || mesh_desc_problem(&q->mesh) ||
      (q->texture_key && (!q->texture_rgb8 || q->tex_rows <= 0 || q->tex_cols <= 0)))
    return MR_E_INVALID;
  Request* r = new Request();
  r->req = *q;
  r->mesh_key = q->mesh_key;
  r->tex_key = q->texture_key;
  r->cost = request_footprint(*q);
  const size_t own = r->cost + mesh_footprint(q->mesh) + (size_t)q->tex_rows * q->tex_cols * 3;
  std::lock_guard<std::mutex> lk(s->m);
  if (own > s->o.budget_bytes) {
    s->rejected++;
    delete r;
    return MR_E_BUDGET;
  }
  r->ticket = s->next_ticket++;
  r->t_submit = now_us();
  if (!s->submitted++) s->t_first = r->t_submit;
  s->reqs[r->ticket] = r;
  s->queue.push_back(r);
  *ticket = r->ticket;
  s->cv_work.notify_one();
  return MR_OK;
}

MR_API int mr_server_wait(mr_server* s, uint64_t ticket, int64_t timeout_us, mr_request_info* info) {
  if (!s) return MR_E_INVALID;
  std::unique_lock<std::mutex> lk(s->m);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return MR_E_HANDLE;
  Request* r = it->second;
  if (r->status != 0 && timeout_us > 0)
    s->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), [r] { return r->status == 0; });
  if (r->status != 0) return MR_E_NOT_READY;
  if (info) {
    info->status = r->result;
    info->batch_size = r->batch_size;
    info->queue_us = r->t_launch > 0 ? r->t_launch - r->t_submit : 0;
    info->latency_us = r->t_done - r->t_submit;
  }
  int rc = r->result;
  s->reqs.erase(it);
  delete r;
  return rc;
}

MR_API int mr_server_get_stats(mr_server* s, mr_server_stats* o) {
  if (!s || !o) return MR_E_INVALID;
  std::lock_guard<std::mutex> lk(s->m);
  memset(o, 0, sizeof(*o));
  o->submitted = s->submitted;
  o->completed = s->completed;
  o->rejected = s->rejected;
  o->batches = s->batches;
  o->in_queue = (int64_t)s->queue.size();
  for (Slot* sl : s->slots) o->in_flight += sl->busy ? (int64_t)sl->reqs.size() : 0;
  o->mean_batch = s->batches ? (double)s->batched / (double)s->batches : 0;
  if (!s->lat.empty()) {
    std::vector<double> v = s->lat;
    std::sort(v.begin(), v.end());
    auto pct = [&v](double p) { return v[std::min(v.size() - 1, (size_t)(p * (double)(v.size() - 1) + 0.5))]; };
    o->p50_us = pct(0.50);
    o->p99_us = pct(0.99);
    o->max_us = v.back();
  }
  if (s->t_last > s->t_first) o->frames_per_s = (double)s->completed / ((s->t_last - s->t_first) * 1e-6);
  o->resident_bytes = s->resident;
  o->committed_bytes = s->committed;
  return MR_OK;
}

MR_API int mr_server_reset_stats(mr_server* s) {
  if (!s) return MR_E_INVALID;
  std::lock_guard<std::mutex> lk(s->m);
  s->lat.clear();
  s->submitted = s->completed = s->rejected = s->batches = s->batched = 0;
  s->t_first = s->t_last = 0;
  return MR_OK;
}

MR_API int mr_server_destroy(mr_server* s) {
  if (!s) return MR_E_INVALID;
  {
    std::lock_guard<std::mutex> lk(s->m);
    s->stop = true;
  }
  s->cv_work.notify_all();
  s->worker.join();
  {
    std::lock_guard<std::recursive_mutex> g(s->c->mu);
    cudaSetDevice(s->c->device);
    if (s->upload) cudaStreamSynchronize(s->upload);
    for (Slot* sl : s->slots) cudaStreamSynchronize(sl->stream);
    for (auto& kv : s->meshes) {
      mesh_destroy(s->c, kv.second.handle, s->slots[0]->stream);
      if (kv.second.ready) cudaEventDestroy(kv.second.ready);
    }
    for (auto& kv : s->textures) {
      texture_destroy(s->c, kv.second.handle, s->slots[0]->stream);
      if (kv.second.ready) cudaEventDestroy(kv.second.ready);
    }
    for (Slot* sl : s->slots) {
      cudaStreamSynchronize(sl->stream);
      sl->b.release();
      cudaStreamDestroy(sl->stream);
      delete sl;
    }
    if (s->upload) cudaStreamDestroy(s->upload);
    if (s->pool) cudaMemPoolDestroy(s->pool);  // every allocation from it has been freed
  }
  for (auto& kv : s->reqs) delete kv.second;
  delete s;
  return MR_OK;
}

}  // extern "C"
