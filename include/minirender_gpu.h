/*
 * minirender_gpu.h -- C ABI of the GB300 (sm_103a) rasterisation path that
 * sits behind minirender's C++ Renderer.
 *
 * The reference exposes no C ABI: its interface is the C++ class
 * minirender::Renderer (include/minirender/Renderer.h:17-64) fed by the scene
 * model of include/minirender/Scene.h.  Each entry point below names the
 * reference member or function whose work it takes over.  Plain pointers and
 * sizes only; every call returns MR_OK (0) or a negative MR_E_* code, and
 * mr_last_error() gives a one-line reason.
 *
 * Threading: a context may be shared between threads; calls on one context
 * are serialised by an internal lock.  Device work is queued on the context's
 * CUDA stream (mr_set_stream) and completes in call order.
 *
 * Numerics: all arithmetic is IEEE binary32 without fused multiply-add and in
 * the reference's operation order, so coverage, depth and the visible
 * triangle per pixel equal the reference CPU renderer bit for bit; colour may
 * differ by rounding of powf/sqrtf/division only.
 */
#ifndef MINIRENDER_GPU_H
#define MINIRENDER_GPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define MR_API __declspec(dllexport)
#else
#define MR_API __attribute__((visibility("default")))
#endif

#define MR_ABI_VERSION 2

/* Status codes. */
#define MR_OK 0
#define MR_E_INVALID -1      /* bad argument or inconsistent sizes */
#define MR_E_CUDA -2         /* a CUDA runtime call failed */
#define MR_E_NOMEM -3        /* device allocation failed */
#define MR_E_HANDLE -4       /* unknown mesh / texture / context handle */
#define MR_E_BAD_INDEX -5    /* a mesh index was out of range (kernel-checked) */
#define MR_E_BUDGET -6       /* request does not fit the device-memory budget */
#define MR_E_TIMEOUT -7      /* a bounded device wait gave up */
#define MR_E_NOT_READY -8    /* asynchronous result not available yet */
#define MR_E_NO_DEVICE -9    /* no usable CUDA device */
#define MR_E_NOALLOC_LIMIT -10 /* frame or mesh larger than mr_render_noalloc's fixed scratch */
#define MR_E_IO -11          /* a file could not be read, written or parsed */

/* Background sentinel in the per-pixel triangle-id image. */
#define MR_NO_TRIANGLE 0xFFFFFFFFu

typedef struct mr_ctx mr_ctx;

/* Material (include/minirender/Scene.h:38-45, defaults src/Scene.cpp:65-71).
 * texture: handle from mr_texture_upload_* or -1 for none. */
typedef struct mr_material {
    float diffuse[3];
    float specular[3];
    float emissive[3];
    float shininess;
    int32_t texture;
} mr_material;

/* TriMesh arrays exactly as the reference holds them
 * (include/minirender/Scene.h:73-87): Vec3 = 3 floats, Vec2 = 2 floats, one
 * int per index.  n_* count elements (vertices, not floats).  texcoords are
 * used only when both texcoords and texcoordsI are non-empty
 * (src/Renderer.cpp:371). */
typedef struct mr_mesh_desc {
    const float* vertices;     int32_t n_vertices;
    const float* normals;      int32_t n_normals;
    const float* texcoords;    int32_t n_texcoords;
    const int32_t* indices;    int32_t n_indices;
    const int32_t* normalsI;   int32_t n_normalsI;
    const int32_t* texcoordsI; int32_t n_texcoordsI;
} mr_mesh_desc;

/* One entry of Renderer::_renderables after Scene::collectShapes
 * (include/minirender/Scene.h:47-53, src/Scene.cpp:13-36): the mesh, its
 * world transform (row-major, m[4*i+j] = row i, column j) and the material
 * paintMesh would use (mesh->material, or the default, src/Renderer.cpp:336).
 * flags (0 for scene renderables):
 *   MR_RS_MODELVIEW  transform is the modelview itself: the frame's view is
 *                    not applied (Renderer::paintTriangle's view-space
 *                    vertices are a one-triangle mesh with the identity here)
 *   MR_RS_NO_CLIP    no near-plane clipping (paintTriangle(..., world=false),
 *                    src/Renderer.cpp:163-173)
 *   MR_RS_OWN_STATE  the renderable carries the switches its paint call saw
 *                    (paintTriangle reads _lighting, _texturing and
 *                    _lightIsPoint at the call, src/Renderer.cpp:264-289):
 *                    MR_RS_LIGHTING, MR_RS_TEXTURING and MR_RS_POINT_LIGHT
 *                    replace the frame's lighting, texturing and
 *                    light_is_point for its fragments.  The light's position
 *                    stays the frame's (placed as render() places it,
 *                    :317-320, from the frame's view, light and
 *                    light_is_point). */
#define MR_RS_MODELVIEW   1
#define MR_RS_NO_CLIP     2
#define MR_RS_OWN_STATE   4
#define MR_RS_LIGHTING    8
#define MR_RS_TEXTURING   16
#define MR_RS_POINT_LIGHT 32
typedef struct mr_renderable {
    int32_t mesh;
    int32_t flags;
    float transform[16];
    mr_material material;
} mr_renderable;

/* Scene-graph node for mr_collect_shapes: nodes in pre-order, node 0 the
 * root Scene, parent < own index.  mesh = -1 for a plain SceneNode. */
typedef struct mr_node {
    int32_t parent;
    int32_t mesh;
    float transform[16];
    int32_t has_material;      /* 0: the Renderer's default material */
    mr_material material;
    float opacity;             /* Material::opacity (OBJ "d", src/io.cpp:288-289;
                                  1 by default); the renderer does not use it */
} mr_node;

/* Renderer state read by Renderer::render() (src/Renderer.cpp:311-332). */
typedef struct mr_frame {
    int32_t width, height;          /* setSize */
    float projection[16];           /* setProjection */
    float view[16];                 /* setView */
    float light[3];                 /* setLight */
    int32_t light_is_point;
    float ambient;                  /* Scene::ambientLight */
    float background[3];            /* setBackground */
    int32_t lighting;               /* setLighting */
    int32_t texturing;              /* setTexturing */
    int32_t save_normals;           /* setSaveNormals */
} mr_frame;

/* Device-side outputs of the last frame (device pointers, valid until the
 * next mr_render on the context).  rgb8: H*W*3 bytes (savePPM quantisation,
 * src/io.cpp:358-362); depth: H*W floats (getDepth); rgb_f32: H*W*3 floats
 * (getImage), only when requested; tri_id: H*W u32 visible sub-triangle id
 * 2*(global triangle index)+clip sub-triangle, MR_NO_TRIANGLE for
 * background; normals: H*W*3 floats when save_normals. */
typedef struct mr_outputs {
    int32_t width, height;
    uint8_t* rgb8;
    float* depth;
    float* rgb_f32;
    uint32_t* tri_id;
    float* normals;
} mr_outputs;

/* Output selection for mr_render (bit mask). */
#define MR_OUT_RGB8    1
#define MR_OUT_DEPTH   2
#define MR_OUT_RGB_F32 4
#define MR_OUT_TRI_ID  8
#define MR_OUT_DEFAULT (MR_OUT_RGB8 | MR_OUT_DEPTH | MR_OUT_TRI_ID)

/* Per-frame counters (device-side, read at the next synchronisation). */
typedef struct mr_stats {
    int64_t triangles;        /* submitted triangles */
    int64_t clipped;          /* triangles that crossed the near plane */
    int64_t rasterised;       /* sub-triangles past cull and reject */
    int64_t small_direct;     /* rasterised in the setup kernel */
    int64_t binned;           /* large sub-triangles (records) */
    int64_t bin_entries;      /* their work items: 32-row blocks (mr_render),
                                 (tile, sub-triangle) pairs (mr_render_batch) */
    int64_t error_flags;      /* nonzero: MR_E_BAD_INDEX seen */
    float stage_ms[8];        /* when profiling: clear+vertex, setup, large raster, -, resolve */
    int32_t n_stages;
} mr_stats;

/* ---- library / context --------------------------------------------- */
MR_API int mr_abi_version(void);
MR_API const char* mr_status_string(int status);
MR_API const char* mr_last_error(const mr_ctx* ctx);

/* Replaces: constructing a minirender::Renderer (src/Renderer.cpp:85-98). */
MR_API int mr_create(int device, mr_ctx** out);
MR_API int mr_destroy(mr_ctx* ctx);
/* cudaStream_t passed as void*; NULL = the context's own stream. */
MR_API int mr_set_stream(mr_ctx* ctx, void* cuda_stream);
MR_API int mr_synchronize(mr_ctx* ctx);
/* Stream for mr_mesh_update / mr_texture_update (NULL: the context's own
 * stream).  An update waits on the device for the frames already queued on
 * the context (they read the old contents); the next frame waits for the
 * update.  Contexts that share one upload stream send their updates over
 * the host link one at a time, each at the link's full rate, while their
 * frames render on their own streams. */
MR_API int mr_set_upload_stream(mr_ctx* ctx, void* cuda_stream);
/* Small-triangle bounding-box limit (pixels) of mr_render.  `tile` (8, 16
 * or 32) is validated and kept for source compatibility; single frames no
 * longer bin into tiles. */
MR_API int mr_set_tuning(mr_ctx* ctx, int tile, int small_max);
MR_API int mr_set_profiling(mr_ctx* ctx, int on);

/* ---- resident data ----------------------------------------------------- */
/* Replaces: the per-frame reads of TriMesh arrays in Renderer::paintMesh
 * (src/Renderer.cpp:334-381); the mesh stays on the device. */
MR_API int mr_mesh_upload(mr_ctx* ctx, const mr_mesh_desc* desc, int32_t* mesh_out);
/* Re-copies the arrays of an existing mesh (same element counts). */
MR_API int mr_mesh_update(mr_ctx* ctx, int32_t mesh, const mr_mesh_desc* desc);
MR_API int mr_mesh_free(mr_ctx* ctx, int32_t mesh);
/* Replaces: Material::texture filled by loadPPM (src/io.cpp:367-415): each
 * texel is byte/255.0f, kept as RGB8 on the device. */
MR_API int mr_texture_upload_rgb8(mr_ctx* ctx, const uint8_t* rgb, int32_t rows, int32_t cols,
                                  int32_t* tex_out);
/* Material::texture given as floats (Array2<Vec3>, row-major rows x cols x 3). */
MR_API int mr_texture_upload_f32(mr_ctx* ctx, const float* rgb, int32_t rows, int32_t cols,
                                 int32_t* tex_out);
/* Re-copies the texels of an existing texture (same size and format). */
MR_API int mr_texture_update(mr_ctx* ctx, int32_t tex, const void* texels);
MR_API int mr_texture_free(mr_ctx* ctx, int32_t tex);

/* ---- frame ------------------------------------------------------------- */
/* Replaces: Renderer::render() after collectShapes (src/Renderer.cpp:311-332)
 * with paintMesh/paintTriangle/clipTriangle (src/Renderer.cpp:121-381).
 * Asynchronous: queued on the context stream. outputs: MR_OUT_* mask. */
MR_API int mr_render(mr_ctx* ctx, const mr_frame* frame, const mr_renderable* renderables,
                     int32_t n_renderables, int32_t outputs);
/* Replaces: getImage/getDepth (include/minirender/Renderer.h:60-63) plus the
 * savePPM byte conversion (src/io.cpp:358-362).  Copies the requested
 * outputs of the last frame to host memory (NULL = skip) and waits. */
MR_API int mr_read(mr_ctx* ctx, uint8_t* rgb8, float* depth, float* rgb_f32, uint32_t* tri_id,
                   float* normals);
/* mr_read without the wait: queues the copies of the last frame's outputs
 * (pinned host buffers make them asynchronous) and returns.  mr_wait -- or
 * the next mr_read / mr_render / mr_get_stats on this context -- completes
 * them; the buffers must stay valid until then.  Several contexts, each on
 * its own stream, keep frames in flight: one context's upload and render
 * overlap another's read-back (see mr_set_upload_stream). */
MR_API int mr_read_async(mr_ctx* ctx, uint8_t* rgb8, float* depth, float* rgb_f32, uint32_t* tri_id,
                         float* normals);
MR_API int mr_wait(mr_ctx* ctx);
MR_API int mr_get_outputs(mr_ctx* ctx, mr_outputs* out);
MR_API int mr_get_stats(mr_ctx* ctx, mr_stats* out);
/* Replaces: Renderer::getRangeImage (src/Renderer.cpp:388-415): view-space
 * XYZ per pixel from the last depth buffer, H*W*3 floats to host memory. */
MR_API int mr_read_range_image(mr_ctx* ctx, float* xyz);

/* ---- batches -------------------------------------------------------------
 * No single counterpart in the reference: many Renderer::render() calls
 * (src/Renderer.cpp:311-332), one per scene, done in one launch sequence --
 * vertex pass, setup of every scene's triangles into records binned per
 * screen tile, and one persistent fused bin-raster-shade kernel over the
 * tiles of all scenes.  Results per scene are identical to mr_render's. */
typedef struct mr_batch_scene {
    mr_frame frame;                 /* the scene's Renderer state */
    int32_t first_renderable;       /* its renderables: renderables[first .. first+n) */
    int32_t n_renderables;
} mr_batch_scene;

/* Tile edge (8/16/32), threads per tile block (64/128/256) and records
 * staged per pass in shared memory (16..256) for mr_render_batch. */
MR_API int mr_set_batch_tuning(mr_ctx* ctx, int tile, int threads, int chunk);
/* As mr_set_batch_tuning with a rectangular screen tile: power-of-two sides,
 * width 4..256, height 2..64, 64..4096 pixels.  Wide tiles shorten the
 * column-by-column edge-function replay of triangles that cross tiles. */
MR_API int mr_set_batch_tiling(mr_ctx* ctx, int tile_w, int tile_h, int threads, int chunk);
/* Sub-triangles whose bounding box holds at most small_max pixels (0..4096,
 * default 64) are rasterised by the batch's setup kernel into a per-scene
 * visibility buffer; larger ones are binned into the fused tile kernel.
 * 0: every sub-triangle is binned (no visibility buffer is allocated). */
MR_API int mr_set_batch_small_max(mr_ctx* ctx, int small_max);
/* graphs != 0: the launch sequence is captured once per batch shape (scene
 * count, sizes, renderable and triangle counts, tuning) into a CUDA graph and
 * replayed; cameras, lights and materials may change between replays. */
MR_API int mr_set_batch_graphs(mr_ctx* ctx, int graphs);
/* Queues the batch; outputs: MR_OUT_RGB8 | MR_OUT_DEPTH | MR_OUT_TRI_ID.
 * A batch whose (tile, record) list overflowed is re-run when it is first
 * waited for (mr_read_batch / mr_get_batch_stats), so the meshes and textures
 * it reads must not be updated before then. */
MR_API int mr_render_batch(mr_ctx* ctx, const mr_batch_scene* scenes, int32_t n_scenes,
                           const mr_renderable* renderables, int32_t n_renderables, int32_t outputs);
/* Waits for the last batch and copies scene `scene`'s outputs to host memory. */
MR_API int mr_read_batch(mr_ctx* ctx, int32_t scene, uint8_t* rgb8, float* depth, uint32_t* tri_id);
/* Device pointers of scene `scene`'s outputs (valid until the next batch). */
MR_API int mr_get_batch_outputs(mr_ctx* ctx, int32_t scene, mr_outputs* out);
/* Waits for the last batch; counters and stage times (vertex, setup, fused). */
MR_API int mr_get_batch_stats(mr_ctx* ctx, mr_stats* out);

/* ---- render server ---------------------------------------------------------
 * No counterpart in the reference (one synchronous Renderer::render() per
 * frame).  A worker thread keeps meshes, textures and framebuffers resident,
 * admits queued requests against a device-memory budget and renders them in
 * batches as they arrive: while some batches run on the device the next ones
 * are formed and launched on other streams (continuous batching).  Each
 * request renders one mesh (one renderable of Renderer::render) and its
 * result is identical whether it ran alone or in a mix. */
typedef struct mr_server mr_server;

typedef struct mr_server_opts {
    uint64_t budget_bytes;   /* device memory the server may commit (resident meshes + in-flight requests) */
    int32_t slots;           /* batches in flight at once (>= 1) */
    int32_t max_batch;       /* requests per batch (>= 1) */
    int32_t tile, threads, chunk;   /* batch tuning, as mr_set_batch_tuning (0: defaults) */
    int32_t tile_h;          /* tile height; 0: square tiles of edge `tile` (as mr_set_batch_tiling) */
    int32_t small_max;       /* as mr_set_batch_small_max; negative: the default (64) */
} mr_server_opts;

typedef struct mr_request {
    mr_frame frame;
    uint64_t mesh_key;        /* caller's id of the mesh; a resident key is re-rendered without upload */
    mr_mesh_desc mesh;        /* host arrays, read when the mesh is not resident; valid until done */
    float transform[16];      /* world transform of the mesh */
    mr_material material;     /* material.texture is ignored: see texture_key */
    uint64_t texture_key;     /* 0: no texture */
    const uint8_t* texture_rgb8;   /* rows x cols x 3, read when the texture is not resident */
    int32_t tex_rows, tex_cols;
    int32_t outputs;          /* MR_OUT_RGB8 | MR_OUT_DEPTH | MR_OUT_TRI_ID */
    uint8_t* rgb8;            /* host destinations (page-locked memory lets copies overlap), or NULL */
    float* depth;
    uint32_t* tri_id;
} mr_request;

typedef struct mr_request_info {
    int32_t status;           /* MR_OK, or the request's error */
    int32_t batch_size;       /* requests in the batch it ran in */
    double queue_us;          /* submit -> launch */
    double latency_us;        /* submit -> outputs in host memory */
} mr_request_info;

typedef struct mr_server_stats {
    int64_t submitted, completed, rejected, batches, in_queue, in_flight;
    double mean_batch, p50_us, p99_us, max_us, frames_per_s;
    uint64_t resident_bytes, committed_bytes;
} mr_server_stats;

MR_API int mr_server_create(mr_ctx* ctx, const mr_server_opts* opts, mr_server** out);
/* Queues a request; MR_E_BUDGET if it can never fit the budget. */
MR_API int mr_server_submit(mr_server* srv, const mr_request* req, uint64_t* ticket);
/* Waits up to timeout_us (0: poll) for a request; MR_E_NOT_READY if not done.
 * A request is forgotten once it has been reported done. */
MR_API int mr_server_wait(mr_server* srv, uint64_t ticket, int64_t timeout_us, mr_request_info* info);
/* Latency percentiles over the requests completed since the last reset. */
MR_API int mr_server_get_stats(mr_server* srv, mr_server_stats* out);
MR_API int mr_server_reset_stats(mr_server* srv);
/* Drains the queue, stops the worker and releases the server's memory. */
MR_API int mr_server_destroy(mr_server* srv);

/* ---- rendering without any device allocation ----------------------------
 * No counterpart in the reference (its CPU Renderer never touches device
 * memory).  For callers that must not allocate device memory themselves or
 * through this library: code running under a framework whose pool owns all
 * device memory, or a real-time loop that cannot afford cudaMalloc/cudaFree
 * and the device-wide synchronisation cudaFree implies.  Renders one mesh
 * (one renderable of Renderer::render, src/Renderer.cpp:311-381) with every
 * piece of working memory -- visibility buffer, counters, per-triangle
 * index-check mask, renderable record, triangle-base table and a fixed store
 * of large-triangle records (32768; further large triangles are rasterised
 * by the setup kernel, as small ones are) -- taken from one
 * file-scope device array of MR_NOALLOC_SCRATCH_BYTES that the library
 * reserves on each GPU it is loaded on, until the process exits.
 *
 * Limits: width, height <= MR_NOALLOC_MAX_SIDE, width*height <=
 * MR_NOALLOC_MAX_PIXELS, triangles <= MR_NOALLOC_MAX_TRIANGLES; anything
 * larger returns MR_E_NOALLOC_LIMIT before any device work.
 * Inputs and outputs are DEVICE pointers owned by the caller: the mesh arrays
 * in *mesh (same layout as mr_mesh_upload's), the texture (rows x cols x 3
 * bytes decoded as b/255, or floats; NULL for none), and the outputs rgb8
 * (H*W*3), depth (H*W), tri_id (H*W), any of which may be NULL.  Results are
 * bit-identical to mr_render of the same renderable.
 * Arguments (null arrays with non-zero counts, negative counts, short index
 * arrays) are checked before any device work and give MR_E_INVALID.
 * The first call on a device looks up the scratch array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  The address is kept for the life of the
 * process, so the device must not be reset (cudaDeviceReset) while the
 * library is in use.  The call is synchronous on `cuda_stream`
 * (NULL = legacy default stream).  All calls in the process share the one
 * scratch array, which keeps the previous call's contents: calls whose GPU
 * work overlaps (other host threads, other streams) race on it and must be
 * serialised by the caller. */
#define MR_NOALLOC_SCRATCH_BYTES (20u << 20)
#define MR_NOALLOC_MAX_SIDE 4096
#define MR_NOALLOC_MAX_PIXELS (1 << 21)
#define MR_NOALLOC_MAX_TRIANGLES (1 << 22)
MR_API int mr_render_noalloc(const mr_frame* frame, const mr_mesh_desc* mesh, const float* transform,
                             const mr_material* material, const void* texture, int32_t tex_rows,
                             int32_t tex_cols, int32_t tex_is_rgb8, uint8_t* rgb8, float* depth,
                             uint32_t* tri_id, void* cuda_stream);

/* ---- model and image files (host only, no device work) -------------------
 * loadMesh (src/io.cpp:111-132) for .stl (loadSTL :134-153, ASCII :16-60 or
 * binary :62-109), .obj (+ .mtl, loadOBJ :187-335) and .x3d (src/x3d.cpp:
 * 35-200); any other extension gives an empty node, as the reference does.
 * The model is the scene tree the reference builds: mr_node array in
 * pre-order (node 0 the returned node; a TriMesh without material has
 * has_material 0; material.texture indexes the model's textures), one
 * mr_mesh_desc per TriMesh (host arrays owned by the model), RGB8 textures
 * read with loadPPM's rules (:364-415; decode b/255.0f happens on the
 * device).  Large OBJ and binary STL files are parsed on all host threads. */
typedef struct mr_model mr_model;
MR_API int mr_model_load(const char* path, mr_model** out);
MR_API int mr_model_counts(const mr_model* model, int32_t* n_nodes, int32_t* n_meshes, int32_t* n_textures);
MR_API int mr_model_nodes(const mr_model* model, mr_node* out, int32_t cap);
MR_API int mr_model_mesh(const mr_model* model, int32_t mesh, mr_mesh_desc* out);
MR_API int mr_model_texture(const mr_model* model, int32_t texture, const uint8_t** rgb8, int32_t* rows,
                            int32_t* cols);
MR_API void mr_model_free(mr_model* model);
/* loadPPM (src/io.cpp:364-415) as bytes: rows/cols always, pixels when rgb8
 * is given and cap_bytes >= rows*cols*3. */
MR_API int mr_ppm_load(const char* path, uint8_t* rgb8, int64_t cap_bytes, int32_t* rows, int32_t* cols);
/* savePPM (src/io.cpp:337-362) of an RGB8 image (mr_read's bytes are already
 * quantised as savePPM does). */
MR_API int mr_ppm_save(const char* path, const uint8_t* rgb8, int32_t rows, int32_t cols);
/* saveSTL (src/io.cpp:155-183): binary STL of the mesh's triangles under a
 * row-major transform (NULL: identity). */
MR_API int mr_stl_save(const char* path, const mr_mesh_desc* mesh, const float* transform);
/* saveXYZ (src/io.cpp:417-431): the points of a rows x cols x 3 float image
 * (mr_read_range_image's) whose z < -1e-5, one "x y z" line each (printf
 * "%f"), in row order, after transform (row-major; NULL = identity). */
MR_API int mr_xyz_save(const char* path, const float* xyz, int32_t rows, int32_t cols, const float* transform);

/* ---- host helpers (no device work) -------------------------------------- */
/* Scene::collectShapes (src/Scene.cpp:13-36) over a pre-order node array.
 * Writes at most cap renderables; *n_out = number produced. */
MR_API int mr_collect_shapes(const mr_node* nodes, int32_t n_nodes, mr_renderable* out,
                             int32_t cap, int32_t* n_out);
/* Matrix4 product and inverse in the operation order the device path uses. */
MR_API void mr_mat4_mul(const float* a, const float* b, float* out);
MR_API void mr_mat4_inverse(const float* a, float* out);
/* Projection builders (src/Renderer.cpp:40-83). */
MR_API void mr_projection_ortho(float l, float r, float b, float t, float n, float f, float* out);
MR_API void mr_projection_perspective(float l, float r, float b, float t, float n, float f,
                                      float* out);
MR_API void mr_projection_frustum(float fov, float aspect, float n, float f, float* out);
MR_API void mr_projection_frustum_h(float fov, float aspect, float n, float f, float* out);
MR_API void mr_projection_ortho_fov(float fov, float aspect, float n, float f, float* out);
MR_API void mr_projection_cv(const float* K, float w, float h, float n, float f, float* out);

#ifdef __cplusplus
}
#endif
#endif /* MINIRENDER_GPU_H */
