/*
 * ORACLE -- test infrastructure only.  Nothing in the product library links,
 * loads or calls this code; tests, __graft_entry__.smoke() and the CPU
 * baseline of bench.py use it as the oracle.
 *
 * Plain-C restatement of minirender's Renderer::render() hot path
 * (src/Renderer.cpp:13-20, 113-381 and src/Scene.cpp:13-36) with one
 * addition the reference lacks: the id of the triangle that won each pixel.
 *
 * Parity pin: mr_oracle.c is checked bit for bit (image, depth) against the
 * reference's own src/Renderer.cpp, src/Scene.cpp and src/primitives.cpp
 * compiled unmodified against a from-scratch stand-in for the ASL library
 * (oracle/asl_shim, recipe oracle/Makefile), and against the committed
 * fixtures in tests/golden.  ASL (aslze/asl 1.11.14) itself is absent, so
 * the operation order of its Vec/Matrix operators is restated, not pinned.
 */
#ifndef MR_ORACLE_H
#define MR_ORACLE_H
#include <stdint.h>
#include "../include/minirender_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mro_texture {
    const float* rgb; /* rows*cols*3 floats, row-major */
    int32_t rows, cols;
} mro_texture;

int mro_collect_shapes(const mr_node* nodes, int32_t n_nodes, mr_renderable* out, int32_t cap,
                       int32_t* n_out);

/* image: H*W*3, depth: H*W, ids: H*W (MR_NO_TRIANGLE = background),
 * normals: H*W*3 or NULL. */
int mro_render(const mr_frame* f, const mr_renderable* rs, int32_t n, const mr_mesh_desc* meshes,
               int32_t n_meshes, const mro_texture* tex, int32_t n_tex, float* image, float* depth,
               uint32_t* ids, float* normals);

/* savePPM conversion (src/io.cpp:358-362) of n_px pixels. */
void mro_quantize_rgb8(const float* image, int64_t n_px, uint8_t* out);
/* loadPPM conversion (src/io.cpp:407-410) of n_px texels. */
void mro_decode_rgb8(const uint8_t* rgb, int64_t n_px, float* out);
/* getRangeImage (src/Renderer.cpp:388-415). */
void mro_range_image(const mr_frame* f, const float* depth, float* xyz);

void mro_mat4_mul(const float* a, const float* b, float* out);
void mro_mat4_inverse(const float* a, float* out);
void mro_projection_frustum(float fov, float aspect, float n, float f, float* out);
void mro_projection_perspective(float l, float r, float b, float t, float n, float f, float* out);
void mro_projection_ortho(float l, float r, float b, float t, float n, float f, float* out);

/* Multi-threaded throughput harness for the CPU baseline: renders n_frames
 * independent frames of the same scene on n_threads threads, each with its
 * own buffers, and returns elapsed seconds. */
double mro_render_frames_mt(const mr_frame* f, const mr_renderable* rs, int32_t n,
                            const mr_mesh_desc* meshes, int32_t n_meshes, const mro_texture* tex,
                            int32_t n_tex, int32_t n_frames, int32_t n_threads);

#ifdef __cplusplus
}
#endif
#endif
