/*
 * ORACLE -- test infrastructure only (see mr_oracle.h).  Plain C,
 * compiled with -O2 -ffp-contract=off and without -ffast-math, so every
 * float operation below is one IEEE binary32 operation in source order.
 *
 * Each function cites the reference lines it restates.  The reference's
 * Vec2/Vec3/Matrix4 come from ASL (aslze/asl 1.11.14, not available here);
 * the operator semantics restated for them are:
 *   dot products sum x, y, z terms left to right; Vec2 cross a^b =
 *   a.x*b.y - a.y*b.x; perpend(v) = (-v.y, v.x); v.normalized() = v/|v|
 *   component-wise; Matrix4*Vec3 = affine rows, no w divide;
 *   min(a,b) = b<a ? b : a; max(a,b) = a<b ? b : a;
 *   clamp(x,lo,hi) = x<lo ? lo : (x>hi ? hi : x); fract(x) = x-floor(x).
 * Deviation from the reference (which has undefined behaviour there): a
 * texel index is clamped to the texture, and triangles with an index
 * outside the mesh arrays are skipped.
 */
#include "mr_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef struct { float x, y, z; } V3;
typedef struct { float x, y; } V2;
typedef struct { V3 pos, nrm; V2 uv; } Vtx; /* Vertex, include/minirender/Scene.h:14-24 */

static V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
static V2 v2(float x, float y) { V2 r; r.x = x; r.y = y; return r; }
static V3 v3_add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static V3 v3_sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static V3 v3_ks(float k, V3 v) { return v3(k * v.x, k * v.y, k * v.z); }
static float v3_dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static float v3_len(V3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
static V3 v3_normalized(V3 a) { float l = v3_len(a); return v3(a.x / l, a.y / l, a.z / l); }
static V2 v2_add(V2 a, V2 b) { return v2(a.x + b.x, a.y + b.y); }
static V2 v2_sub(V2 a, V2 b) { return v2(a.x - b.x, a.y - b.y); }
static V2 v2_ks(float k, V2 v) { return v2(k * v.x, k * v.y); }
static float fminr(float a, float b) { return (b < a) ? b : a; }
static float fmaxr(float a, float b) { return (a < b) ? b : a; }
static float clampr(float x, float lo, float hi) { return (x < lo) ? lo : ((x > hi) ? hi : x); }
static float fractr(float x) { return x - floorf(x); }

/* Matrix4 * Vec3, affine (used by src/Renderer.cpp:318, 345, 348). */
static V3 m4_apply(const float* m, V3 p) {
    return v3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3],
              m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
              m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
}

void mro_mat4_mul(const float* a, const float* b, float* out) {
    float r[16];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            r[4 * i + j] = a[4 * i + 0] * b[0 + j] + a[4 * i + 1] * b[4 + j] +
                           a[4 * i + 2] * b[8 + j] + a[4 * i + 3] * b[12 + j];
    memcpy(out, r, sizeof(r));
}

/* 4x4 inverse by adjugate over 2x2 complementary minors. */
void mro_mat4_inverse(const float* a, float* out) {
#define M(i, j) a[4 * (i) + (j)]
    float s0 = M(0, 0) * M(1, 1) - M(1, 0) * M(0, 1);
    float s1 = M(0, 0) * M(1, 2) - M(1, 0) * M(0, 2);
    float s2 = M(0, 0) * M(1, 3) - M(1, 0) * M(0, 3);
    float s3 = M(0, 1) * M(1, 2) - M(1, 1) * M(0, 2);
    float s4 = M(0, 1) * M(1, 3) - M(1, 1) * M(0, 3);
    float s5 = M(0, 2) * M(1, 3) - M(1, 2) * M(0, 3);
    float c5 = M(2, 2) * M(3, 3) - M(3, 2) * M(2, 3);
    float c4 = M(2, 1) * M(3, 3) - M(3, 1) * M(2, 3);
    float c3 = M(2, 1) * M(3, 2) - M(3, 1) * M(2, 2);
    float c2 = M(2, 0) * M(3, 3) - M(3, 0) * M(2, 3);
    float c1 = M(2, 0) * M(3, 2) - M(3, 0) * M(2, 2);
    float c0 = M(2, 0) * M(3, 1) - M(3, 0) * M(2, 1);
    float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    float id = 1 / det;
    float r[16];
    r[0] = (M(1, 1) * c5 - M(1, 2) * c4 + M(1, 3) * c3) * id;
    r[1] = (-M(0, 1) * c5 + M(0, 2) * c4 - M(0, 3) * c3) * id;
    r[2] = (M(3, 1) * s5 - M(3, 2) * s4 + M(3, 3) * s3) * id;
    r[3] = (-M(2, 1) * s5 + M(2, 2) * s4 - M(2, 3) * s3) * id;
    r[4] = (-M(1, 0) * c5 + M(1, 2) * c2 - M(1, 3) * c1) * id;
    r[5] = (M(0, 0) * c5 - M(0, 2) * c2 + M(0, 3) * c1) * id;
    r[6] = (-M(3, 0) * s5 + M(3, 2) * s2 - M(3, 3) * s1) * id;
    r[7] = (M(2, 0) * s5 - M(2, 2) * s2 + M(2, 3) * s1) * id;
    r[8] = (M(1, 0) * c4 - M(1, 1) * c2 + M(1, 3) * c0) * id;
    r[9] = (-M(0, 0) * c4 + M(0, 1) * c2 - M(0, 3) * c0) * id;
    r[10] = (M(3, 0) * s4 - M(3, 1) * s2 + M(3, 3) * s0) * id;
    r[11] = (-M(2, 0) * s4 + M(2, 1) * s2 - M(2, 3) * s0) * id;
    r[12] = (-M(1, 0) * c3 + M(1, 1) * c1 - M(1, 2) * c0) * id;
    r[13] = (M(0, 0) * c3 - M(0, 1) * c1 + M(0, 2) * c0) * id;
    r[14] = (-M(3, 0) * s3 + M(3, 1) * s1 - M(3, 2) * s0) * id;
    r[15] = (M(2, 0) * s3 - M(2, 1) * s1 + M(2, 2) * s0) * id;
#undef M
    memcpy(out, r, sizeof(r));
}

static void m4_transpose(const float* a, float* out) {
    float r[16];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r[4 * i + j] = a[4 * j + i];
    memcpy(out, r, sizeof(r));
}

/* src/Renderer.cpp:40-47 */
void mro_projection_ortho(float l, float r, float b, float t, float n, float f, float* o) {
    float m[16] = {2 / (r - l), 0, 0, -(r + l) / (r - l),
                   0, 2 / (t - b), 0, -(t + b) / (t - b),
                   0, 0, -2 / (f - n), -(f + n) / (f - n),
                   0, 0, 0, 1};
    memcpy(o, m, sizeof(m));
}
/* src/Renderer.cpp:49-56 */
void mro_projection_perspective(float l, float r, float b, float t, float n, float f, float* o) {
    float m[16] = {2 * n / (r - l), 0, (r + l) / (r - l), 0,
                   0, 2 * n / (t - b), (t + b) / (t - b), 0,
                   0, 0, -(f + n) / (f - n), -2 * f * n / (f - n),
                   0, 0, -1, 0};
    memcpy(o, m, sizeof(m));
}
/* src/Renderer.cpp:68-72 */
void mro_projection_frustum(float fov, float aspect, float n, float f, float* o) {
    float t = tanf(fov / 2);
    mro_projection_perspective(-n * t * aspect, n * t * aspect, -n * t, n * t, n, f, o);
}

/* Scene::collectShapes / TriMesh::collectShapes, src/Scene.cpp:13-36:
 * world(root) = I * T(root); world(child) = world(parent) * T(child); a mesh
 * node is listed before its children, children in insertion order. */
int mro_collect_shapes(const mr_node* nodes, int32_t n_nodes, mr_renderable* out, int32_t cap,
                       int32_t* n_out) {
    static const float I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    static const mr_material def = {{0.7f, 0.7f, 0.9f}, {0.8f, 0.8f, 0.8f}, {0, 0, 0}, 12.0f, -1};
    if (n_nodes <= 0 || nodes[0].parent != -1) return MR_E_INVALID;
    float* world = (float*)malloc(sizeof(float) * 16 * (size_t)n_nodes);
    int32_t n = 0;
    for (int32_t i = 0; i < n_nodes; i++) {
        const float* parent = I;
        if (i > 0) {
            if (nodes[i].parent < 0 || nodes[i].parent >= i) { free(world); return MR_E_INVALID; }
            parent = world + 16 * nodes[i].parent;
        }
        mro_mat4_mul(parent, nodes[i].transform, world + 16 * i);
        if (nodes[i].mesh >= 0) {
            if (n < cap) {
                out[n].mesh = nodes[i].mesh;
                out[n].flags = 0;
                memcpy(out[n].transform, world + 16 * i, sizeof(float) * 16);
                out[n].material = nodes[i].has_material ? nodes[i].material : def;
            }
            n++;
        }
    }
    free(world);
    *n_out = n;
    return MR_OK;
}

typedef struct {
    int W, H;
    const float* P;
    int persp;
    float znear;
    V3 lightdir;
    int point;
    float ambient;
    int lighting, texturing, save_normals;
    float* image;
    float* depth;
    uint32_t* ids;
    float* normals;
    const mr_material* mat;
    const mro_texture* tex; /* NULL when the material has none */
} Frame;

/* htransform, src/Renderer.cpp:13-20 */
static V3 htransform(const float* m, V3 p) {
    float iw = 1 / (m[12] * p.x + m[13] * p.y + m[14] * p.z + m[15]);
    return v3((m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3]) * iw,
              (m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7]) * iw,
              (m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]) * iw);
}

static void paint_triangle(Frame* F, const Vtx* v0, const Vtx* v1, const Vtx* v2, int world, uint32_t id);

/* clip, src/Renderer.cpp:121-129 */
static Vtx clip_vtx(float z, const Vtx* a, const Vtx* b) {
    float k = (fabsf(b->pos.z - a->pos.z) < 1e-6f) ? 0.5f : (z - a->pos.z) / (b->pos.z - a->pos.z);
    Vtx v;
    v.pos = v3_add(v3_ks(k, b->pos), v3_ks(1 - k, a->pos));
    v.nrm = v3_add(v3_ks(k, b->nrm), v3_ks(1 - k, a->nrm));
    v.uv = v2_add(v2_ks(k, b->uv), v2_ks(1 - k, a->uv));
    return v;
}

/* clipTriangle, src/Renderer.cpp:131-161.  Sub-triangle ids: id+0 for the
 * first paintTriangle call, id+1 for the second (quad case). */
static void clip_triangle(Frame* F, float z, Vtx* v, uint32_t id) {
    if (v[0].pos.z > z && v[1].pos.z > z && v[2].pos.z > z) return;
    while (v[0].pos.z < v[1].pos.z || v[0].pos.z < v[2].pos.z) {
        Vtx t = v[0]; v[0] = v[1]; v[1] = t;
        t = v[0]; v[0] = v[2]; v[2] = t;
    }
    if (v[1].pos.z > z) {
        Vtx v02 = clip_vtx(z, &v[0], &v[2]);
        Vtx v12 = clip_vtx(z, &v[1], &v[2]);
        paint_triangle(F, &v02, &v12, &v[2], 0, id);
    } else if (v[2].pos.z > z) {
        Vtx v01 = clip_vtx(z, &v[0], &v[1]);
        Vtx v12 = clip_vtx(z, &v[1], &v[2]);
        paint_triangle(F, &v01, &v[1], &v12, 0, id);
    } else {
        Vtx v01 = clip_vtx(z, &v[0], &v[1]);
        Vtx v02 = clip_vtx(z, &v[0], &v[2]);
        paint_triangle(F, &v01, &v[1], &v[2], 0, id);
        paint_triangle(F, &v01, &v[2], &v02, 0, id + 1);
    }
}

/* paintTriangle, src/Renderer.cpp:163-309 (PREMULT and FAST_LIGHT defined,
 * src/Renderer.cpp:4-5). */
static void paint_triangle(Frame* F, const Vtx* a, const Vtx* b, const Vtx* c, int world, uint32_t id) {
    V3 vertices[3] = {a->pos, b->pos, c->pos};
    V3 normals[3] = {a->nrm, b->nrm, c->nrm};
    V2 texcoords[3] = {a->uv, b->uv, c->uv};
    float zn = F->znear;
    /* near-plane test, :169-177 */
    if (world && (vertices[0].z > zn || vertices[1].z > zn || vertices[2].z > zn)) {
        if (vertices[0].z > zn && vertices[1].z > zn && vertices[2].z > zn) return;
        Vtx verts[3] = {*a, *b, *c};
        clip_triangle(F, zn, verts, id);
        return;
    }
    float w = (float)F->W, h = (float)F->H;
    V3 ndc[3];
    V2 p[3];
    V2 pmin = v2(1e30f, 1e30f), pmax = v2(-1e30f, -1e30f);
    for (int i = 0; i < 3; i++) ndc[i] = htransform(F->P, vertices[i]); /* :186-189 */
    for (int i = 0; i < 3; i++) {                                          /* :193-200 */
        p[i].x = (1 + ndc[i].x) * (w / 2);
        p[i].y = (1 - ndc[i].y) * (h / 2);
        pmin = v2(fminr(pmin.x, p[i].x), fminr(pmin.y, p[i].y));
        pmax = v2(fmaxr(pmax.x, p[i].x), fmaxr(pmax.y, p[i].y));
    }
    if (pmax.x < 0 || pmax.y < 0 || pmin.x > w || pmin.y > h) return; /* :202-203 */
    V2 d0 = v2_sub(p[0], p[1]), d2 = v2_sub(p[2], p[1]);
    float area = d0.x * d2.y - d0.y * d2.x; /* :205 */
    if (area <= 0) return;                  /* :207-210 back-face cull */
    float i2a = (area == 0) ? 0.0f : -1.0f / area;
    V2 e02 = v2_sub(p[0], p[2]), e10 = v2_sub(p[1], p[0]);
    V2 n1 = v2(-e02.y * i2a, e02.x * i2a); /* :215 perpend()*i2a */
    V2 n2 = v2(-e10.y * i2a, e10.x * i2a); /* :216 */
    pmin.x = clampr(pmin.x, 0.f, w - 1);   /* :218-221 */
    pmax.x = clampr(pmax.x, 0.f, w - 1);
    pmin.y = clampr(pmin.y, 0.f, h - 1);
    pmax.y = clampr(pmax.y, 0.f, h - 1);
    float zz[4] = {ndc[0].z, ndc[1].z, ndc[2].z, 1};
    float iz[4] = {-1 / vertices[0].z, -1 / vertices[1].z, -1 / vertices[2].z, 1};
    int persp = F->persp;
    const mr_material* M = F->mat;
    int hasspecular = M->shininess != 0;
    int hastexture = F->texturing && F->tex != NULL && F->tex->rows > 0;
    V3 color = v3(M->diffuse[0], M->diffuse[1], M->diffuse[2]);
    V3 emissive = v3(M->emissive[0], M->emissive[1], M->emissive[2]);
    V3 mspecular = v3(M->specular[0], M->specular[1], M->specular[2]);
    float shininess = M->shininess;
    float k[4] = {0, 0, 0, 0};
    const int W = F->W;
    /* raster, :238-269 */
    for (float y = floorf(pmin.y) + 0.5f; y <= pmax.y + 0.5f; y++) {
        V2 pt = v2(floorf(pmin.x) + 0.5f, y);
        V2 q2 = v2_sub(pt, p[2]), q0 = v2_sub(pt, p[0]);
        float e1 = n1.x * q2.x + n1.y * q2.y;
        float e2 = n2.x * q0.x + n2.y * q0.y;
        for (float x = pt.x; x <= pmax.x + 0.5f; x++, e1 += n1.x, e2 += n2.x) {
            if (e1 < 0 || e2 < 0 || 1 - e1 - e2 < 0) continue;
            k[0] = 1.f - e1 - e2;
            k[1] = e1;
            k[2] = e2;
            float z;
            if (persp) {
                z = 1.f / (k[0] * iz[0] + k[1] * iz[1] + k[2] * iz[2]);
                k[0] *= iz[0] * z;
                k[1] *= iz[1] * z;
                k[2] *= iz[2] * z;
            } else {
                z = k[0] * zz[0] + k[1] * zz[1] + k[2] * zz[2] + k[3] * zz[3];
            }
            int i = (int)y, j = (int)x;
            size_t px = (size_t)i * W + j;
            if (!(z < F->depth[px])) continue; /* :267 strict less */
            F->depth[px] = z;
            F->ids[px] = id;
            /* shade, :271-305 */
            if (hastexture) {
                V2 uv = v2_add(v2_add(v2_ks(k[0], texcoords[0]), v2_ks(k[1], texcoords[1])),
                               v2_ks(k[2], texcoords[2]));
                int ti = (int)(fractr(uv.y) * F->tex->rows);
                int tj = (int)(fractr(uv.x) * F->tex->cols);
                if (ti < 0) ti = 0;
                if (ti >= F->tex->rows) ti = F->tex->rows - 1;
                if (tj < 0) tj = 0;
                if (tj >= F->tex->cols) tj = F->tex->cols - 1;
                const float* t = F->tex->rgb + 3 * ((size_t)ti * F->tex->cols + tj);
                color = v3(t[0], t[1], t[2]);
            }
            V3 value = emissive;
            if (F->lighting) {
                V3 position = v3_add(v3_add(v3_ks(k[0], vertices[0]), v3_ks(k[1], vertices[1])),
                                     v3_ks(k[2], vertices[2]));
                V3 lightdir = F->point ? v3_normalized(v3_sub(F->lightdir, position)) : F->lightdir;
                V3 normal = v3_add(v3_add(v3_ks(k[0], normals[0]), v3_ks(k[1], normals[1])),
                                   v3_ks(k[2], normals[2]));
                float s = fmaxr(0.0f, v3_dot(normal, lightdir)) / v3_len(normal) + F->ambient;
                value = v3_add(value, v3_ks(s, color));
                if (hasspecular) {
                    V3 viewDir = v3_normalized(position);
                    V3 lv = v3_sub(lightdir, viewDir);
                    float specular = powf(fmaxr(v3_dot(lv, normal), 0.0f) / (v3_len(lv) * v3_len(normal)),
                                          shininess);
                    value = v3_add(value, v3_ks(specular, mspecular));
                }
                if (F->save_normals && F->normals) {
                    F->normals[3 * px + 0] = normal.x;
                    F->normals[3 * px + 1] = normal.y;
                    F->normals[3 * px + 2] = normal.z;
                }
            }
            F->image[3 * px + 0] = value.x;
            F->image[3 * px + 1] = value.y;
            F->image[3 * px + 2] = value.z;
        }
    }
}

static int idx_ok(int32_t i, int32_t n) { return i >= 0 && i < n; }

/* paintMesh, src/Renderer.cpp:334-381 (PREMULT). */
static void paint_mesh(Frame* F, const float* view, const mr_renderable* r, const mr_mesh_desc* m,
                       uint32_t tri_base) {
    float mv[16], inv[16], nm[16];
    if (r->flags & MR_RS_MODELVIEW) /* paintTriangle's view-space vertices (identity here) */
        memcpy(mv, r->transform, sizeof(mv));
    else
        mro_mat4_mul(view, r->transform, mv); /* :337 */
    mro_mat4_inverse(mv, inv);           /* :338 */
    m4_transpose(inv, nm);
    V3* vv = (V3*)malloc(sizeof(V3) * (size_t)(m->n_vertices > 0 ? m->n_vertices : 1));
    V3* nn = (V3*)malloc(sizeof(V3) * (size_t)(m->n_normals > 0 ? m->n_normals : 1));
    for (int32_t i = 0; i < m->n_vertices; i++) /* :344-345 */
        vv[i] = m4_apply(mv, v3(m->vertices[3 * i], m->vertices[3 * i + 1], m->vertices[3 * i + 2]));
    for (int32_t i = 0; i < m->n_normals; i++) /* :347-348 */
        nn[i] = m4_apply(nm, v3(m->normals[3 * i], m->normals[3 * i + 1], m->normals[3 * i + 2]));
    int has_uv = m->n_texcoords > 0 && m->n_texcoordsI > 0; /* :371 */
    int32_t ntri = m->n_indices / 3;
    for (int32_t t = 0; t < ntri; t++) {
        int32_t i = 3 * t;
        int32_t ia = m->indices[i], ib = m->indices[i + 1], ic = m->indices[i + 2];
        int32_t na = m->normalsI[i], nb = m->normalsI[i + 1], nc = m->normalsI[i + 2];
        if (!idx_ok(ia, m->n_vertices) || !idx_ok(ib, m->n_vertices) || !idx_ok(ic, m->n_vertices) ||
            !idx_ok(na, m->n_normals) || !idx_ok(nb, m->n_normals) || !idx_ok(nc, m->n_normals))
            continue;
        Vtx A, B, C;
        A.pos = vv[ia]; B.pos = vv[ib]; C.pos = vv[ic];
        A.nrm = nn[na]; B.nrm = nn[nb]; C.nrm = nn[nc];
        A.uv = B.uv = C.uv = v2(0, 0);
        if (has_uv) {
            int32_t ta = m->texcoordsI[i], tb = m->texcoordsI[i + 1], tc = m->texcoordsI[i + 2];
            if (!idx_ok(ta, m->n_texcoords) || !idx_ok(tb, m->n_texcoords) || !idx_ok(tc, m->n_texcoords))
                continue;
            A.uv = v2(m->texcoords[2 * ta], m->texcoords[2 * ta + 1]);
            B.uv = v2(m->texcoords[2 * tb], m->texcoords[2 * tb + 1]);
            C.uv = v2(m->texcoords[2 * tc], m->texcoords[2 * tc + 1]);
        }
        /* world = false (no near-plane clipping) for MR_RS_NO_CLIP, :163-173 */
        paint_triangle(F, &A, &B, &C, (r->flags & MR_RS_NO_CLIP) ? 0 : 1, 2u * (tri_base + (uint32_t)t));
    }
    free(vv);
    free(nn);
}

/* Renderer::render, src/Renderer.cpp:311-332, with clear() :113-119. */
int mro_render(const mr_frame* f, const mr_renderable* rs, int32_t n, const mr_mesh_desc* meshes,
               int32_t n_meshes, const mro_texture* tex, int32_t n_tex, float* image, float* depth,
               uint32_t* ids, float* normals) {
    if (f->width <= 0 || f->height <= 0) return MR_E_INVALID;
    size_t npx = (size_t)f->width * f->height;
    for (size_t i = 0; i < npx; i++) {
        image[3 * i] = f->background[0];
        image[3 * i + 1] = f->background[1];
        image[3 * i + 2] = f->background[2];
        depth[i] = 1e11f;
        ids[i] = MR_NO_TRIANGLE;
        if (f->save_normals && normals) {
            normals[3 * i] = 0; normals[3 * i + 1] = 0; normals[3 * i + 2] = 1;
        }
    }
    Frame F;
    memset(&F, 0, sizeof(F));
    F.W = f->width;
    F.H = f->height;
    F.P = f->projection;
    F.point = f->light_is_point;
    V3 L = v3(f->light[0], f->light[1], f->light[2]);
    F.lightdir = F.point ? m4_apply(f->view, L) : v3_normalized(L); /* :317-320 */
    F.ambient = f->ambient;                                         /* :322 */
    F.persp = f->projection[15] == 0;                               /* :324-326 */
    F.znear = F.persp ? f->projection[11] / (f->projection[10] - 1)
                      : (f->projection[11] + 1) / f->projection[10];
    F.znear = -F.znear;
    F.lighting = f->lighting;
    F.texturing = f->texturing;
    F.save_normals = f->save_normals;
    F.image = image;
    F.depth = depth;
    F.ids = ids;
    F.normals = normals;
    uint32_t base = 0;
    for (int32_t r = 0; r < n; r++) {
        if (rs[r].mesh < 0 || rs[r].mesh >= n_meshes) return MR_E_HANDLE;
        const mr_mesh_desc* m = &meshes[rs[r].mesh];
        /* the switches of the renderable's paint call (MR_RS_OWN_STATE) or
           the frame's; the light's position stays the frame's (:264-289) */
        if (rs[r].flags & MR_RS_OWN_STATE) {
            F.lighting = (rs[r].flags & MR_RS_LIGHTING) != 0;
            F.texturing = (rs[r].flags & MR_RS_TEXTURING) != 0;
            F.point = (rs[r].flags & MR_RS_POINT_LIGHT) != 0;
        } else {
            F.lighting = f->lighting;
            F.texturing = f->texturing;
            F.point = f->light_is_point;
        }
        F.mat = &rs[r].material;
        F.tex = NULL;
        if (rs[r].material.texture >= 0) {
            if (rs[r].material.texture >= n_tex) return MR_E_HANDLE;
            F.tex = &tex[rs[r].material.texture];
        }
        paint_mesh(&F, f->view, &rs[r], m, base);
        base += (uint32_t)(m->n_indices / 3);
    }
    return MR_OK;
}

/* savePPM, src/io.cpp:358-362: (byte)clamp(v*255, 0, 255). */
void mro_quantize_rgb8(const float* image, int64_t n_px, uint8_t* out) {
    for (int64_t i = 0; i < 3 * n_px; i++) out[i] = (uint8_t)clampr(image[i] * 255.0f, 0.0f, 255.0f);
}

/* loadPPM, src/io.cpp:407-410: Vec3(r,g,b)/255.0f. */
void mro_decode_rgb8(const uint8_t* rgb, int64_t n_px, float* out) {
    for (int64_t i = 0; i < 3 * n_px; i++) out[i] = (float)rgb[i] / 255.0f;
}

/* getRangeImage, src/Renderer.cpp:388-415. */
void mro_range_image(const mr_frame* f, const float* depth, float* xyz) {
    const float* P = f->projection;
    int persp = P[15] == 0;
    float zfar = persp ? P[11] / (P[10] + 1) : (P[11] - 1) / P[10];
    float fardepth = persp ? zfar : 1.0f;
    float w = (float)f->width, h = (float)f->height;
    for (int i = 0; i < f->height; i++)
        for (int j = 0; j < f->width; j++) {
            size_t px = (size_t)i * f->width + j;
            float* o = xyz + 3 * px;
            if (depth[px] > fardepth) {
                o[0] = 0; o[1] = 0; o[2] = 0;
            } else {
                float u = (j + 0.5f) / (w / 2) - 1;
                float v = -(i + 0.5f) / (h / 2) + 1;
                float z = -depth[px];
                o[0] = -(u + P[2]) * z / P[0];
                o[1] = -(v + P[6]) * z / P[5];
                o[2] = z;
            }
        }
}

/* ---- multi-threaded throughput harness (CPU baseline) ---------------- */
typedef struct {
    const mr_frame* f;
    const mr_renderable* rs;
    int32_t n;
    const mr_mesh_desc* meshes;
    int32_t n_meshes;
    const mro_texture* tex;
    int32_t n_tex;
    int32_t frames;
} Job;

static void* job_main(void* arg) {
    Job* j = (Job*)arg;
    size_t npx = (size_t)j->f->width * j->f->height;
    float* image = (float*)malloc(sizeof(float) * 3 * npx);
    float* depth = (float*)malloc(sizeof(float) * npx);
    uint32_t* ids = (uint32_t*)malloc(sizeof(uint32_t) * npx);
    for (int32_t k = 0; k < j->frames; k++)
        mro_render(j->f, j->rs, j->n, j->meshes, j->n_meshes, j->tex, j->n_tex, image, depth, ids, NULL);
    free(image);
    free(depth);
    free(ids);
    return NULL;
}

double mro_render_frames_mt(const mr_frame* f, const mr_renderable* rs, int32_t n,
                            const mr_mesh_desc* meshes, int32_t n_meshes, const mro_texture* tex,
                            int32_t n_tex, int32_t n_frames, int32_t n_threads) {
    if (n_threads < 1) n_threads = 1;
    if (n_threads > n_frames) n_threads = n_frames;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * n_threads);
    Job* jobs = (Job*)malloc(sizeof(Job) * n_threads);
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int32_t t = 0; t < n_threads; t++) {
        Job j = {f, rs, n, meshes, n_meshes, tex, n_tex, n_frames / n_threads + (t < n_frames % n_threads)};
        jobs[t] = j;
        pthread_create(&th[t], NULL, job_main, &jobs[t]);
    }
    for (int32_t t = 0; t < n_threads; t++) pthread_join(th[t], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    free(th);
    free(jobs);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
