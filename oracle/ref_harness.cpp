// ORACLE -- test infrastructure only.  C entry points that drive the
// reference's own minirender::Renderer (src/Renderer.cpp), Scene
// (src/Scene.cpp) and primitive generators (src/primitives.cpp), compiled
// unmodified against the ASL stand-in in oracle/asl_shim by oracle/Makefile.
// The product never loads this; tests use it to pin mr_oracle.c.
#include <string.h>

#include <vector>

#include "minirender/Renderer.h"
#include "minirender/io.h"
#include "minirender/primitives.h"
#include "../include/minirender_gpu.h"

using namespace asl;
using namespace minirender;

static Matrix4 to_m4(const float* m) {
  return Matrix4(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8], m[9], m[10], m[11], m[12],
                 m[13], m[14], m[15]);
}
static void from_m4(const Matrix4& a, float* m) {
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) m[4 * i + j] = a(i, j);
}

struct RefTexture {
  const float* rgb;
  int32_t rows, cols;
};

static Shared<TriMesh> make_mesh(const mr_mesh_desc& d) {
  Shared<TriMesh> m = new TriMesh();
  for (int i = 0; i < d.n_vertices; i++)
    m->vertices << Vec3(d.vertices[3 * i], d.vertices[3 * i + 1], d.vertices[3 * i + 2]);
  for (int i = 0; i < d.n_normals; i++)
    m->normals << Vec3(d.normals[3 * i], d.normals[3 * i + 1], d.normals[3 * i + 2]);
  for (int i = 0; i < d.n_texcoords; i++) m->texcoords << Vec2(d.texcoords[2 * i], d.texcoords[2 * i + 1]);
  for (int i = 0; i < d.n_indices; i++) m->indices << d.indices[i];
  for (int i = 0; i < d.n_normalsI; i++) m->normalsI << d.normalsI[i];
  for (int i = 0; i < d.n_texcoordsI; i++) m->texcoordsI << d.texcoordsI[i];
  return m;
}

extern "C" {

// Builds a Scene from a pre-order node array (node 0 = the Scene root) and
// renders it with the reference Renderer.  normals may be NULL.
int ref_render(const mr_frame* f, const mr_node* nodes, int32_t n_nodes, const mr_mesh_desc* meshes,
               int32_t n_meshes, const RefTexture* tex, int32_t n_tex, float* image, float* depth,
               float* normals, float* range_xyz) {
  if (n_nodes < 1 || nodes[0].parent != -1 || nodes[0].mesh != -1) return MR_E_INVALID;
  Shared<Scene> scene = new Scene();
  scene->transform = to_m4(nodes[0].transform);
  scene->ambientLight = f->ambient;
  std::vector<Shared<SceneNode>> made(n_nodes);
  made[0] = scene;
  for (int i = 1; i < n_nodes; i++) {
    const mr_node& nd = nodes[i];
    if (nd.parent < 0 || nd.parent >= i) return MR_E_INVALID;
    Shared<SceneNode> node;
    if (nd.mesh >= 0) {
      if (nd.mesh >= n_meshes) return MR_E_HANDLE;
      Shared<TriMesh> m = make_mesh(meshes[nd.mesh]);
      if (nd.has_material) {
        Shared<Material> mat = new Material();
        mat->diffuse = Vec3(nd.material.diffuse[0], nd.material.diffuse[1], nd.material.diffuse[2]);
        mat->specular = Vec3(nd.material.specular[0], nd.material.specular[1], nd.material.specular[2]);
        mat->emissive = Vec3(nd.material.emissive[0], nd.material.emissive[1], nd.material.emissive[2]);
        mat->shininess = nd.material.shininess;
        int t = nd.material.texture;
        if (t >= 0) {
          if (t >= n_tex) return MR_E_HANDLE;
          mat->texture.resize(tex[t].rows, tex[t].cols);
          for (int a = 0; a < tex[t].rows; a++)
            for (int b = 0; b < tex[t].cols; b++) {
              const float* p = tex[t].rgb + 3 * ((size_t)a * tex[t].cols + b);
              mat->texture(a, b) = Vec3(p[0], p[1], p[2]);
            }
        }
        m->material = mat;
      }
      node = m;
    } else {
      node = new SceneNode();
    }
    node->transform = to_m4(nd.transform);
    made[nd.parent]->children << node;
    made[i] = node;
  }
  Renderer r;
  r.setSaveNormals(f->save_normals != 0);
  r.setBackground(Vec3(f->background[0], f->background[1], f->background[2]));
  r.setSize(f->width, f->height);
  r.setScene(scene);
  r.setProjection(to_m4(f->projection));
  r.setView(to_m4(f->view));
  r.setLight(Vec3(f->light[0], f->light[1], f->light[2]), f->light_is_point != 0);
  r.setLighting(f->lighting != 0);
  r.setTexturing(f->texturing != 0);
  r.render();
  Array2<Vec3> img = r.getImage();
  Array2<float> dep = r.getDepth();
  size_t npx = (size_t)f->width * f->height;
  for (size_t i = 0; i < npx; i++) {
    const Vec3& v = img.data()[i];
    image[3 * i] = v.x;
    image[3 * i + 1] = v.y;
    image[3 * i + 2] = v.z;
    depth[i] = dep.data()[i];
  }
  if (normals && f->save_normals) {
    Array2<Vec3> nrm = r.getNormalsImage();
    for (size_t i = 0; i < npx; i++) {
      normals[3 * i] = nrm.data()[i].x;
      normals[3 * i + 1] = nrm.data()[i].y;
      normals[3 * i + 2] = nrm.data()[i].z;
    }
  }
  if (range_xyz) {
    Array2<Vec3> pts = r.getRangeImage();
    for (size_t i = 0; i < npx; i++) {
      range_xyz[3 * i] = pts.data()[i].x;
      range_xyz[3 * i + 1] = pts.data()[i].y;
      range_xyz[3 * i + 2] = pts.data()[i].z;
    }
  }
  return MR_OK;
}

// Reference primitive generators.  kind: 0 cube(a), 1 cylinder(a, b, seg,
// hseg, caps), 2 sphere(a, lat=seg, lon=hseg).  Call with NULL buffers to get
// the counts (vertices, normals, texcoords, indices).
int ref_primitive(int kind, float a, float b, int seg, int hseg, int caps, int32_t* counts,
                  float* vertices, float* normals, float* texcoords, int32_t* indices,
                  int32_t* normalsI) {
  Shared<TriMesh> m;
  if (kind == 0) m = createCube(a);
  else if (kind == 1) m = createCylinder(a, b, seg, hseg, caps != 0);
  else if (kind == 2) m = createSphere(a, seg, hseg);
  else return MR_E_INVALID;
  counts[0] = m->vertices.length();
  counts[1] = m->normals.length();
  counts[2] = m->texcoords.length();
  counts[3] = m->indices.length();
  counts[4] = m->normalsI.length();
  if (vertices)
    for (int i = 0; i < counts[0]; i++) {
      vertices[3 * i] = m->vertices[i].x; vertices[3 * i + 1] = m->vertices[i].y; vertices[3 * i + 2] = m->vertices[i].z;
    }
  if (normals)
    for (int i = 0; i < counts[1]; i++) {
      normals[3 * i] = m->normals[i].x; normals[3 * i + 1] = m->normals[i].y; normals[3 * i + 2] = m->normals[i].z;
    }
  if (texcoords)
    for (int i = 0; i < counts[2]; i++) {
      texcoords[2 * i] = m->texcoords[i].x; texcoords[2 * i + 1] = m->texcoords[i].y;
    }
  if (indices) memcpy(indices, m->indices.ptr(), sizeof(int32_t) * counts[3]);
  if (normalsI) memcpy(normalsI, m->normalsI.ptr(), sizeof(int32_t) * counts[4]);
  return MR_OK;
}

// Reference projection builders (src/Renderer.cpp:40-83).  kind: 0 ortho,
// 1 perspective (l,r,b,t,n,f); 2 frustum, 3 frustumH, 4 ortho-fov (fov,
// aspect, n, f in p[0..3]).
void ref_projection(int kind, const float* p, float* out) {
  Matrix4 m;
  switch (kind) {
    case 0: m = projectionOrtho(p[0], p[1], p[2], p[3], p[4], p[5]); break;
    case 1: m = projectionPerspective(p[0], p[1], p[2], p[3], p[4], p[5]); break;
    case 2: m = projectionFrustum(p[0], p[1], p[2], p[3]); break;
    case 3: m = projectionFrustumH(p[0], p[1], p[2], p[3]); break;
    default: m = projectionOrtho(p[0], p[1], p[2], p[3]); break;
  }
  from_m4(m, out);
}

// Matrix4 product / inverse as the stand-in ASL computes them.
void ref_mat4_mul(const float* a, const float* b, float* out) { from_m4(to_m4(a) * to_m4(b), out); }
void ref_mat4_inverse(const float* a, float* out) { from_m4(to_m4(a).inverse(), out); }

// ---- loaders: the reference's loadMesh / loadPPM / savePPM / saveSTL
// (src/io.cpp, src/x3d.cpp), flattened for comparison.
struct RefModel {
  std::vector<mr_node> nodes;
  std::vector<TriMesh*> meshes;
  std::vector<const Material*> textures;  // materials with a non-empty texture
  Shared<SceneNode> root;
};

static void flatten(RefModel& M, const Shared<SceneNode>& n, int parent) {
  mr_node nd;
  memset(&nd, 0, sizeof nd);
  nd.parent = parent;
  nd.mesh = -1;
  from_m4(n->transform, nd.transform);
  nd.material.texture = -1;
  nd.opacity = 1.0f;
  if (TriMesh* t = dynamic_cast<TriMesh*>(n.ptr())) {
    nd.mesh = (int32_t)M.meshes.size();
    M.meshes.push_back(t);
    if (t->material) {
      const Material& m = *t->material;
      nd.has_material = 1;
      nd.material.diffuse[0] = m.diffuse.x; nd.material.diffuse[1] = m.diffuse.y; nd.material.diffuse[2] = m.diffuse.z;
      nd.material.specular[0] = m.specular.x; nd.material.specular[1] = m.specular.y;
      nd.material.specular[2] = m.specular.z;
      nd.material.emissive[0] = m.emissive.x; nd.material.emissive[1] = m.emissive.y;
      nd.material.emissive[2] = m.emissive.z;
      nd.material.shininess = m.shininess;
      nd.opacity = m.opacity;
      if (m.texture.rows() > 0) {
        int id = -1;
        for (size_t k = 0; k < M.textures.size(); k++)
          if (M.textures[k] == &m) id = (int)k;
        if (id < 0) {
          id = (int)M.textures.size();
          M.textures.push_back(&m);
        }
        nd.material.texture = id;
      }
    }
  }
  const int self = (int)M.nodes.size();
  M.nodes.push_back(nd);
  for (int i = 0; i < n->children.length(); i++) flatten(M, n->children[i], self);
}

void* ref_model_load(const char* path) {
  Shared<SceneNode> root = loadMesh(path);
  if (!root) return nullptr;
  RefModel* M = new RefModel();
  M->root = root;
  flatten(*M, root, -1);
  return M;
}
void ref_model_counts(void* h, int32_t* n_nodes, int32_t* n_meshes, int32_t* n_textures) {
  RefModel* M = (RefModel*)h;
  *n_nodes = (int32_t)M->nodes.size();
  *n_meshes = (int32_t)M->meshes.size();
  *n_textures = (int32_t)M->textures.size();
}
void ref_model_nodes(void* h, mr_node* out) {
  RefModel* M = (RefModel*)h;
  memcpy(out, M->nodes.data(), sizeof(mr_node) * M->nodes.size());
}
// counts: vertices, normals, texcoords, indices, normalsI, texcoordsI; arrays may be NULL
void ref_model_mesh(void* h, int i, int32_t* counts, float* vertices, float* normals, float* texcoords,
                    int32_t* indices, int32_t* normalsI, int32_t* texcoordsI) {
  TriMesh* m = ((RefModel*)h)->meshes[i];
  counts[0] = m->vertices.length(); counts[1] = m->normals.length(); counts[2] = m->texcoords.length();
  counts[3] = m->indices.length(); counts[4] = m->normalsI.length(); counts[5] = m->texcoordsI.length();
  for (int k = 0; vertices && k < counts[0]; k++) {
    vertices[3 * k] = m->vertices[k].x; vertices[3 * k + 1] = m->vertices[k].y; vertices[3 * k + 2] = m->vertices[k].z;
  }
  for (int k = 0; normals && k < counts[1]; k++) {
    normals[3 * k] = m->normals[k].x; normals[3 * k + 1] = m->normals[k].y; normals[3 * k + 2] = m->normals[k].z;
  }
  for (int k = 0; texcoords && k < counts[2]; k++) {
    texcoords[2 * k] = m->texcoords[k].x; texcoords[2 * k + 1] = m->texcoords[k].y;
  }
  if (indices && counts[3]) memcpy(indices, m->indices.ptr(), sizeof(int32_t) * counts[3]);
  if (normalsI && counts[4]) memcpy(normalsI, m->normalsI.ptr(), sizeof(int32_t) * counts[4]);
  if (texcoordsI && counts[5]) memcpy(texcoordsI, m->texcoordsI.ptr(), sizeof(int32_t) * counts[5]);
}
// rgb: rows*cols*3 floats (NULL: sizes only)
void ref_model_texture(void* h, int i, int32_t* rows, int32_t* cols, float* rgb) {
  const Array2<Vec3>& t = ((RefModel*)h)->textures[i]->texture;
  *rows = t.rows();
  *cols = t.cols();
  for (int r = 0; rgb && r < t.rows(); r++)
    for (int c = 0; c < t.cols(); c++) {
      const Vec3& v = t(r, c);
      float* o = rgb + 3 * ((size_t)r * t.cols() + c);
      o[0] = v.x; o[1] = v.y; o[2] = v.z;
    }
}
void ref_model_free(void* h) { delete (RefModel*)h; }

// loadPPM: sizes always; floats when rgb is given.  Returns 0 for an empty image.
int ref_ppm_load(const char* path, int32_t* rows, int32_t* cols, float* rgb) {
  Array2<Vec3> t = loadPPM(path);
  *rows = t.rows();
  *cols = t.cols();
  for (int r = 0; rgb && r < t.rows(); r++)
    for (int c = 0; c < t.cols(); c++) {
      float* o = rgb + 3 * ((size_t)r * t.cols() + c);
      o[0] = t(r, c).x; o[1] = t(r, c).y; o[2] = t(r, c).z;
    }
  return t.rows() > 0;
}
void ref_ppm_save(const char* path, const float* rgb, int32_t rows, int32_t cols) {
  Array2<Vec3> t(rows, cols);
  for (int r = 0; r < rows; r++)
    for (int c = 0; c < cols; c++) {
      const float* v = rgb + 3 * ((size_t)r * cols + c);
      t(r, c) = Vec3(v[0], v[1], v[2]);
    }
  savePPM(t, path);
}
void ref_xyz_save(const char* path, const float* xyz, int32_t rows, int32_t cols, const float* transform) {
  Array2<Vec3> t(rows, cols);
  for (int r = 0; r < rows; r++)
    for (int c = 0; c < cols; c++) {
      const float* v = xyz + 3 * ((size_t)r * cols + c);
      t(r, c) = Vec3(v[0], v[1], v[2]);
    }
  if (transform) saveXYZ(t, path, to_m4(transform));
  else saveXYZ(t, path);
}
void ref_stl_save(const char* path, const mr_mesh_desc* d, const float* transform) {
  Shared<TriMesh> m = make_mesh(*d);
  if (transform) m->transform = to_m4(transform);
  saveSTL(m, path);
}

// Material of a paint: diffuse/specular/emissive/shininess and a texture
// index into tex (or -1).
static Shared<Material> make_material(const mr_material& mm, const RefTexture* tex, int32_t n_tex) {
  Shared<Material> mat = new Material();
  mat->diffuse = Vec3(mm.diffuse[0], mm.diffuse[1], mm.diffuse[2]);
  mat->specular = Vec3(mm.specular[0], mm.specular[1], mm.specular[2]);
  mat->emissive = Vec3(mm.emissive[0], mm.emissive[1], mm.emissive[2]);
  mat->shininess = mm.shininess;
  if (mm.texture >= 0 && mm.texture < n_tex) {
    const RefTexture& t = tex[mm.texture];
    mat->texture.resize(t.rows, t.cols);
    for (int a = 0; a < t.rows; a++)
      for (int b = 0; b < t.cols; b++) {
        const float* q = t.rgb + 3 * ((size_t)a * t.cols + b);
        mat->texture(a, b) = Vec3(q[0], q[1], q[2]);
      }
  }
  return mat;
}

// render() of an empty scene with the frame's state (which sets the light
// direction, ambient and near plane paintMesh uses), optionally clear(),
// then n_ops paints in order: kind 0 = paintMesh(meshes[mesh[i]] with
// material[i], transform[16 i..]), kind 1 = setMaterial(material[i]) and
// paintTriangle of tri[24 i..] (3 x position, normal, uv) with world[i],
// kind 2 = setView(transform[16 i..]), kind 3 = setLighting(world[i]),
// kind 4 = setTexturing(world[i]), kind 5 = setLight(transform[16 i..16 i+2],
// point = world[i]), kind 6 = setBackground(transform[16 i..16 i+2]); each
// for the calls after it.
int ref_paint(const mr_frame* f, const mr_mesh_desc* meshes, int32_t n_meshes, const RefTexture* tex,
              int32_t n_tex, int do_clear, int32_t n_ops, const int32_t* kind, const int32_t* mesh,
              const float* transform, const mr_material* material, const float* tri, const int32_t* world,
              float* image, float* depth) {
  Shared<Scene> scene = new Scene();
  scene->ambientLight = f->ambient;
  Renderer r;
  r.setBackground(Vec3(f->background[0], f->background[1], f->background[2]));
  r.setSize(f->width, f->height);
  r.setScene(scene);
  r.setProjection(to_m4(f->projection));
  r.setView(to_m4(f->view));
  r.setLight(Vec3(f->light[0], f->light[1], f->light[2]), f->light_is_point != 0);
  r.setLighting(f->lighting != 0);
  r.setTexturing(f->texturing != 0);
  r.render();
  if (do_clear) r.clear();
  std::vector<Shared<TriMesh>> keep;
  for (int32_t i = 0; i < n_ops; i++) {
    const float* q16 = transform + 16 * i;
    if (kind[i] == 2) {
      r.setView(to_m4(q16));
      continue;
    }
    if (kind[i] == 3) {
      r.setLighting(world[i] != 0);
      continue;
    }
    if (kind[i] == 4) {
      r.setTexturing(world[i] != 0);
      continue;
    }
    if (kind[i] == 5) {
      r.setLight(Vec3(q16[0], q16[1], q16[2]), world[i] != 0);
      continue;
    }
    if (kind[i] == 6) {
      r.setBackground(Vec3(q16[0], q16[1], q16[2]));
      continue;
    }
    Shared<Material> mat = make_material(material[i], tex, n_tex);
    if (kind[i] == 0) {
      if (mesh[i] < 0 || mesh[i] >= n_meshes) return MR_E_HANDLE;
      Shared<TriMesh> m = make_mesh(meshes[mesh[i]]);
      m->material = mat;
      keep.push_back(m);
      r.paintMesh(m.ptr(), to_m4(transform + 16 * i));
    } else {
      r.setMaterial(mat);
      const float* q = tri + 24 * i;
      Vertex v[3];
      for (int c = 0; c < 3; c++) {
        const float* e = q + 8 * c;
        v[c] = Vertex(Vec3(e[0], e[1], e[2]), Vec3(e[3], e[4], e[5]), Vec2(e[6], e[7]));
      }
      r.paintTriangle(v[0], v[1], v[2], world[i] != 0);
    }
  }
  Array2<Vec3> img = r.getImage();
  Array2<float> dep = r.getDepth();
  size_t npx = (size_t)f->width * f->height;
  for (size_t i = 0; i < npx; i++) {
    image[3 * i] = img.data()[i].x;
    image[3 * i + 1] = img.data()[i].y;
    image[3 * i + 2] = img.data()[i].z;
    depth[i] = dep.data()[i];
  }
  return MR_OK;
}

}  // extern "C"
