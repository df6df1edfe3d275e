// GpuRenderer: minirender's Renderer on the GB300 path (see GpuRenderer.h).
#include "GpuRenderer.h"

#include <string.h>

#include <set>

namespace minirender {

namespace {

void rowMajor(const asl::Matrix4& m, float* o) {
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) o[4 * i + j] = m(i, j);
}

bool sameMatrix(const asl::Matrix4& a, const asl::Matrix4& b) {
  float x[16], y[16];
  rowMajor(a, x);
  rowMajor(b, y);
  return memcmp(x, y, sizeof(x)) == 0;
}

template <class T>
const void* first(const asl::Array<T>& a) {
  return a.length() ? (const void*)&a[0] : nullptr;
}

mr_material toMaterial(const Material& m) {
  mr_material r;
  r.diffuse[0] = m.diffuse.x; r.diffuse[1] = m.diffuse.y; r.diffuse[2] = m.diffuse.z;
  r.specular[0] = m.specular.x; r.specular[1] = m.specular.y; r.specular[2] = m.specular.z;
  r.emissive[0] = m.emissive.x; r.emissive[1] = m.emissive.y; r.emissive[2] = m.emissive.z;
  r.shininess = m.shininess;
  r.texture = -1;
  return r;
}

}  // namespace

void GpuRenderer::check(int status, const char* what) const {
  if (status != MR_OK)
    throw GpuError(status, std::string(what) + ": " + mr_status_string(status) + " (" + mr_last_error(_ctx) + ")");
}

// Renderer::Renderer (src/Renderer.cpp:85-98): 800x600, the orthographic
// projection (-40, 40, -30, 30, 50, 120), the light (-0.15, 0.6, 1)
// normalised, the default material, lighting and texturing on, black
// background.  The view starts as the identity.
GpuRenderer::GpuRenderer(int device) {
  const int rc = mr_create(device, &_ctx);
  if (rc != MR_OK) {
    _ctx = nullptr;
    throw GpuError(rc, std::string("mr_create: ") + mr_status_string(rc));
  }
  float p[16];
  mr_projection_ortho(-40, 40, -30, 30, 50, 120, p);
  _projection = asl::Matrix4(p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8], p[9], p[10], p[11], p[12],
                             p[13], p[14], p[15]);
  _view = asl::Matrix4::identity();
  _light = asl::Vec3(-0.15f, 0.6f, 1).normalized();
  _bgcolor = asl::Vec3(0, 0, 0);
  _defmaterial = new Material();
  _material = _defmaterial;
  setSize(800, 600);
}

GpuRenderer::~GpuRenderer() {
  if (_ctx) mr_destroy(_ctx);  // frees every mesh and texture of the context
}

void GpuRenderer::setSize(int w, int h) {
  if (w <= 0 || h <= 0) throw GpuError(MR_E_INVALID, "setSize: sizes must be positive");
  _w = w;
  _h = h;
  clear();
}

void GpuRenderer::setScene(asl::Shared<Scene> scene) {
  // a new scene brings new meshes; the frame drawn so far keeps its own
  // reference to the old scene until the next render() or clear()
  for (auto& e : _meshes)
    if (e.second.handle >= 0) mr_mesh_free(_ctx, e.second.handle);
  _meshes.clear();
  _scene = scene;
}

// Renderer::clear (src/Renderer.cpp:113-119): the next frame read holds the
// background, depth 1e11 and, with normals saved, (0, 0, 1).
void GpuRenderer::clear() {
  _items.clear();
  for (auto& r : _runs)
    if (r.handle >= 0) mr_mesh_free(_ctx, r.handle);
  _runs.clear();
  _drawn = asl::Shared<Scene>();
  _haveFrame = false;
  _clearBg = _bgcolor;  // the image clear() fills (src/Renderer.cpp:113-119)
  _rendered = false;
  _have = false;
}

// Renderer::render (src/Renderer.cpp:311-332): the scene's renderables in
// collectShapes order, each in its mesh's material or the default one
// (src/Renderer.cpp:336), rendered now with the current state.
void GpuRenderer::render() {
  if (!_scene) throw GpuError(MR_E_INVALID, "render: setScene() first");
  asl::Array<Renderable> list;
  _scene->collectShapes(list, asl::Matrix4::identity());
  clear();
  _drawn = _scene;
  fixFrame();  // the light is placed now (src/Renderer.cpp:317-320)
  for (int i = 0; i < list.length(); i++) {
    Item it;
    it.mesh = list[i].mesh;
    it.transform = list[i].transform;
    it.material = it.mesh->material ? it.mesh->material : _defmaterial;
    _items.push_back(it);
  }
  if (!_items.empty()) _material = _items.back().material;  // paintMesh's side effect
  flush();
}

// Renderer::paintMesh (src/Renderer.cpp:334-381): over what is drawn, with
// the current view and `transform`, in the mesh's material or the default.
void GpuRenderer::paintMesh(TriMesh* mesh, const asl::Matrix4& transform) {
  if (!mesh) throw GpuError(MR_E_INVALID, "paintMesh: null mesh");
  if (!_haveFrame) fixFrame();
  Item it;
  it.mesh = mesh;
  it.transform = transform;
  it.flags = paintFlags();
  if (!sameMatrix(_view, _frameView)) {
    // the view changed since the frame's light was placed: the modelview
    // of this call, _view * transform (src/Renderer.cpp:337), composed as
    // the library composes it
    float v[16], t[16], m[16];
    rowMajor(_view, v);
    rowMajor(transform, t);
    mr_mat4_mul(v, t, m);
    it.transform = asl::Matrix4(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8], m[9], m[10], m[11], m[12],
                                m[13], m[14], m[15]);
    it.flags |= MR_RS_MODELVIEW;
  }
  it.material = mesh->material ? mesh->material : _defmaterial;
  _material = it.material;
  _items.push_back(it);
  _rendered = false;
  _have = false;
}

// Renderer::paintTriangle (src/Renderer.cpp:163-309): one triangle of
// view-space vertices in the current material; world = false skips the
// near-plane clip.  Calls in a row that share material and clip mode form
// one mesh whose modelview is the identity (MR_RS_MODELVIEW).
void GpuRenderer::paintTriangle(const Vertex& a, const Vertex& b, const Vertex& c, bool world) {
  if (!_haveFrame) fixFrame();
  const int32_t flags = MR_RS_MODELVIEW | (world ? 0 : MR_RS_NO_CLIP) | paintFlags();
  asl::Shared<Material> mat = _material ? _material : _defmaterial;
  if (_items.empty() || _items.back().run < 0 || _items.back().flags != flags ||
      _items.back().material.operator->() != mat.operator->()) {
    Item it;
    it.run = (int)_runs.size();
    it.transform = asl::Matrix4::identity();
    it.material = mat;
    it.flags = flags;
    _runs.push_back(TriangleRun());
    _items.push_back(it);
  }
  TriangleRun& r = _runs[_items.back().run];
  const Vertex* v[3] = {&a, &b, &c};
  for (int k = 0; k < 3; k++) {
    r.pos.insert(r.pos.end(), {v[k]->position.x, v[k]->position.y, v[k]->position.z});
    r.nrm.insert(r.nrm.end(), {v[k]->normal.x, v[k]->normal.y, v[k]->normal.z});
    r.uv.insert(r.uv.end(), {v[k]->uv.x, v[k]->uv.y});
    r.idx.push_back((int32_t)r.idx.size());
  }
  _rendered = false;
  _have = false;
}

// Renderer::render places the light with the view, light and light type of
// the moment (src/Renderer.cpp:317-320); paints keep it until the next.
void GpuRenderer::fixFrame() {
  _frameView = _view;
  _frameLight = _light;
  _frameLightIsPoint = _lightIsPoint;
  _frameLighting = _lighting;
  _frameTexturing = _texturing;
  _haveFrame = true;
}

// MR_RS_OWN_STATE and the switches of this paint call when they differ from
// the frame's (paintTriangle reads them per call, src/Renderer.cpp:264-289).
int32_t GpuRenderer::paintFlags() const {
  if (_lighting == _frameLighting && _texturing == _frameTexturing && _lightIsPoint == _frameLightIsPoint) return 0;
  return MR_RS_OWN_STATE | (_lighting ? MR_RS_LIGHTING : 0) | (_texturing ? MR_RS_TEXTURING : 0) |
         (_lightIsPoint ? MR_RS_POINT_LIGHT : 0);
}

void GpuRenderer::meshChanged(TriMesh* mesh) {
  auto it = _meshes.find(mesh);
  if (it != _meshes.end()) it->second.stale = true;
  _rendered = false;
  _have = false;
}

void GpuRenderer::textureChanged(Material* material) {
  auto it = _textures.find(material);
  if (it != _textures.end()) it->second.stale = true;
  _rendered = false;
  _have = false;
}

int32_t GpuRenderer::meshHandle(TriMesh* m) {
  const void* arrays[6] = {first(m->vertices), first(m->normals), first(m->texcoords),
                           first(m->indices), first(m->normalsI), first(m->texcoordsI)};
  const int lengths[6] = {m->vertices.length(), m->normals.length(), m->texcoords.length(),
                          m->indices.length(), m->normalsI.length(), m->texcoordsI.length()};
  MeshEntry& e = _meshes[m];
  bool same = e.handle >= 0 && !e.stale;
  for (int k = 0; k < 6 && same; k++) same = e.arrays[k] == arrays[k] && e.lengths[k] == lengths[k];
  if (same) return e.handle;
  // the arrays exactly as the TriMesh holds them: Vec3 = 3 floats, Vec2 = 2
  mr_mesh_desc d;
  d.vertices = (const float*)arrays[0]; d.n_vertices = lengths[0];
  d.normals = (const float*)arrays[1]; d.n_normals = lengths[1];
  d.texcoords = (const float*)arrays[2]; d.n_texcoords = lengths[2];
  d.indices = (const int32_t*)arrays[3]; d.n_indices = lengths[3];
  d.normalsI = (const int32_t*)arrays[4]; d.n_normalsI = lengths[4];
  d.texcoordsI = (const int32_t*)arrays[5]; d.n_texcoordsI = lengths[5];
  // same counts (and the same arrays shared with the indices): copy in
  // place; otherwise a new device mesh
  if (e.handle < 0 || mr_mesh_update(_ctx, e.handle, &d) != MR_OK) {
    if (e.handle >= 0) mr_mesh_free(_ctx, e.handle);
    e.handle = -1;
    check(mr_mesh_upload(_ctx, &d, &e.handle), "mesh upload");
  }
  for (int k = 0; k < 6; k++) {
    e.arrays[k] = arrays[k];
    e.lengths[k] = lengths[k];
  }
  e.stale = false;
  return e.handle;
}

// Material::texture (Array2<Vec3>, as loadPPM fills it, src/io.cpp:407-410),
// sent as floats once per Material.
int32_t GpuRenderer::textureHandle(const asl::Shared<Material>& mat) {
  const asl::Array2<asl::Vec3>& t = mat->texture;
  TexEntry& e = _textures[mat.operator->()];
  const void* data = &t(0, 0);
  if (e.handle >= 0 && !e.stale && e.data == data && e.rows == t.rows() && e.cols == t.cols()) return e.handle;
  std::vector<float> f((size_t)t.rows() * t.cols() * 3);
  for (int i = 0; i < t.rows(); i++)
    for (int j = 0; j < t.cols(); j++) {
      const asl::Vec3& v = t(i, j);
      float* o = &f[3 * ((size_t)i * t.cols() + j)];
      o[0] = v.x;
      o[1] = v.y;
      o[2] = v.z;
    }
  if (e.handle >= 0 && e.rows == t.rows() && e.cols == t.cols()) {
    check(mr_texture_update(_ctx, e.handle, f.data()), "texture update");
  } else {
    if (e.handle >= 0) mr_texture_free(_ctx, e.handle);
    e.handle = -1;
    check(mr_texture_upload_f32(_ctx, f.data(), t.rows(), t.cols(), &e.handle), "texture upload");
  }
  e.owner = mat;
  e.data = data;
  e.rows = t.rows();
  e.cols = t.cols();
  e.stale = false;
  return e.handle;
}

int32_t GpuRenderer::runHandle(TriangleRun& r) {
  const int n = (int)r.idx.size() / 3;
  if (r.handle >= 0 && r.sent == n) return r.handle;
  if (r.handle >= 0) mr_mesh_free(_ctx, r.handle);
  r.handle = -1;
  const int nv = (int)r.idx.size();
  // one index array for positions, normals and texcoords: the library
  // keeps one device copy of it
  mr_mesh_desc d = {r.pos.data(), nv, r.nrm.data(), nv, r.uv.data(), nv,
                    r.idx.data(), nv, r.idx.data(), nv, r.idx.data(), nv};
  check(mr_mesh_upload(_ctx, &d, &r.handle), "triangle upload");
  r.sent = n;
  return r.handle;
}

// The Renderer state render() reads (src/Renderer.cpp:311-326).
mr_frame GpuRenderer::frame() const {
  mr_frame f;
  f.width = _w;
  f.height = _h;
  rowMajor(_projection, f.projection);
  const bool fixed = _haveFrame;
  rowMajor(fixed ? _frameView : _view, f.view);
  const asl::Vec3& light = fixed ? _frameLight : _light;
  f.light[0] = light.x;
  f.light[1] = light.y;
  f.light[2] = light.z;
  f.light_is_point = fixed ? _frameLightIsPoint : _lightIsPoint;
  f.ambient = _drawn ? _drawn->ambientLight : (_scene ? _scene->ambientLight : 0.1f);
  f.background[0] = _clearBg.x;
  f.background[1] = _clearBg.y;
  f.background[2] = _clearBg.z;
  f.lighting = fixed ? _frameLighting : _lighting;
  f.texturing = fixed ? _frameTexturing : _texturing;
  f.save_normals = _saveNormals;
  return f;
}

// Renders the draw list (the last render()'s renderables and the paints
// since, in order) as one frame; an empty list gives the cleared frame.
void GpuRenderer::flush() {
  std::vector<mr_renderable> rs(_items.size());
  for (size_t i = 0; i < _items.size(); i++) {
    const Item& it = _items[i];
    mr_renderable& r = rs[i];
    r.mesh = it.mesh ? meshHandle(it.mesh) : runHandle(_runs[it.run]);
    r.flags = it.flags;
    rowMajor(it.transform, r.transform);
    r.material = toMaterial(*it.material);
    if (it.material->texture.rows() > 0 && it.material->texture.cols() > 0) r.material.texture = textureHandle(it.material);
  }
  const mr_frame f = frame();
  check(mr_render(_ctx, &f, rs.data(), (int32_t)rs.size(), MR_OUT_RGB8 | MR_OUT_DEPTH | MR_OUT_RGB_F32 | MR_OUT_TRI_ID),
        "render");
  _rendered = true;
  _have = false;
  prune();
}

// Frees the cached meshes and textures the frame just drawn does not use.
void GpuRenderer::prune() {
  std::set<TriMesh*> meshes;
  std::set<Material*> materials;
  for (const Item& it : _items) {
    if (it.mesh) meshes.insert(it.mesh);
    materials.insert(it.material.operator->());
  }
  for (auto i = _meshes.begin(); i != _meshes.end();) {
    if (meshes.count(i->first)) {
      ++i;
      continue;
    }
    if (i->second.handle >= 0) mr_mesh_free(_ctx, i->second.handle);
    i = _meshes.erase(i);
  }
  for (auto i = _textures.begin(); i != _textures.end();) {
    if (materials.count(i->first)) {
      ++i;
      continue;
    }
    if (i->second.handle >= 0) mr_texture_free(_ctx, i->second.handle);
    i = _textures.erase(i);
  }
}

void GpuRenderer::read() {
  if (!_rendered) flush();
  if (_have) return;
  const size_t n = (size_t)_w * _h;
  _image.resize(3 * n);
  _depth.resize(n);
  _rgb8.resize(3 * n);
  _ids.resize(n);
  _normals.assign(_saveNormals ? 3 * n : 0, 0.0f);
  check(mr_read(_ctx, _rgb8.data(), _depth.data(), _image.data(), _ids.data(),
                _saveNormals ? _normals.data() : nullptr),
        "read");
  _have = true;
}

asl::Array2<float> GpuRenderer::getDepth() {
  read();
  asl::Array2<float> d(_h, _w);
  for (int i = 0; i < _h; i++)
    for (int j = 0; j < _w; j++) d(i, j) = _depth[(size_t)i * _w + j];
  return d;
}

asl::Array2<asl::Vec3> GpuRenderer::getImage() {
  read();
  asl::Array2<asl::Vec3> a(_h, _w);
  for (int i = 0; i < _h; i++)
    for (int j = 0; j < _w; j++) {
      const float* p = &_image[3 * ((size_t)i * _w + j)];
      a(i, j) = asl::Vec3(p[0], p[1], p[2]);
    }
  return a;
}

// With normals not saved the image is (0, 0, 1) everywhere (the reference
// returns whatever its normals buffer last held).
asl::Array2<asl::Vec3> GpuRenderer::getNormalsImage() {
  read();
  asl::Array2<asl::Vec3> a(_h, _w);
  for (int i = 0; i < _h; i++)
    for (int j = 0; j < _w; j++) {
      if (_saveNormals) {
        const float* p = &_normals[3 * ((size_t)i * _w + j)];
        a(i, j) = asl::Vec3(p[0], p[1], p[2]);
      } else {
        a(i, j) = asl::Vec3(0, 0, 1);
      }
    }
  return a;
}

// Renderer::getRangeImage (src/Renderer.cpp:388-415), computed on the device.
asl::Array2<asl::Vec3> GpuRenderer::getRangeImage() {
  read();
  std::vector<float> xyz(3 * (size_t)_w * _h);
  check(mr_read_range_image(_ctx, xyz.data()), "range image");
  asl::Array2<asl::Vec3> a(_h, _w);
  for (int i = 0; i < _h; i++)
    for (int j = 0; j < _w; j++) {
      const float* p = &xyz[3 * ((size_t)i * _w + j)];
      a(i, j) = asl::Vec3(p[0], p[1], p[2]);
    }
  return a;
}

std::vector<uint8_t> GpuRenderer::getImageRGB8() {
  read();
  return _rgb8;
}

std::vector<uint32_t> GpuRenderer::getTriangleIds() {
  read();
  return _ids;
}

}  // namespace minirender
