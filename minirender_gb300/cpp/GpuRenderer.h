// GpuRenderer: minirender's Renderer interface (include/minirender/Renderer.h:
// 17-64) rendering on the GB300 path through the C ABI of
// libminirender_gpu.so (include/minirender_gpu.h).
//
// A maintainer adds this file and GpuRenderer.cpp to the reference's build
// and uses GpuRenderer where the code used Renderer: the same public methods
// with the same argument meaning, over the reference's own scene model
// (minirender/Scene.h) and ASL types.  Scene::collectShapes (src/Scene.cpp:
// 13-36) still flattens the scene; meshes and textures become resident on
// the device and only the renderables, matrices and materials travel per
// frame.
//
// Differences a caller sees:
//  * Errors are reported, not hidden: the constructor throws GpuError when
//    no CUDA device can be used (there is no CPU fallback), and every
//    failing library call throws GpuError with the library's status and
//    reason.
//  * Meshes are cached by TriMesh pointer together with the addresses and
//    lengths of their six arrays; a mesh whose arrays were reallocated or
//    resized is sent again automatically.  A mesh edited in place (the same
//    arrays, new contents, e.g. after TriMesh::applyTransform) must be
//    announced with meshChanged().  setScene() forgets the cached meshes.
//  * Textures are cached by Material; the cache holds a reference to the
//    Material, so an entry can never outlive it.  A texture edited in place
//    is announced with textureChanged().
//  * paintMesh / paintTriangle after render() or clear() are recorded and
//    rendered with the frame, in call order, when an image is next read: the
//    same pixels as painting them one after the other.  State follows the
//    reference call by call: paintMesh uses the view current at the call,
//    every paint the lighting, texturing and light-type switches current at
//    the call; the light is placed as the last render() placed it (with no
//    render() since clear(), as the first paint finds it); the background
//    is the one of the last clear() / render().  Projection and the normals
//    switch are the frame's: the state when the image is read.
//  * The caches hold the meshes and textures of the frame last drawn:
//    entries the next frame does not use are freed.  A TriMesh or Material
//    destroyed and replaced by another at the same address with arrays of
//    the same addresses and lengths is taken for the old one unless
//    meshChanged() / textureChanged() says otherwise.
//  * Beyond the reference: getImageRGB8() (savePPM's bytes, src/io.cpp:
//    358-362, computed on the device) and getTriangleIds().
#ifndef MINIRENDER_GPU_RENDERER_H
#define MINIRENDER_GPU_RENDERER_H

#include <asl/Array2.h>
#include <minirender/Scene.h>
#include <minirender_gpu.h>

#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace minirender {

// A failing library call: status is the library's MR_E_* code.
class GpuError : public std::runtime_error {
 public:
  GpuError(int status, const std::string& what) : std::runtime_error(what), status(status) {}
  int status;
};

class GpuRenderer {
 public:
  explicit GpuRenderer(int device = 0);
  ~GpuRenderer();
  GpuRenderer(const GpuRenderer&) = delete;
  GpuRenderer& operator=(const GpuRenderer&) = delete;

  void setSize(int w, int h);
  float aspect() const { return (float)_w / _h; }
  void setScene(asl::Shared<Scene> scene);
  void setProjection(const asl::Matrix4& m) { _projection = m; }
  void setView(const asl::Matrix4& m) { _view = m; }
  void setLight(const asl::Vec3& v, bool point = false) {
    _light = v;
    _lightIsPoint = point;
  }
  void setMaterial(asl::Shared<Material> material) { _material = material; }
  void setLighting(bool on) { _lighting = on; }
  void setTexturing(bool on) { _texturing = on; }
  void setSaveNormals(bool on) { _saveNormals = on; }
  void setBackground(const asl::Vec3& color) { _bgcolor = color; }
  void clear();
  void render();
  void paintMesh(TriMesh* mesh, const asl::Matrix4& transform = asl::Matrix4::identity());
  void paintTriangle(const Vertex& a, const Vertex& b, const Vertex& c, bool world = true);
  asl::Array2<float> getDepth();
  asl::Array2<asl::Vec3> getImage();
  asl::Array2<asl::Vec3> getRangeImage();
  asl::Array2<asl::Vec3> getNormalsImage();

  // Beyond the reference.
  std::vector<uint8_t> getImageRGB8();      // rows x cols x 3 bytes
  std::vector<uint32_t> getTriangleIds();   // MR_NO_TRIANGLE for background
  void meshChanged(TriMesh* mesh);          // re-send a mesh edited in place
  void textureChanged(Material* material);  // re-send a texture edited in place
  mr_ctx* context() const { return _ctx; }

 private:
  struct MeshEntry {
    int32_t handle = -1;
    const void* arrays[6] = {};
    int lengths[6] = {};
    bool stale = false;
  };
  struct TexEntry {
    int32_t handle = -1;
    asl::Shared<Material> owner;  // keeps the Material (and the key) alive
    const void* data = nullptr;
    int rows = 0, cols = 0;
    bool stale = false;
  };
  // paintTriangle calls in a row with one material and clip mode: one
  // mesh of view-space vertices (3 per triangle).
  struct TriangleRun {
    std::vector<float> pos, nrm, uv;
    std::vector<int32_t> idx;
    int32_t handle = -1;
    int sent = -1;  // triangles on the device
  };
  struct Item {
    TriMesh* mesh = nullptr;  // null: triangle run `run`
    int run = -1;
    asl::Matrix4 transform;
    asl::Shared<Material> material;
    int32_t flags = 0;
  };

  void check(int status, const char* what) const;
  void prune();
  void fixFrame();
  int32_t paintFlags() const;
  int32_t meshHandle(TriMesh* m);
  int32_t textureHandle(const asl::Shared<Material>& mat);
  int32_t runHandle(TriangleRun& r);
  mr_frame frame() const;
  void flush();
  void read();

  mr_ctx* _ctx = nullptr;
  int _w = 0, _h = 0;
  asl::Matrix4 _projection, _view;
  // the state that placed the frame's light (render(), or the first paint
  // after clear()): view, light and the default switches of the frame
  asl::Matrix4 _frameView;
  asl::Vec3 _frameLight, _clearBg;
  bool _frameLightIsPoint = false, _frameLighting = true, _frameTexturing = true;
  bool _haveFrame = false;
  asl::Vec3 _light, _bgcolor;
  bool _lightIsPoint = false, _lighting = true, _texturing = true, _saveNormals = false;
  asl::Shared<Scene> _scene;
  asl::Shared<Scene> _drawn;     // the scene of the draw list (kept alive with its meshes)
  asl::Shared<Material> _material, _defmaterial;
  std::map<TriMesh*, MeshEntry> _meshes;
  std::map<Material*, TexEntry> _textures;
  std::vector<TriangleRun> _runs;
  std::vector<Item> _items;      // the frame's draw list, in draw order
  bool _rendered = false;        // the draw list is on the device
  bool _have = false;            // host copies below hold that frame
  std::vector<float> _image, _depth, _normals;
  std::vector<uint8_t> _rgb8;
  std::vector<uint32_t> _ids;
};

}  // namespace minirender

#endif
