// TEST INFRASTRUCTURE.  Stand-in for the scene model of the reference's
// include/minirender/Scene.h, for building the C++ binding
// (minirender_gb300/cpp/GpuRenderer.*) and its test driver where the
// reference sources are absent.  The binding is written against the
// reference's type and member names, so these are the same: Vertex,
// Material, Renderable, SceneNode, Shape, TriMesh, Scene and the members the
// binding and the driver use (no bounding boxes, no texture names).  Where
// the reference is present the binding is compiled against its own header.
#ifndef MR_TEST_SCENE_STANDIN_H
#define MR_TEST_SCENE_STANDIN_H
#include <asl/Array.h>
#include <asl/Array2.h>
#include <asl/Matrix4.h>
#include <asl/Pointer.h>
#include <asl/Vec2.h>
#include <asl/Vec3.h>

namespace minirender {

struct Vertex {
  asl::Vec3 position, normal;
  asl::Vec2 uv;
  Vertex() {}
  Vertex(const asl::Vec3& p, const asl::Vec3& n, const asl::Vec2& t) : position(p), normal(n), uv(t) {}
};

struct TriMesh;

struct Material {
  asl::Vec3 diffuse, specular, emissive;
  float shininess, opacity;
  asl::Array2<asl::Vec3> texture;
  Material();
};

struct Renderable {
  TriMesh* mesh;
  asl::Matrix4 transform;
  Renderable() : mesh(0) {}
  Renderable(TriMesh* m, const asl::Matrix4& t) : mesh(m), transform(t) {}
};

struct SceneNode {
  bool visible;
  asl::Matrix4 transform;
  asl::Array<asl::Shared<SceneNode>> children;
  SceneNode();
  virtual ~SceneNode() {}
  virtual void collectShapes(asl::Array<Renderable>& list, const asl::Matrix4& xform);
};

struct Shape : public SceneNode {
  asl::Shared<Material> material;
};

struct TriMesh : public Shape {
  asl::Array<asl::Vec3> vertices, normals;
  asl::Array<asl::Vec2> texcoords;
  asl::Array<int> indices, normalsI, texcoordsI;
  void collectShapes(asl::Array<Renderable>& list, const asl::Matrix4& xform) override;
};

struct Scene : public SceneNode {
  float ambientLight;
  Scene();
  void add(const asl::Shared<SceneNode>& node) { children << node; }
};

}  // namespace minirender
#endif
