// TEST INFRASTRUCTURE.  The scene-model behaviour the C++ binding relies on,
// for the stand-in header beside this file: the flattening order of
// Scene::collectShapes (src/Scene.cpp:13-36: the node's transform applied
// after its parent's, a mesh listed before its children) and the defaults
// of Material, SceneNode and Scene (src/Scene.cpp:7-11, 65-75).
#include "minirender/Scene.h"

namespace minirender {

SceneNode::SceneNode() : visible(true), transform(asl::Matrix4::identity()) {}

void SceneNode::collectShapes(asl::Array<Renderable>& list, const asl::Matrix4& xform) {
  const asl::Matrix4 tr = xform * transform;
  for (int i = 0; i < children.length(); i++) children[i]->collectShapes(list, tr);
}

void TriMesh::collectShapes(asl::Array<Renderable>& list, const asl::Matrix4& xform) {
  const asl::Matrix4 tr = xform * transform;
  list << Renderable(this, tr);
  for (int i = 0; i < children.length(); i++) children[i]->collectShapes(list, tr);
}

Material::Material()
    : diffuse(0.7f, 0.7f, 0.9f), specular(0.8f, 0.8f, 0.8f), emissive(0, 0, 0), shininess(12.0f), opacity(1.0f) {}

Scene::Scene() : ambientLight(0.1f) {}

}  // namespace minirender
