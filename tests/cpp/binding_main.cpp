// TEST INFRASTRUCTURE.  Drives minirender_gb300/cpp/GpuRenderer (the C++
// binding a maintainer adds beside the reference's Renderer) from a scene
// description written by tests/test_cpp_binding.py, and writes what the
// Renderer getters return so the test can compare it with the oracle.
//
//   binding_main <scene.txt>
//
// scene.txt holds one command per line, executed in order:
//   size W H | projection p0..p15 | view v0..v15 | light x y z point
//   background r g b | switches lighting texturing save_normals
//   lighting B | texturing B       (setLighting / setTexturing alone)
//   texture K ROWS COLS FILE       (float32 RGB texels, as loadPPM leaves them)
//   mesh K FILE NV NN NT NI NNI NTI (float32 vertices, normals, texcoords,
//                                    then int32 indices, normalsI, texcoordsI)
//   node PARENT MESH HAS_MATERIAL d0 d1 d2 s0 s1 s2 e0 e1 e2 SHININESS TEXTURE t0..t15
//                                  (node 0: the Scene; MESH -1: a plain node)
//   ambient A | render | clear
//   paintmesh MESH HAS_MATERIAL d0..e2 SHININESS TEXTURE t0..t15
//   material d0..e2 SHININESS TEXTURE            (setMaterial)
//   triangle WORLD x y z nx ny nz u v x y z nx ny nz u v x y z nx ny nz u v
//   scale NODE F   scales the node's mesh vertices by F in place, then
//                  GpuRenderer::meshChanged (same arrays, new contents)
//   grow NODE T    appends one triangle (a copy of triangle T, pushed 0.5
//                  along +z) to the node's mesh: the arrays are reallocated
//                  and longer, which the binding must notice
//   detach NODE  removes the node from its parent's children (the binding
//                frees the meshes the next frame does not use)
//   attach NODE  appends it to its parent's children again
//   out PREFIX   -> PREFIX.image/.depth/.rgb8/.ids/.range[/.normals]
// Exit status 3 with the message on stdout when the binding throws GpuError.
#include <stdio.h>

#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "GpuRenderer.h"

using namespace minirender;

namespace {

struct MeshData {
  std::vector<float> v, n, t;
  std::vector<int> i, ni, ti;
};

template <class T>
void read_block(FILE* f, std::vector<T>& out, size_t count) {
  out.resize(count);
  if (count && fread(out.data(), sizeof(T), count, f) != count) throw std::runtime_error("short mesh file");
}

MeshData load_mesh(const std::string& path, size_t nv, size_t nn, size_t nt, size_t ni, size_t nni, size_t nti) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) throw std::runtime_error("cannot open " + path);
  MeshData m;
  read_block(f, m.v, 3 * nv);
  read_block(f, m.n, 3 * nn);
  read_block(f, m.t, 2 * nt);
  read_block(f, m.i, ni);
  read_block(f, m.ni, nni);
  read_block(f, m.ti, nti);
  fclose(f);
  return m;
}

asl::Shared<TriMesh> make_mesh(const MeshData& d) {
  asl::Shared<TriMesh> m = new TriMesh();
  for (size_t k = 0; k < d.v.size(); k += 3) m->vertices << asl::Vec3(d.v[k], d.v[k + 1], d.v[k + 2]);
  for (size_t k = 0; k < d.n.size(); k += 3) m->normals << asl::Vec3(d.n[k], d.n[k + 1], d.n[k + 2]);
  for (size_t k = 0; k < d.t.size(); k += 2) m->texcoords << asl::Vec2(d.t[k], d.t[k + 1]);
  for (int x : d.i) m->indices << x;
  for (int x : d.ni) m->normalsI << x;
  for (int x : d.ti) m->texcoordsI << x;
  return m;
}

asl::Matrix4 read_matrix(std::istream& in) {
  float a[16];
  for (float& x : a) in >> x;
  return asl::Matrix4(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10], a[11], a[12], a[13], a[14],
                      a[15]);
}

asl::Vec3 read_vec3(std::istream& in) {
  float x, y, z;
  in >> x >> y >> z;
  return asl::Vec3(x, y, z);
}

asl::Shared<Material> read_material(std::istream& in, const std::vector<asl::Array2<asl::Vec3>>& textures) {
  asl::Shared<Material> m = new Material();
  m->diffuse = read_vec3(in);
  m->specular = read_vec3(in);
  m->emissive = read_vec3(in);
  int tex;
  in >> m->shininess >> tex;
  if (tex >= 0) m->texture = textures[tex];
  return m;
}

template <class T>
void write(const std::string& path, const T* data, size_t count) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f || fwrite(data, sizeof(T), count, f) != count) throw std::runtime_error("cannot write " + path);
  fclose(f);
}

void write_vec3(const std::string& path, const asl::Array2<asl::Vec3>& a) {
  std::vector<float> out;
  for (int i = 0; i < a.rows(); i++)
    for (int j = 0; j < a.cols(); j++) {
      out.push_back(a(i, j).x);
      out.push_back(a(i, j).y);
      out.push_back(a(i, j).z);
    }
  write(path, out.data(), out.size());
}

int run(const char* scene_file) {
  std::ifstream file(scene_file);
  if (!file) throw std::runtime_error("cannot open scene file");
  GpuRenderer r(0);
  std::vector<MeshData> meshes;
  std::vector<asl::Array2<asl::Vec3>> textures;
  std::vector<asl::Shared<SceneNode>> nodes;
  std::vector<int> parents;
  std::vector<asl::Shared<TriMesh>> painted;  // paintMesh meshes stay alive until exit
  asl::Shared<Scene> scene;
  bool save_normals = false, scene_set = false;
  std::string line;
  while (std::getline(file, line)) {
    std::istringstream in(line);
    std::string cmd;
    if (!(in >> cmd)) continue;
    if (cmd == "size") {
      int w, h;
      in >> w >> h;
      r.setSize(w, h);
    } else if (cmd == "projection") {
      r.setProjection(read_matrix(in));
    } else if (cmd == "view") {
      r.setView(read_matrix(in));
    } else if (cmd == "light") {
      asl::Vec3 v = read_vec3(in);
      int point;
      in >> point;
      r.setLight(v, point != 0);
    } else if (cmd == "background") {
      r.setBackground(read_vec3(in));
    } else if (cmd == "switches") {
      int l, t, n;
      in >> l >> t >> n;
      r.setLighting(l != 0);
      r.setTexturing(t != 0);
      r.setSaveNormals(n != 0);
      save_normals = n != 0;
    } else if (cmd == "lighting" || cmd == "texturing") {
      int on;
      in >> on;
      if (cmd == "lighting") r.setLighting(on != 0);
      else r.setTexturing(on != 0);
    } else if (cmd == "texture") {
      int k, rows, cols;
      std::string path;
      in >> k >> rows >> cols >> path;
      std::vector<float> texels;
      FILE* f = fopen(path.c_str(), "rb");
      if (!f) throw std::runtime_error("cannot open " + path);
      read_block(f, texels, (size_t)rows * cols * 3);
      fclose(f);
      asl::Array2<asl::Vec3> t(rows, cols);
      for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++) {
          const float* p = &texels[3 * ((size_t)i * cols + j)];
          t(i, j) = asl::Vec3(p[0], p[1], p[2]);
        }
      textures.resize(k + 1);
      textures[k] = t;
    } else if (cmd == "mesh") {
      int k;
      std::string path;
      size_t nv, nn, nt, ni, nni, nti;
      in >> k >> path >> nv >> nn >> nt >> ni >> nni >> nti;
      meshes.resize(k + 1);
      meshes[k] = load_mesh(path, nv, nn, nt, ni, nni, nti);
    } else if (cmd == "node") {
      int parent, mesh, has_material;
      in >> parent >> mesh >> has_material;
      asl::Shared<Material> mat = read_material(in, textures);
      asl::Shared<SceneNode> node;
      if (parent < 0) {
        scene = new Scene();
        node = scene;
      } else if (mesh >= 0) {
        asl::Shared<TriMesh> m = make_mesh(meshes[mesh]);
        if (has_material) m->material = mat;
        node = m;
      } else {
        node = new SceneNode();
      }
      node->transform = read_matrix(in);
      if (parent >= 0) nodes[parent]->children << node;
      nodes.push_back(node);
      parents.push_back(parent);
    } else if (cmd == "ambient") {
      in >> scene->ambientLight;
    } else if (cmd == "render") {
      if (!scene_set) r.setScene(scene);  // once: setScene forgets the mesh cache
      scene_set = true;
      r.render();
    } else if (cmd == "clear") {
      r.clear();
    } else if (cmd == "paintmesh") {
      int mesh, has_material;
      in >> mesh >> has_material;
      asl::Shared<Material> mat = read_material(in, textures);
      asl::Shared<TriMesh> m = make_mesh(meshes[mesh]);
      if (has_material) m->material = mat;
      painted.push_back(m);
      r.paintMesh(m.operator->(), read_matrix(in));
    } else if (cmd == "material") {
      r.setMaterial(read_material(in, textures));
    } else if (cmd == "triangle") {
      int world;
      in >> world;
      Vertex v[3];
      for (auto& x : v) {
        x.position = read_vec3(in);
        x.normal = read_vec3(in);
        float u, w;
        in >> u >> w;
        x.uv = asl::Vec2(u, w);
      }
      r.paintTriangle(v[0], v[1], v[2], world != 0);
    } else if (cmd == "scale") {
      int k;
      float f;
      in >> k >> f;
      TriMesh* m = dynamic_cast<TriMesh*>(nodes[k].operator->());
      if (!m) throw std::runtime_error("scale: not a mesh node");
      for (int i = 0; i < m->vertices.length(); i++)
        m->vertices[i] = asl::Vec3(m->vertices[i].x * f, m->vertices[i].y * f, m->vertices[i].z * f);
      r.meshChanged(m);
    } else if (cmd == "grow") {
      int k, t;
      in >> k >> t;
      TriMesh* m = dynamic_cast<TriMesh*>(nodes[k].operator->());
      if (!m) throw std::runtime_error("grow: not a mesh node");
      const int nv = m->vertices.length(), nn = m->normals.length(), nt = m->texcoords.length();
      for (int c = 0; c < 3; c++) {
        const asl::Vec3 v = m->vertices[m->indices[3 * t + c]];
        m->vertices << asl::Vec3(v.x, v.y, v.z + 0.5f);
        m->normals << m->normals[m->normalsI[3 * t + c]];
        if (nt && m->texcoordsI.length()) m->texcoords << m->texcoords[m->texcoordsI[3 * t + c]];
      }
      for (int c = 0; c < 3; c++) {
        m->indices << nv + c;
        m->normalsI << nn + c;
        if (nt && m->texcoordsI.length()) m->texcoordsI << nt + c;
      }
    } else if (cmd == "detach" || cmd == "attach") {
      int k;
      in >> k;
      if (k <= 0 || k >= (int)nodes.size()) throw std::runtime_error(cmd + ": no such node");
      asl::Array<asl::Shared<SceneNode>>& children = nodes[parents[k]]->children;
      if (cmd == "attach") {
        children << nodes[k];
      } else {
        asl::Array<asl::Shared<SceneNode>> keep;
        for (int i = 0; i < children.length(); i++)
          if (children[i].operator->() != nodes[k].operator->()) keep << children[i];
        children.clear();
        for (int i = 0; i < keep.length(); i++) children << keep[i];
      }
    } else if (cmd == "out") {
      std::string prefix;
      in >> prefix;
      const asl::Array2<float> depth = r.getDepth();
      std::vector<float> d;
      for (int i = 0; i < depth.rows(); i++)
        for (int j = 0; j < depth.cols(); j++) d.push_back(depth(i, j));
      write(prefix + ".depth", d.data(), d.size());
      write_vec3(prefix + ".image", r.getImage());
      const std::vector<uint8_t> rgb8 = r.getImageRGB8();
      write(prefix + ".rgb8", rgb8.data(), rgb8.size());
      const std::vector<uint32_t> ids = r.getTriangleIds();
      write(prefix + ".ids", ids.data(), ids.size());
      write_vec3(prefix + ".range", r.getRangeImage());
      if (save_normals) write_vec3(prefix + ".normals", r.getNormalsImage());
    } else {
      throw std::runtime_error("unknown command " + cmd);
    }
  }
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 2) {
    fprintf(stderr, "usage: binding_main scene.txt\n");
    return 2;
  }
  try {
    return run(argv[1]);
  } catch (const GpuError& e) {
    printf("GpuError %d %s\n", e.status, e.what());
    return 3;
  } catch (const std::exception& e) {
    printf("error %s\n", e.what());
    return 1;
  }
}
