// Model and image files on either side of the rendering path (host code, no
// device work): the reference's loaders src/io.cpp (loadMesh :111-132, loadSTL
// :134-153 with loadSTLa :16-60 and loadSTLb :62-109, saveSTL :155-183,
// loadOBJ :187-335, savePPM :337-362, loadPPM :364-415) and src/x3d.cpp
// (triangulateIndices :17-33, the X3D reader :35-200), producing the scene
// tree, TriMesh arrays and materials the reference builds, as plain arrays
// (mr_node tree in pre-order, mr_mesh_desc per TriMesh, RGB8 textures).
//
// Text is converted the way the reference's string helpers do it here:
// numbers with strtod (then float) / strtol, tokens split at whitespace,
// '/'-separated fields keep empty ones, lines end at '\n' with one trailing
// '\r' dropped.  Large OBJ and binary STL files are parsed on all host
// threads: OBJ lines in contiguous chunks (vertex data and face records per
// chunk, concatenated in file order), STL facets in contiguous ranges.
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include <algorithm>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/minirender_gpu.h"

namespace {

// ------------------------------------------------------------ text helpers
float to_float(const std::string& s) { return (float)strtod(s.c_str(), nullptr); }
int to_int(const std::string& s) { return (int)strtol(s.c_str(), nullptr, 10); }

std::vector<std::string> split_ws(const char* b, const char* e) {
  std::vector<std::string> out;
  while (b < e) {
    while (b < e && isspace((unsigned char)*b)) b++;
    const char* t = b;
    while (b < e && !isspace((unsigned char)*b)) b++;
    if (b > t) out.emplace_back(t, b);
  }
  return out;
}
std::vector<std::string> split_ws(const std::string& s) { return split_ws(s.data(), s.data() + s.size()); }

std::vector<std::string> split_char(const std::string& s, char c) {
  std::vector<std::string> out;
  size_t i = 0;
  for (;;) {
    size_t j = s.find(c, i);
    if (j == std::string::npos) {
      out.push_back(s.substr(i));
      return out;
    }
    out.push_back(s.substr(i, j - i));
    i = j + 1;
  }
}

std::vector<float> floats_of(const std::string& s) {
  std::vector<float> out;
  for (auto& t : split_ws(s)) out.push_back(to_float(t));
  return out;
}
float at(const std::vector<float>& v, size_t i) { return i < v.size() ? v[i] : 0.0f; }
float fat(const std::vector<std::string>& v, size_t i) { return i < v.size() ? to_float(v[i]) : 0.0f; }

bool read_file(const std::string& path, std::string& out) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  out.clear();
  long size = -1;
  if (fseek(f, 0, SEEK_END) == 0) size = ftell(f);
  if (size > 0 && fseek(f, 0, SEEK_SET) == 0) {  // one read into a buffer of the file's size
    out.resize((size_t)size);
    out.resize(fread(&out[0], 1, (size_t)size, f));
  }
  char buf[1 << 16];  // the rest (or all, for a stream without a size)
  size_t k;
  while ((k = fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, k);
  fclose(f);
  return true;
}

std::string directory_of(const std::string& p) {
  size_t s = p.rfind('/');
  return s == std::string::npos ? std::string() : p.substr(0, s);
}
size_t ext_dot(const std::string& p) {
  size_t s = p.rfind('/');
  size_t n = s == std::string::npos ? 0 : s + 1;
  size_t d = p.rfind('.');
  return (d == std::string::npos || d < n) ? std::string::npos : d;
}
bool has_ext(const std::string& p, const char* e) {
  size_t d = ext_dot(p);
  return d != std::string::npos && strcasecmp(p.c_str() + d + 1, e) == 0;
}
std::string no_ext(const std::string& p) {
  size_t d = ext_dot(p);
  return d == std::string::npos ? p : p.substr(0, d);
}

int n_threads() {
  unsigned h = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(h, 64u));
}

// ------------------------------------------------------------ float vectors
struct F3 {
  float x, y, z;
};
F3 sub(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
F3 cross(F3 a, F3 b) { return F3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
F3 normalized(F3 v) {
  float l = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
  return F3{v.x / l, v.y / l, v.z / l};
}

// Matrix4 (row-major) products and constructors in the order the reference's
// matrix helpers sum.
struct M4 {
  float m[16];
};
M4 identity() {
  M4 r{};
  r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1;
  return r;
}
M4 mul(const M4& a, const M4& b) {
  M4 r;
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++)
      r.m[4 * i + j] = a.m[4 * i] * b.m[j] + a.m[4 * i + 1] * b.m[4 + j] + a.m[4 * i + 2] * b.m[8 + j] +
                       a.m[4 * i + 3] * b.m[12 + j];
  return r;
}
M4 translate(float x, float y, float z) {
  M4 r = identity();
  r.m[3] = x;
  r.m[7] = y;
  r.m[11] = z;
  return r;
}
M4 scale(float x, float y, float z) {
  M4 r = identity();
  r.m[0] = x;
  r.m[5] = y;
  r.m[10] = z;
  return r;
}
// rotation by angle t about the (normalized) axis a
M4 rotate(F3 a, float t) {
  F3 u = normalized(a);
  float c = cosf(t), s = sinf(t), k = 1 - c;
  M4 r = identity();
  r.m[0] = k * u.x * u.x + c;
  r.m[1] = k * u.x * u.y - s * u.z;
  r.m[2] = k * u.x * u.z + s * u.y;
  r.m[4] = k * u.x * u.y + s * u.z;
  r.m[5] = k * u.y * u.y + c;
  r.m[6] = k * u.y * u.z - s * u.x;
  r.m[8] = k * u.x * u.z - s * u.y;
  r.m[9] = k * u.y * u.z + s * u.x;
  r.m[10] = k * u.z * u.z + c;
  return r;
}
F3 affine(const float* m, F3 p) {
  return F3{m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
            m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]};
}

// ------------------------------------------------------------ model
struct Mesh {
  std::shared_ptr<std::vector<float>> pos, nrm, uv;  // may be shared between meshes (OBJ)
  std::vector<int32_t> idx, nidx, tidx;
  Mesh()
      : pos(std::make_shared<std::vector<float>>()), nrm(std::make_shared<std::vector<float>>()),
        uv(std::make_shared<std::vector<float>>()) {}
};
struct Texture {
  std::vector<uint8_t> rgb;
  int32_t rows = 0, cols = 0;
};
// The reference's Material defaults (src/Scene.cpp:65-71).
mr_material default_material() {
  mr_material m;
  m.diffuse[0] = 0.7f; m.diffuse[1] = 0.7f; m.diffuse[2] = 0.9f;
  m.specular[0] = m.specular[1] = m.specular[2] = 0.8f;
  m.emissive[0] = m.emissive[1] = m.emissive[2] = 0.0f;
  m.shininess = 12.0f;
  m.texture = -1;
  return m;
}

// Fan triangulation of -1-terminated polygons (src/x3d.cpp:17-33).
std::vector<int32_t> triangulate(const std::vector<int32_t>& ind) {
  std::vector<int32_t> tris;
  tris.reserve(ind.size());
  const int n = (int)ind.size();
  int i = 0, j = 0;
  while (i < n) {
    for (j = i + 1; j < n - 1; j++) {
      if (ind[j] == -1 || ind[j + 1] == -1) break;
      tris.push_back(ind[i]);
      tris.push_back(ind[j]);
      tris.push_back(ind[j + 1]);
    }
    i = j + 2;
  }
  return tris;
}

// Per-face normals (b-a)^(c-a) normalized, one per triangle (src/io.cpp:318-329,
// src/x3d.cpp:151-162).
void face_normals(Mesh& m) {
  auto nrm = std::make_shared<std::vector<float>>();
  m.nidx.clear();
  const std::vector<float>& P = *m.pos;
  auto v = [&](int i) { return F3{P[3 * (size_t)i], P[3 * (size_t)i + 1], P[3 * (size_t)i + 2]}; };
  const size_t nv = P.size() / 3;
  for (size_t i = 0, j = 0; i + 2 < m.idx.size(); i += 3, j++) {
    int32_t ia = m.idx[i], ib = m.idx[i + 1], ic = m.idx[i + 2];
    F3 n{0, 0, 0};
    if (ia >= 0 && ib >= 0 && ic >= 0 && (size_t)ia < nv && (size_t)ib < nv && (size_t)ic < nv)
      n = normalized(cross(sub(v(ib), v(ia)), sub(v(ic), v(ia))));
    nrm->push_back(n.x);
    nrm->push_back(n.y);
    nrm->push_back(n.z);
    m.nidx.push_back((int32_t)j);
    m.nidx.push_back((int32_t)j);
    m.nidx.push_back((int32_t)j);
  }
  m.nrm = nrm;
}

}  // namespace

struct mr_model {
  std::vector<mr_node> nodes;
  std::vector<Mesh> meshes;
  std::vector<Texture> textures;
  std::map<std::string, int32_t> texture_of_path;

  int add_node(int parent, int mesh, const M4& xf, bool has_mat, const mr_material& mat, float opacity = 1.0f) {
    mr_node n;
    memset(&n, 0, sizeof n);
    n.parent = parent;
    n.mesh = mesh;
    memcpy(n.transform, xf.m, sizeof n.transform);
    n.has_material = has_mat ? 1 : 0;
    n.material = has_mat ? mat : default_material();
    n.opacity = has_mat ? opacity : 1.0f;
    nodes.push_back(n);
    return (int)nodes.size() - 1;
  }
  // loadPPM of a material's texture: index into textures, -1 if it cannot be read
  int32_t texture(const std::string& path);
};

namespace {

// ------------------------------------------------------------ PPM
// loadPPM (src/io.cpp:364-415): header characters up to the third newline
// outside comments, exactly four tokens "P6 cols rows max", then rows of
// cols*3 bytes (a short row ends the read; rows not read stay zero).
int ppm_read(const std::string& path, Texture& t) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return MR_E_IO;
  std::string header;
  int nl = 0;
  bool comment = false;
  for (;;) {
    int c = fgetc(f);
    if (c == EOF) break;
    if (c == '\n') {
      if (!comment) nl++;
      comment = false;
    } else if (c == '#') {
      comment = true;
    }
    if (!comment) header += (char)c;
    if (nl >= 3) break;
  }
  std::vector<std::string> parts = split_ws(header);
  if (parts.size() != 4 || parts[0] != "P6") {
    fclose(f);
    return MR_E_IO;
  }
  const int rows = to_int(parts[2]), cols = to_int(parts[1]);
  if (rows <= 0 || cols <= 0 || rows > 65536 || cols > 65536) {
    fclose(f);
    return MR_E_IO;
  }
  t.rows = rows;
  t.cols = cols;
  t.rgb.assign((size_t)rows * cols * 3, 0);
  for (int i = 0; i < rows; i++) {
    size_t n = fread(t.rgb.data() + (size_t)i * cols * 3, 1, (size_t)cols * 3, f);
    if (n < (size_t)cols * 3) {
      memset(t.rgb.data() + (size_t)i * cols * 3, 0, (size_t)cols * 3);  // a short row is not used
      break;
    }
  }
  fclose(f);
  return MR_OK;
}

}  // namespace

int32_t mr_model::texture(const std::string& path) {
  auto it = texture_of_path.find(path);
  if (it != texture_of_path.end()) return it->second;
  Texture t;
  int32_t id = -1;
  if (ppm_read(path, t) == MR_OK) {
    textures.push_back(std::move(t));
    id = (int32_t)textures.size() - 1;
  }
  texture_of_path[path] = id;
  return id;
}

namespace {

// ------------------------------------------------------------ STL
// ASCII STL (loadSTLa): whitespace tokens; "normal" and "vertex" take the
// numbers of the rest of their line; "endfacet" closes a triangle when it
// had three vertices.
bool stl_ascii(const std::string& s, Mesh& m) {
  size_t i = 0;
  const size_t n = s.size();
  auto token = [&](std::string& t) {
    while (i < n && isspace((unsigned char)s[i])) i++;
    size_t b = i;
    while (i < n && !isspace((unsigned char)s[i])) i++;
    t.assign(s, b, i - b);
  };
  auto rest_of_line = [&]() {
    size_t b = i;
    while (i < n && s[i] != '\n') i++;
    size_t e = i;
    if (i < n) i++;
    if (e > b && s[e - 1] == '\r') e--;
    return std::string(s, b, e - b);
  };
  std::string tag;
  token(tag);
  if (tag != "solid") return false;
  int np = 0, iv = 0, in = 0;
  std::vector<float>& P = *m.pos;
  std::vector<float>& N = *m.nrm;
  while (i < n) {
    token(tag);
    if (tag == "endfacet") {
      if (np == 3) {
        m.idx.insert(m.idx.end(), {iv - 3, iv - 2, iv - 1});
        m.nidx.insert(m.nidx.end(), {in - 1, in - 1, in - 1});
      }
      np = 0;
    } else if (tag == "normal") {
      std::vector<float> a = floats_of(rest_of_line());
      N.insert(N.end(), {at(a, 0), at(a, 1), at(a, 2)});
      in++;
    } else if (tag == "vertex") {
      std::vector<float> a = floats_of(rest_of_line());
      P.insert(P.end(), {at(a, 0), at(a, 1), at(a, 2)});
      np++;
      iv++;
    }
  }
  return true;
}

// Binary STL (loadSTLb): 80-byte header, facet count, 50-byte facets (normal,
// three vertices, 2 attribute bytes); facets parsed in parallel ranges.
bool stl_binary(const std::string& s, Mesh& m) {
  int32_t nf;
  memcpy(&nf, s.data() + 80, 4);
  if (nf > 100000000 || nf < 0) return false;
  std::vector<float>& P = *m.pos;
  std::vector<float>& N = *m.nrm;
  P.resize((size_t)nf * 9);
  N.resize((size_t)nf * 3);
  m.idx.resize((size_t)nf * 3);
  m.nidx.resize((size_t)nf * 3);
  auto work = [&](int64_t f0, int64_t f1) {
    for (int64_t f = f0; f < f1; f++) {
      const char* r = s.data() + 84 + f * 50;
      memcpy(&N[(size_t)f * 3], r, 12);
      memcpy(&P[(size_t)f * 9], r + 12, 36);
      for (int c = 0; c < 3; c++) {
        m.idx[(size_t)f * 3 + c] = (int32_t)(3 * f + c);
        m.nidx[(size_t)f * 3 + c] = (int32_t)f;
      }
    }
  };
  const int T = nf > 200000 ? n_threads() : 1;
  std::vector<std::thread> th;
  for (int t = 0; t < T; t++) th.emplace_back(work, (int64_t)nf * t / T, (int64_t)nf * (t + 1) / T);
  for (auto& x : th) x.join();
  return true;
}

// loadSTL: binary when the size is exactly 84 + 50 x (facet count), else ASCII.
int load_stl(const std::string& path, Mesh& m) {
  std::string s;
  if (!read_file(path, s) || s.size() < 5) return MR_E_IO;
  bool binary = false;
  if (s.size() > 84) {
    int32_t nf;
    memcpy(&nf, s.data() + 80, 4);
    if ((int64_t)s.size() == 84 + (int64_t)nf * 50) binary = true;
  }
  return (binary ? stl_binary(s, m) : stl_ascii(s, m)) ? MR_OK : MR_E_IO;
}

// ------------------------------------------------------------ OBJ
struct ObjEvent {
  enum Kind { FACES, USEMTL, MTLLIB } kind;
  std::string name;
  std::vector<int32_t> idx, tidx, nidx;  // FACES: corners with -1 after each face
};
struct ObjChunk {
  std::vector<float> v, vn, vt;
  std::vector<ObjEvent> ev;
};

void obj_parse_lines(const char* b, const char* e, ObjChunk& c) {
  ObjEvent* faces = nullptr;
  while (b < e) {
    const char* le = (const char*)memchr(b, '\n', (size_t)(e - b));
    const char* next = le ? le + 1 : e;
    if (!le) le = e;
    const char* lend = le;
    if (lend > b && lend[-1] == '\r') lend--;
    if (b < lend && *b != '#') {
      std::vector<std::string> parts = split_ws(b, lend);
      if (!parts.empty()) {
        const std::string& k = parts[0];
        if (k == "v") {
          c.v.insert(c.v.end(), {fat(parts, 1), fat(parts, 2), fat(parts, 3)});
        } else if (k == "vn") {
          c.vn.insert(c.vn.end(), {fat(parts, 1), fat(parts, 2), fat(parts, 3)});
        } else if (k == "vt") {
          c.vt.insert(c.vt.end(), {fat(parts, 1), 1.0f - fat(parts, 2)});
        } else if (k == "f") {
          if (!faces) {
            c.ev.push_back(ObjEvent{ObjEvent::FACES, std::string(), {}, {}, {}});
            faces = &c.ev.back();
          }
          for (size_t i = 1; i < parts.size(); i++) {
            std::vector<std::string> f = split_char(parts[i], '/');
            faces->idx.push_back(to_int(f[0]) - 1);
            if (f.size() > 1) faces->tidx.push_back(to_int(f[1]) - 1);
            if (f.size() > 2) faces->nidx.push_back(to_int(f[2]) - 1);
          }
          faces->idx.push_back(-1);
          faces->tidx.push_back(-1);
          faces->nidx.push_back(-1);
        } else if (k == "usemtl" || k == "mtllib") {
          c.ev.push_back(ObjEvent{k == "usemtl" ? ObjEvent::USEMTL : ObjEvent::MTLLIB,
                                  parts.size() > 1 ? parts[1] : std::string(), {}, {}, {}});
          faces = nullptr;
        }
      }
    }
    b = next;
  }
}

// Material library (the mtllib block of src/io.cpp:258-290).  Materials are
// objects: newmtl puts a new one under its name, a mesh keeps the object it
// was given when it was created, and lines before any newmtl modify the
// default material.
struct ObjMaterial {
  mr_material m = default_material();
  float opacity = 1.0f;
  std::string texture_name;
};
using MatPtr = std::shared_ptr<ObjMaterial>;
void obj_mtllib(const std::string& path, std::map<std::string, MatPtr>& mats) {
  std::string s;
  if (!read_file(path, s)) return;
  MatPtr cur = mats[""];
  size_t i = 0;
  while (i < s.size()) {
    size_t j = s.find('\n', i);
    if (j == std::string::npos) j = s.size();
    size_t e = j;
    if (e > i && s[e - 1] == '\r') e--;
    std::vector<std::string> parts = split_ws(s.data() + i, s.data() + e);
    i = j + 1;
    if (parts.empty()) continue;
    const std::string& k = parts[0];
    if (k == "newmtl") {
      cur = std::make_shared<ObjMaterial>();
      mats[parts.size() > 1 ? parts[1] : std::string()] = cur;
      continue;
    }
    ObjMaterial& mt = *cur;
    if (k == "Kd") {
      for (int c = 0; c < 3; c++) mt.m.diffuse[c] = fat(parts, 1 + c);
    } else if (k == "Ks") {
      for (int c = 0; c < 3; c++) mt.m.specular[c] = fat(parts, 1 + c);
    } else if (k == "Ke") {
      for (int c = 0; c < 3; c++) mt.m.emissive[c] = fat(parts, 1 + c);
    } else if (k == "Ns") {
      mt.m.shininess = fat(parts, 1);
      if (mt.m.shininess < 0.0001f) mt.m.shininess = 10;
    } else if (k == "d") {
      mt.opacity = fat(parts, 1);
    } else if (k == "map_Kd") {
      mt.texture_name = parts.size() > 1 ? parts[1] : std::string();
    }
  }
}

int load_obj(const std::string& path, mr_model& M) {
  std::string s;
  if (!read_file(path, s)) return MR_E_IO;
  // 1. chunks of whole lines, parsed in parallel
  const int T = s.size() > (4u << 20) ? n_threads() : 1;
  std::vector<size_t> cut(T + 1, 0);
  cut[T] = s.size();
  for (int t = 1; t < T; t++) {
    size_t p = std::max(cut[t - 1], s.size() * t / T);
    while (p < s.size() && s[p - 1] != '\n') p++;
    cut[t] = p;
  }
  std::vector<ObjChunk> ch(T);
  {
    std::vector<std::thread> th;
    for (int t = 0; t < T; t++)
      th.emplace_back(obj_parse_lines, s.data() + cut[t], s.data() + cut[t + 1], std::ref(ch[t]));
    for (auto& x : th) x.join();
  }
  // 2. vertex data in file order, shared by every mesh
  auto pos = std::make_shared<std::vector<float>>();
  auto nrm = std::make_shared<std::vector<float>>();
  auto uv = std::make_shared<std::vector<float>>();
  for (auto& c : ch) {
    pos->insert(pos->end(), c.v.begin(), c.v.end());
    nrm->insert(nrm->end(), c.vn.begin(), c.vn.end());
    uv->insert(uv->end(), c.vt.begin(), c.vt.end());
  }
  // 3. faces into one mesh per material, in file order
  std::map<std::string, MatPtr> mats;
  mats[""] = std::make_shared<ObjMaterial>();
  struct Group {
    MatPtr material;  // the material object when the group was created
    std::vector<int32_t> idx, tidx, nidx;
  };
  std::map<std::string, Group> groups;
  groups[""] = Group{mats[""], {}, {}, {}};
  Group* cur = &groups[""];
  const std::string dir = directory_of(path);
  for (auto& c : ch)
    for (auto& ev : c.ev) {
      if (ev.kind == ObjEvent::FACES) {
        cur->idx.insert(cur->idx.end(), ev.idx.begin(), ev.idx.end());
        cur->tidx.insert(cur->tidx.end(), ev.tidx.begin(), ev.tidx.end());
        cur->nidx.insert(cur->nidx.end(), ev.nidx.begin(), ev.nidx.end());
      } else if (ev.kind == ObjEvent::USEMTL) {
        if (!groups.count(ev.name)) groups[ev.name] = Group{mats.count(ev.name) ? mats[ev.name] : mats[""], {}, {}, {}};
        cur = &groups[ev.name];
      } else {
        obj_mtllib(dir + "/" + ev.name, mats);
      }
    }
  // 4. textures of the materials still in the library (map_Kd, read as PPM
  //    next to the OBJ)
  std::map<const ObjMaterial*, int32_t> tex_of_mat;
  for (auto& kv : mats)
    if (!kv.second->texture_name.empty()) tex_of_mat[kv.second.get()] = M.texture(dir + "/" + kv.second->texture_name);
  // 5. the scene: a node with one TriMesh per material, in name order
  const int root = M.add_node(-1, -1, identity(), false, default_material());
  for (auto& kv : groups) {
    Group& g = kv.second;
    Mesh m;
    m.pos = pos;
    m.nrm = nrm;
    m.uv = uv;
    m.idx = triangulate(g.idx);
    m.tidx = triangulate(g.tidx);
    m.nidx = triangulate(g.nidx);
    if (nrm->empty()) face_normals(m);
    mr_material mat = g.material->m;
    auto t = tex_of_mat.find(g.material.get());
    mat.texture = t == tex_of_mat.end() ? -1 : t->second;
    M.meshes.push_back(std::move(m));
    M.add_node(root, (int)M.meshes.size() - 1, identity(), true, mat, g.material->opacity);
  }
  return MR_OK;
}

// ------------------------------------------------------------ X3D
// A small XML element tree: elements and attributes (prolog, comments,
// DOCTYPE and CDATA skipped, text ignored, the five predefined entities
// decoded in attribute values).
struct XNode {
  std::string tag;
  std::vector<std::pair<std::string, std::string>> attrs;
  std::vector<std::shared_ptr<XNode>> kids;
  std::string attr(const char* a) const {
    for (auto& kv : attrs)
      if (kv.first == a) return kv.second;
    return std::string();
  }
  bool has(const char* a) const {
    for (auto& kv : attrs)
      if (kv.first == a) return true;
    return false;
  }
  std::shared_ptr<XNode> child(const char* t) const {
    for (auto& k : kids)
      if (k->tag == t) return k;
    return nullptr;
  }
};
using XPtr = std::shared_ptr<XNode>;

struct XmlParser {
  const std::string& s;
  size_t i = 0;
  int depth = 0;
  explicit XmlParser(const std::string& t) : s(t) {}
  bool starts(const char* p) const { return s.compare(i, strlen(p), p) == 0; }
  void ws() { while (i < s.size() && isspace((unsigned char)s[i])) i++; }
  static std::string decode(const std::string& v) {
    std::string r;
    for (size_t k = 0; k < v.size(); k++) {
      if (v[k] == '&') {
        size_t e = v.find(';', k);
        if (e != std::string::npos) {
          std::string ent = v.substr(k + 1, e - k - 1);
          const char* rep = ent == "quot" ? "\"" : ent == "apos" ? "'" : ent == "lt" ? "<" : ent == "gt" ? ">"
                            : ent == "amp" ? "&" : nullptr;
          if (rep) {
            r += rep;
            k = e;
            continue;
          }
        }
      }
      r += v[k];
    }
    return r;
  }
  void misc() {
    for (;;) {
      while (i < s.size() && s[i] != '<') i++;
      if (i >= s.size()) return;
      size_t e;
      if (starts("<!--")) { e = s.find("-->", i); i = e == std::string::npos ? s.size() : e + 3; }
      else if (starts("<![CDATA[")) { e = s.find("]]>", i); i = e == std::string::npos ? s.size() : e + 3; }
      else if (starts("<?")) { e = s.find("?>", i); i = e == std::string::npos ? s.size() : e + 2; }
      else if (starts("<!")) {
        int d = 0;
        for (; i < s.size(); i++) {
          if (s[i] == '[') d++;
          else if (s[i] == ']') d--;
          else if (s[i] == '>' && d <= 0) { i++; break; }
        }
      } else return;
    }
  }
  XPtr element() {
    auto n = std::make_shared<XNode>();
    if (++depth > 4096) {  // bounded nesting
      i = s.size();
      return n;
    }
    i++;
    size_t b = i;
    while (i < s.size() && !isspace((unsigned char)s[i]) && s[i] != '>' && s[i] != '/') i++;
    n->tag = s.substr(b, i - b);
    for (;;) {
      ws();
      if (i >= s.size()) { depth--; return n; }
      if (s[i] == '/') {
        i = s.find('>', i);
        i = i == std::string::npos ? s.size() : i + 1;
        depth--;
        return n;
      }
      if (s[i] == '>') { i++; break; }
      size_t a = i;
      while (i < s.size() && s[i] != '=' && !isspace((unsigned char)s[i]) && s[i] != '>' && s[i] != '/') i++;
      std::string name = s.substr(a, i - a);
      ws();
      std::string val;
      if (i < s.size() && s[i] == '=') {
        i++;
        ws();
        char q = i < s.size() ? s[i] : 0;
        if (q == '"' || q == '\'') {
          size_t e = s.find(q, i + 1);
          if (e == std::string::npos) e = s.size();
          val = decode(s.substr(i + 1, e - i - 1));
          i = e + 1;
        }
      }
      if (!name.empty()) n->attrs.push_back({name, val});
      if (name.empty() && i < s.size() && s[i] != '>' && s[i] != '/') i++;  // stray character
    }
    for (;;) {
      misc();
      if (i >= s.size()) break;
      if (starts("</")) {
        i = s.find('>', i);
        i = i == std::string::npos ? s.size() : i + 1;
        break;
      }
      n->kids.push_back(element());
    }
    depth--;
    return n;
  }
};

XPtr xml_read(const std::string& path) {
  std::string s;
  if (!read_file(path, s)) return nullptr;
  XmlParser p(s);
  p.misc();
  if (p.i >= s.size()) return nullptr;
  return p.element();
}

XPtr xml_find_def(const XPtr& n, const std::string& def) {
  if (n->has("DEF") ? n->attr("DEF") == def : def.empty()) return n;
  for (auto& k : n->kids) {
    XPtr r = xml_find_def(k, def);
    if (r) return r;
  }
  return nullptr;
}

std::string or_default(const std::string& v, const char* d) { return v.empty() ? std::string(d) : v; }

F3 to_f3(const std::string& s) {
  std::vector<float> a = floats_of(s);
  return F3{at(a, 0), at(a, 1), at(a, 2)};
}
std::vector<float> number_list(const std::string& s) {
  std::string t = s;
  std::replace(t.begin(), t.end(), ',', ' ');
  return floats_of(t);
}
std::vector<int32_t> int_list(const std::string& s) {
  std::vector<int32_t> out;
  for (auto& t : split_ws(s)) out.push_back(to_int(t));
  return out;
}

// The reference's X3D reader (src/x3d.cpp:35-200), including its state: an
// Inline element re-targets the document and file name used by later
// lookups, as the reference's reader does.
struct X3dReader {
  mr_model& M;
  std::string filename;
  XPtr doc;
  int inline_depth = 0;
  explicit X3dReader(mr_model& m) : M(m) {}

  XPtr get(const XPtr& item) const {
    if (item && item->has("USE")) {
      const std::string use = item->attr("USE");
      return doc ? xml_find_def(doc, use) : nullptr;
    }
    return item;
  }

  // Adds the node for element e under parent; false when e yields nothing.
  bool item(const XPtr& e, int parent) {
    if (e->tag == "Transform" || e->tag == "Group") {
      std::vector<std::string> rot = split_ws(or_default(e->attr("rotation"), "0 0 1 0"));
      std::vector<std::string> tr = split_ws(or_default(e->attr("translation"), "0 0 0"));
      std::vector<std::string> sc = split_ws(or_default(e->attr("scale"), "1 1 1"));
      M4 xf = mul(mul(translate(fat(tr, 0), fat(tr, 1), fat(tr, 2)),
                      rotate(F3{fat(rot, 0), fat(rot, 1), fat(rot, 2)}, fat(rot, 3))),
                  scale(fat(sc, 0), fat(sc, 1), fat(sc, 2)));
      const int self = M.add_node(parent, -1, xf, false, default_material());
      std::vector<XPtr> kids = e->kids;  // a copy, as the reference iterates
      for (auto& k : kids) item(k, self);
      return true;
    }
    if (e->tag == "Shape") {
      Mesh m;
      mr_material mat = default_material();
      XPtr appx = get(e->child("Appearance"));
      if (XPtr mt = get(appx ? appx->child("Material") : nullptr)) {
        F3 d = to_f3(or_default(mt->attr("diffuseColor"), "0.7 0.75 0.8"));
        F3 s = to_f3(or_default(mt->attr("specularColor"), "0.4 0.4 0.4"));
        F3 em = to_f3(or_default(mt->attr("emissiveColor"), "0 0 0"));
        mat.diffuse[0] = d.x; mat.diffuse[1] = d.y; mat.diffuse[2] = d.z;
        mat.specular[0] = s.x; mat.specular[1] = s.y; mat.specular[2] = s.z;
        mat.emissive[0] = em.x; mat.emissive[1] = em.y; mat.emissive[2] = em.z;
        mat.shininess = to_float(or_default(mt->attr("shininess"), "0.5")) * 8;
      }
      if (XPtr tx = get(appx ? appx->child("ImageTexture") : nullptr)) {
        std::string name = no_ext(tx->attr("url")) + ".ppm";
        mat.texture = M.texture(directory_of(filename) + "/" + name);
      }
      XPtr ifs = get(e->child("IndexedFaceSet"));
      XPtr its = get(e->child("IndexedTriangleSet"));
      if (XPtr g = ifs ? ifs : its) {
        XPtr co = get(g->child("Coordinate")), no = get(g->child("Normal")), tc = get(g->child("TextureCoordinate"));
        std::vector<float> verts = number_list(co ? co->attr("point") : std::string());
        std::vector<float> normals = number_list(no ? no->attr("vector") : std::string());
        std::vector<float> uvs = number_list(tc ? tc->attr("point") : std::string());
        for (size_t i = 0; i < verts.size(); i += 3) m.pos->insert(m.pos->end(), {at(verts, i), at(verts, i + 1), at(verts, i + 2)});
        for (size_t i = 0; i < normals.size(); i += 3)
          m.nrm->insert(m.nrm->end(), {at(normals, i), at(normals, i + 1), at(normals, i + 2)});
        for (size_t i = 0; i < uvs.size(); i += 2) m.uv->insert(m.uv->end(), {at(uvs, i), 1 - at(uvs, i + 1)});
        if (ifs) {
          m.idx = triangulate(int_list(g->attr("coordIndex")));
          std::vector<int32_t> t = int_list(g->attr("texCoordIndex")), nn = int_list(g->attr("normalIndex"));
          m.tidx = t.empty() ? m.idx : triangulate(t);
          m.nidx = nn.empty() ? m.idx : triangulate(nn);
        } else {
          m.idx = int_list(g->attr("index"));
          m.tidx = m.idx;
          m.nidx = m.idx;
        }
        if (m.nrm->empty()) face_normals(m);
        if (m.uv->empty()) {
          m.uv->insert(m.uv->end(), {0.0f, 0.0f});
          m.tidx.assign(m.idx.size(), 0);
        }
      }
      M.meshes.push_back(std::move(m));
      M.add_node(parent, (int)M.meshes.size() - 1, identity(), true, mat);
      return true;
    }
    if (e->tag == "Inline") {
      std::string url = e->attr("url");
      url.erase(std::remove(url.begin(), url.end(), '"'), url.end());
      return load(directory_of(filename) + "/" + url, parent);
    }
    return false;
  }

  // Reads an X3D file: its Scene's elements become children of a new node
  // under parent (or the root when parent < 0).  False if it is not X3D.
  bool load(const std::string& path, int parent) {
    if (++inline_depth > 64) return false;  // bounded Inline recursion
    XPtr d = xml_read(path);
    doc = d;  // replaced before the checks, as the reference's reader does
    if (!d || d->tag != "X3D") return false;
    XPtr scene = d->child("Scene");
    if (!scene) return false;
    filename = path;
    const int self = M.add_node(parent, -1, identity(), false, default_material());
    std::vector<XPtr> kids = scene->kids;
    for (auto& k : kids) item(k, self);
    return true;
  }
};

int load_x3d(const std::string& path, mr_model& M) {
  X3dReader r(M);
  return r.load(path, -1) ? MR_OK : MR_E_IO;
}

}  // namespace

extern "C" {

MR_API int mr_model_load(const char* path, mr_model** out) {
  if (!path || !out) return MR_E_INVALID;
  *out = nullptr;
  std::unique_ptr<mr_model> M(new mr_model());
  const std::string p(path);
  int rc = MR_OK;
  if (has_ext(p, "stl")) {
    Mesh m;
    rc = load_stl(p, m);
    if (rc == MR_OK) {
      M->meshes.push_back(std::move(m));
      const int root = M->add_node(-1, -1, identity(), false, default_material());
      M->add_node(root, 0, identity(), false, default_material());
    }
  } else if (has_ext(p, "obj")) {
    rc = load_obj(p, *M);
  } else if (has_ext(p, "x3d")) {
    rc = load_x3d(p, *M);
  } else {
    M->add_node(-1, -1, identity(), false, default_material());  // an empty node, as the reference returns
  }
  if (rc != MR_OK) return rc;
  *out = M.release();
  return MR_OK;
}

MR_API int mr_model_counts(const mr_model* m, int32_t* n_nodes, int32_t* n_meshes, int32_t* n_textures) {
  if (!m) return MR_E_INVALID;
  if (n_nodes) *n_nodes = (int32_t)m->nodes.size();
  if (n_meshes) *n_meshes = (int32_t)m->meshes.size();
  if (n_textures) *n_textures = (int32_t)m->textures.size();
  return MR_OK;
}

MR_API int mr_model_nodes(const mr_model* m, mr_node* out, int32_t cap) {
  if (!m || (!out && cap > 0) || cap < (int32_t)m->nodes.size()) return MR_E_INVALID;
  if (!m->nodes.empty()) memcpy(out, m->nodes.data(), sizeof(mr_node) * m->nodes.size());
  return MR_OK;
}

MR_API int mr_model_mesh(const mr_model* m, int32_t i, mr_mesh_desc* out) {
  if (!m || !out || i < 0 || i >= (int32_t)m->meshes.size()) return MR_E_INVALID;
  const Mesh& s = m->meshes[i];
  auto p = [](const std::vector<float>& v) { return v.empty() ? nullptr : v.data(); };
  auto q = [](const std::vector<int32_t>& v) { return v.empty() ? nullptr : v.data(); };
  out->vertices = p(*s.pos);
  out->n_vertices = (int32_t)(s.pos->size() / 3);
  out->normals = p(*s.nrm);
  out->n_normals = (int32_t)(s.nrm->size() / 3);
  out->texcoords = p(*s.uv);
  out->n_texcoords = (int32_t)(s.uv->size() / 2);
  out->indices = q(s.idx);
  out->n_indices = (int32_t)s.idx.size();
  out->normalsI = q(s.nidx);
  out->n_normalsI = (int32_t)s.nidx.size();
  out->texcoordsI = q(s.tidx);
  out->n_texcoordsI = (int32_t)s.tidx.size();
  return MR_OK;
}

MR_API int mr_model_texture(const mr_model* m, int32_t i, const uint8_t** rgb8, int32_t* rows, int32_t* cols) {
  if (!m || i < 0 || i >= (int32_t)m->textures.size()) return MR_E_INVALID;
  if (rgb8) *rgb8 = m->textures[i].rgb.data();
  if (rows) *rows = m->textures[i].rows;
  if (cols) *cols = m->textures[i].cols;
  return MR_OK;
}

MR_API void mr_model_free(mr_model* m) { delete m; }

MR_API int mr_ppm_load(const char* path, uint8_t* rgb8, int64_t cap_bytes, int32_t* rows, int32_t* cols) {
  if (!path) return MR_E_INVALID;
  Texture t;
  int rc = ppm_read(path, t);
  if (rc != MR_OK) return rc;
  if (rows) *rows = t.rows;
  if (cols) *cols = t.cols;
  if (rgb8) {
    if (cap_bytes < (int64_t)t.rgb.size()) return MR_E_INVALID;
    memcpy(rgb8, t.rgb.data(), t.rgb.size());
  }
  return MR_OK;
}

// savePPM (src/io.cpp:337-362) of bytes already quantised as it does.
MR_API int mr_ppm_save(const char* path, const uint8_t* rgb8, int32_t rows, int32_t cols) {
  if (!path || !rgb8 || rows <= 0 || cols <= 0) return MR_E_INVALID;
  FILE* f = fopen(path, "wb");
  if (!f) return MR_E_IO;
  fprintf(f, "P6\n%d %d\n255\n", cols, rows);
  size_t n = fwrite(rgb8, 1, (size_t)rows * cols * 3, f);
  fclose(f);
  return n == (size_t)rows * cols * 3 ? MR_OK : MR_E_IO;
}

// saveSTL (src/io.cpp:155-183): binary STL of the mesh's triangles under
// transform (row-major, NULL = identity), facet normal ((c-a)^(b-a)) normalized.
MR_API int mr_stl_save(const char* path, const mr_mesh_desc* d, const float* transform) {
  if (!path || !d || d->n_indices < 0 || d->n_indices % 3 || (d->n_indices && !d->indices) ||
      (d->n_vertices && !d->vertices))
    return MR_E_INVALID;
  for (int32_t i = 0; i < d->n_indices; i++)
    if (d->indices[i] < 0 || d->indices[i] >= d->n_vertices) return MR_E_BAD_INDEX;
  M4 xf = identity();
  if (transform) memcpy(xf.m, transform, sizeof xf.m);
  FILE* f = fopen(path, "wb");
  if (!f) return MR_E_IO;
  std::string buf(80, ' ');
  int32_t nf = d->n_indices / 3;
  buf.append((const char*)&nf, 4);
  for (int32_t i = 0; i < d->n_indices; i += 3) {
    auto v = [&](int k) {
      const float* p = d->vertices + 3 * (size_t)d->indices[i + k];
      return affine(xf.m, F3{p[0], p[1], p[2]});
    };
    F3 a = v(0), b = v(1), c = v(2);
    F3 n = normalized(cross(sub(c, a), sub(b, a)));
    float rec[12] = {n.x, n.y, n.z, a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z};
    buf.append((const char*)rec, sizeof rec);
    buf.append(2, '\0');
  }
  size_t w = fwrite(buf.data(), 1, buf.size(), f);
  fclose(f);
  return w == buf.size() ? MR_OK : MR_E_IO;
}

// saveXYZ (src/io.cpp:417-431): one "x y z" line (printf %f) per point of the
// rows x cols image whose z < -1e-5, in row order, after transform
// (row-major, NULL = identity; m * p, no w divide).
MR_API int mr_xyz_save(const char* path, const float* xyz, int32_t rows, int32_t cols, const float* transform) {
  if (!path || rows < 0 || cols < 0 || ((size_t)rows * cols && !xyz)) return MR_E_INVALID;
  M4 xf = identity();
  if (transform) memcpy(xf.m, transform, sizeof xf.m);
  FILE* f = fopen(path, "w");
  if (!f) return MR_E_IO;
  bool ok = true;
  const size_t n = (size_t)rows * cols;
  for (size_t i = 0; i < n && ok; i++) {
    const float* q = xyz + 3 * i;
    if (q[2] < -1e-5f) {
      const F3 p = affine(xf.m, F3{q[0], q[1], q[2]});
      ok = fprintf(f, "%f %f %f\n", p.x, p.y, p.z) > 0;
    }
  }
  ok = fclose(f) == 0 && ok;
  return ok ? MR_OK : MR_E_IO;
}

}  // extern "C"
