// yh_scene.cpp -- seeded procedural scenes that stand in for Yune's OBJ/MTL input.
//
// The output is what Scene::loadModel produces (src/Scene.cpp:133-383): TriangleGPU
// records with points at w = 1, normals at w = 0 and a material index, plus Material
// records whose colours carry w = 1 (src/Scene.cpp:173-200). Lights are quads, the
// form the reference kernels intersect analytically (kernels/legacy/udpt.cl:97-106).
// Every random draw comes from std::mt19937_64 mapped to [0,1) by the top 53 bits, so
// the same seed gives the same scene on every host.
#include "yune_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <cstdlib>
#include <map>
#include <new>
#include <random>
#include <utility>
#include <vector>

namespace {
struct D3 { double x, y, z; };
}  // namespace

struct yh_scene {
  std::vector<yc_triangle> tris;
  std::vector<yc_material> mats;
  std::vector<yc_quad_light> lights;
  // unit icosphere per subdivision level (vertices, faces), built on first use
  std::map<int, std::pair<std::vector<D3>, std::vector<int>>> ico;
};

namespace {
inline D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 operator*(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 cross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline D3 unit(D3 a) { const double l = std::sqrt(dot(a, a)); return l > 0 ? a * (1.0 / l) : a; }

inline double u01(std::mt19937_64& g) { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }

yc_float4 pt(D3 p) { return yc_float4{(float)p.x, (float)p.y, (float)p.z, 1.0f}; }
yc_float4 vec(D3 v) { return yc_float4{(float)v.x, (float)v.y, (float)v.z, 0.0f}; }

yc_material base_material() {
  yc_material m;
  std::memset(&m, 0, sizeof(m));
  m.ke = yc_float4{0, 0, 0, 1};
  m.kd = yc_float4{0.3f, 0.3f, 0.3f, 1};
  m.ks = yc_float4{0, 0, 0, 1};
  m.n = 1; m.k = 1; m.px = 1; m.py = 1; m.alpha_x = 100; m.alpha_y = 100;   // newMaterial()
  return m;
}

void push_tri(yh_scene* s, D3 a, D3 b, D3 c, D3 na, D3 nb, D3 nc, int mat) {
  yc_triangle t;
  std::memset(&t, 0, sizeof(t));
  t.v1 = pt(a); t.v2 = pt(b); t.v3 = pt(c);
  t.vn1 = vec(na); t.vn2 = vec(nb); t.vn3 = vec(nc);
  t.matID = mat;
  s->tris.push_back(t);
}

// quad a-b-c-d (counter-clockwise seen from the side the normal points to)
void push_quad(yh_scene* s, D3 a, D3 b, D3 c, D3 d, D3 n, int mat) {
  push_tri(s, a, b, c, n, n, n, mat);
  push_tri(s, a, c, d, n, n, n, mat);
}

void push_box(yh_scene* s, D3 center, D3 half, double yaw, int mat) {
  const double cy = std::cos(yaw), sy = std::sin(yaw);
  auto xf = [&](D3 p) {   // rotate about +y then translate
    return D3{cy * p.x + sy * p.z + center.x, p.y + center.y, -sy * p.x + cy * p.z + center.z};
  };
  auto xn = [&](D3 n) { return D3{cy * n.x + sy * n.z, n.y, -sy * n.x + cy * n.z}; };
  const double hx = half.x, hy = half.y, hz = half.z;
  D3 p[8] = {{-hx, -hy, -hz}, {hx, -hy, -hz}, {hx, hy, -hz}, {-hx, hy, -hz},
             {-hx, -hy, hz},  {hx, -hy, hz},  {hx, hy, hz},  {-hx, hy, hz}};
  for (auto& q : p) q = xf(q);
  push_quad(s, p[4], p[5], p[6], p[7], xn({0, 0, 1}), mat);    // +z
  push_quad(s, p[1], p[0], p[3], p[2], xn({0, 0, -1}), mat);   // -z
  push_quad(s, p[5], p[1], p[2], p[6], xn({1, 0, 0}), mat);    // +x
  push_quad(s, p[0], p[4], p[7], p[3], xn({-1, 0, 0}), mat);   // -x
  push_quad(s, p[7], p[6], p[2], p[3], xn({0, 1, 0}), mat);    // +y
  push_quad(s, p[0], p[1], p[5], p[4], xn({0, -1, 0}), mat);   // -y
}

// Unit icosphere: the 12 icosahedron vertices, faces found as the triples at the
// edge length, then `level` midpoint subdivisions projected back to the sphere.
void icosphere(int level, std::vector<D3>& v, std::vector<int>& f) {
  const double phi = (1.0 + std::sqrt(5.0)) / 2.0;
  v.clear(); f.clear();
  for (int s1 = -1; s1 <= 1; s1 += 2)
    for (int s2 = -1; s2 <= 1; s2 += 2) {
      v.push_back(unit({(double)s1, s2 * phi, 0}));
      v.push_back(unit({0, (double)s1, s2 * phi}));
      v.push_back(unit({s2 * phi, 0, (double)s1}));
    }
  double min_d = 1e9;
  for (size_t i = 0; i < v.size(); ++i)
    for (size_t j = i + 1; j < v.size(); ++j) min_d = std::min(min_d, dot(v[i] - v[j], v[i] - v[j]));
  auto adj = [&](int i, int j) { return std::fabs(dot(v[i] - v[j], v[i] - v[j]) - min_d) < 1e-9; };
  for (int i = 0; i < 12; ++i)
    for (int j = i + 1; j < 12; ++j)
      for (int k = j + 1; k < 12; ++k)
        if (adj(i, j) && adj(j, k) && adj(i, k)) {
          D3 n = cross(v[j] - v[i], v[k] - v[i]);
          if (dot(n, v[i] + v[j] + v[k]) > 0) { f.push_back(i); f.push_back(j); f.push_back(k); }
          else { f.push_back(i); f.push_back(k); f.push_back(j); }
        }
  for (int l = 0; l < level; ++l) {
    std::map<std::pair<int, int>, int> mid;
    auto midpoint = [&](int i, int j) {
      std::pair<int, int> key(std::min(i, j), std::max(i, j));
      auto it = mid.find(key);
      if (it != mid.end()) return it->second;
      v.push_back(unit(v[i] + v[j]));
      const int idx = (int)v.size() - 1;
      mid.emplace(key, idx);
      return idx;
    };
    std::vector<int> nf;
    nf.reserve(f.size() * 4);
    for (size_t t = 0; t < f.size(); t += 3) {
      const int i = f[t], j = f[t + 1], k = f[t + 2];
      const int ij = midpoint(i, j), jk = midpoint(j, k), ki = midpoint(k, i);
      const int quad[12] = {i, ij, ki, ij, j, jk, ki, jk, k, ij, jk, ki};
      nf.insert(nf.end(), quad, quad + 12);
    }
    f.swap(nf);
  }
}

}  // namespace

extern "C" int yh_scene_new(yh_scene** out) {
  if (!out) return YH_E_INVALID;
  *out = new (std::nothrow) yh_scene;
  return *out ? YH_OK : YH_E_NOMEM;
}
extern "C" void yh_scene_free(yh_scene* s) { delete s; }

extern "C" int yh_scene_add_material(yh_scene* s, const yc_material* m, int* mat_id) {
  if (!s || !m) return YH_E_INVALID;
  s->mats.push_back(*m);
  if (mat_id) *mat_id = (int)s->mats.size() - 1;
  return YH_OK;
}

extern "C" int yh_scene_add_light(yh_scene* s, const yc_quad_light* l) {
  if (!s || !l) return YH_E_INVALID;
  s->lights.push_back(*l);
  return YH_OK;
}

extern "C" int yh_scene_add_cornell(yh_scene* s, uint64_t seed, float on_sigma2, float phong_exp,
                                    float light_emission, int with_boxes) {
  if (!s) return YH_E_INVALID;
  std::mt19937_64 g(seed);
  const int m0 = (int)s->mats.size();
  yc_material white = base_material();
  white.kd = yc_float4{0.73f, 0.73f, 0.73f, 1};
  white.alpha_x = white.alpha_y = on_sigma2;
  yc_material red = white;
  red.kd = yc_float4{0.63f, 0.065f, 0.05f, 1};
  yc_material green = white;
  green.kd = yc_float4{0.14f, 0.45f, 0.091f, 1};
  yc_material phong = base_material();
  phong.kd = yc_float4{0.35f, 0.35f, 0.35f, 1};
  phong.ks = yc_float4{0.45f, 0.45f, 0.45f, 1};
  phong.px = phong_exp * 0.5f;
  phong.py = phong_exp * 0.5f;
  phong.alpha_x = phong.alpha_y = 0.0f;
  s->mats.push_back(white);
  s->mats.push_back(red);
  s->mats.push_back(green);
  s->mats.push_back(phong);
  const int W = m0, R = m0 + 1, G = m0 + 2, P = m0 + 3;
  const double h = 0.5;
  push_quad(s, {-h, -h, -h}, {-h, -h, h}, {h, -h, h}, {h, -h, -h}, {0, 1, 0}, W);    // floor
  push_quad(s, {-h, h, -h}, {h, h, -h}, {h, h, h}, {-h, h, h}, {0, -1, 0}, W);       // ceiling
  push_quad(s, {-h, -h, -h}, {h, -h, -h}, {h, h, -h}, {-h, h, -h}, {0, 0, 1}, W);    // back
  push_quad(s, {-h, -h, -h}, {-h, h, -h}, {-h, h, h}, {-h, -h, h}, {1, 0, 0}, R);    // left
  push_quad(s, {h, -h, -h}, {h, -h, h}, {h, h, h}, {h, h, -h}, {-1, 0, 0}, G);       // right
  const double yaw0 = (10.0 + 15.0 * u01(g)) * M_PI / 180.0;
  const double yaw1 = -(10.0 + 15.0 * u01(g)) * M_PI / 180.0;
  if (with_boxes) {
    push_box(s, {-0.18, -0.2, -0.15}, {0.14, 0.3, 0.14}, yaw0, P);
    push_box(s, {0.18, -0.36, 0.14}, {0.14, 0.14, 0.14}, yaw1, W);
  }
  yc_quad_light l;
  std::memset(&l, 0, sizeof(l));
  l.pos = yc_float4{-0.125f, 0.499f, -0.125f, 1.0f};
  l.normal = yc_float4{0, -1, 0, 0};
  l.ke = yc_float4{light_emission, light_emission, light_emission, 0};
  l.edge_l = yc_float4{0.25f, 0, 0, 0};
  l.edge_w = yc_float4{0, 0, 0.25f, 0};
  s->lights.push_back(l);
  return YH_OK;
}

extern "C" int yh_scene_add_icosphere(yh_scene* s, const float c[3], float r, int level, float disp,
                                      uint64_t seed, int mat_id) {
  if (!s || !c || level < 0 || level > 9 || !(r > 0)) return YH_E_INVALID;
  try {
    auto it = s->ico.find(level);
    if (it == s->ico.end()) {
      std::pair<std::vector<D3>, std::vector<int>> vf;
      icosphere(level, vf.first, vf.second);
      it = s->ico.emplace(level, std::move(vf)).first;
    }
    const std::vector<D3>& v = it->second.first;
    const std::vector<int>& f = it->second.second;
    std::mt19937_64 g(seed);
    std::vector<D3> p(v.size()), n(v.size(), D3{0, 0, 0});
    const D3 cc{c[0], c[1], c[2]};
    for (size_t i = 0; i < v.size(); ++i) {
      const double k = disp > 0 ? 1.0 + disp * (2.0 * u01(g) - 1.0) : 1.0;
      p[i] = cc + v[i] * (r * k);
    }
    if (disp > 0) {
      for (size_t t = 0; t < f.size(); t += 3) {
        const D3 fn = cross(p[f[t + 1]] - p[f[t]], p[f[t + 2]] - p[f[t]]);   // area weighted
        for (int q = 0; q < 3; ++q) n[f[t + q]] = n[f[t + q]] + fn;
      }
      for (auto& x : n) x = unit(x);
    } else {
      n = v;
    }
    const size_t need = s->tris.size() + f.size() / 3;   // grow geometrically: many spheres append here
    if (need > s->tris.capacity()) s->tris.reserve(std::max(need, 2 * s->tris.capacity()));
    for (size_t t = 0; t < f.size(); t += 3)
      push_tri(s, p[f[t]], p[f[t + 1]], p[f[t + 2]], n[f[t]], n[f[t + 1]], n[f[t + 2]], mat_id);
  } catch (const std::bad_alloc&) {
    return YH_E_NOMEM;
  }
  return YH_OK;
}

extern "C" int yh_scene_counts(const yh_scene* s, int* n_tri, int* n_mat, int* n_light) {
  if (!s) return YH_E_INVALID;
  if (n_tri) *n_tri = (int)s->tris.size();
  if (n_mat) *n_mat = (int)s->mats.size();
  if (n_light) *n_light = (int)s->lights.size();
  return YH_OK;
}

extern "C" int yh_scene_copy(const yh_scene* s, yc_triangle* tris, yc_material* mats, yc_quad_light* lights) {
  if (!s) return YH_E_INVALID;
  if (tris && !s->tris.empty()) std::memcpy(tris, s->tris.data(), s->tris.size() * sizeof(yc_triangle));
  if (mats && !s->mats.empty()) std::memcpy(mats, s->mats.data(), s->mats.size() * sizeof(yc_material));
  if (lights && !s->lights.empty()) std::memcpy(lights, s->lights.data(), s->lights.size() * sizeof(yc_quad_light));
  return YH_OK;
}

// ---- OBJ/MTL ingestion: Scene::loadModel (src/Scene.cpp:133-383) restated ----
//
// Rules kept from the reference, so that the triangle, material and BVH arrays equal its
// own for the same files:
//   * the material file is named by an `mtllib` line that must be the first line of the
//     OBJ that is neither empty nor a comment (Scene::getMatFileName, :385-410), and is
//     read from the OBJ's directory; without one the scene gets the default material
//     (newMaterial, include/CL_headers.h:109-124) as material 0 "default" (the reference
//     also writes that default material file to disk; this loader writes nothing);
//   * material keys ke/kd/ks (w = 1), n, k, alpha_x, alpha_y, is_specular,
//     is_transmissive; `px` sets the py field and `py` the px field (:215-218);
//     numbers that fail to parse keep the previous line's value, as the reference's
//     shared x, y, z do;
//   * OBJ: `v` (w = 1) and `vn` (w = 0) append to lists that `o` does not reset; `o`
//     forgets the current material name; `usemtl` selects a material by name (an unknown
//     name: material 0); a face before any `usemtl` takes material 0; a face reads its
//     first three vertices `v`, `v//vn` or `v/vt/vn` (texture indices are skipped,
//     further vertices ignored);
//   * lines whose first character is '#' and empty lines are skipped.
// Departures: a face without normal indices gets zero normals (the reference leaves them
// undefined); an index outside the lists read so far is an error (the reference reads out
// of bounds).
namespace {

bool read_float(std::istringstream& ss, float& v) {
  std::string tok;
  if (!(ss >> tok)) return false;
  char* end = nullptr;
  const float f = std::strtof(tok.c_str(), &end);
  if (end == tok.c_str()) return false;
  v = f;
  return true;
}

bool read_int(std::istringstream& ss, int& v) {
  std::string tok;
  if (!(ss >> tok)) return false;
  char* end = nullptr;
  const long x = std::strtol(tok.c_str(), &end, 10);
  if (end == tok.c_str()) return false;
  v = (int)x;
  return true;
}

yc_material default_material() {
  yc_material m;
  std::memset(&m, 0, sizeof(m));
  m.ke = yc_float4{0, 0, 0, 1};
  m.kd = yc_float4{0.3f, 0.3f, 0.3f, 1};
  m.ks = yc_float4{0, 0, 0, 1};
  m.n = 1; m.k = 1; m.px = 1; m.py = 1; m.alpha_x = 100; m.alpha_y = 100;
  return m;
}

// first line of the OBJ that is neither empty nor a comment, if it is `mtllib <name>`
std::string mtllib_of(const std::string& obj_path) {
  std::ifstream f(obj_path);
  std::string line;
  while (std::getline(f, line)) {
    if (line.empty() || line[0] == '#') continue;
    std::istringstream ss(line);
    std::string key, name;
    ss >> key;
    if (key != "mtllib") return "";
    ss >> name;
    return name;
  }
  return "";
}

int load_materials(const std::string& path, std::vector<yc_material>& mats, std::map<std::string, int>& index) {
  std::ifstream f(path);
  if (!f.is_open()) return YH_E_INVALID;
  std::string line;
  float x = 0, y = 0, z = 0;
  const size_t first = mats.size();
  while (std::getline(f, line)) {
    if (line.empty() || line[0] == '#') continue;
    std::istringstream ss(line);
    std::string key;
    ss >> key;
    if (key == "newmtl") {
      std::string id;
      ss >> id;
      index[id] = (int)(mats.size() - first);
      mats.push_back(default_material());
      continue;
    }
    if (mats.size() == first) continue;   // keys before the first newmtl
    yc_material& m = mats.back();
    if (key == "ke" || key == "kd" || key == "ks") {
      read_float(ss, x) && read_float(ss, y) && read_float(ss, z);
      yc_float4& c = key == "ke" ? m.ke : (key == "kd" ? m.kd : m.ks);
      c = yc_float4{x, y, z, 1.0f};
    } else if (key == "n") read_float(ss, m.n);
    else if (key == "k") read_float(ss, m.k);
    else if (key == "px") read_float(ss, m.py);   // swapped as in the reference
    else if (key == "py") read_float(ss, m.px);
    else if (key == "alpha_x") read_float(ss, m.alpha_x);
    else if (key == "alpha_y") read_float(ss, m.alpha_y);
    else if (key == "is_specular") read_int(ss, m.is_specular);
    else if (key == "is_transmissive") read_int(ss, m.is_transmissive);
  }
  return mats.size() > first ? YH_OK : YH_E_INVALID;   // "Bad Material file."
}

}  // namespace

extern "C" int yh_scene_load_obj(yh_scene* s, const char* obj_path, int* n_tri_loaded) {
  if (!s || !obj_path) return YH_E_INVALID;
  try {
    const std::string path(obj_path);
    const size_t slash = path.find_last_of('/');
    const std::string dir = slash == std::string::npos ? std::string() : path.substr(0, slash + 1);
    const int mat_base = (int)s->mats.size();
    std::map<std::string, int> index;
    const std::string mtl = mtllib_of(path);
    if (mtl.empty()) {
      index["default"] = 0;
      s->mats.push_back(default_material());
    } else if (int r = load_materials(dir + mtl, s->mats, index)) {
      s->mats.resize(mat_base);
      return r;
    }
    std::ifstream f(path);
    if (!f.is_open()) { s->mats.resize(mat_base); return YH_E_INVALID; }
    std::vector<D3> v, vn;
    std::string line, mat_name;
    int idx = -1;
    const size_t tri_base = s->tris.size();
    while (std::getline(f, line)) {
      if (line.empty() || line[0] == '#') continue;
      std::istringstream ss(line);
      std::string key;
      ss >> key;
      if (key == "o") {
        mat_name.clear();
      } else if (key == "v" || key == "vn") {
        float c[3] = {0, 0, 0};
        for (int k = 0; k < 3 && read_float(ss, c[k]); ++k) {}
        (key == "v" ? v : vn).push_back(D3{c[0], c[1], c[2]});
      } else if (key == "usemtl") {
        ss >> mat_name;
        const auto it = index.find(mat_name);
        idx = it != index.end() ? it->second : 0;
      } else if (key == "f") {
        if (idx < 0) {
          const auto it = index.find(mat_name);
          idx = it != index.end() ? it->second : 0;
        }
        D3 p[3] = {}, n[3] = {};
        for (int i = 0; i < 3; ++i) {
          std::string tok;
          if (!(ss >> tok)) { s->tris.resize(tri_base); s->mats.resize(mat_base); return YH_E_INVALID; }
          std::istringstream ts(tok);
          std::string part;
          for (int j = 0; std::getline(ts, part, '/'); ++j) {
            if (j == 1 || part.empty() || j > 2) continue;
            const long k = std::strtol(part.c_str(), nullptr, 10) - 1;
            const std::vector<D3>& list = j == 0 ? v : vn;
            if (k < 0 || k >= (long)list.size()) { s->tris.resize(tri_base); s->mats.resize(mat_base); return YH_E_RANGE; }
            (j == 0 ? p[i] : n[i]) = list[k];
          }
        }
        yc_triangle t;
        std::memset(&t, 0, sizeof(t));
        t.v1 = yc_float4{(float)p[0].x, (float)p[0].y, (float)p[0].z, 1.0f};
        t.v2 = yc_float4{(float)p[1].x, (float)p[1].y, (float)p[1].z, 1.0f};
        t.v3 = yc_float4{(float)p[2].x, (float)p[2].y, (float)p[2].z, 1.0f};
        t.vn1 = yc_float4{(float)n[0].x, (float)n[0].y, (float)n[0].z, 0.0f};
        t.vn2 = yc_float4{(float)n[1].x, (float)n[1].y, (float)n[1].z, 0.0f};
        t.vn3 = yc_float4{(float)n[2].x, (float)n[2].y, (float)n[2].z, 0.0f};
        t.matID = mat_base + idx;
        s->tris.push_back(t);
      }
    }
    if (n_tri_loaded) *n_tri_loaded = (int)(s->tris.size() - tri_base);
  } catch (const std::bad_alloc&) {
    return YH_E_NOMEM;
  }
  return YH_OK;
}
