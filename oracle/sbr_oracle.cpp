// CPU restatement of SBRSolver's shoot-bounce-reflect path (TEST
// INFRASTRUCTURE: the oracle).  Only the tests, the smoke check and the
// benchmark's CPU-baseline leg use this file; the product never links it.
//
// It follows the reference step by step in FP64 with the same operation
// order (built with -ffp-contract=off), so on the same host it reproduces the
// compiled reference bit for bit; that equality is checked against
// oracle/_ref (the reference's own sources) by tests/golden/make_golden.py.
// Differences from the reference are structural only: trees are traced for
// all launches first, then every receiver is processed on its own (capture,
// image correction, duplicate removal, field) so memory stays O(tree nodes)
// instead of Paths[launches][receivers] (RTSolver.cpp:461-468), and both
// phases run on all host threads.
//
// Reference map (SBRSolver_rev2/...):
//   STL read + vertex merge      StlReader.h:448-508,529-700
//   coplanar ids                 Preprocessor.cpp:116-246
//   triangle frame / bbox        Triangle.cpp:37-70
//   SAH BVH build                BVH/BVH.h:135-274
//   closest hit                  BVH/BVH.h:276-328, BVH/BVHNode.h:64-85,
//                                Triangle.cpp:80-124
//   icosahedron launch dirs      Icosahedron.cpp:3-109
//   ray tree                     RTSolver.cpp:128-257
//   reception sphere + capture   RTSolver.cpp:259-297,805-863
//   BFS path order               Ray.cpp:136-182
//   image correction             RTSolver.cpp:299-433,910-924
//   duplicate removal            RTSolver.cpp:435-459,875-883
//   field                        FieldCompute.cpp:11-25,71-302, VecMatDef.h:51-155
#include "sbr_oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <numeric>
#include <queue>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace orc {

typedef std::complex<double> cd;
// The reference takes pi from Eigen's EIGEN_PI, a long double literal, so the
// expressions that mix it in (Constants.h:6-23, VecMatDef.h:69,152) are
// evaluated in long double and rounded once; kept that way here.
const long double kPiL = 3.141592653589793238462643383279502884197169399375105820974944592307816406L;
const double kPi = kPiL;
const double kC = 2.99792458e8;
const double kU0 = 4 * kPiL * 1e-7;
const double kE0 = 1.0 / (kU0 * kC * kC);
const double kEta0 = kU0 * kC;
const double kTwoPi = 2 * kPiL;
const double kEps = std::numeric_limits<float>::epsilon();
const double kInf = std::numeric_limits<double>::infinity();

// ---------------------------------------------------------------- vectors
struct V3 {
  double x = 0, y = 0, z = 0;
  V3() {}
  V3(double a, double b, double c) : x(a), y(b), z(c) {}
  double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(const V3& a, const V3& b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(const V3& a, const V3& b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator-(const V3& a) { return V3(-a.x, -a.y, -a.z); }
inline V3 operator*(const V3& a, double s) { return V3(a.x * s, a.y * s, a.z * s); }
inline V3 operator*(double s, const V3& a) { return V3(s * a.x, s * a.y, s * a.z); }
inline bool operator==(const V3& a, const V3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline double dot(const V3& a, const V3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline double sqnorm(const V3& a) { return (a.x * a.x + a.y * a.y) + a.z * a.z; }
inline double norm(const V3& a) { return std::sqrt(sqnorm(a)); }
inline V3 normalized(const V3& a) {
  double z = sqnorm(a);
  if (z > 0) {
    double s = std::sqrt(z);
    return V3(a.x / s, a.y / s, a.z / s);
  }
  return a;
}
inline V3 cross(const V3& a, const V3& b) {
  return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
struct M3 {  // row-major
  double m[9];
  double& operator()(int i, int j) { return m[3 * i + j]; }
  double operator()(int i, int j) const { return m[3 * i + j]; }
  static M3 I() {
    M3 r;
    for (int i = 0; i < 9; ++i) r.m[i] = (i % 4 == 0) ? 1.0 : 0.0;
    return r;
  }
  V3 row(int i) const { return V3(m[3 * i], m[3 * i + 1], m[3 * i + 2]); }
};
inline M3 mul(const M3& a, const M3& b) {
  M3 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      r(i, j) = (a(i, 0) * b(0, j) + a(i, 1) * b(1, j)) + a(i, 2) * b(2, j);
  return r;
}
inline M3 transpose(const M3& a) {
  M3 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r(i, j) = a(j, i);
  return r;
}
inline V3 mul(const M3& a, const V3& v) {
  return V3((a(0, 0) * v.x + a(0, 1) * v.y) + a(0, 2) * v.z,
            (a(1, 0) * v.x + a(1, 1) * v.y) + a(1, 2) * v.z,
            (a(2, 0) * v.x + a(2, 1) * v.y) + a(2, 2) * v.z);
}
struct C3 {
  cd v[3];
};
inline C3 mul(const M3& a, const C3& c) {
  C3 r;
  for (int i = 0; i < 3; ++i) {
    cd acc = a(i, 0) * c.v[0];
    acc = acc + a(i, 1) * c.v[1];
    acc = acc + a(i, 2) * c.v[2];
    r.v[i] = acc;
  }
  return r;
}

// VecMatDef.h:56-77
double angle_between(V3 v1, V3 v2) {
  v1 = normalized(v1);
  v2 = normalized(v2);
  double ratio = dot(v1, v2);
  if (ratio < 0) return static_cast<double>(kPiL - 2.0 * std::asin(norm(-v1 - v2) / 2.0));
  return static_cast<double>(2.0 * std::asin(norm(v1 - v2) / 2.0));
}
// VecMatDef.h:85-99 (sph2cart form; transposed for cart2sph)
M3 transformation(double theta, double phi) {
  double st = std::sin(theta), sp = std::sin(phi), ct = std::cos(theta), cp = std::cos(phi);
  M3 t;
  t(0, 0) = st * cp; t(0, 1) = ct * cp; t(0, 2) = -1 * sp;
  t(1, 0) = st * sp; t(1, 1) = ct * sp; t(1, 2) = cp;
  t(2, 0) = ct;      t(2, 1) = -1 * st; t(2, 2) = 0.0;
  return t;
}
// VecMatDef.h:132-155
V3 cart_to_sph(const V3& v) {
  V3 r;
  r.x = norm(v);
  if (v.x == 0.0 && v.y == 0.0 && v.z == 0.0) r.y = kPiL / 2;
  else r.y = std::atan2(std::sqrt(v.x * v.x + v.y * v.y), v.z);
  r.z = std::atan2(v.y, v.x);
  if (r.z < 0) r.z += 2 * kPiL;
  return r;
}

// ---------------------------------------------------------------- scene
struct Tri {
  V3 v1, v2, v3, n;
  M3 cs;
  double bb[6];  // min xyz, max xyz
  V3 center;
  int id = -1, cop = -1, mat = 0;
};

struct Scene {
  std::vector<Tri> tris;        // by triangle id (file order)
  std::vector<int> mesh_order;  // caller's vector after BVH build: position -> id
  struct Node {
    double bb[6];
    int c0 = -1, c1 = -1;
    std::vector<int> objs;  // triangle ids
  };
  std::vector<Node> nodes;
};

// Triangle.cpp:37-70
void finish_tri(Tri& t) {
  V3 zw = t.n;
  V3 yw = normalized(t.v2 - t.v1);
  V3 xw = cross(yw, zw);
  for (int j = 0; j < 3; ++j) {
    t.cs(0, j) = xw[j];
    t.cs(1, j) = yw[j];
    t.cs(2, j) = zw[j];
  }
  for (int a = 0; a < 3; ++a) {
    t.bb[a] = std::min({t.v1[a], t.v2[a], t.v3[a]});
    t.bb[3 + a] = std::max({t.v1[a], t.v2[a], t.v3[a]});
    t.center[a] = (t.bb[a] + t.bb[3 + a]) / 2.0;
  }
}

// Coplanar components (Preprocessor.cpp:116-246): triangles are adjacent when
// they share an edge of merged vertices and their file normals are exactly
// equal or exactly opposite; ids number the components by lowest member.
void coplanar_ids(std::vector<Tri>& tris, const std::vector<int>& vidx) {
  const int n = int(tris.size());
  std::vector<int> parent(n);
  std::iota(parent.begin(), parent.end(), 0);
  auto find = [&](int a) {
    while (parent[a] != a) a = parent[a] = parent[parent[a]];
    return a;
  };
  std::map<std::pair<int, int>, std::vector<int>> edges;
  for (int t = 0; t < n; ++t) {
    int a = vidx[3 * t], b = vidx[3 * t + 1], c = vidx[3 * t + 2];
    std::pair<int, int> es[3] = {a < b ? std::make_pair(a, b) : std::make_pair(b, a),
                                 b < c ? std::make_pair(b, c) : std::make_pair(c, b),
                                 a < c ? std::make_pair(a, c) : std::make_pair(c, a)};
    for (auto& e : es) {
      auto& lst = edges[e];
      for (int o : lst)
        if (tris[o].n == tris[t].n || tris[o].n == -tris[t].n) parent[find(o)] = find(t);
      lst.push_back(t);
    }
  }
  std::vector<int> comp(n, -1);
  int next = 0;
  for (int t = 0; t < n; ++t) {
    int r = find(t);
    if (comp[r] < 0) comp[r] = next++;
    tris[t].cop = comp[r];
  }
}

// Exact vertex merge (StlReader.h:448-508): equal float triples share an id;
// triangles whose corners collapse are dropped while their normals stay in
// place, as in the reference reader.  Then frames, boxes, coplanar ids.
bool tris_from_soup(const std::vector<float>& coords, const std::vector<float>& normals,
                    std::vector<Tri>& tris) {
  const size_t nvtx = coords.size() / 3;
  std::vector<size_t> order(nvtx);
  std::iota(order.begin(), order.end(), 0);
  auto key = [&](size_t i) { return std::make_tuple(coords[3 * i], coords[3 * i + 1], coords[3 * i + 2]); };
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return key(a) < key(b); });
  std::vector<int> uid(nvtx);
  int cur = -1;
  for (size_t k = 0; k < nvtx; ++k) {
    if (k == 0 || key(order[k]) != key(order[k - 1])) ++cur;
    uid[order[k]] = cur;
  }
  std::vector<int> vidx;
  std::vector<size_t> src;  // first vertex slot of each kept triangle
  for (size_t t = 0; t < nvtx / 3; ++t) {
    int a = uid[3 * t], b = uid[3 * t + 1], c = uid[3 * t + 2];
    if (a != b && a != c && b != c) {
      vidx.push_back(a);
      vidx.push_back(b);
      vidx.push_back(c);
      src.push_back(3 * t);
    }
  }
  tris.clear();
  for (size_t t = 0; t < src.size(); ++t) {
    Tri tr;
    const float* p = &coords[3 * src[t]];
    tr.v1 = V3(p[0], p[1], p[2]);
    tr.v2 = V3(p[3], p[4], p[5]);
    tr.v3 = V3(p[6], p[7], p[8]);
    tr.n = V3(normals[3 * t], normals[3 * t + 1], normals[3 * t + 2]);
    tr.id = int(t);
    finish_tri(tr);
    tris.push_back(tr);
  }
  coplanar_ids(tris, vidx);
  return true;
}

bool read_stl(const std::string& path, std::vector<Tri>& tris) {
  std::ifstream in(path, std::ios::binary);
  if (!in) return false;
  std::string head(256, '\0');
  in.read(&head[0], 256);
  head.resize(size_t(in.gcount()));
  std::string low = head;
  for (auto& ch : low) ch = char(std::tolower((unsigned char)ch));
  const bool ascii = low.find("solid") != std::string::npos && low.find('\n') != std::string::npos &&
                     low.find("facet") != std::string::npos && low.find("normal") != std::string::npos;
  std::vector<float> coords, normals;  // 3 per vertex / per facet
  in.clear();
  in.seekg(0);
  if (ascii) {
    std::string line, tok;
    int nv = 0;
    while (std::getline(in, line)) {
      std::istringstream ls(line);
      std::vector<std::string> toks;
      while (ls >> tok) toks.push_back(tok);
      if (toks.empty()) continue;
      if (toks[0] == "vertex" && toks.size() >= 4) {
        for (int i = 0; i < 3; ++i) coords.push_back(float(std::atof(toks[1 + i].c_str())));
        ++nv;
      } else if (toks[0] == "facet" && toks.size() >= 5) {
        for (int i = 0; i < 3; ++i) normals.push_back(float(std::atof(toks[2 + i].c_str())));
        nv = 0;
      }
    }
  } else {
    char hdr[80];
    in.read(hdr, 80);
    uint32_t n = 0;
    in.read(reinterpret_cast<char*>(&n), 4);
    for (uint32_t t = 0; t < n; ++t) {
      float d[12];
      in.read(reinterpret_cast<char*>(d), 48);
      char attr[2];
      in.read(attr, 2);
      if (!in) return false;
      for (int i = 0; i < 3; ++i) normals.push_back(d[i]);
      for (int i = 3; i < 12; ++i) coords.push_back(d[i]);
    }
  }
  return tris_from_soup(coords, normals, tris);
}

// BVH/BVH.h:251-267
double surface_area(const double* b) {
  if (b[3] <= b[0] || b[4] <= b[1] || b[5] <= b[2]) return 0.0;
  const double dx = b[3] - b[0], dy = b[4] - b[1], dz = b[5] - b[2];
  return 2.0 * (dx * dy + dy * dz + dz * dx);
}
void empty_box(double* b) {
  for (int a = 0; a < 3; ++a) {
    b[a] = std::numeric_limits<float>::max();
    b[3 + a] = -std::numeric_limits<float>::max();
  }
}
void merge_box(const double* b1, const double* b2, double* r) {
  for (int a = 0; a < 3; ++a) {
    r[a] = std::min(b1[a], b2[a]);
    r[3 + a] = std::max(b1[3 + a], b2[3 + a]);
  }
}

// BVH/BVH.h:135-230 (including its in-place sorts of the object vector)
void build_node(Scene& s, std::vector<const Tri*>& objs, int idx) {
  empty_box(s.nodes[idx].bb);
  for (const Tri* o : objs) merge_box(o->bb, s.nodes[idx].bb, s.nodes[idx].bb);
  double best_cost = 1.0 * objs.size();
  int best_axis = -1, best_split = -1;
  const double sa_root = surface_area(s.nodes[idx].bb);
  const int n = int(objs.size());
  for (int axis = 0; axis < 3; ++axis) {
    std::sort(objs.begin(), objs.end(),
              [axis](const Tri* a, const Tri* b) { return a->center[axis] < b->center[axis]; });
    double b1[6];
    empty_box(b1);
    std::vector<double> sa1(n + 1, std::numeric_limits<double>::max());
    sa1[0] = surface_area(b1);
    for (int i = 0; i < n; ++i) {
      merge_box(b1, objs[i]->bb, b1);
      sa1[i] = surface_area(b1);
    }
    double b2[6];
    empty_box(b2);
    std::vector<double> sa2(n + 1, std::numeric_limits<double>::max());
    sa2[n] = surface_area(b2);
    for (int i = n - 1; i >= 0; --i) {
      merge_box(b2, objs[i]->bb, b2);
      sa2[i] = surface_area(b2);
    }
    for (int i = 1; i < n - 1; ++i) {
      const int j = n - i;
      const double cost = 2 * 1.0 + (i * sa1[i] + j * sa2[i]) * 1.0 / sa_root;
      if (cost < best_cost) {
        best_cost = cost;
        best_axis = axis;
        best_split = i;
      }
    }
  }
  if (best_axis == -1) {
    s.nodes[idx].c0 = s.nodes[idx].c1 = -1;
    for (const Tri* o : objs) s.nodes[idx].objs.push_back(o->id);
    return;
  }
  std::sort(objs.begin(), objs.end(), [best_axis](const Tri* a, const Tri* b) {
    return a->center[best_axis] < b->center[best_axis];
  });
  s.nodes[idx].c0 = int(s.nodes.size());
  s.nodes.emplace_back();
  s.nodes[idx].c1 = int(s.nodes.size());
  s.nodes.emplace_back();
  std::vector<const Tri*> left(objs.begin(), objs.begin() + best_split);
  std::vector<const Tri*> right(objs.begin() + best_split, objs.end());
  int c0 = s.nodes[idx].c0, c1 = s.nodes[idx].c1;
  build_node(s, left, c0);
  build_node(s, right, c1);
}

void build_bvh(Scene& s) {
  std::vector<const Tri*> objs;
  for (const Tri& t : s.tris) objs.push_back(&t);
  s.nodes.assign(1, Scene::Node());
  build_node(s, objs, 0);  // sorts objs in place like the caller's vector
  s.mesh_order.clear();
  for (const Tri* t : objs) s.mesh_order.push_back(t->id);
}

// ---------------------------------------------------------------- tracing
struct Hit {
  V3 n, p;
  int mat = -1, tri = -1, cop = -1;
  double dist = kInf;
};

// Triangle.cpp:80-124
bool tri_intersect(const Tri& t, const V3& o, const V3& d, Hit& info) {
  V3 e1 = t.v2 - t.v1, e2 = t.v3 - t.v1;
  V3 h = cross(d, e2);
  double a = dot(e1, h);
  if (a > -kEps && a < kEps) return false;
  double f = 1.0 / a;
  V3 s = o - t.v1;
  double u = f * dot(s, h);
  if (u < 0.0 || u > 1.0) return false;
  V3 q = cross(s, e1);
  double v = f * dot(d, q);
  if (v < 0.0 || u + v > 1.0) return false;
  double tt = f * dot(e2, q);
  if (tt > kEps) {
    info.p = o + d * tt;
    info.dist = norm(info.p - o);
    info.n = t.n;
    info.mat = t.mat;
    info.tri = t.id;
    info.cop = t.cop;
    return true;
  }
  return false;
}

// BVH/BVHNode.h:64-85 (std::min/std::max argument order kept: NaN slabs drop out)
bool box_hit(const double* bb, const V3& o, const V3& d) {
  double tmax = kInf, tmin = -kInf;
  for (int i = 0; i < 3; ++i) {
    double t1 = (bb[i] - o[i]) / d[i];
    double t2 = (bb[3 + i] - o[i]) / d[i];
    double tn = std::min(t1, t2), tf = std::max(t1, t2);
    tmax = std::min(tmax, tf);
    tmin = std::max(tmin, tn);
    if (tmin > tmax) return false;
  }
  return true;
}

// BVH/BVH.h:276-328
bool bvh_hit(const Scene& s, int idx, const V3& o, const V3& d, Hit& info) {
  const Scene::Node& nd = s.nodes[idx];
  if (!box_hit(nd.bb, o, d)) return false;
  if (nd.c0 != -1) {
    bool any = false;
    if (bvh_hit(s, nd.c0, o, d, info)) any = true;
    if (bvh_hit(s, nd.c1, o, d, info)) any = true;
    return any;
  }
  bool any = false;
  for (int id : nd.objs) {
    Hit cur;
    if (tri_intersect(s.tris[id], o, d, cur) && cur.dist < info.dist) {
      any = true;
      info = cur;
    }
  }
  return any;
}

// Icosahedron.cpp:3-109
std::vector<V3> icosphere(int level) {
  const double X = .525731112119133606, Z = .850650808352039932, N = 0.0;
  std::vector<V3> v = {{-X, N, Z}, {X, N, Z},  {-X, N, -Z}, {X, N, -Z}, {N, Z, X},  {N, Z, -X},
                       {N, -Z, X}, {N, -Z, -X}, {Z, X, N},  {-Z, X, N}, {Z, -X, N}, {-Z, -X, N}};
  std::vector<std::array<int, 3>> f = {
      {0, 4, 1},  {0, 9, 4},  {9, 5, 4},  {4, 5, 8},  {4, 8, 1},  {8, 10, 1}, {8, 3, 10},
      {5, 3, 8},  {5, 2, 3},  {2, 7, 3},  {7, 10, 3}, {7, 6, 10}, {7, 11, 6}, {11, 0, 6},
      {0, 1, 6},  {6, 1, 10}, {9, 0, 11}, {9, 11, 2}, {9, 2, 5},  {7, 2, 11}};
  for (int l = 0; l < level; ++l) {
    std::map<std::pair<int, int>, int> lookup;
    std::vector<std::array<int, 3>> nf;
    nf.reserve(f.size() * 4);
    auto mid = [&](int a, int b) {
      std::pair<int, int> k(std::min(a, b), std::max(a, b));
      auto ins = lookup.insert({k, int(v.size())});
      if (ins.second) v.push_back(normalized(v[a] + v[b]));
      return ins.first->second;
    };
    for (auto& t : f) {
      int m0 = mid(t[0], t[1]), m1 = mid(t[1], t[2]), m2 = mid(t[2], t[0]);
      nf.push_back({t[0], m0, m2});
      nf.push_back({t[1], m1, m0});
      nf.push_back({t[2], m2, m1});
      nf.push_back({m0, m1, m2});
    }
    f.swap(nf);
  }
  for (auto& d : v) d = normalized(d);
  return v;
}

// One node of a launch's ray tree (PathTreeNode, Ray.h:38-43).  Children by
// index; kind: 0 root, 1 reflected, 2 transmitted.
struct TNode {
  V3 src, tgt;
  double path_len;  // Ray::pathLength as stored by RayLaunch
  int tri, cop, mat, kind;
  int child_t = -1, child_r = -1;
};

struct Tracer {
  const Scene& s;
  int max_r, max_t;
  std::vector<TNode>* out;
  // RTSolver.cpp:128-257
  void launch(int node, V3 src, V3 dir, int trans_mat, int ref_mat, int rc, int tc, double total,
              bool is_root) {
    if (rc > max_r && tc > max_t) return;
    Hit hit;
    bool has = bvh_hit(s, 0, src, dir, hit);
    std::vector<TNode>& t = *out;
    if (has) {
      int nn = node;
      if (!is_root) {
        TNode x;
        x.src = src;
        x.tgt = hit.p;
        x.tri = hit.tri;
        x.cop = hit.cop;
        x.path_len = total + hit.dist;
        x.kind = ref_mat >= 0 ? 1 : 2;
        x.mat = ref_mat >= 0 ? ref_mat : trans_mat;
        t.push_back(x);
        nn = int(t.size()) - 1;
        if (ref_mat >= 0) t[node].child_r = nn;
        else t[node].child_t = nn;
      } else {
        t[node].src = src;
        t[node].tgt = hit.p;
        t[node].tri = hit.tri;
        t[node].cop = hit.cop;
        t[node].path_len = hit.dist;
        t[node].kind = 0;
        t[node].mat = -1;
      }
      if (rc < max_r) {
        V3 nd = normalized(dir - 2.0 * hit.n * dot(hit.n, dir));
        launch(nn, hit.p, nd, -1, hit.mat, rc + 1, tc, total + hit.dist, false);
      }
      if (tc < max_t) launch(nn, hit.p, dir, hit.mat, -1, rc, tc + 1, total + hit.dist, false);
    } else {
      if (rc > 0 || tc > 0) {
        TNode x;
        x.src = src;
        x.tgt = src + (dir * 1E2);
        x.tri = -1;
        x.cop = -1;
        x.path_len = kInf;
        x.kind = ref_mat >= 0 ? 1 : 2;
        x.mat = ref_mat >= 0 ? ref_mat : trans_mat;
        t.push_back(x);
        if (ref_mat >= 0) t[node].child_r = int(t.size()) - 1;
        else if (trans_mat >= 0) t[node].child_t = int(t.size()) - 1;
      }
      if (is_root) {
        t[node].src = src;
        t[node].tgt = src + (dir * 1E10);
        t[node].tri = -1;
        t[node].cop = -1;
        t[node].path_len = kInf;
        t[node].kind = 0;
        t[node].mat = -1;
      }
    }
  }
};

// RTSolver.cpp:805-863 with beta and tan(beta) precomputed per request.
bool reception(const V3& s, const V3& t, const V3& c, double path_len, double tan_beta) {
  V3 d = t - s;
  double t0 = dot(d, c - s) / sqnorm(d);
  if (t0 < 0) return false;
  if (t0 >= 1) t0 = 1;
  double unfolded = path_len + norm(s + t0 * d);
  double radius = unfolded * tan_beta;
  double dist = norm(c - (s + t0 * d));
  return dist <= radius;
}

// ---------------------------------------------------------------- field
struct PathRay {
  V3 src, tgt;
  int tri, cop, kind, mat;
};

cd ctrans_angle(double ti, cd ei, cd et) {  // FieldCompute.cpp:294-302
  cd theta_i(ti, 0);
  cd ni = std::sqrt(ei), nt = std::sqrt(et);
  return std::asin((ni / nt) * std::sin(theta_i));
}
// FieldCompute.cpp:237-292: returns (ref, tran) for TE (te=true) or TM.
void fresnel(bool te, cd ti, cd tt, cd ei, cd et, double lam, double width, bool inf_wall, cd& rc,
             cd& tc) {
  const cd J(0.0, 1.0);
  cd ni = std::sqrt(ei), nt = std::sqrt(et);
  cd etai = kEta0 / ni, etat = kEta0 / nt;
  cd ci = std::cos(ti), ct = std::cos(tt), si = std::sin(ti);
  cd g = te ? -((etat / ct) - (etai / ci)) / ((etat / ct) + (etai / ci))
            : (-etat * ct + etai * ci) / (etat * ct + etai * ci);
  if (inf_wall) {
    rc = g;
    tc = 0;
  } else {
    cd q = (kTwoPi * width / lam) * std::sqrt(nt - (si * si));
    cd ph = std::exp(-J * 2.0 * q);
    cd den = 1.0 - (g * g * ph);
    rc = (g * (1.0 - ph)) / den;
    tc = ((1.0 - g * g) * ph) / den;
  }
}
C3 interact(bool reflect, const C3& e, double rel_perm, double sigma, double freq, double ti,
            double width, bool inf_wall) {  // FieldCompute.cpp:185-235
  cd et;
  et.real(rel_perm);
  et.imag(-1 * sigma / (kE0 * 2 * kPi * freq));
  double lam = kC / freq;
  cd ei(1, 0);
  cd tt = ctrans_angle(ti, ei, et);
  cd rte, rtm, tte, ttm;
  fresnel(false, ti, tt, ei, et, lam, width, inf_wall, rtm, ttm);
  fresnel(true, ti, tt, ei, et, lam, width, inf_wall, rte, tte);
  C3 r;
  r.v[0] = e.v[0];
  r.v[1] = e.v[1] * (reflect ? rtm : ttm);
  r.v[2] = e.v[2] * (reflect ? rte : tte);
  return r;
}
C3 pattern(int type, double theta, double pt) {  // FieldCompute.cpp:153-183
  C3 e;
  if (type == 0) e.v[0] = cd(0, std::sqrt(60 * pt));
  if (type == 1) e.v[1] = cd(0, std::sqrt(60 * pt * 1.5) * std::sin(theta));
  else if (type == 2)
    e.v[1] = cd(0, std::sqrt(60 * pt) * (std::cos(kPi * std::cos(theta) / 2.0) / std::sin(theta)));
  // (PI in that expression is the double constant, Constants.h:21)
  return e;
}

// Antenna type 3: a tabulated pattern on a regular (theta, phi) grid in
// degrees, the TXPattern.dat layout (Preprocessor.cpp:3-35,
// common/DataStructures.h:32-37).  The reference reads such a table but never
// applies it; this project defines its use: each grid point's complex
// amplitude 10^(g/20) e^(j arg) is interpolated bilinearly (theta clamped to
// the grid, phi periodic) and E_theta, E_phi = sqrt(60 Pt) * amplitude, the
// scaling of the analytic patterns (sqrt(60 Pt G)).  E_r = 0.
struct Pattern {
  const float* gp = nullptr;  // nt * np * 4: g_theta, arg_theta, g_phi, arg_phi
  int nt = 0, np = 0;
  double dt = 1, dp = 1;

  cd amplitude(int i, int j, int c) const {
    const float* g = gp + 4 * (size_t(i) * np + j) + 2 * c;
    const double mag = std::pow(10.0, double(g[0]) / 20.0);
    const double arg = double(g[1]) * (3.14159265358979323846 / 180.0);
    return cd(mag * std::cos(arg), mag * std::sin(arg));
  }
  C3 field(double theta, double phi, double pt) const {
    const double deg = 180.0 / kPi;
    double u = std::min(std::max(theta * deg / dt, 0.0), double(nt - 1));
    int i0 = nt > 1 ? std::min(int(std::floor(u)), nt - 2) : 0;
    const int i1 = nt > 1 ? i0 + 1 : 0;
    const double wu = nt > 1 ? u - i0 : 0.0;
    double v = phi * deg / dp;
    v -= std::floor(v / np) * np;  // into [0, np)
    int j0 = std::min(int(std::floor(v)), np - 1);
    const int j1 = (j0 + 1) % np;
    const double wv = v - j0;
    const double s = std::sqrt(60 * pt);
    C3 e;
    for (int c = 0; c < 2; ++c) {
      const cd a = (1 - wu) * ((1 - wv) * amplitude(i0, j0, c) + wv * amplitude(i0, j1, c)) +
                   wu * ((1 - wv) * amplitude(i1, j0, c) + wv * amplitude(i1, j1, c));
      e.v[1 + c] = s * a;
    }
    return e;
  }
};

struct FieldCtx {
  const Scene* s;
  const std::vector<MaterialProperties_c>* mats;
  M3 txcs;
  double freq, pt;
  bool fresnel;
  int antenna;
  Pattern pat;
};

// FieldCompute.cpp:71-151; triangle frames are looked up by position in the
// caller's mesh vector (mesh_order), as the reference does.
C3 field_for_path(const FieldCtx& c, const std::vector<PathRay>& path) {
  const cd J(0.0, 1.0);
  double lam = kC / c.freq;
  double k = (2 * kPi) / lam;
  M3 glob = M3::I(), cur = glob, next = c.txcs;
  C3 inc, tot;
  double L = 0.0;
  for (int i = 0; i < int(path.size()); ++i) {
    const PathRay& r = path[i];
    V3 vg = r.tgt - r.src;
    V3 vl = mul(mul(next, transpose(glob)), vg);
    V3 sph = cart_to_sph(vl);
    double rr = sph.x, th = sph.y, ph = sph.z;
    L += rr;
    cur = next;
    if (r.tri == -1) next = glob;
    else next = c.s->tris[c.s->mesh_order[r.tri]].cs;
    if (i == 0) {
      inc = c.antenna == 3 ? c.pat.field(th, ph, c.pt) : pattern(c.antenna, th, c.pt);
    } else {
      inc = mul(mul(glob, transpose(cur)), tot);
      inc = mul(transpose(transformation(th, ph)), inc);
    }
    if (r.kind != 0) {
      double ang = angle_between(vg, cur.row(2));
      const MaterialProperties_c& m = (*c.mats)[r.mat];
      tot = interact(r.kind == 1, inc, m.relPermittivityRe, m.relConductivity, c.freq, ang,
                     m.width, c.fresnel);
    } else {
      tot = inc;
    }
    tot = mul(transformation(th, ph), tot);
    tot = mul(mul(glob, transpose(cur)), tot);
  }
  cd sc = std::exp(-J * k * L);
  for (int i = 0; i < 3; ++i) tot.v[i] = tot.v[i] * sc / L;
  return tot;
}

// ---------------------------------------------------------------- solve
V3 image_point(const Tri& t, const V3& src) {  // RTSolver.cpp:910-924
  double d = dot(t.n, src - t.v1);
  return src - (2 * d * t.n);
}

struct Solver {
  const Scene& s;
  const oracle_request& rq;
  std::vector<MaterialProperties_c> mats;
  std::vector<std::vector<TNode>> trees;
  std::vector<V3> rx;
  double tan_beta = 0;
  unsigned threads = 1;

  Solver(const Scene& sc, const oracle_request& r) : s(sc), rq(r) {}

  void trace() {
    std::vector<V3> dirs = icosphere(rq.tessellation);
    trees.assign(dirs.size(), {});
    std::atomic<size_t> next(0);
    auto work = [&]() {
      Tracer tr{s, rq.max_reflection, rq.max_transmission, nullptr};
      for (size_t i; (i = next.fetch_add(1)) < dirs.size();) {
        trees[i].emplace_back();
        tr.out = &trees[i];
        trees[i][0].child_t = trees[i][0].child_r = -1;
        tr.launch(0, V3(rq.tx[0], rq.tx[1], rq.tx[2]), dirs[i], -1, -1, 0, 0, 0, true);
      }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < threads; ++t) pool.emplace_back(work);
    for (auto& th : pool) th.join();
  }

  // RayCapture (RTSolver.cpp:259-297) then the BFS flatten of Paths
  // (Ray.cpp:136-182): captured node ids of one launch for one receiver,
  // in BFS order (transmit child before reflect child).
  void capture(const std::vector<TNode>& t, const V3& c, std::vector<int>& out,
               std::vector<int>& parent) const {
    out.clear();
    struct Item { int node; double len; };
    std::vector<Item> stack;
    std::vector<char> cap(t.size(), 0);
    parent.assign(t.size(), -1);
    stack.push_back({0, 0.0});
    while (!stack.empty()) {
      Item it = stack.back();
      stack.pop_back();
      const TNode& n = t[it.node];
      if (reception(n.src, n.tgt, c, it.len, tan_beta)) {
        cap[it.node] = 1;
        continue;  // descendants deleted
      }
      double nl = it.len + n.path_len;
      if (n.child_r >= 0) { parent[n.child_r] = it.node; stack.push_back({n.child_r, nl}); }
      if (n.child_t >= 0) { parent[n.child_t] = it.node; stack.push_back({n.child_t, nl}); }
    }
    std::queue<int> q;
    q.push(0);
    while (!q.empty()) {
      int u = q.front();
      q.pop();
      if (cap[u]) { out.push_back(u); continue; }
      if (t[u].child_t >= 0) q.push(t[u].child_t);
      if (t[u].child_r >= 0) q.push(t[u].child_r);
    }
  }

  struct RxOut {
    C3 field;
    std::vector<oracle_path> paths;
    std::vector<int> tri, cop, kind;
    std::vector<double> pts;
    long captured = 0, corrected = 0;
  };

  // ImagePathCorrection + RemoveDuplicatePath + FieldAtReceiver for one receiver.
  void receiver(int k, RxOut& o) const {
    const V3 c = rx[k];
    const V3 tx(rq.tx[0], rq.tx[1], rq.tx[2]);
    FieldCtx fc{&s, &mats, M3(), rq.frequency, rq.pt, rq.use_fresnel != 0, rq.antenna, Pattern()};
    if (rq.antenna == 3) {
      fc.pat.gp = rq.pattern;
      fc.pat.nt = rq.pat_nt;
      fc.pat.np = rq.pat_np;
      fc.pat.dt = rq.pat_dt;
      fc.pat.dp = rq.pat_dp;
    }
    for (int i = 0; i < 9; ++i) fc.txcs.m[i] = rq.tx_coord_sys[i];
    std::map<std::vector<int>, int> seen;
    std::vector<int> caps, parent;
    std::vector<PathRay> path;
    std::vector<int> chain;
    for (size_t L = 0; L < trees.size(); ++L) {
      const std::vector<TNode>& t = trees[L];
      capture(t, c, caps, parent);
      for (int leaf : caps) {
        ++o.captured;
        chain.clear();
        for (int u = leaf; u >= 0; u = parent[u]) chain.push_back(u);
        std::reverse(chain.begin(), chain.end());
        path.clear();
        for (size_t q = 0; q < chain.size(); ++q) {
          const TNode& n = t[chain[q]];
          PathRay r{n.src, n.tgt, n.tri, n.cop, n.kind, n.mat};
          if (q + 1 == chain.size()) r.tri = r.cop = -1;  // captured: ids cleared
          path.push_back(r);
        }
        if (!correct(path, tx, c)) continue;
        ++o.corrected;
        std::vector<int> key;
        for (auto& r : path) key.push_back(r.cop);
        if (seen.count(key)) continue;
        seen.insert({key, 0});
        C3 e = field_for_path(fc, path);
        for (int a = 0; a < 3; ++a) o.field.v[a] += e.v[a];
        oracle_path op;
        op.receiver = k;
        op.launch = long(L);
        op.n_rays = int(path.size());
        op.field[0] = e.v[0].real(); op.field[1] = e.v[0].imag();
        op.field[2] = e.v[1].real(); op.field[3] = e.v[1].imag();
        op.field[4] = e.v[2].real(); op.field[5] = e.v[2].imag();
        for (auto& r : path) {
          o.tri.push_back(r.tri);
          o.cop.push_back(r.cop);
          o.kind.push_back(r.kind);
          for (int a = 0; a < 3; ++a) o.pts.push_back(r.src[a]);
          for (int a = 0; a < 3; ++a) o.pts.push_back(r.tgt[a]);
        }
        o.paths.push_back(op);
      }
    }
  }

  // RTSolver.cpp:330-433 (DirectPathCorrection for one-ray paths)
  bool correct(std::vector<PathRay>& p, const V3& tx, const V3& rxp) const {
    if (p.size() == 1) {
      Hit res;
      V3 d = rxp - tx;
      bool has = bvh_hit(s, 0, tx, d, res);
      if (!has || norm(d) < res.dist) {
        p[0].src = tx;
        p[0].tgt = rxp;
        return true;
      }
      return false;
    }
    std::vector<std::pair<int, V3>> img{{-1, tx}};
    V3 cur = tx;
    for (size_t i = 0; i + 1 < p.size(); ++i) {
      int sid = p[i].tri;
      if (sid < 0) break;
      if (p[i + 1].kind == 1) {
        cur = image_point(s.tris[s.mesh_order[sid]], cur);
        img.push_back({sid, cur});
      } else if (p[i + 1].kind == 2) {
        img.push_back({sid, cur});
      } else {
        break;
      }
    }
    Hit res;
    V3 target = rxp;
    for (int i = int(p.size()) - 1; i >= 0; --i) {
      // (imgSources.at(i) throws in the reference when the list is short;
      // that cannot happen for paths built by the tracer.)
      int sid = img.at(i).first;
      V3 src = img.at(i).second;
      V3 d = target - src;
      if (sid < 0) {
        p[i].src = src;
        p[i].tgt = target;
      } else {
        if (tri_intersect(s.tris[s.mesh_order[sid]], src, d, res)) {
          p[i].src = res.p;
          p[i].tgt = target;
          target = res.p;
        } else {
          return false;
        }
      }
    }
    return true;
  }
};

}  // namespace orc

// ---------------------------------------------------------------- C API
struct oracle_scene {
  orc::Scene s;
};

struct oracle_result {
  long segments = 0, captured = 0, corrected = 0;
  std::vector<double> field;  // 6 per receiver
  std::vector<oracle_path> paths;
  std::vector<int> tri, cop, kind;
  std::vector<double> pts;
  std::vector<long> ray_offset;  // per path, into tri/cop/kind (pts: x6)
};

extern "C" {

int oracle_scene_from_stl(const char* path, oracle_scene** out) {
  auto* sc = new oracle_scene();
  if (!orc::read_stl(path, sc->s.tris)) {
    delete sc;
    return 1;
  }
  orc::build_bvh(sc->s);
  *out = sc;
  return 0;
}

int oracle_scene_from_triangles(int n, const float* v, const float* nrm, oracle_scene** out) {
  auto* sc = new oracle_scene();
  std::vector<float> coords(v, v + 9 * size_t(n));
  std::vector<float> normals(nrm, nrm + 3 * size_t(n));
  if (!orc::tris_from_soup(coords, normals, sc->s.tris)) {
    delete sc;
    return 1;
  }
  orc::build_bvh(sc->s);
  *out = sc;
  return 0;
}

int oracle_scene_set_materials(oracle_scene* sc, const int* mat_ids) {
  for (size_t i = 0; i < sc->s.tris.size(); ++i) sc->s.tris[i].mat = mat_ids[i];
  return 0;
}

int oracle_scene_info(const oracle_scene* sc, int* n_tri, int* n_nodes) {
  *n_tri = int(sc->s.tris.size());
  *n_nodes = int(sc->s.nodes.size());
  return 0;
}

int oracle_scene_mesh_order(const oracle_scene* sc, int* out) {
  for (size_t i = 0; i < sc->s.mesh_order.size(); ++i) out[i] = sc->s.mesh_order[i];
  return 0;
}

int oracle_scene_coplanar(const oracle_scene* sc, int* out) {
  for (size_t i = 0; i < sc->s.tris.size(); ++i) out[i] = sc->s.tris[i].cop;
  return 0;
}

void oracle_scene_destroy(oracle_scene* sc) { delete sc; }

int oracle_icosphere(int level, double* out, long cap) {
  std::vector<orc::V3> v = orc::icosphere(level);
  if (long(v.size()) > cap) return -1;
  for (size_t i = 0; i < v.size(); ++i) {
    out[3 * i] = v[i].x;
    out[3 * i + 1] = v[i].y;
    out[3 * i + 2] = v[i].z;
  }
  return int(v.size());
}

int oracle_solve(const oracle_scene* sc, const oracle_request* rq, int threads,
                 oracle_result** out) {
  if (rq->antenna == 3 && (!rq->pattern || rq->pat_nt < 1 || rq->pat_np < 1 ||
                           !(rq->pat_dt > 0) || !(rq->pat_dp > 0)))
    return 2;
  orc::Solver sv(sc->s, *rq);
  sv.threads = threads > 0 ? unsigned(threads) : std::max(1u, std::thread::hardware_concurrency());
  for (int i = 0; i < rq->n_materials; ++i) sv.mats.push_back(rq->materials[i]);
  for (int i = 0; i < rq->n_rx; ++i)
    sv.rx.emplace_back(rq->rx[3 * i], rq->rx[3 * i + 1], rq->rx[3 * i + 2]);
  const int tess = rq->tessellation + 1;  // RTSolver.cpp:70
  const double beta = 1.0 / (3.0 * tess) * std::acos(-1.0 / std::sqrt(5.0));
  sv.tan_beta = std::tan(beta);
  sv.trace();
  auto* res = new oracle_result();
  for (auto& t : sv.trees) res->segments += long(t.size());
  std::vector<orc::Solver::RxOut> per(sv.rx.size());
  std::atomic<int> next(0);
  auto work = [&]() {
    for (int k; (k = next.fetch_add(1)) < int(sv.rx.size());) sv.receiver(k, per[k]);
  };
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < sv.threads; ++t) pool.emplace_back(work);
  for (auto& th : pool) th.join();
  for (auto& o : per) {
    res->captured += o.captured;
    res->corrected += o.corrected;
    for (int a = 0; a < 3; ++a) {
      res->field.push_back(o.field.v[a].real());
      res->field.push_back(o.field.v[a].imag());
    }
    long off = long(res->tri.size());
    for (auto& p : o.paths) {
      res->ray_offset.push_back(off);
      off += p.n_rays;
      res->paths.push_back(p);
    }
    res->tri.insert(res->tri.end(), o.tri.begin(), o.tri.end());
    res->cop.insert(res->cop.end(), o.cop.begin(), o.cop.end());
    res->kind.insert(res->kind.end(), o.kind.begin(), o.kind.end());
    res->pts.insert(res->pts.end(), o.pts.begin(), o.pts.end());
  }
  res->ray_offset.push_back(long(res->tri.size()));
  *out = res;
  return 0;
}

void oracle_result_counts(const oracle_result* r, long* segments, long* captured, long* corrected,
                          long* n_paths, long* n_rays) {
  *segments = r->segments;
  *captured = r->captured;
  *corrected = r->corrected;
  *n_paths = long(r->paths.size());
  *n_rays = long(r->tri.size());
}

void oracle_result_copy(const oracle_result* r, double* field, oracle_path* paths, long* ray_offset,
                        int* tri, int* cop, int* kind, double* pts) {
  if (field) std::memcpy(field, r->field.data(), r->field.size() * sizeof(double));
  if (paths) std::memcpy(paths, r->paths.data(), r->paths.size() * sizeof(oracle_path));
  if (ray_offset) std::memcpy(ray_offset, r->ray_offset.data(), r->ray_offset.size() * sizeof(long));
  if (tri) std::memcpy(tri, r->tri.data(), r->tri.size() * sizeof(int));
  if (cop) std::memcpy(cop, r->cop.data(), r->cop.size() * sizeof(int));
  if (kind) std::memcpy(kind, r->kind.data(), r->kind.size() * sizeof(int));
  if (pts) std::memcpy(pts, r->pts.data(), r->pts.size() * sizeof(double));
}

void oracle_result_destroy(oracle_result* r) { delete r; }

}  // extern "C"
