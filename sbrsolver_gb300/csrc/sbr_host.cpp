// Host-side scene preparation (see sbr_host.h).  Compiled with
// -ffp-contract=off: every FP64 expression below is evaluated in the order
// written, which is the reference's order, so results are bit-identical to
// the reference on any host.
#include "sbr_host.h"

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <limits>
#include <numeric>
#include <sstream>
#include <thread>
#include <unordered_map>
#include <utility>

namespace sbr {
namespace {

inline double sqn(const double* a) { return (a[0] * a[0] + a[1] * a[1]) + a[2] * a[2]; }

// Eigen's normalized(): v / sqrt(|v|^2) when |v|^2 > 0.
inline void normalize3(const double* a, double* out) {
  double z = sqn(a);
  if (z > 0) {
    double s = std::sqrt(z);
    out[0] = a[0] / s;
    out[1] = a[1] / s;
    out[2] = a[2] / s;
  } else {
    out[0] = a[0];
    out[1] = a[1];
    out[2] = a[2];
  }
}

void finish_tri(HostTri& t) {
  double e[3] = {t.v2[0] - t.v1[0], t.v2[1] - t.v1[1], t.v2[2] - t.v1[2]};
  double y[3];
  normalize3(e, y);
  const double* z = t.n;
  double x[3] = {y[1] * z[2] - y[2] * z[1], y[2] * z[0] - y[0] * z[2], y[0] * z[1] - y[1] * z[0]};
  for (int j = 0; j < 3; ++j) {
    t.cs[j] = x[j];
    t.cs[3 + j] = y[j];
    t.cs[6 + j] = z[j];
  }
  for (int a = 0; a < 3; ++a) {
    t.bb[a] = std::min({t.v1[a], t.v2[a], t.v3[a]});
    t.bb[3 + a] = std::max({t.v1[a], t.v2[a], t.v3[a]});
    t.center[a] = (t.bb[a] + t.bb[3 + a]) / 2.0;
  }
}

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

// A triangle as the SAH build sees it: its box (float values: the box of
// float vertices) and id.  The build permutes one array of these in place, a
// node owning a contiguous range, so its sorts and sweeps read memory in
// order instead of chasing ids into the triangle records.
struct BuildRec {
  float lo[3], hi[3];
  int id, pad;
  // the box centre exactly as the reference computes it (bb min + max) / 2
  double center(int a) const { return (double(lo[a]) + double(hi[a])) / 2.0; }
};

struct BuildNode {
  double bb[6];
  int c0 = -1, c1 = -1;
  int lo = 0, hi = 0;  // range of the build array; a leaf's triangles in the reference's order
};

struct SplitScratch {
  std::vector<std::pair<double, int>> kv;
  std::vector<BuildRec> tmp;
  std::vector<double> sa1, sa2;
};

// One step of the reference's SAH build (BVH/BVH.h:135-230) on the node whose
// objects are R[lo, hi) (sorted in place exactly as the reference sorts its
// object list).  Returns the split index (relative to lo), or -1 for a leaf.
int sah_split(std::vector<BuildRec>& R, int lo, int hi, double* bb, SplitScratch& s) {
  const int n = hi - lo;
  BuildRec* r = R.data() + lo;
  empty_box(bb);
  for (int i = 0; i < n; ++i) {
    const double b[6] = {r[i].lo[0], r[i].lo[1], r[i].lo[2], r[i].hi[0], r[i].hi[1], r[i].hi[2]};
    merge_box(b, bb, bb);
  }
  double best_cost = 1.0 * n;
  int best_axis = -1, best_split = -1;
  const double sa_root = surface_area(bb);
  s.sa1.assign(size_t(n) + 1, std::numeric_limits<double>::max());
  s.sa2.assign(size_t(n) + 1, std::numeric_limits<double>::max());
  s.kv.resize(size_t(n));
  s.tmp.resize(size_t(n));
  // std::sort's result depends only on the outcomes of its comparisons, so
  // sorting (key, position) pairs by key and then moving the records leaves
  // them in exactly the order the reference's sort of ids by
  // tris[id].center[axis] does.
  auto sort_axis = [&](int axis) {
    for (int i = 0; i < n; ++i) s.kv[size_t(i)] = {r[i].center(axis), i};
    std::sort(s.kv.begin(), s.kv.end(), [](const std::pair<double, int>& a,
                                           const std::pair<double, int>& b) { return a.first < b.first; });
    for (int i = 0; i < n; ++i) s.tmp[size_t(i)] = r[s.kv[size_t(i)].second];
    std::copy(s.tmp.begin(), s.tmp.end(), r);
  };
  for (int axis = 0; axis < 3; ++axis) {
    sort_axis(axis);
    double b1[6];
    empty_box(b1);
    s.sa1[0] = surface_area(b1);
    for (int i = 0; i < n; ++i) {
      const double b[6] = {r[i].lo[0], r[i].lo[1], r[i].lo[2], r[i].hi[0], r[i].hi[1], r[i].hi[2]};
      merge_box(b1, b, b1);
      s.sa1[size_t(i)] = surface_area(b1);
    }
    double b2[6];
    empty_box(b2);
    s.sa2[size_t(n)] = surface_area(b2);
    for (int i = n - 1; i >= 0; --i) {
      const double b[6] = {r[i].lo[0], r[i].lo[1], r[i].lo[2], r[i].hi[0], r[i].hi[1], r[i].hi[2]};
      merge_box(b2, b, b2);
      s.sa2[size_t(i)] = surface_area(b2);
    }
    for (int i = 1; i < n - 1; ++i) {
      const int j = n - i;
      const double cost = 2 * 1.0 + (i * s.sa1[size_t(i)] + j * s.sa2[size_t(i)]) * 1.0 / sa_root;
      if (cost < best_cost) {
        best_cost = cost;
        best_axis = axis;
        best_split = i;
      }
    }
  }
  if (best_axis == -1) return -1;
  sort_axis(best_axis);
  return best_split;
}

}  // namespace

bool read_stl(const std::string& path, std::vector<float>& v, std::vector<float>& n,
              std::string& err) {
  std::ifstream in(path, std::ios::binary);
  if (!in) {
    err = "cannot open " + path;
    return false;
  }
  std::string head(256, '\0');
  in.read(&head[0], 256);
  head.resize(size_t(in.gcount()));
  for (auto& ch : head) ch = char(std::tolower(static_cast<unsigned char>(ch)));
  const bool ascii = head.find("solid") != std::string::npos &&
                     head.find('\n') != std::string::npos &&
                     head.find("facet") != std::string::npos &&
                     head.find("normal") != std::string::npos;
  in.clear();
  in.seekg(0);
  v.clear();
  n.clear();
  if (ascii) {
    std::string line, tok;
    size_t nv = 0;
    while (std::getline(in, line)) {
      std::istringstream ls(line);
      std::vector<std::string> toks;
      while (ls >> tok) toks.push_back(tok);
      if (toks.empty()) continue;
      if (toks[0] == "vertex") {
        if (toks.size() < 4) {
          err = "malformed vertex line in " + path;
          return false;
        }
        for (int i = 0; i < 3; ++i) v.push_back(float(std::atof(toks[1 + i].c_str())));
        ++nv;
      } else if (toks[0] == "facet") {
        if (toks.size() < 5 || toks[1] != "normal") {
          err = "malformed facet line in " + path;
          return false;
        }
        for (int i = 0; i < 3; ++i) n.push_back(float(std::atof(toks[2 + i].c_str())));
        nv = 0;
      } else if (toks[0] == "endfacet") {
        if (nv != 3) {
          err = "facet without 3 vertices in " + path;
          return false;
        }
      }
    }
  } else {
    char hdr[80];
    uint32_t cnt = 0;
    in.read(hdr, 80);
    in.read(reinterpret_cast<char*>(&cnt), 4);
    if (!in) {
      err = "truncated binary STL header in " + path;
      return false;
    }
    // the header's facet count must fit the file (84-byte header, 50 bytes
    // per facet) before any storage is sized from it
    in.seekg(0, std::ios::end);
    const unsigned long long size = (unsigned long long)(std::streamoff)in.tellg();
    in.seekg(84);
    if (size < 84ull + 50ull * cnt) {
      err = "truncated binary STL in " + path + ": header counts " + std::to_string(cnt) +
            " facets, the file holds " + std::to_string((size - 84) / 50);
      return false;
    }
    v.resize(size_t(cnt) * 9);
    n.resize(size_t(cnt) * 3);
    for (uint32_t t = 0; t < cnt; ++t) {
      float d[12];
      char attr[2];
      in.read(reinterpret_cast<char*>(d), 48);
      in.read(attr, 2);
      if (!in) {
        err = "truncated binary STL facet in " + path;
        return false;
      }
      std::memcpy(&n[3 * size_t(t)], d, 12);
      std::memcpy(&v[9 * size_t(t)], d + 3, 36);
    }
  }
  if (n.size() * 3 != v.size()) {
    err = "facet/vertex count mismatch in " + path;
    return false;
  }
  return true;
}

namespace {
void build_search_bvh_ids(const float* v, int n_tri, SearchBVH& out);
}  // namespace

bool prepare_scene(int n_tri, const float* v, const float* nrm, const int* mat, HostScene& out,
                   std::string& err, bool host_tables, bool ref_bvh) {
  out = HostScene();
  if (n_tri <= 0 || !v || !nrm) {
    err = "empty triangle list";
    return false;
  }
  // The search BVH depends only on the triangles' float boxes, so it is built
  // over triangle ids on its own thread while the reference BVH is built, and
  // its leaves are mapped to depth-first ranks at the end.
  SearchBVH search;
  std::thread search_thread;
  if (host_tables) search_thread = std::thread([&] { build_search_bvh_ids(v, n_tri, search); });
  struct Joiner {
    std::thread& t;
    ~Joiner() {
      if (t.joinable()) t.join();
    }
  } joiner{search_thread};
  // Exact vertex merge (StlReader.h:448-508): equal float triples share an id.
  struct Key {
    float x, y, z;
    bool operator==(const Key& o) const { return x == o.x && y == o.y && z == o.z; }
  };
  struct KeyHash {
    size_t operator()(const Key& k) const {
      // +0.0 and -0.0 compare equal, so hash them alike.
      float a = k.x == 0.0f ? 0.0f : k.x, b = k.y == 0.0f ? 0.0f : k.y,
            c = k.z == 0.0f ? 0.0f : k.z;
      uint32_t u[3];
      std::memcpy(&u[0], &a, 4);
      std::memcpy(&u[1], &b, 4);
      std::memcpy(&u[2], &c, 4);
      uint64_t h = 1469598103934665603ull;
      for (uint32_t w : u) h = (h ^ w) * 1099511628211ull;
      return size_t(h);
    }
  };
  const size_t nv = size_t(n_tri) * 3;
  std::vector<int> uid(nv);
  if (host_tables) {
    std::unordered_map<Key, int, KeyHash> ids;
    ids.reserve(nv);
    for (size_t i = 0; i < nv; ++i) {
      Key k{v[3 * i], v[3 * i + 1], v[3 * i + 2]};
      auto it = ids.emplace(k, int(ids.size())).first;
      uid[i] = it->second;
    }
  } else {  // merged on the device; the ids here only need to be distinct
    for (size_t i = 0; i < nv; ++i) uid[i] = int(i);
  }
  std::vector<int> vidx;
  std::vector<size_t> src;
  for (size_t t = 0; t < size_t(n_tri); ++t) {
    int a = uid[3 * t], b = uid[3 * t + 1], c = uid[3 * t + 2];
    if (a != b && a != c && b != c) {
      vidx.push_back(a);
      vidx.push_back(b);
      vidx.push_back(c);
      src.push_back(t);
    }
  }
  // A collapsed facet shifts later normals in the reference reader; reject
  // such input instead of reproducing the misalignment silently.
  if (src.size() != size_t(n_tri)) {
    err = "degenerate triangle(s) after vertex merge: " + std::to_string(size_t(n_tri) - src.size());
    return false;
  }
  out.tris.resize(src.size());
  // triangle records (frames, boxes) in parallel slices
  const unsigned n_slices =
      std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 32u));
  std::vector<double> slice_ext(n_slices, 0.0);
  {
    auto fill = [&](unsigned k) {
      const size_t b = src.size() * k / n_slices, e = src.size() * (k + 1) / n_slices;
      double ext = 0;
      for (size_t t = b; t < e; ++t) {
        HostTri& tr = out.tris[t];
        const float* p = &v[9 * src[t]];
        for (int a = 0; a < 3; ++a) {
          tr.v1[a] = p[a];
          tr.v2[a] = p[3 + a];
          tr.v3[a] = p[6 + a];
          tr.n[a] = nrm[3 * t + a];
          ext = std::max({ext, std::fabs(tr.v1[a]), std::fabs(tr.v2[a]), std::fabs(tr.v3[a])});
        }
        tr.id = int(t);
        tr.mat = mat ? mat[src[t]] : 0;
        finish_tri(tr);
      }
      slice_ext[k] = ext;
    };
    std::vector<std::thread> pool;
    for (unsigned k = 1; k < n_slices; ++k) pool.emplace_back(fill, k);
    fill(0);
    for (auto& th : pool) th.join();
  }
  out.extent = *std::max_element(slice_ext.begin(), slice_ext.end());

  // Coplanar ids (Preprocessor.cpp:116-246), unless the device builds them.
  const int nt = int(out.tris.size());
  if (host_tables) {
  std::vector<int> parent(nt);
  std::iota(parent.begin(), parent.end(), 0);
  auto find = [&](int a) {
    while (parent[a] != a) a = parent[a] = parent[parent[a]];
    return a;
  };
  auto same_or_opposite = [&](int a, int b) {
    const double* p = out.tris[a].n;
    const double* q = out.tris[b].n;
    return (p[0] == q[0] && p[1] == q[1] && p[2] == q[2]) ||
           (p[0] == -q[0] && p[1] == -q[1] && p[2] == -q[2]);
  };
  // Triangles sharing an edge (of merged vertex ids) are adjacent when their
  // facet normals are equal or opposite; the components do not depend on the
  // order the pairs are joined in, so the edges are grouped by sorting.
  std::vector<std::pair<uint64_t, int>> edges;
  edges.reserve(3 * size_t(nt));
  for (int t = 0; t < nt; ++t) {
    int a = vidx[3 * t], b = vidx[3 * t + 1], c = vidx[3 * t + 2];
    int es[3][2] = {{std::min(a, b), std::max(a, b)},
                    {std::min(b, c), std::max(b, c)},
                    {std::min(a, c), std::max(a, c)}};
    for (auto& e : es) edges.push_back({(uint64_t(uint32_t(e[0])) << 32) | uint32_t(e[1]), t});
  }
  std::sort(edges.begin(), edges.end());
  for (size_t i = 0; i < edges.size();) {
    size_t j = i + 1;
    while (j < edges.size() && edges[j].first == edges[i].first) ++j;
    for (size_t x = i; x < j; ++x)
      for (size_t y = x + 1; y < j; ++y)
        if (same_or_opposite(edges[x].second, edges[y].second))
          parent[find(edges[x].second)] = find(edges[y].second);
    i = j;
  }
  std::vector<int> comp(nt, -1);
  int next = 0;
  for (int t = 0; t < nt; ++t) {
    int r = find(t);
    if (comp[r] < 0) comp[r] = next++;
    out.tris[t].cop = comp[r];
  }
  }

  if (!ref_bvh) return true;  // the device builds the reference BVH

  // SAH BVH with the reference's splits; nodes renumbered depth-first.  Every
  // node's split depends only on its own object list, so the tree does not
  // depend on the order nodes are split in: nodes above a size threshold are
  // split here, the subtrees below it in parallel, then merged.
  std::vector<BuildRec> R(static_cast<size_t>(nt));
  for (int t = 0; t < nt; ++t) {
    const HostTri& tr = out.tris[size_t(t)];
    BuildRec& b = R[size_t(t)];
    for (int a = 0; a < 3; ++a) {
      b.lo[a] = float(tr.bb[a]);  // float vertices: the box values are floats
      b.hi[a] = float(tr.bb[3 + a]);
    }
    b.id = t;
    b.pad = 0;
  }
  std::vector<BuildNode> bn;
  bn.reserve(size_t(2) * nt);
  bn.emplace_back();
  bn[0].lo = 0;
  bn[0].hi = nt;
  const int big = std::max(4096, nt / 64);
  const unsigned nthreads =
      std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 32u));
  // runs f(0..n-1) on up to nthreads threads
  auto parallel_for = [nthreads](size_t n, const std::function<void(size_t)>& f) {
    std::atomic<size_t> next{0};
    auto run = [&]() {
      for (size_t k = next++; k < n; k = next++) f(k);
    };
    std::vector<std::thread> pool;
    for (unsigned i = 1; i < nthreads && i < n; ++i) pool.emplace_back(run);
    run();
    for (auto& t : pool) t.join();
  };
  std::vector<int> subtrees;  // roots left to the parallel subtree phase
  {
    // the large nodes level by level, the nodes of a level split in parallel
    std::vector<int> frontier{0};
    while (!frontier.empty()) {
      std::vector<int> split(frontier.size());
      parallel_for(frontier.size(), [&](size_t k) {
        SplitScratch sc;
        BuildNode& b = bn[size_t(frontier[k])];
        split[k] = sah_split(R, b.lo, b.hi, b.bb, sc);
      });
      if (frontier[0] == 0) {  // the caller's vector after ConstructBVH
        out.mesh_order.resize(size_t(nt));
        for (int t = 0; t < nt; ++t) out.mesh_order[size_t(t)] = R[size_t(t)].id;
      }
      std::vector<int> next;
      for (size_t k = 0; k < frontier.size(); ++k) {
        const int idx = frontier[k];
        if (split[k] < 0) continue;  // a leaf keeps its objects
        const int c0 = int(bn.size());
        bn.emplace_back();
        const int c1 = int(bn.size());
        bn.emplace_back();
        BuildNode& b = bn[size_t(idx)];
        b.c0 = c0;
        b.c1 = c1;
        bn[size_t(c0)].lo = b.lo;
        bn[size_t(c0)].hi = b.lo + split[k];
        bn[size_t(c1)].lo = b.lo + split[k];
        bn[size_t(c1)].hi = b.hi;
        for (int c : {c0, c1})
          (bn[size_t(c)].hi - bn[size_t(c)].lo >= big ? next : subtrees).push_back(c);
      }
      frontier.swap(next);
    }
  }
  {
    // each subtree into its own node list (local index 0 = the subtree root);
    // the subtrees own disjoint ranges of R
    std::vector<std::vector<BuildNode>> local(subtrees.size());
    parallel_for(subtrees.size(), [&](size_t k) {
      SplitScratch sc;
      std::vector<BuildNode>& ln = local[k];
      ln.emplace_back();
      ln[0].lo = bn[size_t(subtrees[k])].lo;
      ln[0].hi = bn[size_t(subtrees[k])].hi;
      std::vector<int> work{0};
      while (!work.empty()) {
        const int idx = work.back();
        work.pop_back();
        const int lo = ln[size_t(idx)].lo, hi = ln[size_t(idx)].hi;
        double bb[6];
        const int split = sah_split(R, lo, hi, bb, sc);
        std::memcpy(ln[size_t(idx)].bb, bb, sizeof bb);
        if (split < 0) continue;
        const int c0 = int(ln.size());
        ln.emplace_back();
        const int c1 = int(ln.size());
        ln.emplace_back();
        ln[size_t(idx)].c0 = c0;
        ln[size_t(idx)].c1 = c1;
        ln[size_t(c0)].lo = lo;
        ln[size_t(c0)].hi = lo + split;
        ln[size_t(c1)].lo = lo + split;
        ln[size_t(c1)].hi = hi;
        work.push_back(c1);
        work.push_back(c0);
      }
    });
    for (size_t k = 0; k < subtrees.size(); ++k) {
      std::vector<BuildNode>& ln = local[k];
      const int off = int(bn.size()) - 1;  // local j >= 1 goes to bn[off + j]
      auto map = [&](int c) { return c < 0 ? -1 : (c == 0 ? subtrees[k] : off + c); };
      for (size_t j = 1; j < ln.size(); ++j) {
        ln[j].c0 = map(ln[j].c0);
        ln[j].c1 = map(ln[j].c1);
        bn.push_back(ln[j]);
      }
      BuildNode& r = bn[size_t(subtrees[k])];
      std::memcpy(r.bb, ln[0].bb, sizeof r.bb);
      r.c0 = map(ln[0].c0);
      r.c1 = map(ln[0].c1);
    }
  }
  // Depth-first renumbering, children[0] first.
  out.nodes.clear();
  out.nodes.reserve(bn.size());
  struct Item {
    int b, parent, depth, slot_parent, which;
  };
  std::vector<Item> st{{0, -1, 0, -1, 0}};
  while (!st.empty()) {
    Item it = st.back();
    st.pop_back();
    int me = int(out.nodes.size());
    out.nodes.emplace_back();
    HostNode& hn = out.nodes.back();
    std::memcpy(hn.bb, bn[it.b].bb, sizeof hn.bb);
    hn.parent = it.parent;
    hn.depth = it.depth;
    out.max_depth = std::max(out.max_depth, it.depth);
    if (it.slot_parent >= 0) {
      if (it.which == 0) out.nodes[it.slot_parent].c0 = me;
      else out.nodes[it.slot_parent].c1 = me;
    }
    if (bn[it.b].c0 < 0) {
      hn.first = int(out.dfs_tris.size());
      hn.count = bn[it.b].hi - bn[it.b].lo;
      for (int q = bn[it.b].lo; q < bn[it.b].hi; ++q) out.dfs_tris.push_back(R[size_t(q)].id);
    } else {
      st.push_back({bn[it.b].c1, me, it.depth + 1, me, 1});
      st.push_back({bn[it.b].c0, me, it.depth + 1, me, 0});
    }
  }
  if (host_tables) {
    search_thread.join();
    out.search = std::move(search);
    map_search_order(out);
  }
  return true;
}

void map_search_order(HostScene& H) {
  std::vector<int> rank_of(H.tris.size());
  for (size_t r = 0; r < H.dfs_tris.size(); ++r) rank_of[size_t(H.dfs_tris[r])] = int(r);
  for (int& o : H.search.order) o = rank_of[size_t(o)];
}

namespace {

struct FBox {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  void add(const float* l, const float* h) {
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], l[a]);
      hi[a] = std::max(hi[a], h[a]);
    }
  }
  void add_point(const float* p) { add(p, p); }
  float area() const {
    const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return dx < 0 ? 0.0f : 2.0f * (dx * dy + dy * dz + dz * dx);
  }
};

struct SearchBuild {
  std::vector<float> blo, bhi, cen;  // per triangle
  SearchBVH* out;
  int max_depth = 0;

  int leaf(int b, int n) { return ~((b << 3) | n); }

  // Builds [b, e) of out->order; returns the child ref and its box.
  int build(int b, int e, int depth, FBox& box) {
    std::vector<int>& ord = out->order;
    FBox cb;
    box = FBox();
    for (int i = b; i < e; ++i) {
      const int p = ord[i];
      box.add(&blo[3 * p], &bhi[3 * p]);
      cb.add_point(&cen[3 * p]);
    }
    max_depth = std::max(max_depth, depth);
    const int n = e - b;
    if (n <= 2) return leaf(b, n);
    int ax = 0;
    for (int a = 1; a < 3; ++a)
      if (cb.hi[a] - cb.lo[a] > cb.hi[ax] - cb.lo[ax]) ax = a;
    const float ext = cb.hi[ax] - cb.lo[ax];
    int mid = -1;
    if (ext > 0) {
      constexpr int kBins = 32;
      FBox bins[kBins];
      int cnt[kBins] = {0};
      const float k = kBins / ext;
      auto bin_of = [&](int p) {
        return std::min(kBins - 1, std::max(0, int((cen[3 * p + ax] - cb.lo[ax]) * k)));
      };
      for (int i = b; i < e; ++i) {
        const int p = ord[i], q = bin_of(p);
        ++cnt[q];
        bins[q].add(&blo[3 * p], &bhi[3 * p]);
      }
      float right_area[kBins];
      int right_cnt[kBins];
      FBox acc;
      int c = 0;
      for (int i = kBins - 1; i > 0; --i) {
        acc.add(bins[i].lo, bins[i].hi);
        c += cnt[i];
        right_area[i] = acc.area();
        right_cnt[i] = c;
      }
      FBox lacc;
      int lc = 0, best = -1;
      float best_cost = INFINITY;
      for (int i = 0; i < kBins - 1; ++i) {
        lacc.add(bins[i].lo, bins[i].hi);
        lc += cnt[i];
        if (lc == 0 || right_cnt[i + 1] == 0) continue;
        const float cost = lacc.area() * lc + right_area[i + 1] * right_cnt[i + 1];
        if (cost < best_cost) {
          best_cost = cost;
          best = i;
        }
      }
      // cost of a node relative to its leaf: one box test per triangle saved
      const float leaf_cost = box.area() * n;
      if (best >= 0 && (n > 7 || best_cost + box.area() < leaf_cost)) {
        // stable, so the leaf order is a function of the input alone (the
        // device build reproduces it)
        mid = int(std::stable_partition(ord.begin() + b, ord.begin() + e,
                                        [&](int p) { return bin_of(p) <= best; }) -
                  ord.begin());
      } else if (n <= 7) {
        return leaf(b, n);
      }
    } else if (n <= 7) {
      return leaf(b, n);
    }
    if (depth > 48) mid = -1;  // keep the tree shallow enough for the traversal stack
    if (mid <= b || mid >= e) {  // no usable SAH split: median along the axis
      mid = b + n / 2;
      // ordered by (centroid, triangle id): no ties, so the halves are
      // determined by the input alone
      std::sort(ord.begin() + b, ord.begin() + e, [&](int x, int y) {
        const float cx = cen[3 * x + ax], cy = cen[3 * y + ax];
        return cx < cy || (cx == cy && x < y);
      });
    }
    const int me = int(out->nodes.size());
    out->nodes.emplace_back();
    FBox lb, rb;
    const int l = build(b, mid, depth + 1, lb);
    const int r = build(mid, e, depth + 1, rb);
    SearchNode& nd = out->nodes[me];
    for (int a = 0; a < 3; ++a) {
      nd.lo[0][a] = lb.lo[a];
      nd.hi[0][a] = lb.hi[a];
      nd.lo[1][a] = rb.lo[a];
      nd.hi[1][a] = rb.hi[a];
    }
    nd.child[0] = l;
    nd.child[1] = r;
    return me;
  }
};

// Builds `out` over triangles 0..n_tri-1 with vertices v (9 floats each);
// out.order holds triangle ids.
void build_search_bvh_ids(const float* v, int n_tri, SearchBVH& out) {
  const int n = n_tri;
  SearchBuild sb;
  sb.out = &out;
  out.nodes.clear();
  out.order.resize(n);
  sb.blo.resize(3 * size_t(n));
  sb.bhi.resize(3 * size_t(n));
  sb.cen.resize(3 * size_t(n));
  // -0 is read as +0 (they compare equal; the boxes then do not depend on
  // which of the two a min or max met first, so the device build matches)
  auto pz = [](float x) { return x == 0.0f ? 0.0f : x; };
  for (int t = 0; t < n; ++t) {
    const float* p = v + 9 * size_t(t);
    for (int a = 0; a < 3; ++a) {
      const float x = pz(p[a]), y = pz(p[3 + a]), z = pz(p[6 + a]);
      sb.blo[3 * t + a] = std::min({x, y, z});
      sb.bhi[3 * t + a] = std::max({x, y, z});
      sb.cen[3 * t + a] = 0.5f * (sb.blo[3 * t + a] + sb.bhi[3 * t + a]);
    }
    out.order[t] = t;
  }
  out.nodes.reserve(size_t(n) / 2 + 2);
  out.nodes.emplace_back();  // root
  FBox box;
  const int ref = sb.build(0, n, 1, box);
  SearchNode& root = out.nodes[0];
  if (ref >= 0) {  // the root's children become node 0's children
    root = out.nodes[size_t(ref)];
    // node `ref` stays as an unreachable copy
  } else {  // the whole scene is one leaf: one child, the other an empty leaf
    for (int a = 0; a < 3; ++a) {
      root.lo[0][a] = root.lo[1][a] = box.lo[a];
      root.hi[0][a] = root.hi[1][a] = box.hi[a];
    }
    root.child[0] = ref;
    root.child[1] = ~0;  // first 0, count 0
  }
  out.max_depth = sb.max_depth;
}

}  // namespace

void build_search_bvh(HostScene& H) {
  std::vector<float> v(9 * H.tris.size());
  for (size_t t = 0; t < H.tris.size(); ++t)
    for (int a = 0; a < 3; ++a) {
      // vertices are float values, so the float copies are exact
      v[9 * t + a] = float(H.tris[t].v1[a]);
      v[9 * t + 3 + a] = float(H.tris[t].v2[a]);
      v[9 * t + 6 + a] = float(H.tris[t].v3[a]);
    }
  build_search_bvh_ids(v.data(), int(H.tris.size()), H.search);
  std::vector<int> rank_of(H.tris.size());
  for (size_t r = 0; r < H.dfs_tris.size(); ++r) rank_of[size_t(H.dfs_tris[r])] = int(r);
  for (int& o : H.search.order) o = rank_of[size_t(o)];
}

void icosphere(int level, std::vector<double>& dirs) {
  const double X = .525731112119133606, Z = .850650808352039932, N = 0.0;
  std::vector<double> v = {-X, N, Z, X, N, Z,  -X, N, -Z, X, N, -Z, N, Z, X,  N, Z, -X,
                           N,  -Z, X, N, -Z, -X, Z,  X, N, -Z, X,  N, Z, -X, N, -Z, -X, N};
  std::vector<int> f = {0, 4, 1,  0, 9, 4,  9, 5, 4,  4, 5, 8,  4, 8, 1,  8, 10, 1, 8, 3, 10,
                        5, 3, 8,  5, 2, 3,  2, 7, 3,  7, 10, 3, 7, 6, 10, 7, 11, 6, 11, 0, 6,
                        0, 1, 6,  6, 1, 10, 9, 0, 11, 9, 11, 2, 9, 2, 5,  7, 2, 11};
  for (int l = 0; l < level; ++l) {
    std::unordered_map<uint64_t, int> lookup;
    lookup.reserve(f.size());
    std::vector<int> nf;
    nf.reserve(f.size() * 4);
    auto mid = [&](int a, int b) {
      uint64_t key = (uint64_t(uint32_t(std::min(a, b))) << 32) | uint32_t(std::max(a, b));
      auto ins = lookup.emplace(key, int(v.size() / 3));
      if (ins.second) {
        double s[3] = {v[3 * a] + v[3 * b], v[3 * a + 1] + v[3 * b + 1], v[3 * a + 2] + v[3 * b + 2]};
        double m[3];
        normalize3(s, m);
        v.insert(v.end(), m, m + 3);
      }
      return ins.first->second;
    };
    for (size_t t = 0; t < f.size(); t += 3) {
      int a = f[t], b = f[t + 1], c = f[t + 2];
      int m0 = mid(a, b), m1 = mid(b, c), m2 = mid(c, a);
      int add[12] = {a, m0, m2, b, m1, m0, c, m2, m1, m0, m1, m2};
      nf.insert(nf.end(), add, add + 12);
    }
    f.swap(nf);
  }
  dirs.resize(v.size());
  for (size_t i = 0; i < v.size(); i += 3) normalize3(&v[i], &dirs[i]);
}

}  // namespace sbr
