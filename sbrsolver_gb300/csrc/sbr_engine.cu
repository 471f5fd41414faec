// GB300 SBR engine: device-resident scenes, workspaces and the solve behind
// the C ABI declared in include/sbr.h.  The kernels live in
//   sbr_grid.cuh     receivers -> uniform grid (bbox, count, scan, scatter)
//   sbr_trace.cuh    RayLaunch (RTSolver.cpp:128-257) as a wavefront: per bounce
//                    depth an FP32 candidate search (k_find) and the FP64
//                    closest hit, tree node and children (k_trace); then each
//                    path class's correction cone in FP64 (k_class_cones)
//   sbr_capture.cuh  RayCapture (RTSolver.cpp:259-297, 805-863) with image
//                    correction's first step as a prefilter (k_capture), FP64
//                    decisions, MultiPathCorrection (its outcome kept per
//                    (class, receiver)) and ancestor suppression
//                    (k_capture_finish)
//   sbr_paths.cuh    DirectPathCorrection per receiver (k_direct, on a side
//                    stream during the trace), duplicate removal
//                    (RTSolver.cpp:435-459), the survivors' corrected
//                    geometry (k_path), field terms per segment (k_seg) and
//                    field (k_combine) (FieldCompute.cpp:71-151), and the
//                    per-receiver sum in (launch, BFS) order
//                    (FieldCompute.cpp:11-25)
// Each workspace has a stream and a side stream; the host synchronises once
// per solve, after the capacity counters (a solve whose tables overflowed is
// repeated with larger ones).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <functional>
#include <thread>
#include <vector>

#include "../../include/sbr.h"
#include "sbr_device.h"
#include "sbr_field.cuh"
#include "sbr_host.h"
#include "sbr_kernels.cuh"

#include "sbr_common.cuh"
#include "sbr_grid.cuh"
#include "sbr_trace.cuh"
#include "sbr_capture.cuh"
#include "sbr_paths.cuh"
#include "sbr_prep.cuh"
#include "sbr_refbvh.cuh"

namespace sbr {

// ------------------------------------------------------------ error state
static thread_local std::string g_err;
static void set_err(const std::string& s) { g_err = s; }
void set_error_message(const std::string& s) { g_err = s; }

struct CudaError {
  cudaError_t e;
  std::string where;
};
#define CK(x)                                                             \
  do {                                                                    \
    cudaError_t _e = (x);                                                 \
    if (_e != cudaSuccess) throw CudaError{_e, std::string(#x)};          \
  } while (0)

// ------------------------------------------------------------ fault injection
// Host-side fault injection for tests (sbr_fault_inject_alloc): when armed
// with n >= 0, the (n+1)-th device allocation the library attempts fails as
// cudaMalloc fails on an exhausted device, without calling it.  -1 = off.
static std::atomic<long long> g_alloc_fault{-1};

static bool injected_alloc_failure() {
  long long v = g_alloc_fault.load(std::memory_order_relaxed);
  while (v >= 0) {
    if (g_alloc_fault.compare_exchange_weak(v, v - 1, std::memory_order_relaxed)) return v == 0;
  }
  return false;
}

// ------------------------------------------------------------ device buffer
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void ensure(size_t want) {
    if (want <= n) return;
    release();
    if (want == 0) return;
    void* q = nullptr;
    cudaError_t e = injected_alloc_failure() ? cudaErrorMemoryAllocation
                                             : cudaMalloc(&q, want * sizeof(T));
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw CudaError{e, "cudaMalloc " + std::to_string(want * sizeof(T)) + " bytes"};
    }
    p = static_cast<T*>(q);
    n = want;
  }
  void upload(const T* src, size_t cnt, cudaStream_t st) {
    ensure(cnt);
    if (cnt) CK(cudaMemcpyAsync(p, src, cnt * sizeof(T), cudaMemcpyHostToDevice, st));
  }
};

// Pinned host buffer: the staging of what a solve uploads (a captured graph
// copies from it when it replays).
template <class T>
struct HBuf {
  T* p = nullptr;
  size_t n = 0;
  ~HBuf() {
    if (p) cudaFreeHost(p);
  }
  void ensure(size_t want) {
    if (want <= n) return;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    void* q = nullptr;
    cudaError_t e = injected_alloc_failure() ? cudaErrorMemoryAllocation
                                             : cudaMallocHost(&q, want * sizeof(T));
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw CudaError{e, "cudaMallocHost " + std::to_string(want * sizeof(T)) + " bytes"};
    }
    p = static_cast<T*>(q);
    n = want;
  }
};

static uint32_t next_pow2(uint64_t x) {
  uint64_t p = 1;
  while (p < x) p <<= 1;
  return uint32_t(std::min<uint64_t>(p, 1ull << 31));
}

// ============================================================ host side

// Buffers, stream and capacities of one solve in flight.  A scene keeps a
// pool of these so that solves issued from several host threads run on
// separate streams and overlap on the GPU.
struct Workspace {
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;  // the direct-path test, concurrent with the trace
  cudaEvent_t ev[8] = {};
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaEvent_t cap_ev[2] = {};  // around the capture kernel
  std::vector<cudaEvent_t> tr_ev;  // before and after each k_trace launch
  DBuf<TxParams> txp;
  DBuf<double> rx;
  DBuf<int> rx_req;
  DBuf<int> rx_bad;  // set when a device-resident receiver has a non-finite coordinate
  DBuf<double> path_bound, field_bound;  // FP32 field mode: error bounds per path / receiver
  DBuf<int> rx_flag;                     // FP32 field mode: receivers recomputed in FP64
  DBuf<unsigned long long> fstat;
  DBuf<GridBuild> gb;
  DBuf<RxGrid> grids;
  DBuf<int> cell_base, cell_counts, cell_starts, cell_cursor;
  DBuf<float4> rx32;
  DBuf<RayRec> q0, q1;
  DBuf<RayF32> ray32;                  // FP32 copies of a chunk's rays (k_find -> k_trace)
  DBuf<NodeHot> nodes;
  DBuf<NodeCold> nodes_cold;
  DBuf<unsigned long long> cls_keys, cop_keys, dd_keys, dd_rank;
  DBuf<unsigned long long> cc_keys;    // (class, receiver) correction cache
  DBuf<uint32_t> cls_list;             // interned classes, for their correction cones
  DBuf<unsigned char> cc_val;
  DBuf<ClassInfo> cls_info;
  DBuf<ClassCap> cls_cap;
  DBuf<Corrected> corr_list;
  DBuf<uint2> pairs;  // capture pairs left to the FP64 pass
  DBuf<unsigned char> direct_ok;
  DBuf<Survivor> surv;
  DBuf<int> s_counts, s_starts, s_cursor, s_order;
  DBuf<double> path_field, path_pts, field;
  DBuf<SegTerms> seg;                  // field terms per path segment
  DBuf<int> path_mat;                  // material of each ray's start per path
  DBuf<double> path_field64, field64;  // FP64 shadow of an FP32 field (field_check)
  DBuf<int> path_nray, path_tri, path_cop, path_kind, path_near;
  DBuf<Counters> ctr;
  DBuf<unsigned long long> seg_tx;
  DBuf<uint2> cand;                    // FP32 search contenders, kCand per ray of a chunk
  DBuf<unsigned char> ncand;
  DBuf<unsigned long long> find_work;  // work counter of the running search launch
  // pinned staging of a solve's uploads
  HBuf<TxParams> h_txp;
  HBuf<int> h_rxreq;
  HBuf<double> h_rx;
  HBuf<GridBuild> h_gb;
  HBuf<unsigned char> h_res;  // a solve's results on their way to the host
  // the device pipeline as a CUDA graph: captured the second time the same
  // pipeline (pipeline_key) runs, replayed whenever it comes again.  A few
  // graphs are kept (the passes of a split batch, a serving loop's request
  // mixes alternate); the least recently used one goes first.
  struct PipelineGraph {
    std::string key;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long kernels = 0;      // kernel launches the graph holds
    unsigned long long used = 0;
  };
  std::vector<PipelineGraph> graphs;
  std::vector<std::string> seen;  // keys that ran eagerly, most recent last
  unsigned long long graph_tick = 0;
  long long pipeline_kernels = 0;  // kernels the last pipeline ran
  // capacities (grown from occupancy and on overflow)
  unsigned long long cap_nodes = 1 << 20, cap_queue = 1 << 19, cap_surv = 1 << 14;
  unsigned long long cap_corr = 1 << 16, cap_pairs = 1 << 20;
  uint32_t cap_cls = 1 << 16, cap_cop = 1 << 14, cap_dd = 1 << 14, cap_cc = 1 << 14;
  // occupancy seen per executed segment in earlier solves, used to size the
  // tables of the next solve before it runs
  // (first solve: values typical of the urban canyon, so most first solves
  // need no retry)
  double r_cls = 0.01, r_cop = 0.004, r_corr = 0.01, r_dd = 5e-4, r_surv = 5e-4, r_pairs = 0.1,
         r_cc = 0.01;
  ~Workspace() {
    for (auto& g : graphs) {
      if (g.exec) cudaGraphExecDestroy(g.exec);
      if (g.graph) cudaGraphDestroy(g.graph);
    }
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    for (auto& e : cap_ev)
      if (e) cudaEventDestroy(e);
    for (auto& e : tr_ev) cudaEventDestroy(e);
    if (join) cudaEventDestroy(join);
    if (stream) cudaStreamDestroy(stream);
    if (side) cudaStreamDestroy(side);
  }
};

// Launch shapes of the trace and capture kernels (sbr_tuning); 0 = default.
struct Tuning {
  int find_steps = 0, find_refill = 0, find_bps = 0, trace_bps = 0, capture_bps = 0;
  int chunk_log2 = 0;
  int trace_kernel = 0;  // FP64 resolution: 1 = k_trace (a ray per lane), 2 = k_trace_pool
  int graph = 0;         // pipeline as a CUDA graph on repeat: 1 (0 = default), -1 = never
  int find_tris = 0;     // FP32 search: leaf triangles per step, 1 or 2 (0 = default)
};

// A request mix's identity for the autotuner's cache: the sorted
// (level, reflections, transmissions) of its requests.
static std::string mix_key(const sbr_request* reqs, int n) {
  std::vector<long long> k;
  k.reserve(size_t(n));
  for (int i = 0; i < n; ++i)
    k.push_back((long long)reqs[i].tessellation << 40 | (long long)reqs[i].max_reflection << 20 |
                reqs[i].max_transmission);
  std::sort(k.begin(), k.end());
  std::string s;
  for (long long v : k) s += std::to_string(v) + ",";
  return s;
}

struct SceneImpl {
  HostScene host;
  // launch shapes: the scene default and autotuned choices per request mix
  std::mutex tune_mu;
  Tuning tuning;
  std::map<std::string, Tuning> tuned;
  std::vector<sbr_material> materials;
  int device = 0;
  cudaStream_t stream = nullptr;  // scene uploads
  DBuf<Node32> node32;
  DBuf<RefNode> ref;
  DBuf<Tri32> tri32;
  DBuf<Tri64> tri64;
  DBuf<Node4> snode4;
  DBuf<Tri32> stri;
  DBuf<int> srank;
  DBuf<AncBox> anc;
  DBuf<int> anc_off;
  DBuf<CorrTri> corr;
  DBuf<Tri32> corr32;
  DBuf<Material> mats;
  DBuf<int> tri_cop;     // by rank
  DBuf<int> rank_to_id;
  DevScene dev{};
  long long dev_bytes = 0;
  int n_cop = 0;
  double prep_ms[6] = {};  // sbr_scene_info prep_* in order
  // launch directions per icosahedron level (0..12), resident once built
  std::mutex dirs_mu;
  std::vector<std::unique_ptr<DBuf<double>>> dirs;
  DBuf<const double*> dir_table;  // 13 entries, allocated once
  std::mutex pool_mu;  // held while the mesh order is replaced
};

// Process-wide pool of idle workspaces per device, shared by all scenes
// (a workspace holds no scene data).
struct WorkspacePool {
  std::mutex mu;
  std::vector<std::unique_ptr<Workspace>> idle[64];
};
static WorkspacePool& ws_pool() {
  static WorkspacePool* p = new WorkspacePool();  // intentionally never destroyed
  return *p;
}

}  // namespace sbr

struct sbr_scene {
  sbr::SceneImpl impl;
};

struct sbr_result {
  std::vector<double> field;
  std::vector<double> field64;  // FP64 shadow field (field_check requests), else empty
  std::vector<double> field_bound;  // per receiver (sbr_result_field_bound)
  std::vector<sbr_path> paths;
  std::vector<int> tri, cop, kind;
  std::vector<double> points;
  sbr_counts counts{};
  sbr_timing timing{};
  std::vector<long long> segments_per_request;
  std::vector<long long> launches_per_request;
  std::vector<int> rx_per_request;
};

namespace sbr {

void pattern_fields(const sbr_pattern* p, const float** dev, int* nt, int* np, double* dt,
                    double* dp, int* device);  // sbr_pattern.cpp

static void pattern_params(const sbr_pattern* p, int scene_device, TxParams& P) {
  const float* dev = nullptr;
  int device = -1;
  pattern_fields(p, &dev, &P.pat_nt, &P.pat_np, &P.pat_dt, &P.pat_dp, &device);
  if (device != scene_device) throw std::string("the pattern was created on another device");
  P.pat = reinterpret_cast<const float4*>(dev);
}

// Runs f(b, e) over slices of [0, n) on the host's cores.
static void host_parallel(size_t n, const std::function<void(size_t, size_t)>& f) {
  const size_t T = std::max<size_t>(1, std::min<size_t>(std::thread::hardware_concurrency(), 32));
  if (n < 8192 || T == 1) {
    f(0, n);
    return;
  }
  std::vector<std::thread> pool;
  for (size_t k = 1; k < T; ++k) pool.emplace_back(f, n * k / T, n * (k + 1) / T);
  f(0, n / T);
  for (auto& t : pool) t.join();
}

static void upload_scene(SceneImpl& S) {
  const HostScene& H = S.host;
  const int nt = int(H.tris.size()), nn = int(H.nodes.size());
  std::vector<Node32> n32(nn);
  std::vector<RefNode> ref(nn);
  const double margin_m = std::ldexp(H.extent + 1.0, -14);
  host_parallel(size_t(nn), [&](size_t b, size_t e) {
    for (int i = int(b); i < int(e); ++i) {
      const HostNode& h = H.nodes[i];
      RefNode& r = ref[i];
      std::memcpy(r.bb, h.bb, sizeof r.bb);
      r.flat = 0;
      for (int a = 0; a < 6; ++a) r.fb[a] = float(h.bb[a]);
      for (int a = 0; a < 3; ++a) {
        // boxes of float vertices are floats; a non-float bound (empty box
        // sentinel) disables the FP32 decision for that node
        if (double(r.fb[a]) != h.bb[a] || double(r.fb[3 + a]) != h.bb[3 + a]) r.flat |= 8;
        if (h.bb[a] == h.bb[3 + a]) r.flat |= 1 << a;
      }
      r.c0 = h.c0;
      r.c1 = h.c1;
      r.first = h.first;
      r.count = h.count;
      r.parent = h.parent;
      Node32& m = n32[i];
      std::memset(&m, 0, sizeof m);
      if (h.c0 >= 0) {
        const int cs[2] = {h.c0, h.c1};
        for (int k = 0; k < 2; ++k) {
          const HostNode& c = H.nodes[cs[k]];
          float* lo = k == 0 ? m.lo0 : m.lo1;
          float* hi = k == 0 ? m.hi0 : m.hi1;
          for (int a = 0; a < 3; ++a) {
            // outward rounding keeps the FP32 box around the FP64 one
            lo[a] = std::nextafter(float(c.bb[a]), -INFINITY);
            hi[a] = std::nextafter(float(c.bb[3 + a]), INFINITY);
          }
          m.child[k] = c.c0 >= 0 ? cs[k] : ~cs[k];
        }
      }
    }
  });
  std::vector<Tri32> t32(nt);
  std::vector<Tri64> t64(nt);
  std::vector<int> cop(nt), r2i(nt);
  host_parallel(size_t(nt), [&](size_t b, size_t e) {
    for (int r = int(b); r < int(e); ++r) {
      const HostTri& t = H.tris[H.dfs_tris[r]];
      Tri64& d = t64[r];
      Tri32& f = t32[r];
      for (int a = 0; a < 3; ++a) {
        d.v1[a] = t.v1[a];
        d.e1[a] = t.v2[a] - t.v1[a];
        d.e2[a] = t.v3[a] - t.v1[a];
        d.n[a] = t.n[a];
        f.v1[a] = float(d.v1[a]);
        f.e1[a] = float(d.e1[a]);
        f.e2[a] = float(d.e2[a]);
      }
      f.nv1 = float(std::sqrt(d.v1[0] * d.v1[0] + d.v1[1] * d.v1[1] + d.v1[2] * d.v1[2])) * 1.0001f;
      f.ne1 = float(std::sqrt(d.e1[0] * d.e1[0] + d.e1[1] * d.e1[1] + d.e1[2] * d.e1[2])) * 1.0001f;
      f.ne2 = float(std::sqrt(d.e2[0] * d.e2[0] + d.e2[1] * d.e2[1] + d.e2[2] * d.e2[2])) * 1.0001f;
      d.id = t.id;
      d.cop = t.cop;
      d.mat = t.mat;
      d.node = -1;
      cop[r] = t.cop;
      r2i[r] = t.id;
    }
  });
  host_parallel(size_t(nn), [&](size_t b, size_t e) {
    for (int i = int(b); i < int(e); ++i)
      if (H.nodes[i].c0 < 0)
        for (int r = H.nodes[i].first; r < H.nodes[i].first + H.nodes[i].count; ++r)
          t64[r].node = i;
  });
  S.n_cop = 0;
  for (auto& t : H.tris) S.n_cop = std::max(S.n_cop, t.cop + 1);
  std::vector<Material> mats(S.materials.size());
  for (size_t i = 0; i < mats.size(); ++i)
    mats[i] = Material{S.materials[i].rel_permittivity_re, S.materials[i].rel_conductivity,
                       S.materials[i].width};
  cudaStream_t st = S.stream;
  S.node32.upload(n32.data(), n32.size(), st);
  S.ref.upload(ref.data(), ref.size(), st);
  S.tri32.upload(t32.data(), t32.size(), st);
  S.tri64.upload(t64.data(), t64.size(), st);
  S.mats.upload(mats.data(), mats.size(), st);
  {  // search BVH, collapsed to four-wide nodes
    const SearchBVH& B = H.search;
    // A node's two child slots are widened by replacing the internal child
    // with the largest box (surface area) by its two children, until four
    // slots or only leaves; the boxes are the binary tree's own.  Nodes are
    // numbered depth-first (parent first).
    struct Slot {
      float lo[3], hi[3];
      int ref;
    };
    auto area = [](const Slot& x) {
      const float dx = x.hi[0] - x.lo[0], dy = x.hi[1] - x.lo[1], dz = x.hi[2] - x.lo[2];
      return dx * dy + dy * dz + dz * dx;
    };
    std::vector<Node4> sn;
    sn.reserve(B.nodes.size());
    std::function<int(int)> build4 = [&](int b) -> int {
      Slot s[4];
      int ns = 0;
      for (int k = 0; k < 2; ++k) {
        for (int a = 0; a < 3; ++a) {
          s[ns].lo[a] = B.nodes[size_t(b)].lo[k][a];
          s[ns].hi[a] = B.nodes[size_t(b)].hi[k][a];
        }
        s[ns++].ref = B.nodes[size_t(b)].child[k];
      }
      while (ns < 4) {
        int pick = -1;
        float best = -1.0f;
        for (int i = 0; i < ns; ++i)
          if (s[i].ref >= 0 && area(s[i]) > best) {
            best = area(s[i]);
            pick = i;
          }
        if (pick < 0) break;
        const SearchNode& c = B.nodes[size_t(s[pick].ref)];
        for (int i = ns; i > pick + 1; --i) s[i] = s[i - 1];
        for (int k = 0; k < 2; ++k) {
          Slot& o = s[pick + k];
          for (int a = 0; a < 3; ++a) {
            o.lo[a] = c.lo[k][a];
            o.hi[a] = c.hi[k][a];
          }
          o.ref = c.child[k];
        }
        ++ns;
      }
      const int me = int(sn.size());
      sn.emplace_back();
      int refs[4];
      for (int i = 0; i < ns; ++i) refs[i] = s[i].ref >= 0 ? build4(s[i].ref) : s[i].ref;
      Node4& o = sn[size_t(me)];
      std::memset(&o, 0, sizeof o);
      for (int i = 0; i < 4; ++i) {
        for (int a = 0; a < 3; ++a) {
          o.lo[a][i] = i < ns ? s[i].lo[a] : INFINITY;
          o.hi[a][i] = i < ns ? s[i].hi[a] : -INFINITY;
        }
        o.child[i] = i < ns ? refs[i] : kEmptyChild;
      }
      return me;
    };
    build4(0);
    std::vector<Tri32> st32(B.order.size());
    host_parallel(B.order.size(), [&](size_t lo, size_t hi) {
      for (size_t j = lo; j < hi; ++j) st32[j] = t32[B.order[j]];
    });
    S.snode4.upload(sn.data(), sn.size(), st);
    S.stri.upload(st32.data(), st32.size(), st);
    S.srank.upload(B.order.data(), B.order.size(), st);
    S.dev.snode4 = S.snode4.p;
    S.dev.stri = S.stri.p;
    S.dev.srank = S.srank.p;
    CK(cudaStreamSynchronize(st));  // the host vectors above go out of scope
  }
  {  // every reference leaf's boxes up to the root, one run per leaf
    // (the leaf, its ancestors to the root, then an end marker), written on
    // the device from the reference nodes uploaded above
    std::vector<int> off(nn, -1);
    size_t total = 0;
    for (int i = 0; i < nn; ++i) {
      if (H.nodes[i].c0 >= 0) continue;
      off[i] = int(total);
      total += size_t(H.nodes[i].depth) + 2;
    }
    if (total > size_t(INT_MAX)) throw std::string("reference BVH too deep for the ancestor table");
    S.anc.ensure(std::max<size_t>(1, total));
    S.anc_off.upload(off.data(), off.size(), st);
    prep::k_anc_fill<<<std::max(1, std::min(4096, (nn + 255) / 256)), 256, 0, st>>>(
        S.ref.p, nn, S.anc_off.p, S.anc.p);
    CK(cudaGetLastError());
    S.dev.anc = S.anc.p;
    S.dev.anc_off = S.anc_off.p;
    CK(cudaStreamSynchronize(st));
  }
  S.tri_cop.upload(cop.data(), cop.size(), st);
  S.rank_to_id.upload(r2i.data(), r2i.size(), st);
  S.dev.node32 = S.node32.p;
  S.dev.ref = S.ref.p;
  S.dev.tri32 = S.tri32.p;
  S.dev.tri64 = S.tri64.p;
  S.dev.mats = S.mats.p;
  S.dev.rank_to_id = S.rank_to_id.p;
  S.dev.n_tri = nt;
  S.dev.n_nodes = nn;
  S.dev.n_mats = int(mats.size());
  S.dev.root_leaf = H.nodes[0].c0 < 0 ? 1 : 0;
  S.dev.box_margin = float(margin_m);
  S.dev_bytes = (long long)(n32.size() * sizeof(Node32) + ref.size() * sizeof(RefNode) +
                            t32.size() * sizeof(Tri32) + t64.size() * sizeof(Tri64) +
                            2 * nt * sizeof(int) + nt * sizeof(CorrTri) +
                            S.snode4.n * sizeof(Node4) + S.stri.n * sizeof(Tri32) +
                            S.srank.n * sizeof(int) + S.anc.n * sizeof(AncBox) +
                            S.anc_off.n * sizeof(int));
  CK(cudaStreamSynchronize(st));
}

// corr[id] = the triangle at mesh position id (what triangleMesh[id] returns).
static void upload_mesh_order(SceneImpl& S, const std::vector<int>& order) {
  const HostScene& H = S.host;
  const int nt = int(H.tris.size());
  std::vector<CorrTri> c(nt);
  std::vector<Tri32> c32(nt);
  host_parallel(size_t(nt), [&](size_t lo, size_t hi) {
    for (int i = int(lo); i < int(hi); ++i) {
      const HostTri& t = H.tris[order[i]];
      CorrTri& d = c[i];
      for (int a = 0; a < 3; ++a) {
        d.v1[a] = t.v1[a];
        d.e1[a] = t.v2[a] - t.v1[a];
        d.e2[a] = t.v3[a] - t.v1[a];
        d.n[a] = t.n[a];
      }
      std::memcpy(d.cs, t.cs, sizeof d.cs);
      d.mat = t.mat;
      d.pad = 0;
    }
    for (int i = int(lo); i < int(hi); ++i) {
      Tri32& f = c32[i];
      for (int a = 0; a < 3; ++a) {
        f.v1[a] = float(c[i].v1[a]);
        f.e1[a] = float(c[i].e1[a]);
        f.e2[a] = float(c[i].e2[a]);
      }
      auto n3 = [](const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); };
      f.nv1 = float(n3(c[i].v1)) * 1.0001f;
      f.ne1 = float(n3(c[i].e1)) * 1.0001f;
      f.ne2 = float(n3(c[i].e2)) * 1.0001f;
    }
  });
  S.corr.upload(c.data(), c.size(), S.stream);
  S.corr32.upload(c32.data(), c32.size(), S.stream);
  S.dev.corr = S.corr.p;
  S.dev.corr32 = S.corr32.p;
  CK(cudaStreamSynchronize(S.stream));
}

static void ensure_dirs(SceneImpl& S, int level) {
  if (level < 0 || level > 12) throw std::string("tessellation level must be 0..12");
  std::lock_guard<std::mutex> lock(S.dirs_mu);
  if (S.dirs.size() < 13) S.dirs.resize(13);
  if (!S.dir_table.p) {
    S.dir_table.ensure(13);
    CK(cudaMemset(S.dir_table.p, 0, 13 * sizeof(const double*)));
  }
  if (!S.dirs[level]) {
    std::vector<double> d;
    icosphere(level, d);
    auto b = std::make_unique<DBuf<double>>();
    b->ensure(d.size());
    CK(cudaMemcpy(b->p, d.data(), d.size() * sizeof(double), cudaMemcpyHostToDevice));
    const double* ptr = b->p;
    CK(cudaMemcpy(S.dir_table.p + level, &ptr, sizeof ptr, cudaMemcpyHostToDevice));
    S.dirs[level] = std::move(b);
  }
}

static long long n_launch_of(int level) { return 10LL * (1LL << (2 * level)) + 2; }

// Bounds of one launch's ray tree (RTSolver.cpp:186-221): nodes with r
// reflections and t transmissions exist for r <= R, t <= T, C(r+t, t) of each.
static double tree_nodes(int R, int T) {
  double n = 0;
  for (int r = 0; r <= R; ++r) {
    double c = 1;  // C(r + t, t), t = 0
    for (int t = 0; t <= T; ++t) {
      n += c;
      c = c * double(r + t + 1) / double(t + 1);
    }
  }
  return n;
}
// widest bounce depth: nodes with r + t = d
static double tree_width(int R, int T) {
  double w = 1;
  for (int d = 0; d <= R + T; ++d) {
    double n = 0, c = 1;  // C(d, t)
    for (int t = 0; t <= std::min(d, T); ++t) {
      if (d - t <= R) n += c;
      c = c * double(d - t) / double(t + 1);
    }
    w = std::max(w, n);
  }
  return w;
}
// Device bytes a request may need (node records at the tree bound, queues,
// receivers): used to split batches into passes and to size buffers.
double request_bytes(const sbr_request& q) {
  const double L = double(n_launch_of(std::min(std::max(q.tessellation, 0), 12)));
  const int R = std::max(q.max_reflection, 0), T = std::max(q.max_transmission, 0);
  return L * tree_nodes(R, T) * (sizeof(NodeHot) + sizeof(NodeCold)) +
         L * tree_width(R, T) * 2 * sizeof(RayRec) + double(q.n_rx) * 256.0;
}

// SM count of the current device, queried once per device.
static int device_sms() {
  static std::atomic<int> cache[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  std::atomic<int>& c = cache[dev & 63];
  int n = c.load(std::memory_order_relaxed);
  if (!n) {
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    n = std::max(1, n);
    c.store(n, std::memory_order_relaxed);
  }
  return n;
}

// Resident blocks per SM of a kernel at a block size, queried once per kernel.
template <class K>
static int blocks_per_sm(K kernel, int block) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
  return std::max(1, per_sm);
}

// Persistent grids: `want` resident blocks per SM (0 = as many as fit),
// never more than fit, so every block of a persistent kernel is resident.
static int persistent_grid(int fit, int want) {
  return device_sms() * (want > 0 ? std::min(want, fit) : fit);
}

// Blocks of each persistent kernel that fit on one SM.
static int find_fit() {
  static const int per_sm = blocks_per_sm(k_find, 128);
  return per_sm;
}
static int trace_fit() {
  static const int per_sm = blocks_per_sm(k_trace, 128);
  return per_sm;
}
// k_trace_pool keeps its rays in dynamic shared memory (one PoolSlots per warp).
constexpr size_t kPoolSmem = sizeof(PoolSlots) * kPoolWarps;
static int pool_fit() {
  static const int per_sm = [] {
    cudaFuncSetAttribute(k_trace_pool, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kPoolSmem));
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_trace_pool, 32 * kPoolWarps, kPoolSmem);
    return std::max(1, n);
  }();
  return per_sm;
}
static int capture_fit() {
  static const int per_sm = blocks_per_sm(k_capture_fast, 32 * kCapWarps);
  return per_sm;
}

// FP32 search.
static int find_grid(const Tuning& t) { return persistent_grid(find_fit(), t.find_bps); }

// FP64 resolution.
static int trace_grid(const Tuning& t) { return persistent_grid(trace_fit(), t.trace_bps); }

// Capture: the work counter balances the blocks.
static int capture_grid(const Tuning& t) { return persistent_grid(capture_fit(), t.capture_bps); }

// The FP64 resolution kernel solves use unless tuned otherwise.
constexpr int kDefaultTraceKernel = 1;
constexpr int kFindTris = 2;  // leaf triangles per FP32 search step
// Rays per search/resolution launch pair: 2^25 holds a level-9 launch's
// widest depth at six reflections and one transmission (7 rays per launch)
// in one pair; the chunk never exceeds the depth's queue capacity.
constexpr int kTraceChunkLog2 = 25;

// A tuning with every default filled in (the shapes a solve really uses).
static Tuning resolved(Tuning t) {
  if (t.find_steps <= 0) t.find_steps = kFindSteps;
  if (t.find_refill <= 0) t.find_refill = kFindRefill;
  t.find_refill = std::min(t.find_refill, 32);
  t.find_bps = t.find_bps > 0 ? std::min(t.find_bps, find_fit()) : find_fit();
  t.trace_bps = t.trace_bps > 0 ? std::min(t.trace_bps, trace_fit()) : trace_fit();
  t.capture_bps = t.capture_bps > 0 ? std::min(t.capture_bps, capture_fit()) : capture_fit();
  if (t.chunk_log2 <= 0) t.chunk_log2 = kTraceChunkLog2;
  t.chunk_log2 = std::min(std::max(t.chunk_log2, 16), 26);
  if (t.trace_kernel <= 0 || t.trace_kernel > 2) t.trace_kernel = kDefaultTraceKernel;
  t.graph = t.graph < 0 ? -1 : 1;
  if (t.find_tris <= 0 || t.find_tris > 2) t.find_tris = kFindTris;
  return t;
}

static int grid_for(long long n, int block) {
  const long long g = (n + block - 1) / block;
  return int(std::max<long long>(1, std::min<long long>(g, (long long)device_sms() * 32)));
}

// Blocks to give every one of n items its own thread (no cap: for kernels
// without a grid-stride loop).
static int grid_all(long long n, int block) {
  return int(std::max<long long>(1, (n + block - 1) / block));
}

// ------------------------------------------------------------ scene preparation on the device

// What the device builds of a scene (sbr_prep.cuh): per triangle (file
// order) the coplanar group, frame rows, box and box centre; the search BVH
// over triangle ids, in the host build's node numbering.
struct DeviceTables {
  std::vector<int> cop;
  std::vector<double> cs, bb, center;
  SearchBVH search;
  int degenerate = 0;
  // the reference BVH: nodes depth-first, leaf triangle order, the caller's
  // triangle order after BVH::ConstructBVH
  std::vector<HostNode> nodes;
  std::vector<int> dfs_tris, mesh_order;
  int max_depth = 0;
  double tables_ms = 0, search_ms = 0, ref_ms = 0;  // wall time of each part
};

template <class T>
static void swap_buf(DBuf<T>& a, DBuf<T>& b) {
  std::swap(a.p, b.p);
  std::swap(a.n, b.n);
}

// Exclusive scan of in[0, n) into out[0, n], out[n] = total, over many
// blocks; sums: scratch of at least n / kScanTile + 1 ints.
static void scan_exclusive(const int* in, int* out, int n, int* sums, cudaStream_t st) {
  const int nb = std::max(1, (n + kScanTile - 1) / kScanTile);
  k_tile_sums<<<nb, kScanThreads, 0, st>>>(in, n, sums);
  k_sums_scan<<<1, 1024, 0, st>>>(sums, nb, out + n);
  k_tile_scan<<<nb, kScanThreads, 0, st>>>(in, n, sums, out);
}

// Stable LSD radix sort of perm by word[perm[i]], one varying bit per pass.
static void sort_perm_by(DBuf<int>& perm, DBuf<int>& tmp, DBuf<int>& flags, DBuf<int>& scan,
                         DBuf<int>& sums, DBuf<unsigned>& vb, const uint32_t* word, int n,
                         cudaStream_t st) {
  if (n < 2) return;
  CK(cudaMemsetAsync(vb.p, 0, sizeof(unsigned), st));
  prep::k_varying_bits<<<grid_for(n, 256), 256, 0, st>>>(word, n, vb.p);
  unsigned bits = 0;
  CK(cudaMemcpyAsync(&bits, vb.p, sizeof bits, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  for (int b = 0; b < 32; ++b) {
    if (!((bits >> b) & 1u)) continue;
    prep::k_bit_flags<<<grid_for(n, 256), 256, 0, st>>>(word, perm.p, n, b, flags.p);
    scan_exclusive(flags.p, scan.p, n, sums.p, st);
    prep::k_bit_scatter<<<grid_for(n, 256), 256, 0, st>>>(word, perm.p, n, b, scan.p, tmp.p);
    swap_buf(perm, tmp);
  }
  CK(cudaGetLastError());
}

// The reference BVH on the device (sbr_refbvh.cuh), one tree level at a
// time: each level's nodes get their box, three exact sorts with a surface
// area sweep each, and a final sort along the chosen axis; the host then
// numbers the nodes depth-first as the host build does.  v: the device
// copy of the vertices (9 floats per triangle).
struct RefSort {
  DBuf<double> key;
  DBuf<int> idx, lpos, rpos, tile_seg, cnt_l, cnt_r, off_l, off_r;
  DBuf<int2> totals;
  DBuf<refbvh::SortSeg> big, big_next, small, tiny, heap;
  DBuf<int> ctl;
  int sms = 1;
  int small_cap = 0;  // entries of the small-segment list (both ends)
};

static int read_ctl(RefSort& R, int* h, cudaStream_t st) {
  CK(cudaMemcpyAsync(h, R.ctl.p, sizeof(int) * refbvh::kCtlWords, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (h[refbvh::kError])
    throw std::string("device reference BVH: sort invariant violated (code ") +
        std::to_string(h[refbvh::kError]) + ")";
  return 0;
}

// Sorts the objects of the listed nodes (of their split nodes when `best`
// is given) by key, in the reference sort's order; idx receives the
// permutation.
static void ref_sort(RefSort& R, const refbvh::RNode* nodes, const int* active, int m,
                     const refbvh::NodeBest* best, cudaStream_t st) {
  using namespace refbvh;
  int h[kCtlWords];
  CK(cudaMemsetAsync(R.ctl.p, 0, sizeof(int) * kNodes, st));  // list counters only
  k_file_nodes<<<grid_all(m, 128), 128, 0, st>>>(nodes, active, m, best, R.big.p, R.small.p,
                                                 R.small_cap, R.tiny.p, R.heap.p, R.ctl.p);
  CK(cudaGetLastError());
  read_ctl(R, h, st);
  int n_big = h[kBig], n_tiles = h[kTiles];
  for (int round = 0; n_big > 0; ++round) {
    if (round > 64) throw std::string("device reference BVH: too many partition rounds");
    k_tile_map<<<n_big, 256, 0, st>>>(R.big.p, R.ctl.p + kBig, R.tile_seg.p);
    k_pivot<<<grid_all(n_big, 128), 128, 0, st>>>(R.big.p, n_big, R.key.p, R.idx.p);
    k_count<<<n_tiles, kTileThreads, 0, st>>>(R.big.p, R.tile_seg.p, R.key.p, R.cnt_l.p,
                                              R.cnt_r.p);
    k_tile_offsets<<<grid_all(n_big, 128), 128, 0, st>>>(R.big.p, n_big, R.cnt_l.p, R.cnt_r.p,
                                                         R.off_l.p, R.off_r.p, R.totals.p);
    k_stops<<<n_tiles, kTileThreads, 0, st>>>(R.big.p, R.tile_seg.p, R.key.p, R.off_l.p,
                                              R.off_r.p, R.totals.p, R.lpos.p, R.rpos.p);
    k_exchange<<<n_tiles, kTileThreads, 0, st>>>(R.big.p, R.tile_seg.p, R.totals.p, R.lpos.p,
                                                 R.rpos.p, R.key.p, R.idx.p);
    CK(cudaMemsetAsync(R.ctl.p + kBigNext, 0, sizeof(int), st));
    CK(cudaMemsetAsync(R.ctl.p + kTilesNext, 0, sizeof(int), st));
    k_cut<<<grid_all(n_big, 128), 128, 0, st>>>(R.big.p, n_big, R.totals.p, R.lpos.p, R.rpos.p,
                                                R.big_next.p, R.small.p, R.small_cap, R.tiny.p,
                                                R.heap.p, R.ctl.p);
    CK(cudaGetLastError());
    read_ctl(R, h, st);
    n_big = h[kBigNext];
    n_tiles = h[kTilesNext];
    CK(cudaMemcpyAsync(R.ctl.p + kBig, R.ctl.p + kBigNext, sizeof(int), cudaMemcpyDeviceToDevice,
                       st));
    std::swap(R.big.p, R.big_next.p);
    std::swap(R.big.n, R.big_next.n);
  }
  if (h[kSmall])
    k_small<kSmallMax><<<std::min(h[kSmall], R.sms * 8), 32, small_smem<kSmallMax>(), st>>>(
        R.small.p, R.ctl.p + kSmall, 0, R.key.p, R.idx.p, R.ctl.p);
  if (h[kShort])
    k_small<kShortMax><<<std::min(h[kShort], R.sms * 32), 32, small_smem<kShortMax>(), st>>>(
        R.small.p, R.ctl.p + kShort, R.small_cap, R.key.p, R.idx.p, R.ctl.p);
  if (h[kSmall] + h[kShort] > R.small_cap)
    throw std::string("device reference BVH: small segment list overflow");
  if (h[kTiny])
    k_tiny<<<grid_all(h[kTiny], 128), 128, 0, st>>>(R.tiny.p, R.ctl.p + kTiny, R.key.p, R.idx.p);
  if (h[kHeap])
    k_heap<<<grid_all(h[kHeap], 64), 64, 0, st>>>(R.heap.p, R.ctl.p + kHeap, R.key.p, R.idx.p);
  CK(cudaGetLastError());
}

static void device_ref_bvh(const float* v, int nt, cudaStream_t st, DeviceTables& T) {
  using namespace refbvh;
  const int n = nt;
  const size_t nz = size_t(std::max(1, n));
  DBuf<float4> lo, hi, lo2, hi2;
  lo.ensure(nz);
  hi.ensure(nz);
  lo2.ensure(nz);
  hi2.ensure(nz);
  k_boxes<<<grid_all(n, 256), 256, 0, st>>>(v, nt, lo.p, hi.p);
  RefSort R;
  R.sms = device_sms();
  R.key.ensure(nz);
  R.idx.ensure(nz);
  R.lpos.ensure(nz);
  R.rpos.ensure(nz);
  const size_t tiles = nz / (kTile / 2) + 16, lists = nz / 2 + 16;
  R.tile_seg.ensure(tiles);
  R.cnt_l.ensure(tiles);
  R.cnt_r.ensure(tiles);
  R.off_l.ensure(tiles);
  R.off_r.ensure(tiles);
  R.totals.ensure(nz / kSmallMax + 16);
  R.big.ensure(nz / kSmallMax + 16);
  R.big_next.ensure(nz / kSmallMax + 16);
  R.small.ensure(lists);
  R.small_cap = int(lists);

  R.tiny.ensure(lists);
  R.heap.ensure(lists);
  R.ctl.ensure(kCtlWords);
  CK(cudaMemsetAsync(R.ctl.p, 0, sizeof(int) * kCtlWords, st));
  DBuf<RNode> nodes;
  nodes.ensure(2 * nz + 1);
  DBuf<NodeBest> best;
  best.ensure(nz);
  const size_t tcap = nz + nz / kWarpTile + 16;  // warp tiles of a level
  DBuf<int2> node_tiles;
  node_tiles.ensure(nz);
  DBuf<int> tile_node;
  tile_node.ensure(tcap);
  DBuf<ExactBox> tbox;
  tbox.ensure(tcap);
  DBuf<BoxF> tagg, pre, post;
  tagg.ensure(tcap);
  pre.ensure(tcap);
  post.ensure(tcap);
  DBuf<TileBest> tbest;
  tbest.ensure(tcap);
  DBuf<double> sa_root;
  sa_root.ensure(nz);
  DBuf<int> tiled, small_nodes;  // a level's nodes with tiles / of kNodeSmall or fewer objects
  tiled.ensure(nz);
  small_nodes.ensure(nz);
  DBuf<int> node_of, active, next, ids, mesh;
  node_of.ensure(nz);
  active.ensure(nz);
  next.ensure(nz);
  ids.ensure(nz);
  mesh.ensure(nz);
  {
    RNode root{};
    root.f = 0;
    root.l = n;
    root.c0 = root.c1 = -1;
    nodes.upload(&root, 1, st);
    const int zero = 0, one = 1;
    active.upload(&zero, 1, st);
    CK(cudaMemcpyAsync(R.ctl.p + kNodes, &one, sizeof(int), cudaMemcpyHostToDevice, st));
  }
  int m = 1;
  for (int level = 0; m > 0; ++level) {
    if (level > 4096) throw std::string("device reference BVH: too many levels");
    CK(cudaMemsetAsync(node_of.p, 0xff, sizeof(int) * nz, st));
    CK(cudaMemsetAsync(R.ctl.p + kSweepTiles, 0, 3 * sizeof(int), st));  // tiles, both lists
    k_level_tiles<<<grid_all(m, 128), 128, 0, st>>>(nodes.p, active.p, m, node_tiles.p,
                                                    tile_node.p, tiled.p, small_nodes.p, R.ctl.p);
    int hl[kCtlWords];
    read_ctl(R, hl, st);
    const int n_tiles = hl[kSweepTiles], n_tiled = hl[kTiledNodes], n_small = hl[kSmallNodes];
    const long long tile_threads = 32LL * n_tiles, node_threads = 32LL * n_tiled;
    if (n_tiles) {
      k_tile_exact_box<<<grid_all(tile_threads, 256), 256, 0, st>>>(
          nodes.p, active.p, node_tiles.p, tile_node.p, n_tiles, lo.p, hi.p, node_of.p, tbox.p);
      k_node_box<<<grid_all(node_threads, 256), 256, 0, st>>>(
          nodes.p, active.p, tiled.p, n_tiled, node_tiles.p, tbox.p, sa_root.p, best.p);
    }
    if (n_small)
      k_small_node_box<<<grid_all(n_small, 128), 128, 0, st>>>(nodes.p, active.p, small_nodes.p,
                                                               n_small, lo.p, hi.p, node_of.p,
                                                               sa_root.p, best.p);
    for (int axis = 0; axis <= 3; ++axis) {  // x, y, z, then the chosen axis
      const NodeBest* b = axis == 3 ? best.p : nullptr;
      k_keys<<<grid_all(n, 256), 256, 0, st>>>(lo.p, hi.p, node_of.p, b, axis, n, R.key.p,
                                               R.idx.p);
      ref_sort(R, nodes.p, active.p, m, b, st);
      k_gather<<<grid_all(n, 256), 256, 0, st>>>(lo.p, hi.p, R.idx.p, n, lo2.p, hi2.p);
      std::swap(lo.p, lo2.p);
      std::swap(hi.p, hi2.p);
      if (axis < 3 && n_tiles) {  // the surface area sweep over this order
        k_tile_boxes<<<grid_all(tile_threads, 256), 256, 0, st>>>(
            nodes.p, active.p, node_tiles.p, tile_node.p, n_tiles, lo.p, hi.p, tagg.p);
        k_tile_carries<<<grid_all(node_threads, 256), 256, 0, st>>>(tiled.p, n_tiled,
                                                                    node_tiles.p, tagg.p, pre.p,
                                                                    post.p);
        k_tile_sweep<<<grid_all(tile_threads, 256), 256, 0, st>>>(
            nodes.p, active.p, node_tiles.p, tile_node.p, n_tiles, lo.p, hi.p, pre.p, post.p,
            sa_root.p, tbest.p);
        k_node_best<<<grid_all(node_threads, 256), 256, 0, st>>>(tiled.p, n_tiled, node_tiles.p,
                                                                 tbest.p, axis, best.p);
      }
      if (axis < 3 && n_small)
        k_small_node_sweep<<<grid_all(n_small, 128), 128, 0, st>>>(
            nodes.p, active.p, small_nodes.p, n_small, lo.p, hi.p, sa_root.p, axis, best.p);
    }
    if (level == 0) k_ids<<<grid_all(n, 256), 256, 0, st>>>(lo.p, n, mesh.p);
    CK(cudaMemsetAsync(R.ctl.p + kActiveNext, 0, sizeof(int), st));
    k_children<<<grid_all(m, 128), 128, 0, st>>>(nodes.p, active.p, m, best.p, next.p, R.ctl.p);
    CK(cudaGetLastError());
    int h[kCtlWords];
    read_ctl(R, h, st);
    m = h[kActiveNext];
    std::swap(active.p, next.p);
  }
  int h[kCtlWords];
  read_ctl(R, h, st);
  const int n_nodes = h[kNodes];
  k_ids<<<grid_all(n, 256), 256, 0, st>>>(lo.p, n, ids.p);
  std::vector<RNode> rn(static_cast<size_t>(n_nodes));
  std::vector<int> order(nz);
  T.mesh_order.resize(nz);
  CK(cudaMemcpyAsync(rn.data(), nodes.p, sizeof(RNode) * n_nodes, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(order.data(), ids.p, sizeof(int) * nz, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(T.mesh_order.data(), mesh.p, sizeof(int) * nz, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  T.mesh_order.resize(size_t(n));
  // depth-first numbering, children[0] first (sbr_host.cpp prepare_scene)
  T.nodes.clear();
  T.nodes.reserve(size_t(n_nodes));
  T.dfs_tris.clear();
  T.dfs_tris.reserve(size_t(n));
  T.max_depth = 0;
  struct Item {
    int b, parent, depth, which;
  };
  std::vector<Item> stack{{0, -1, 0, 0}};
  while (!stack.empty()) {
    const Item it = stack.back();
    stack.pop_back();
    const int me = int(T.nodes.size());
    T.nodes.emplace_back();
    HostNode& hn = T.nodes.back();
    const RNode& r = rn[size_t(it.b)];
    std::memcpy(hn.bb, r.bb, sizeof hn.bb);
    hn.parent = it.parent;
    hn.depth = it.depth;
    T.max_depth = std::max(T.max_depth, it.depth);
    if (it.parent >= 0) {
      if (it.which == 0) T.nodes[size_t(it.parent)].c0 = me;
      else T.nodes[size_t(it.parent)].c1 = me;
    }
    if (r.c0 < 0) {
      hn.first = int(T.dfs_tris.size());
      hn.count = r.l - r.f;
      T.dfs_tris.insert(T.dfs_tris.end(), order.begin() + r.f, order.begin() + r.l);
    } else {
      stack.push_back({r.c1, me, it.depth + 1, 1});
      stack.push_back({r.c0, me, it.depth + 1, 0});
    }
  }
}

// Builds the tables on the current device, on stream st.  v: 9 floats per
// triangle, nrm: 3.
static void device_prepare(const float* v_host, const float* n_host, int nt, cudaStream_t st,
                           DeviceTables& T) {
  auto ms_since = [](std::chrono::steady_clock::time_point a) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
  };
  auto t0 = std::chrono::steady_clock::now();
  const int nv = 3 * nt, ne = 3 * nt;
  DBuf<float> v, nrm;
  v.upload(v_host, 9 * size_t(nt), st);
  nrm.upload(n_host, 3 * size_t(nt), st);
  DBuf<uint32_t> wx, wy, wz;
  DBuf<int> perm, tmp, flags, scan, uid, parent, misc, sums;
  DBuf<unsigned> vb;
  const size_t big = size_t(std::max(nv, ne));
  wx.ensure(big);
  wy.ensure(big);
  wz.ensure(big);
  perm.ensure(big);
  tmp.ensure(big);
  flags.ensure(big);
  scan.ensure(big + 1);
  sums.ensure(big / kScanTile + 2);
  uid.ensure(nv);
  parent.ensure(nt);
  misc.ensure(4);
  vb.ensure(1);
  // -- vertex merge: sort the vertices by (x, y, z) bits, number the runs
  prep::k_vertex_words<<<grid_for(nv, 256), 256, 0, st>>>(v.p, nv, wx.p, wy.p, wz.p, perm.p);
  sort_perm_by(perm, tmp, flags, scan, sums, vb, wz.p, nv, st);
  sort_perm_by(perm, tmp, flags, scan, sums, vb, wy.p, nv, st);
  sort_perm_by(perm, tmp, flags, scan, sums, vb, wx.p, nv, st);
  prep::k_run_starts<<<grid_for(nv, 256), 256, 0, st>>>(wx.p, wy.p, wz.p, perm.p, nv, flags.p);
  scan_exclusive(flags.p, scan.p, nv, sums.p, st);
  prep::k_vertex_ids<<<grid_for(nv, 256), 256, 0, st>>>(perm.p, flags.p, scan.p, nv, uid.p);
  // -- edges of merged vertices, grouped by sorting; coplanar groups by
  // hooking roots until no pair of an edge's triangles has two roots
  CK(cudaMemsetAsync(misc.p, 0, 4 * sizeof(int), st));
  prep::k_edges<<<grid_for(nt, 256), 256, 0, st>>>(uid.p, nt, wx.p, wy.p, perm.p, misc.p);
  sort_perm_by(perm, tmp, flags, scan, sums, vb, wy.p, ne, st);  // larger id first (LSD)
  sort_perm_by(perm, tmp, flags, scan, sums, vb, wx.p, ne, st);
  prep::k_run_starts<<<grid_for(ne, 256), 256, 0, st>>>(wx.p, wy.p, nullptr, perm.p, ne, flags.p);
  {
    std::vector<int> id(nt);
    for (int t = 0; t < nt; ++t) id[t] = t;
    parent.upload(id.data(), id.size(), st);
  }
  for (int round = 0;; ++round) {
    if (round > 200) throw std::string("device coplanar grouping did not converge");
    CK(cudaMemsetAsync(misc.p + 1, 0, sizeof(int), st));
    prep::k_hook<<<grid_for(ne, 256), 256, 0, st>>>(wx.p, wy.p, perm.p, flags.p, ne, nrm.p,
                                                    parent.p, misc.p + 1);
    prep::k_compress<<<grid_for(nt, 256), 256, 0, st>>>(parent.p, nt, nullptr);
    int changed = 0;
    CK(cudaMemcpyAsync(&changed, misc.p + 1, sizeof changed, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (!changed) break;
  }
  prep::k_compress<<<grid_for(nt, 256), 256, 0, st>>>(parent.p, nt, tmp.p);
  scan_exclusive(tmp.p, scan.p, nt, sums.p, st);
  DBuf<int> cop;
  cop.ensure(nt);
  prep::k_group_ids<<<grid_for(nt, 256), 256, 0, st>>>(parent.p, scan.p, nt, cop.p);
  // -- frames and boxes
  DBuf<double> cs, bb, center;
  cs.ensure(9 * size_t(nt));
  bb.ensure(6 * size_t(nt));
  center.ensure(3 * size_t(nt));
  prep::k_frames<<<grid_for(nt, 128), 128, 0, st>>>(v.p, nrm.p, nt, cs.p, bb.p, center.p);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  T.tables_ms = ms_since(t0);
  // -- the reference BVH
  t0 = std::chrono::steady_clock::now();
  device_ref_bvh(v.p, nt, st, T);
  T.ref_ms = ms_since(t0);
  t0 = std::chrono::steady_clock::now();
  // -- search BVH, one level of nodes at a time
  DBuf<float> blo, bhi, cen;
  blo.ensure(3 * size_t(nt));
  bhi.ensure(3 * size_t(nt));
  cen.ensure(3 * size_t(nt));
  DBuf<int> ord, otmp;
  ord.ensure(nt);
  otmp.ensure(nt);
  prep::k_tri_boxes<<<grid_for(nt, 256), 256, 0, st>>>(v.p, nt, blo.p, bhi.p, cen.p, ord.p);
  DBuf<prep::Seg> segs, next;
  DBuf<prep::SegPlan> plans;
  DBuf<prep::BNode> nodes;
  const size_t max_nodes = size_t(nt) + 1;
  segs.ensure(max_nodes * 2 + 2);
  next.ensure(max_nodes * 2 + 2);
  plans.ensure(max_nodes * 2 + 2);
  nodes.ensure(max_nodes);
  DBuf<int> ctl;  // [0] nodes, [1] next segments, [2] max depth, [3] root ref, [4] median too big
  ctl.ensure(8);
  DBuf<float> root_box;
  root_box.ensure(6);
  CK(cudaMemsetAsync(ctl.p, 0, 8 * sizeof(int), st));
  {
    const prep::Seg root{0, nt, 1, -1, 0};
    segs.upload(&root, 1, st);
  }
  int n_segs = 1;
  for (int level = 0; n_segs > 0; ++level) {
    if (level > 200) throw std::string("device search BVH deeper than 200 levels");
    prep::k_plan<<<n_segs, 256, 0, st>>>(segs.p, n_segs, ord.p, blo.p, bhi.p, cen.p, nodes.p,
                                         ctl.p, plans.p, ctl.p + 2, ctl.p + 3, root_box.p);
    prep::k_partition<<<n_segs, 256, 0, st>>>(segs.p, n_segs, plans.p, ord.p, otmp.p, cen.p);
    prep::k_median<<<n_segs, 256, 0, st>>>(segs.p, n_segs, plans.p, ord.p, otmp.p, cen.p,
                                           ctl.p + 4);
    CK(cudaMemsetAsync(ctl.p + 1, 0, sizeof(int), st));
    prep::k_children<<<grid_for(n_segs, 256), 256, 0, st>>>(segs.p, n_segs, plans.p, next.p,
                                                            ctl.p + 1);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(&n_segs, ctl.p + 1, sizeof n_segs, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    swap_buf(segs, next);
  }
  int c[8];
  CK(cudaMemcpyAsync(c, ctl.p, sizeof c, cudaMemcpyDeviceToHost, st));
  T.cop.resize(nt);
  T.cs.resize(9 * size_t(nt));
  T.bb.resize(6 * size_t(nt));
  T.center.resize(3 * size_t(nt));
  CK(cudaMemcpyAsync(T.cop.data(), cop.p, sizeof(int) * nt, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(T.cs.data(), cs.p, sizeof(double) * T.cs.size(), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(T.bb.data(), bb.p, sizeof(double) * T.bb.size(), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(T.center.data(), center.p, sizeof(double) * T.center.size(),
                     cudaMemcpyDeviceToHost, st));
  float rb[6];
  CK(cudaMemcpyAsync(rb, root_box.p, sizeof rb, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  CK(cudaMemcpy(&T.degenerate, misc.p, sizeof(int), cudaMemcpyDeviceToHost));
  T.search_ms = ms_since(t0);
  if (c[4]) throw std::string("device search BVH: a median split of more than 8192 triangles");
  const int n_nodes = c[0];
  std::vector<prep::BNode> bn(size_t(std::max(1, n_nodes)));
  if (n_nodes)
    CK(cudaMemcpy(bn.data(), nodes.p, sizeof(prep::BNode) * n_nodes, cudaMemcpyDeviceToHost));
  T.search.order.resize(nt);
  CK(cudaMemcpy(T.search.order.data(), ord.p, sizeof(int) * nt, cudaMemcpyDeviceToHost));
  T.search.max_depth = c[2];
  // depth-first numbering (node 0 = a copy of the root), children[0] first
  T.search.nodes.assign(size_t(n_nodes) + 1, SearchNode{});
  const int root_ref = c[3];
  if (root_ref >= 0) {
    std::vector<int> dfs(size_t(n_nodes), -1);
    std::vector<int> stack{root_ref};
    int id = 1;
    while (!stack.empty()) {
      const int b = stack.back();
      stack.pop_back();
      dfs[size_t(b)] = id++;
      if (bn[size_t(b)].child[1] >= 0) stack.push_back(bn[size_t(b)].child[1]);
      if (bn[size_t(b)].child[0] >= 0) stack.push_back(bn[size_t(b)].child[0]);
    }
    for (int b = 0; b < n_nodes; ++b) {
      SearchNode& o = T.search.nodes[size_t(dfs[size_t(b)])];
      for (int k = 0; k < 2; ++k) {
        for (int a = 0; a < 3; ++a) {
          o.lo[k][a] = bn[size_t(b)].lo[k][a];
          o.hi[k][a] = bn[size_t(b)].hi[k][a];
        }
        const int ch = bn[size_t(b)].child[k];
        o.child[k] = ch >= 0 ? dfs[size_t(ch)] : ch;
      }
    }
    T.search.nodes[0] = T.search.nodes[1];
  } else {  // the whole scene is one leaf
    SearchNode& o = T.search.nodes[0];
    for (int a = 0; a < 3; ++a) {
      o.lo[0][a] = o.lo[1][a] = rb[a];
      o.hi[0][a] = o.hi[1][a] = rb[3 + a];
    }
    o.child[0] = root_ref;
    o.child[1] = ~0;
  }
}

static FieldConsts field_consts() {
  // Constants.h:6-23 evaluated the way the reference evaluates them (EIGEN_PI
  // is a long double literal).
  const long double piL = 3.141592653589793238462643383279502884197169399375105820974944592307816406L;
  const double c = 2.99792458e8;
  const double u0 = 4 * piL * 1e-7;
  FieldConsts K;
  K.e0 = 1.0 / (u0 * c * c);
  K.eta0 = u0 * c;
  K.pi_hi = double(piL);
  K.pi_lo = double(piL - (long double)K.pi_hi);
  return K;
}

// Everything the recorded pipeline's operations depend on besides the
// contents of the staged uploads: the request structure (levels, depths,
// receiver counts and offsets, field precisions, device receiver pointers),
// the capacities, every buffer and scene pointer, the launch shapes and the
// solve's flags.  Two solves with the same key run the same operations.
static std::string pipeline_key(const SceneImpl& S, const Workspace& W, const sbr_request* reqs,
                                const std::vector<TxParams>& tp, int n_req, int rx_total,
                                long long launches, int max_depth, size_t cell_cap,
                                long long chunk, const Tuning& tu, int stage_counts,
                                bool field_check) {
  std::string k;
  auto put = [&k](const void* v, size_t n) { k.append(static_cast<const char*>(v), n); };
  auto put_v = [&put](auto v) { put(&v, sizeof v); };
  put(&S.dev, sizeof S.dev);
  put_v(n_req);
  put_v(rx_total);
  put_v(launches);
  put_v(max_depth);
  put_v(cell_cap);
  put_v(chunk);
  put_v(stage_counts);
  put_v(field_check);
  const Tuning t = resolved(tu);
  put(&t, sizeof t);
  for (int r = 0; r < n_req; ++r) {
    put_v(tp[r].rx_first);
    put_v(tp[r].n_rx);
    put_v(tp[r].n_launch);
    put_v(tp[r].level);
    put_v(tp[r].R);
    put_v(tp[r].T);
    put_v(tp[r].precision);
    put_v(reqs[r].rx_on_device ? reqs[r].rx : nullptr);
  }
  const unsigned long long caps[9] = {W.cap_nodes, W.cap_queue, W.cap_cls, W.cap_cop, W.cap_dd,
                                      W.cap_cc,    W.cap_corr,  W.cap_surv, W.cap_pairs};
  put(caps, sizeof caps);
  const void* ptrs[] = {W.txp.p, W.rx.p, W.rx_req.p, W.rx_bad.p, W.path_bound.p, W.field_bound.p,
                        W.rx_flag.p, W.fstat.p, W.gb.p, W.grids.p, W.cell_base.p, W.cell_counts.p,
                        W.cell_starts.p, W.cell_cursor.p, W.rx32.p, W.q0.p, W.q1.p, W.ray32.p,
                        W.nodes.p, W.nodes_cold.p, W.cls_keys.p, W.cop_keys.p, W.dd_keys.p,
                        W.dd_rank.p, W.cc_keys.p, W.cls_list.p, W.cc_val.p, W.cls_info.p,
                        W.cls_cap.p, W.corr_list.p, W.pairs.p, W.direct_ok.p, W.surv.p,
                        W.s_counts.p, W.s_starts.p, W.s_cursor.p, W.s_order.p, W.path_field.p,
                        W.path_pts.p, W.field.p, W.seg.p, W.path_mat.p, W.path_field64.p,
                        W.field64.p, W.path_nray.p, W.path_tri.p, W.path_cop.p, W.path_kind.p,
                        W.path_near.p, W.ctr.p, W.seg_tx.p, W.cand.p, W.ncand.p, W.find_work.p,
                        W.h_txp.p, W.h_rxreq.p, W.h_rx.p, W.h_gb.p, S.dir_table.p,
                        S.tri_cop.p, S.rank_to_id.p};
  put(ptrs, sizeof ptrs);
  put_v(W.tr_ev.size());
  return k;
}

enum PipelineRun { kEager, kCaptured, kReplayed };
constexpr size_t kPipelineGraphs = 8;  // graphs kept per workspace
constexpr size_t kPipelineSeen = 16;   // eager keys remembered per workspace

// Runs the device pipeline on st: replays the graph captured for the key, or
// captures (then launches) one the second time a key runs, or else runs the
// operations eagerly.  *entry: the graph that ran (captured or replayed).
template <class Record>
static PipelineRun run_pipeline(Workspace& W, cudaStream_t st, Record& record,
                                const std::string& key, bool use_graphs,
                                Workspace::PipelineGraph** entry) {
  *entry = nullptr;
  if (!use_graphs) {
    record();
    return kEager;
  }
  for (auto& g : W.graphs)
    if (g.key == key) {
      CK(cudaGraphLaunch(g.exec, st));
      g.used = ++W.graph_tick;
      *entry = &g;
      return kReplayed;
    }
  auto it = std::find(W.seen.begin(), W.seen.end(), key);
  if (it == W.seen.end()) {
    record();
    if (W.seen.size() == kPipelineSeen) W.seen.erase(W.seen.begin());
    W.seen.push_back(key);
    return kEager;
  }
  W.seen.erase(it);
  if (W.graphs.size() == kPipelineGraphs) {  // drop the least recently used
    auto lru = std::min_element(W.graphs.begin(), W.graphs.end(),
                                [](const auto& a, const auto& b) { return a.used < b.used; });
    CK(cudaGraphExecDestroy(lru->exec));
    CK(cudaGraphDestroy(lru->graph));
    W.graphs.erase(lru);
  }
  Workspace::PipelineGraph g;
  CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  try {
    record();
  } catch (...) {
    cudaGraph_t h = nullptr;
    cudaStreamEndCapture(st, &h);
    if (h) cudaGraphDestroy(h);
    cudaGetLastError();
    throw;
  }
  CK(cudaStreamEndCapture(st, &g.graph));
  const cudaError_t e = cudaGraphInstantiate(&g.exec, g.graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g.graph);
    CK(e);
  }
  g.key = key;
  g.used = ++W.graph_tick;
  W.graphs.push_back(std::move(g));
  *entry = &W.graphs.back();
  CK(cudaGraphLaunch((*entry)->exec, st));
  return kCaptured;
}

// force_check: compute the FP64 shadow field even if no request here asks for
// it (another pass of the same batch did).
static void solve_impl(SceneImpl& S, Workspace& W, const sbr_request* reqs, int n_req,
                       sbr_result& out, const Tuning& tu, bool force_check = false) {
  long long nl = 0;  // kernel launches of this solve (all attempts)
  cudaStream_t st = W.stream;
  if (S.host.mesh_order.empty()) throw std::string("scene is not initialised");
  CK(cudaSetDevice(S.device));
  if (!W.stream) CK(cudaStreamCreateWithFlags(&W.stream, cudaStreamNonBlocking));
  if (!W.side) CK(cudaStreamCreateWithFlags(&W.side, cudaStreamNonBlocking));
  if (!W.ev[0])
    for (auto& e : W.ev) CK(cudaEventCreate(&e));
  if (!W.fork) CK(cudaEventCreateWithFlags(&W.fork, cudaEventDisableTiming));
  if (!W.cap_ev[0])
    for (auto& e : W.cap_ev) CK(cudaEventCreate(&e));
  if (!W.join) CK(cudaEventCreateWithFlags(&W.join, cudaEventDisableTiming));
  st = W.stream;
  // ---- request table
  std::vector<TxParams> tp(n_req);
  long long launches = 0;
  int rx_total = 0, max_depth = 0;
  for (int r = 0; r < n_req; ++r) {
    const sbr_request& q = reqs[r];
    if (q.n_rx < 0 || (q.n_rx > 0 && !q.rx)) throw std::string("receivers missing");
    if (q.max_reflection < 0 || q.max_transmission < 0 ||
        q.max_reflection + q.max_transmission > kMaxDepth)
      throw std::string("max_reflection + max_transmission must be 0..16");
    if (q.tessellation < 0 || q.tessellation > 12) throw std::string("tessellation must be 0..12");
    if (!(q.frequency > 0) || !std::isfinite(q.frequency))
      throw std::string("frequency must be finite and > 0");
    if (!std::isfinite(q.pt)) throw std::string("pt must be finite");
    for (int a = 0; a < 3; ++a)
      if (!std::isfinite(q.tx[a])) throw std::string("transmitter coordinates must be finite");
    for (int a = 0; a < 9; ++a)
      if (!std::isfinite(q.tx_coord_sys[a]))
        throw std::string("tx_coord_sys entries must be finite");
    if (q.n_rx > 0 && !q.rx_on_device)
      for (size_t i = 0; i < 3 * size_t(q.n_rx); ++i)
        if (!std::isfinite(q.rx[i]))
          throw std::string("receiver coordinates must be finite (receiver ") +
              std::to_string(i / 3) + " of request " + std::to_string(r) + ")";
    if (q.antenna < 0 || q.antenna > 3) throw std::string("antenna must be 0, 1, 2 or 3");
    if (q.antenna == SBR_ANTENNA_TABULATED && !q.pattern)
      throw std::string("antenna 3 (tabulated) needs a pattern");
    ensure_dirs(S, q.tessellation);
    TxParams& P = tp[r];
    std::memset(&P, 0, sizeof P);
    for (int a = 0; a < 3; ++a) P.tx[a] = q.tx[a];
    for (int a = 0; a < 9; ++a) P.txcs[a] = q.tx_coord_sys[a];
    P.freq = q.frequency;
    P.pt = q.pt;
    const int tess = q.tessellation + 1;  // RTSolver.cpp:70
    const double beta = 1.0 / (3.0 * tess) * std::acos(-1.0 / std::sqrt(5.0));  // RTSolver.cpp:839
    P.tan_beta = std::tan(beta);
    P.tan_beta32 = float(P.tan_beta);
    P.R = q.max_reflection;
    P.T = q.max_transmission;
    P.antenna = q.antenna;
    P.pat = nullptr;
    P.pat_nt = P.pat_np = 0;
    P.pat_dt = P.pat_dp = 1.0;
    if (q.antenna == SBR_ANTENNA_TABULATED) pattern_params(q.pattern, S.device, P);
    P.fresnel = q.use_fresnel ? 1 : 0;
    P.level = q.tessellation;
    P.n_launch = int(n_launch_of(q.tessellation));
    P.rx_first = rx_total;
    P.n_rx = q.n_rx;
    P.launch_first = launches;
    P.grid = r;
    P.precision = q.field_precision == SBR_FIELD_FP32
                      ? 1
                      : (q.field_precision == SBR_FIELD_FP32_PHASE ? 2 : 0);
    launches += P.n_launch;
    rx_total += q.n_rx;
    max_depth = std::max(max_depth, q.max_reflection + q.max_transmission);
  }
  const int stage_counts = reqs[0].stage_counts ? 1 : 0;
  bool field_check = force_check;
  for (int r = 0; r < n_req; ++r) field_check |= reqs[r].field_check && tp[r].precision != 0;
  if (n_req >= int(0xFFFFFFFFu - kRootBase)) throw std::string("too many requests in one batch");
  auto t0 = std::chrono::steady_clock::now();
  // ---- host staging: everything the device pipeline uploads is staged in
  // pinned memory first, so the pipeline is a fixed sequence of stream
  // operations (a CUDA graph can replay it)
  int max_cells = 64;  // cells per request: the grid aims at ~2 receivers per cell
  for (auto& p : tp)
    max_cells = std::max(max_cells, int(std::min(4.0 * p.n_rx / kMinRxPerCell, 4e6)) + 64);
  max_cells = std::min(max_cells, 1 << 21);
  const size_t cell_cap = size_t(n_req) * (max_cells + 1) + 1;
  int max_rx = 1;
  for (auto& p : tp) max_rx = std::max(max_rx, p.n_rx);
  const dim3 rg(std::min(1024, (max_rx + 255) / 256), n_req);
  W.h_txp.ensure(size_t(n_req));
  std::memcpy(W.h_txp.p, tp.data(), sizeof(TxParams) * n_req);
  W.h_rxreq.ensure(size_t(std::max(1, rx_total)));
  W.h_rx.ensure(3 * size_t(std::max(1, rx_total)));
  for (int r = 0; r < n_req; ++r) {
    const sbr_request& q = reqs[r];
    for (int i = 0; i < q.n_rx; ++i) W.h_rxreq.p[tp[r].rx_first + i] = r;
    if (q.n_rx && !q.rx_on_device)
      std::memcpy(W.h_rx.p + 3 * size_t(tp[r].rx_first), q.rx, 3 * sizeof(double) * q.n_rx);
  }
  W.h_gb.ensure(size_t(n_req));
  for (int r = 0; r < n_req; ++r) {
    GridBuild& g = W.h_gb.p[r];
    for (int a = 0; a < 3; ++a) {
      g.bmin[a] = INT_MAX;
      g.bmax[a] = INT_MIN;
    }
    g.cmax_o = INT_MIN;
    g.cmax = 0;
    g.ncell = 0;
  }
  const FieldConsts K = field_consts();
  {
    // Size node pool and queues at the ray-tree bounds so a pass needs no
    // re-run (the batch splitter keeps each pass within the memory budget).
    double nodes = 0, width = 0;
    for (int r = 0; r < n_req; ++r) {
      const double L = double(tp[r].n_launch);
      nodes += L * tree_nodes(tp[r].R, tp[r].T);
      width += L * tree_width(tp[r].R, tp[r].T);
    }
    W.cap_nodes = std::max<unsigned long long>(W.cap_nodes, (unsigned long long)nodes + 1024);
    W.cap_queue = std::max<unsigned long long>(W.cap_queue, (unsigned long long)width + 1024);
    // Tables from the occupancy ratios learned so far (hash tables half
    // full), each limited to 2% of free device memory: past that the solve
    // grows the table on overflow instead.
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const double cap_bytes = 0.02 * double(free_b);
    auto pow2 = [](double x, double entry_bytes, double limit) {
      x = std::min(x, limit / entry_bytes);
      uint32_t p = 1;
      while (p < x && p < (1u << 30)) p <<= 1;
      return p;
    };
    W.cap_cls = std::max(W.cap_cls, pow2(2.2 * W.r_cls * nodes, 8 + sizeof(ClassInfo) + sizeof(ClassCap), cap_bytes));
    W.cap_cop = std::max(W.cap_cop, pow2(2.2 * W.r_cop * nodes, 8, cap_bytes));
    W.cap_dd = std::max(W.cap_dd, pow2(2.2 * W.r_dd * nodes, 16, cap_bytes));
    W.cap_cc = std::max(W.cap_cc, pow2(2.2 * W.r_cc * nodes, 9, cap_bytes));
    W.cap_corr = std::max<unsigned long long>(
        W.cap_corr, (unsigned long long)std::min(1.2 * W.r_corr * nodes, cap_bytes / sizeof(Corrected)));
    W.cap_surv = std::max<unsigned long long>(
        W.cap_surv, (unsigned long long)std::min(1.2 * W.r_surv * nodes, cap_bytes / 640.0));
    W.cap_pairs = std::max<unsigned long long>(
        W.cap_pairs, (unsigned long long)std::min(1.3 * W.r_pairs * nodes, cap_bytes / sizeof(uint2)));
  }
  for (int attempt = 0;; ++attempt) {
    if (attempt > 6) throw std::string("capacity: tables kept overflowing");
    W.ctr.ensure(1);
    W.nodes.ensure(W.cap_nodes);
    W.nodes_cold.ensure(W.cap_nodes);
    W.q0.ensure(W.cap_queue);
    W.q1.ensure(W.cap_queue);
    W.cls_keys.ensure(W.cap_cls);
    W.cls_info.ensure(W.cap_cls);
    W.cls_cap.ensure(W.cap_cls);
    W.cls_list.ensure(W.cap_cls);
    W.cop_keys.ensure(W.cap_cop);
    W.corr_list.ensure(W.cap_corr);
    W.pairs.ensure(W.cap_pairs);
    W.dd_keys.ensure(W.cap_dd);
    W.cc_keys.ensure(W.cap_cc);
    W.cc_val.ensure(W.cap_cc);
    W.dd_rank.ensure(W.cap_dd);
    W.surv.ensure(W.cap_surv);
    W.seg_tx.ensure(n_req);
    // receivers and their grid
    W.txp.ensure(size_t(n_req));
    W.rx.ensure(std::max(1, 3 * rx_total));
    W.direct_ok.ensure(std::max(1, rx_total));
    W.rx_req.ensure(size_t(std::max(1, rx_total)));
    W.gb.ensure(n_req);
    W.grids.ensure(n_req);
    W.cell_base.ensure(n_req + 1);
    W.cell_counts.ensure(cell_cap);
    W.cell_starts.ensure(cell_cap + 1);
    W.cell_cursor.ensure(cell_cap);
    W.rx32.ensure(std::max(1, rx_total));
    W.rx_bad.ensure(1);
    // trace chunks: each depth runs in chunks of at most kTraceChunk rays
    const long long kTraceChunk =
        1LL << (tu.chunk_log2 > 0 ? std::min(tu.chunk_log2, 26) : kTraceChunkLog2);
    const long long max_width = std::max<long long>(launches, (long long)W.cap_queue);
    const long long chunk = std::max<long long>(1, std::min(kTraceChunk, max_width));
    W.cand.ensure(size_t(chunk) * kCand);
    W.ncand.ensure(size_t(chunk));
    W.ray32.ensure(size_t(chunk));
    W.find_work.ensure(2);  // [0] k_find's work counter, [1] k_trace's
    size_t n_launch_pairs = 0;  // k_find / k_trace launch pairs of the trace
    {
      for (int d = 0; d <= max_depth; ++d) {
        const long long bound = d == 0 ? launches : (long long)W.cap_queue;
        n_launch_pairs += size_t((bound + chunk - 1) / chunk);
      }
      if (2 * n_launch_pairs > W.tr_ev.size()) {
        W.tr_ev.resize(2 * n_launch_pairs, nullptr);
        for (auto& e : W.tr_ev)
          if (!e) CK(cudaEventCreate(&e));
      }
    }
    // the field stage, sized by the survivor capacity
    {
      const size_t nsa = std::max<size_t>(1, W.cap_surv);
      W.path_field.ensure(6 * nsa);
      W.path_nray.ensure(nsa);
      W.path_tri.ensure(nsa * (kMaxDepth + 1));
      W.path_cop.ensure(nsa * (kMaxDepth + 1));
      W.path_kind.ensure(nsa * (kMaxDepth + 1));
      W.path_near.ensure(nsa);
      W.path_pts.ensure(nsa * (kMaxDepth + 2) * 3);
      W.seg.ensure(nsa * (kMaxDepth + 1));
      W.path_mat.ensure(nsa * (kMaxDepth + 1));
      W.field.ensure(std::max(1, 6 * rx_total));
      W.s_counts.ensure(rx_total + 1);
      W.s_starts.ensure(rx_total + 2);
      W.s_cursor.ensure(rx_total + 1);
      W.s_order.ensure(nsa);
      W.path_bound.ensure(nsa);
      W.rx_flag.ensure(std::max(1, rx_total));
      W.field_bound.ensure(std::max(1, rx_total));
      W.fstat.ensure(2);
      if (field_check) {
        W.path_field64.ensure(nsa * 6);
        W.field64.ensure(std::max(1, 6 * rx_total));
      }
    }
    (void)resolved(tu);  // the occupancy queries run before any recording
    (void)pool_fit();
    // ---- the device pipeline: a fixed sequence of stream operations
    const long long nl_before = nl;
    size_t n_tr = 0;  // k_trace launches (timed one by one)
    // Timing events: recorded as event nodes when the pipeline is being
    // captured (a plain record inside a capture only orders the streams; the
    // external flag is refused outside a capture).
    auto mark = [&](cudaEvent_t e) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      CK(cudaStreamIsCapturing(st, &cs));
      if (cs == cudaStreamCaptureStatusActive)
        CK(cudaEventRecordWithFlags(e, st, cudaEventRecordExternal));
      else
        CK(cudaEventRecord(e, st));
    };
    auto record = [&]() {
  mark(W.ev[0]);
  CK(cudaMemcpyAsync(W.txp.p, W.h_txp.p, sizeof(TxParams) * n_req, cudaMemcpyHostToDevice, st));
  for (int r = 0; r < n_req; ++r) {
    const sbr_request& q = reqs[r];
    if (!q.n_rx) continue;
    const size_t o = 3 * size_t(tp[r].rx_first);
    if (q.rx_on_device)
      CK(cudaMemcpyAsync(W.rx.p + o, q.rx, 3 * sizeof(double) * q.n_rx, cudaMemcpyDeviceToDevice, st));
    else
      CK(cudaMemcpyAsync(W.rx.p + o, W.h_rx.p + o, 3 * sizeof(double) * q.n_rx,
                         cudaMemcpyHostToDevice, st));
  }
  CK(cudaMemcpyAsync(W.rx_req.p, W.h_rxreq.p, sizeof(int) * std::max(1, rx_total),
                     cudaMemcpyHostToDevice, st));
  mark(W.ev[1]);
  // ---- receiver grid
  CK(cudaMemcpyAsync(W.gb.p, W.h_gb.p, sizeof(GridBuild) * n_req, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(W.cell_counts.p, 0, sizeof(int) * cell_cap, st));
  CK(cudaMemsetAsync(W.cell_cursor.p, 0, sizeof(int) * cell_cap, st));
  CK(cudaMemsetAsync(W.rx_bad.p, 0, sizeof(int), st));
  ++nl, k_rx_bounds<<<rg, 256, 0, st>>>(W.rx.p, W.txp.p, n_req, W.gb.p, W.rx_bad.p);
  ++nl, k_grid_shape<<<1, 1, 0, st>>>(W.gb.p, W.grids.p, W.txp.p, n_req, max_cells, W.cell_base.p);
  ++nl, k_rx_count<<<rg, 256, 0, st>>>(W.rx.p, W.txp.p, n_req, W.grids.p, W.cell_base.p, W.cell_counts.p);
  ++nl, k_scan_exclusive<<<1, 1024, 0, st>>>(W.cell_counts.p, W.cell_starts.p, int(cell_cap));
  ++nl, k_rx_scatter<<<rg, 256, 0, st>>>(W.rx.p, W.txp.p, n_req, W.grids.p, W.cell_base.p,
                                   W.cell_starts.p, W.cell_cursor.p, W.rx32.p);
  ++nl, k_grid_finish<<<(n_req + 127) / 128, 128, 0, st>>>(W.grids.p, W.cell_starts.p, W.cell_base.p,
                                                    W.rx32.p, n_req);
  CK(cudaGetLastError());

    CK(cudaMemsetAsync(W.ctr.p, 0, sizeof(Counters), st));
    CK(cudaMemsetAsync(W.seg_tx.p, 0, sizeof(unsigned long long) * n_req, st));
    const int fb = 256;
    ++nl, k_fill_u64<<<grid_for(W.cap_cls, fb), fb, 0, st>>>(W.cls_keys.p, W.cap_cls, kEmptyKey);
    ++nl, k_fill_u64<<<grid_for(W.cap_cop, fb), fb, 0, st>>>(W.cop_keys.p, W.cap_cop, kEmptyKey);
    ++nl, k_fill_u64<<<grid_for(W.cap_dd, fb), fb, 0, st>>>(W.dd_keys.p, W.cap_dd, kEmptyKey);
    ++nl, k_fill_u64<<<grid_for(W.cap_dd, fb), fb, 0, st>>>(W.dd_rank.p, W.cap_dd, kEmptyKey);
    ++nl, k_fill_u64<<<grid_for(W.cap_cc, fb), fb, 0, st>>>(W.cc_keys.p, W.cap_cc, kEmptyKey);
    CK(cudaMemsetAsync(W.cc_val.p, 0, W.cap_cc, st));
    mark(W.ev[2]);
    // The direct-path test of every receiver (DirectPathCorrection) needs
    // only the scene and the receivers: it runs on the side stream while the
    // trace runs, and the capture stage waits for it.
    CK(cudaEventRecord(W.fork, st));
    CK(cudaStreamWaitEvent(W.side, W.fork, 0));
    if (rx_total)
      ++nl, k_direct<<<grid_for(rx_total, 64), 64, 0, W.side>>>(S.dev, W.txp.p, W.rx.p, W.rx_req.p,
                                                             rx_total, W.direct_ok.p, W.ctr.p);
    CK(cudaEventRecord(W.join, W.side));
    // ---- trace
    TraceArgs ta;
    ta.sc = S.dev;
    ta.txp = W.txp.p;
    ta.n_tx = n_req;
    ta.dirs = S.dir_table.p;
    ta.nodes = W.nodes.p;
    ta.nodes_cold = W.nodes_cold.p;
    ta.node_cap = W.cap_nodes;
    ta.out_cap = W.cap_queue;
    ta.cls_tab = HashTable{W.cls_keys.p, W.cap_cls - 1};
    ta.cop_tab = HashTable{W.cop_keys.p, W.cap_cop - 1};
    ta.cls_info = W.cls_info.p;
    ta.cls_cap = W.cls_cap.p;
    ta.cls_list = W.cls_list.p;
    ta.tri_cop = S.tri_cop.p;
    ta.ctr = W.ctr.p;
    ta.seg_per_tx = W.seg_tx.p;
    ta.n_root = launches;
    // Each depth runs in chunks (the FP32 search, k_find, stores the chunk's
    // contenders, then k_trace resolves them in FP64 and spawns the next
    // depth).  The ray count of a depth > 0 is on the device; chunks past it
    // return at once.
    FindArgs fnd;
    fnd.sc = S.dev;
    fnd.txp = W.txp.p;
    fnd.n_tx = n_req;
    fnd.dirs = S.dir_table.p;
    fnd.ctr = W.ctr.p;
    fnd.in_cap = W.cap_queue;
    fnd.n_root = launches;
    fnd.work = W.find_work.p;
    fnd.cand = W.cand.p;
    fnd.ncand = W.ncand.p;
    fnd.ray32 = W.ray32.p;
    fnd.steps = tu.find_steps > 0 ? tu.find_steps : kFindSteps;
    fnd.refill = tu.find_refill > 0 ? std::min(tu.find_refill, 32) : kFindRefill;
    fnd.tris_per_step = resolved(tu).find_tris;
    ta.cand = W.cand.p;
    ta.ncand = W.ncand.p;
    ta.ray32 = W.ray32.p;
    ta.work = W.find_work.p + 1;
    n_tr = 0;
    for (int d = 0; d <= max_depth; ++d) {
      ta.depth = fnd.depth = d;
      ta.in = fnd.in = (d % 2 == 0) ? W.q1.p : W.q0.p;
      ta.out = (d % 2 == 0) ? W.q0.p : W.q1.p;
      const long long bound = d == 0 ? launches : (long long)W.cap_queue;
      for (long long lo = 0; lo < bound; lo += chunk) {
        ta.lo = fnd.lo = lo;
        ta.hi = fnd.hi = std::min(bound, lo + chunk);
        CK(cudaMemsetAsync(W.find_work.p, 0, 2 * sizeof(unsigned long long), st));
        ++nl, k_find<<<find_grid(tu), 128, 0, st>>>(fnd);
        mark(W.tr_ev[2 * n_tr]);
        if (resolved(tu).trace_kernel == 2) {
          // one block per 128 rays at most, as k_trace: a small launch still
          // spreads over many warps (each then fills only part of its slots)
          const long long need = (ta.hi - lo + 127) / 128;
          const int grid = int(std::min<long long>(device_sms() * pool_fit(), std::max(1LL, need)));
          ++nl, k_trace_pool<<<grid, 32 * kPoolWarps, kPoolSmem, st>>>(ta);
        } else {
          ++nl, k_trace<<<std::min<long long>(trace_grid(tu), (ta.hi - lo + 127) / 128), 128, 0, st>>>(ta);
        }
        mark(W.tr_ev[2 * n_tr + 1]);
        ++n_tr;
      }
    }
    // correction cones of the classes the trace interned
    ++nl, k_class_cones<<<grid_for(W.cap_cls / 2, 128), 128, 0, st>>>(
        W.cls_list.p, W.ctr.p, W.cap_cls, W.cls_info.p, S.dev, W.cls_cap.p);
    CK(cudaGetLastError());
    mark(W.ev[3]);
    // ---- capture
    CaptureArgs ca;
    ca.sc = S.dev;
    ca.nodes = W.nodes.p;
    ca.nodes_cold = W.nodes_cold.p;
    ca.txp = W.txp.p;
    ca.grids = W.grids.p;
    ca.gb = W.gb.p;
    ca.rx = W.rx.p;
    ca.cls_info = W.cls_info.p;
    ca.cls_cap = W.cls_cap.p;
    ca.direct_ok = W.direct_ok.p;
    ca.corr_list = W.corr_list.p;
    ca.corr_cap = W.cap_corr;
    ca.ctr = W.ctr.p;
    ca.node_cap = W.cap_nodes;
    ca.stage_counts = stage_counts;
    ca.pairs = W.pairs.p;
    ca.pair_cap = W.cap_pairs;
    ca.corr_cache = HashTable{W.cc_keys.p, W.cap_cc - 1};
    ca.corr_val = W.cc_val.p;
    ca.work = W.find_work.p;  // the trace is done with it
    CK(cudaMemsetAsync(W.find_work.p, 0, sizeof(unsigned long long), st));
    CK(cudaStreamWaitEvent(st, W.join, 0));
    mark(W.cap_ev[0]);
    if (stage_counts) {
      ++nl, k_capture<true><<<capture_grid(tu), 32 * kCapWarps, 0, st>>>(ca);
      mark(W.cap_ev[1]);
    } else {
      ++nl, k_capture_fast<<<capture_grid(tu), 32 * kCapWarps, 0, st>>>(ca);
      mark(W.cap_ev[1]);
      ++nl, k_capture_finish<<<device_sms() * 16, 128, 0, st>>>(ca);
    }
    CK(cudaGetLastError());
    mark(W.ev[4]);
    // ---- duplicate removal over the corrected captures
    const HashTable dd{W.dd_keys.p, W.cap_dd - 1};
    ++nl, k_dedup<<<grid_for(W.cap_corr, 256), 256, 0, st>>>(W.corr_list.p, W.cap_corr, W.cls_info.p,
                                                       dd, W.dd_rank.p, W.ctr.p);
    ++nl, k_select<<<grid_for(W.cap_corr, 256), 256, 0, st>>>(W.corr_list.p, W.cap_corr, W.cls_info.p,
                                                        dd, W.dd_rank.p, W.surv.p, W.cap_surv,
                                                        W.ctr.p);
    CK(cudaGetLastError());
    mark(W.ev[5]);
    // ---- field + ordered per-receiver sum, sized by the survivor capacity
    // (the kernels take the count from the device), so the whole solve runs
    // without a host round trip until its results are read
    const unsigned long long ns_cap = W.cap_surv;
    FieldArgs fa;
    fa.sc = S.dev;
    fa.txp = W.txp.p;
    fa.rx = W.rx.p;
    fa.rx_req = W.rx_req.p;
    fa.cls_info = W.cls_info.p;
    fa.rank_to_id = S.rank_to_id.p;
    fa.surv = W.surv.p;
    fa.ctr = W.ctr.p;
    fa.cap = W.cap_surv;
    fa.K = K;
    fa.precision = -1;
    fa.path_field = W.path_field.p;
    fa.path_nray = W.path_nray.p;
    fa.path_tri = W.path_tri.p;
    fa.path_cop = W.path_cop.p;
    fa.path_kind = W.path_kind.p;
    fa.path_near_edge = W.path_near.p;
    fa.path_pts = W.path_pts.p;
    fa.seg = W.seg.p;
    fa.path_mat = W.path_mat.p;
    bool any_fp32 = false;  // a request in the FP32 field mode (error bounds, escalation)
    for (int r = 0; r < n_req; ++r) any_fp32 |= tp[r].precision == 1;
    CK(cudaMemsetAsync(W.rx_flag.p, 0, sizeof(int) * std::max(1, rx_total), st));
    CK(cudaMemsetAsync(W.fstat.p, 0, 2 * sizeof(unsigned long long), st));
    fa.path_bound = W.path_bound.p;
    fa.rx_flag = W.rx_flag.p;
    fa.fstat = W.fstat.p;
    ++nl, k_path<<<grid_for(ns_cap, 64), 64, 0, st>>>(fa);
    ++nl, k_seg<<<grid_for(ns_cap * (kMaxDepth + 1), 64), 64, 0, st>>>(fa);
    ++nl, k_combine<<<grid_for(ns_cap, 64), 64, 0, st>>>(fa);
    CK(cudaMemsetAsync(W.s_counts.p, 0, sizeof(int) * (rx_total + 1), st));
    CK(cudaMemsetAsync(W.s_cursor.p, 0, sizeof(int) * (rx_total + 1), st));
    ++nl, k_surv_hist<<<grid_for(ns_cap, 256), 256, 0, st>>>(W.surv.p, W.ctr.p, W.cap_surv, W.s_counts.p);
    ++nl, k_scan_exclusive<<<1, 1024, 0, st>>>(W.s_counts.p, W.s_starts.p, rx_total);
    ++nl, k_surv_scatter<<<grid_for(ns_cap, 256), 256, 0, st>>>(W.surv.p, W.ctr.p, W.cap_surv,
                                                          W.s_starts.p, W.s_cursor.p, W.s_order.p);
    if (rx_total)
      ++nl, k_rx_sum<<<grid_for(rx_total, 128), 128, 0, st>>>(
          W.surv.p, W.s_starts.p, W.s_order.p, rx_total, W.path_field.p, -1, W.rx_req.p, W.txp.p,
          W.field.p, W.path_bound.p, W.field_bound.p, W.rx_flag.p, W.fstat.p);
    if (any_fp32 && rx_total) {  // receivers the FP32 bound could not certify, in FP64
      ++nl, k_escalate<<<grid_for(ns_cap, 64), 64, 0, st>>>(fa);
      ++nl, k_rx_sum<<<grid_for(rx_total, 128), 128, 0, st>>>(
          W.surv.p, W.s_starts.p, W.s_order.p, rx_total, W.path_field.p, 0, W.rx_req.p, W.txp.p,
          W.field.p, nullptr, W.field_bound.p, nullptr, nullptr, W.rx_flag.p);
    }
    CK(cudaGetLastError());
    mark(W.ev[6]);
    if (field_check) {  // FP64 shadow of the same paths, outside the timed stages
      FieldArgs f64 = fa;
      f64.precision = 0;
      f64.path_field = W.path_field64.p;
      f64.path_bound = nullptr;
      ++nl, k_seg<<<grid_for(ns_cap * (kMaxDepth + 1), 64), 64, 0, st>>>(f64);
      ++nl, k_combine<<<grid_for(ns_cap, 64), 64, 0, st>>>(f64);
      if (rx_total)
        ++nl, k_rx_sum<<<grid_for(rx_total, 128), 128, 0, st>>>(W.surv.p, W.s_starts.p, W.s_order.p,
                                                          rx_total, W.path_field64.p, 0,
                                                          W.rx_req.p, W.txp.p, W.field64.p);
      CK(cudaGetLastError());
    }
    };  // record
    Workspace::PipelineGraph* graph = nullptr;
    const PipelineRun how =
        run_pipeline(W, st, record,
                     pipeline_key(S, W, reqs, tp, n_req, rx_total, launches, max_depth, cell_cap,
                                  chunk, tu, stage_counts, field_check),
                     resolved(tu).graph > 0, &graph);
    if (how == kReplayed) nl = nl_before + graph->kernels;
    if (how == kCaptured) graph->kernels = nl - nl_before;
    W.pipeline_kernels = nl - nl_before;
    n_tr = n_launch_pairs;
    const int graph_run = how == kEager ? 0 : 1;
    Counters c;
    int rx_bad = 0;
    CK(cudaMemcpyAsync(&c, W.ctr.p, sizeof c, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&rx_bad, W.rx_bad.p, sizeof rx_bad, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (rx_bad) throw std::string("receiver coordinates must be finite");
    if (c.overflow & kOvStack) throw std::string("BVH deeper than the traversal stack");
    // keep every hash table at most half full for the next solve
    auto grow = [](uint32_t& cap, unsigned long long used) {
      while (used * 2 > cap && cap < (1u << 30)) cap *= 2;
    };
    grow(W.cap_cls, c.used_cls);
    grow(W.cap_cop, c.used_cop);
    grow(W.cap_dd, c.used_dd);
    grow(W.cap_cc, c.used_cc);  // a full cache only costs recomputation
    if (c.overflow) {
      if (c.overflow & kOvNodes) W.cap_nodes = std::max(W.cap_nodes * 2, c.nodes + c.nodes / 8);
      if (c.overflow & kOvQueue) {
        unsigned long long mx = 0;
        for (auto v : c.queue) mx = std::max(mx, v);
        W.cap_queue = std::max(W.cap_queue * 2, mx + mx / 8);
      }
      // at least 4x, and twice what the refused inserts say was needed (the
      // trace stops at the overflow, so later depths are not counted)
      auto regrow = [](uint32_t& cap, unsigned long long used, unsigned long long lost) {
        const unsigned long long need = std::max<unsigned long long>(4ull * cap, 2 * (used + lost));
        while (cap < need && cap < (1u << 30)) cap *= 2;
      };
      if (c.overflow & kOvClass) regrow(W.cap_cls, c.used_cls, c.lost_cls);
      if (c.overflow & kOvCop) regrow(W.cap_cop, c.used_cop, c.lost_cop);
      if (c.overflow & kOvCorr) W.cap_corr = std::max(W.cap_corr * 2, c.corrected + c.corrected / 4);
      if (c.overflow & kOvDedup) regrow(W.cap_dd, c.used_dd, c.lost_dd);
      if (c.overflow & kOvSurv) W.cap_surv = next_pow2(c.survivors + c.survivors / 4);
      if (c.overflow & kOvPairs) W.cap_pairs = std::max(W.cap_pairs * 2, c.pairs + c.pairs / 4);
      continue;
    }
    if (c.nodes) {
      // ratios of this solve, per bound node (what the next pre-sizing multiplies)
      double bound = 0;
      for (int r = 0; r < n_req; ++r) bound += double(tp[r].n_launch) * tree_nodes(tp[r].R, tp[r].T);
      const double n = std::max(1.0, bound);
      auto upd = [](double& r, double v) { r = std::max(0.9 * r, v); };
      upd(W.r_cls, c.used_cls / n);
      upd(W.r_cop, c.used_cop / n);
      upd(W.r_dd, c.used_dd / n);
      upd(W.r_cc, c.used_cc / n);
      upd(W.r_corr, c.corrected / n);
      upd(W.r_surv, c.survivors / n);
      upd(W.r_pairs, c.pairs / n);
    }
    const unsigned long long ns = c.survivors;
    // ---- results to the host, through the workspace's pinned staging (every
    // array copied by DMA into one area, one synchronisation)
    size_t need = 0;
    auto at = [&need](size_t bytes) {
      const size_t o = need;
      need += (bytes + 15) & ~size_t(15);
      return o;
    };
    const size_t nrs = size_t(ns) * (kMaxDepth + 1), nps = size_t(ns) * (kMaxDepth + 2) * 3;
    const size_t b_field = sizeof(double) * 6 * size_t(rx_total);
    const size_t o_field = at(b_field), o_fb = at(sizeof(double) * size_t(rx_total));
    const size_t o_fst = at(2 * sizeof(unsigned long long));
    const size_t o_f64 = at(field_check ? b_field : 0);
    const size_t o_order = at(sizeof(int) * ns), o_nray = at(sizeof(int) * ns);
    const size_t o_near = at(sizeof(int) * ns), o_sv = at(sizeof(Survivor) * ns);
    const size_t o_pf = at(sizeof(double) * 6 * ns);
    const size_t o_tri = at(sizeof(int) * nrs), o_cop = at(sizeof(int) * nrs);
    const size_t o_kind = at(sizeof(int) * nrs), o_pts = at(sizeof(double) * nps);
    if (need > W.h_res.n) W.h_res.ensure(need + need / 4 + (size_t(64) << 10));  // pinning is slow
    unsigned char* hr = W.h_res.p;
    auto get = [&](size_t o, const void* src, size_t bytes) {
      if (bytes) CK(cudaMemcpyAsync(hr + o, src, bytes, cudaMemcpyDeviceToHost, st));
    };
    get(o_field, W.field.p, b_field);
    get(o_fb, W.field_bound.p, sizeof(double) * size_t(rx_total));
    get(o_fst, W.fstat.p, 2 * sizeof(unsigned long long));
    if (field_check) get(o_f64, W.field64.p, b_field);
    if (ns) {
      get(o_order, W.s_order.p, sizeof(int) * ns);
      get(o_nray, W.path_nray.p, sizeof(int) * ns);
      get(o_near, W.path_near.p, sizeof(int) * ns);
      get(o_sv, W.surv.p, sizeof(Survivor) * ns);
      get(o_pf, W.path_field.p, sizeof(double) * 6 * ns);
      get(o_tri, W.path_tri.p, sizeof(int) * nrs);
      get(o_cop, W.path_cop.p, sizeof(int) * nrs);
      get(o_kind, W.path_kind.p, sizeof(int) * nrs);
      get(o_pts, W.path_pts.p, sizeof(double) * nps);
    }
    CK(cudaEventRecord(W.ev[7], st));
    CK(cudaStreamSynchronize(st));
    const double* hfield = reinterpret_cast<const double*>(hr + o_field);
    out.field.assign(hfield, hfield + 6 * size_t(rx_total));
    const double* hfb = reinterpret_cast<const double*>(hr + o_fb);
    out.field_bound.assign(hfb, hfb + size_t(rx_total));
    unsigned long long fst[2];
    std::memcpy(fst, hr + o_fst, sizeof fst);
    out.field64.clear();
    if (field_check) {
      const double* h64 = reinterpret_cast<const double*>(hr + o_f64);
      out.field64.assign(h64, h64 + 6 * size_t(rx_total));
    }
    const int* order = reinterpret_cast<const int*>(hr + o_order);
    const int* nray = reinterpret_cast<const int*>(hr + o_nray);
    const int* pnear = reinterpret_cast<const int*>(hr + o_near);
    const Survivor* sv = reinterpret_cast<const Survivor*>(hr + o_sv);
    const double* pf = reinterpret_cast<const double*>(hr + o_pf);
    const int* ptri = reinterpret_cast<const int*>(hr + o_tri);
    const int* pcop = reinterpret_cast<const int*>(hr + o_cop);
    const int* pkind = reinterpret_cast<const int*>(hr + o_kind);
    const double* pts = reinterpret_cast<const double*>(hr + o_pts);
    // assemble paths in receiver order, then (launch, BFS) order
    std::vector<int> req_of(rx_total);
    for (int r = 0; r < n_req; ++r)
      for (int i = 0; i < tp[r].n_rx; ++i) req_of[tp[r].rx_first + i] = r;
    out.paths.clear();
    out.tri.clear();
    out.cop.clear();
    out.kind.clear();
    out.points.clear();
    for (size_t k = 0; k < ns; ++k) {
      const int i = order[k];
      sbr_path p;
      p.receiver = int(sv[i].rx) - tp[req_of[sv[i].rx]].rx_first;
      p.request = req_of[sv[i].rx];
      p.n_rays = nray[i];
      p.launch = (long long)(sv[i].rank >> kHeapBits);
      p.heap = int(sv[i].rank & ((1u << kHeapBits) - 1));
      p.ray_offset = (long long)out.tri.size();
      for (int j = 0; j < 6; ++j) p.field[j] = pf[6 * size_t(i) + j];
      p.near_edge = pnear[i];
      p.reserved = 0;
      for (int r = 0; r < p.n_rays; ++r) {
        const size_t b = size_t(i) * (kMaxDepth + 1) + r;
        out.tri.push_back(ptri[b]);
        out.cop.push_back(pcop[b]);
        out.kind.push_back(pkind[b]);
        const size_t q = size_t(i) * (kMaxDepth + 2) * 3 + 3 * r;
        for (int a = 0; a < 6; ++a) out.points.push_back(pts[q + a]);
      }
      out.paths.push_back(p);
    }
    // paths are ordered by survivor order within a receiver; receivers ascend
    // because s_order is grouped by receiver index.
    out.counts.segments = (long long)c.nodes;
    {
      std::vector<unsigned long long> spt(n_req);
      CK(cudaMemcpy(spt.data(), W.seg_tx.p, sizeof(unsigned long long) * n_req,
                    cudaMemcpyDeviceToHost));
      out.segments_per_request.assign(spt.begin(), spt.end());
      out.rx_per_request.resize(n_req);
      out.launches_per_request.resize(n_req);
      for (int r = 0; r < n_req; ++r) {
        out.rx_per_request[r] = tp[r].n_rx;
        out.launches_per_request[r] = tp[r].n_launch;
      }
    }
    out.counts.captured = stage_counts ? (long long)c.events : -1;
    out.counts.corrected = (long long)c.corrected;
    out.counts.paths = (long long)ns;
    out.counts.rays = (long long)out.tri.size();
    out.counts.fp64_triangle_tests = (long long)c.fp64_tri;
    out.counts.fallback_rays = (long long)c.fallback;
    out.counts.fp64_capture_tests = (long long)c.fp64_capture;
    out.counts.launches = launches;
    out.counts.capture_candidates = (long long)c.cand;
    out.counts.ancestor_tests = (long long)c.anc;
    out.counts.classes = (long long)c.used_cls;
    out.counts.groups = -1;
    out.counts.keys = (long long)c.used_dd;
    out.counts.near_edge_paths = 0;
    for (const sbr_path& p : out.paths) out.counts.near_edge_paths += p.near_edge;
    out.counts.gpu_kernels = nl;
    out.counts.pipeline_graph = graph_run;
    out.counts.fp64_field_paths = (long long)fst[0];
    out.counts.fp64_field_receivers = (long long)fst[1];
    float ms[8] = {};
    for (int i = 1; i < 8; ++i) CK(cudaEventElapsedTime(&ms[i], W.ev[i - 1], W.ev[i]));
    out.timing.h2d_ms = ms[1];
    out.timing.trace_ms = ms[3];
    out.timing.capture_ms = ms[4];
    out.timing.correct_ms = ms[5];
    out.timing.field_ms = ms[6];
    out.timing.d2h_ms = ms[7];
    float cap_k = 0;
    CK(cudaEventElapsedTime(&cap_k, W.cap_ev[0], W.cap_ev[1]));
    out.timing.capture_kernel_ms = cap_k;
    double tr_k = 0;
    for (size_t i = 0; i < n_tr; ++i) {
      float x = 0;
      CK(cudaEventElapsedTime(&x, W.tr_ev[2 * i], W.tr_ev[2 * i + 1]));
      tr_k += x;
      if (i == 0) out.timing.trace_kernel_first_ms = x;
    }
    out.timing.trace_kernel_ms = tr_k;
    out.timing.trace_kernel_launches = double(n_tr);
    float all = 0, dev = 0;
    CK(cudaEventElapsedTime(&all, W.ev[0], W.ev[7]));
    CK(cudaEventElapsedTime(&dev, W.ev[1], W.ev[6]));
    out.timing.total_ms = all;
    out.timing.device_ms = dev;
    (void)t0;
    return;
  }
}

}  // namespace sbr

namespace sbr {
// One result per request of a batch result (request order); fields, paths and
// segment counts are the request's own, stage counters the batch's.
std::vector<sbr_result*> split_result(const sbr_result& b) {
  std::vector<sbr_result*> out;
  const int n = int(b.rx_per_request.size());
  size_t f0 = 0;
  for (int r = 0; r < n; ++r) {
    auto* x = new sbr_result();
    const size_t nf = 6 * size_t(b.rx_per_request[r]);
    x->field.assign(b.field.begin() + f0, b.field.begin() + f0 + nf);
    if (!b.field64.empty()) x->field64.assign(b.field64.begin() + f0, b.field64.begin() + f0 + nf);
    if (b.field_bound.size() * 6 == b.field.size())
      x->field_bound.assign(b.field_bound.begin() + f0 / 6, b.field_bound.begin() + (f0 + nf) / 6);
    f0 += nf;
    for (const sbr_path& p : b.paths) {
      if (p.request != r) continue;
      sbr_path q = p;
      q.request = 0;
      q.ray_offset = (long long)x->tri.size();
      const size_t o = size_t(p.ray_offset), m = size_t(p.n_rays);
      x->tri.insert(x->tri.end(), b.tri.begin() + o, b.tri.begin() + o + m);
      x->cop.insert(x->cop.end(), b.cop.begin() + o, b.cop.begin() + o + m);
      x->kind.insert(x->kind.end(), b.kind.begin() + o, b.kind.begin() + o + m);
      x->points.insert(x->points.end(), b.points.begin() + 6 * o, b.points.begin() + 6 * (o + m));
      x->paths.push_back(q);
    }
    x->counts = b.counts;
    x->counts.segments = r < int(b.segments_per_request.size()) ? b.segments_per_request[r] : -1;
    x->counts.paths = (long long)x->paths.size();
    x->counts.near_edge_paths = 0;
    for (const sbr_path& p : x->paths) x->counts.near_edge_paths += p.near_edge;
    x->counts.rays = (long long)x->tri.size();
    x->timing = b.timing;
    x->counts.launches = r < int(b.launches_per_request.size()) ? b.launches_per_request[r] : -1;
    x->segments_per_request = {x->counts.segments};
    x->launches_per_request = {x->counts.launches};
    x->rx_per_request = {b.rx_per_request[r]};
    out.push_back(x);
  }
  return out;
}
}  // namespace sbr

// ============================================================ C ABI

using namespace sbr;

// The launch shapes a solve of this request mix uses: the autotuned choice
// for the mix if there is one, else the scene's default.
static Tuning tuning_for(SceneImpl& S, const sbr_request* reqs, int n) {
  std::lock_guard<std::mutex> lock(S.tune_mu);
  if (reqs && n > 0) {
    auto it = S.tuned.find(mix_key(reqs, n));
    if (it != S.tuned.end()) return it->second;
  }
  return S.tuning;
}

#define ABI_GUARD(...)                                                     \
  try {                                                                     \
    __VA_ARGS__                                                             \
  } catch (const CudaError& e) {                                            \
    set_err(std::string("CUDA error in ") + e.where + ": " + cudaGetErrorString(e.e)); \
    return e.e == cudaErrorMemoryAllocation ? SBR_ERR_OOM : SBR_ERR_CUDA;   \
  } catch (const std::bad_alloc&) {                                         \
    set_err("host allocation failed");                                      \
    return SBR_ERR_OOM;                                                     \
  } catch (const std::string& s) {                                          \
    set_err(s);                                                             \
    return s.rfind("capacity", 0) == 0 ? SBR_ERR_CAPACITY : SBR_ERR_INVALID_ARG; \
  }

extern "C" {

const char* sbr_last_error(void) { return g_err.c_str(); }

sbr_status sbr_fault_inject_alloc(long long after) {
  g_alloc_fault.store(after < 0 ? -1 : after, std::memory_order_relaxed);
  return SBR_OK;
}
const char* sbr_version(void) { return "sbr-gb300 0.1 (sm_103a)"; }

// Wall thicknesses must be finite and non-negative; empty string when valid.
static std::string material_error(const sbr_material* m, int n) {
  for (int i = 0; i < n; ++i)
    if (!(m[i].width >= 0.0) || !std::isfinite(m[i].width))
      return "material " + std::to_string(i) + ": width must be finite and >= 0";
  return std::string();
}

static sbr_status scene_common(std::vector<float>& v, std::vector<float>& n, const int* mat_ids,
                               const sbr_material* materials, int n_materials, unsigned flags,
                               sbr_scene** out) {
  ABI_GUARD({
    if (!out) throw std::string("out is NULL");
    *out = nullptr;
    if (n_materials <= 0 || !materials) throw std::string("at least one material is required");
    if (!material_error(materials, n_materials).empty())
      throw material_error(materials, n_materials);
    const int nt = int(n.size() / 3);
    for (size_t i = 0; i < v.size(); ++i)
      if (!std::isfinite(v[i]))
        throw std::string("vertex coordinates must be finite (triangle ") +
            std::to_string(i / 9) + ")";
    for (size_t i = 0; i < n.size(); ++i)
      if (!std::isfinite(n[i]))
        throw std::string("facet normals must be finite (triangle ") + std::to_string(i / 3) + ")";
    if (mat_ids)
      for (int i = 0; i < nt; ++i)
        if (mat_ids[i] < 0 || mat_ids[i] >= n_materials)
          throw std::string("material id out of range at triangle ") + std::to_string(i);
    const auto t_start = std::chrono::steady_clock::now();
    auto ms_since = [](std::chrono::steady_clock::time_point a) {
      return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a)
          .count();
    };
    auto sc = std::make_unique<sbr_scene>();
    SceneImpl& S = sc->impl;
    std::string err;
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
      cudaGetLastError();
      throw CudaError{cudaErrorNoDevice, "no CUDA device"};
    }
    CK(cudaGetDevice(&S.device));
    CK(cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking));
    // The device builds the coplanar groups, frames, search BVH and
    // reference BVH on its own host thread and stream while this thread forms
    // the triangle records (SBR_SCENE_HOST_PREP: everything on the host).
    const bool on_device = !(flags & SBR_SCENE_HOST_PREP);
    DeviceTables dt;
    std::string dev_err;
    bool dev_failed = false;
    CudaError dev_cuda{cudaSuccess, ""};
    std::thread dev_thread;
    if (on_device)
      dev_thread = std::thread([&] {
        try {
          CK(cudaSetDevice(S.device));
          cudaStream_t st = nullptr;
          CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
          struct Del {
            cudaStream_t s;
            ~Del() { cudaStreamDestroy(s); }
          } del{st};
          device_prepare(v.data(), n.data(), nt, st, dt);
        } catch (const CudaError& e) {
          dev_failed = true;
          dev_cuda = e;
        } catch (const std::string& e) {
          dev_failed = true;
          dev_err = e;
        } catch (...) {
          dev_failed = true;
          dev_err = "device scene preparation failed";
        }
      });
    struct Join {
      std::thread& t;
      ~Join() {
        if (t.joinable()) t.join();
      }
    } join{dev_thread};
    const auto t_host = std::chrono::steady_clock::now();
    const bool host_ok =
        prepare_scene(nt, v.data(), n.data(), mat_ids, S.host, err, !on_device, !on_device);
    S.prep_ms[1] = ms_since(t_host);
    if (dev_thread.joinable()) dev_thread.join();
    S.prep_ms[2] = dt.tables_ms;
    S.prep_ms[3] = dt.search_ms;
    S.prep_ms[4] = dt.ref_ms;
    if (!host_ok) throw err;
    if (on_device) {
      if (dev_failed) {
        if (dev_cuda.e != cudaSuccess) throw dev_cuda;
        throw dev_err;
      }
      if (dt.degenerate)
        throw std::string("degenerate triangle(s) after vertex merge: ") +
            std::to_string(dt.degenerate);
      for (int t = 0; t < nt; ++t) {
        HostTri& tr = S.host.tris[size_t(t)];
        tr.cop = dt.cop[size_t(t)];
        std::memcpy(tr.cs, &dt.cs[9 * size_t(t)], sizeof tr.cs);
      }
      S.host.nodes = std::move(dt.nodes);
      S.host.dfs_tris = std::move(dt.dfs_tris);
      S.host.mesh_order = std::move(dt.mesh_order);
      S.host.max_depth = dt.max_depth;
      S.host.search = std::move(dt.search);
      map_search_order(S.host);
    }
    if (S.host.max_depth + 4 > kStack)
      throw std::string("BVH depth ") + std::to_string(S.host.max_depth) +
          " exceeds the traversal stack (" + std::to_string(kStack) + ")";
    S.materials.assign(materials, materials + n_materials);
    const auto t_up = std::chrono::steady_clock::now();
    upload_scene(S);
    upload_mesh_order(S, S.host.mesh_order);
    CK(cudaStreamSynchronize(S.stream));
    S.prep_ms[5] = ms_since(t_up);
    S.prep_ms[0] = ms_since(t_start);
    *out = sc.release();
    return SBR_OK;
  })
}

sbr_status sbr_scene_create_ex(int n_triangles, const float* vertices, const float* normals,
                               const int* material_ids, const sbr_material* materials,
                               int n_materials, unsigned flags, sbr_scene** out) {
  if (n_triangles <= 0 || !vertices || !normals) {
    set_err("sbr_scene_create: empty triangle list");
    return SBR_ERR_INVALID_ARG;
  }
  if (flags & ~unsigned(SBR_SCENE_HOST_PREP)) {
    set_err("sbr_scene_create_ex: unknown flags");
    return SBR_ERR_INVALID_ARG;
  }
  std::vector<float> v(vertices, vertices + 9 * size_t(n_triangles));
  std::vector<float> n(normals, normals + 3 * size_t(n_triangles));
  return scene_common(v, n, material_ids, materials, n_materials, flags, out);
}

sbr_status sbr_scene_create(int n_triangles, const float* vertices, const float* normals,
                            const int* material_ids, const sbr_material* materials,
                            int n_materials, sbr_scene** out) {
  return sbr_scene_create_ex(n_triangles, vertices, normals, material_ids, materials, n_materials,
                             0u, out);
}

sbr_status sbr_scene_triangle_frames(const sbr_scene* scene, double* frames, double* boxes,
                                     double* centers) {
  if (!scene) {
    set_err("sbr_scene_triangle_frames: NULL scene");
    return SBR_ERR_INVALID_ARG;
  }
  const auto& tris = scene->impl.host.tris;
  for (size_t t = 0; t < tris.size(); ++t) {
    if (frames) std::memcpy(frames + 9 * t, tris[t].cs, sizeof tris[t].cs);
    if (boxes) std::memcpy(boxes + 6 * t, tris[t].bb, sizeof tris[t].bb);
    if (centers) std::memcpy(centers + 3 * t, tris[t].center, sizeof tris[t].center);
  }
  return SBR_OK;
}

sbr_status sbr_scene_search_bvh(const sbr_scene* scene, int* n_nodes, int* max_depth,
                                float* nodes, int* order) {
  if (!scene || !n_nodes) {
    set_err("sbr_scene_search_bvh: NULL argument");
    return SBR_ERR_INVALID_ARG;
  }
  const SearchBVH& B = scene->impl.host.search;
  if (nodes && *n_nodes < int(B.nodes.size())) {
    set_err("sbr_scene_search_bvh: node buffer too small");
    *n_nodes = int(B.nodes.size());
    return SBR_ERR_CAPACITY;
  }
  *n_nodes = int(B.nodes.size());
  if (max_depth) *max_depth = B.max_depth;
  static_assert(sizeof(SearchNode) == 14 * 4, "search node layout");
  if (nodes) std::memcpy(nodes, B.nodes.data(), sizeof(SearchNode) * B.nodes.size());
  if (order) std::memcpy(order, B.order.data(), sizeof(int) * B.order.size());
  return SBR_OK;
}

sbr_status sbr_scene_reference_bvh(const sbr_scene* scene, int* n_nodes, int* max_depth,
                                   double* boxes, int* links, int* order) {
  if (!scene || !n_nodes) {
    set_err("sbr_scene_reference_bvh: NULL argument");
    return SBR_ERR_INVALID_ARG;
  }
  const HostScene& H = scene->impl.host;
  const int nn = int(H.nodes.size());
  if ((boxes || links) && *n_nodes < nn) {
    set_err("sbr_scene_reference_bvh: node buffers too small");
    *n_nodes = nn;
    return SBR_ERR_CAPACITY;
  }
  *n_nodes = nn;
  if (max_depth) *max_depth = H.max_depth;
  for (int k = 0; k < nn; ++k) {
    const HostNode& h = H.nodes[size_t(k)];
    if (boxes) std::memcpy(boxes + 6 * size_t(k), h.bb, sizeof h.bb);
    if (links) {
      int* o = links + 6 * size_t(k);
      o[0] = h.c0;
      o[1] = h.c1;
      o[2] = h.first;
      o[3] = h.count;
      o[4] = h.parent;
      o[5] = h.depth;
    }
  }
  if (order) std::memcpy(order, H.dfs_tris.data(), sizeof(int) * H.dfs_tris.size());
  return SBR_OK;
}

sbr_status sbr_scene_create_from_stl(const char* path, const int* material_ids,
                                     const sbr_material* materials, int n_materials,
                                     sbr_scene** out) {
  std::vector<float> v, n;
  std::string err;
  if (!path || !read_stl(path, v, n, err)) {
    set_err(path ? err : std::string("path is NULL"));
    return SBR_ERR_IO;
  }
  return scene_common(v, n, material_ids, materials, n_materials, 0u, out);
}

sbr_status sbr_scene_info_get(const sbr_scene* scene, sbr_scene_info* out) {
  if (!scene || !out) {
    set_err("NULL argument");
    return SBR_ERR_INVALID_ARG;
  }
  const SceneImpl& S = scene->impl;
  out->n_triangles = int(S.host.tris.size());
  out->n_bvh_nodes = int(S.host.nodes.size());
  out->bvh_depth = S.host.max_depth;
  out->n_coplanar = S.n_cop;
  out->extent = S.host.extent;
  out->device_bytes = S.dev_bytes;
  out->prep_total_ms = S.prep_ms[0];
  out->prep_host_ms = S.prep_ms[1];
  out->prep_device_tables_ms = S.prep_ms[2];
  out->prep_search_bvh_ms = S.prep_ms[3];
  out->prep_reference_bvh_ms = S.prep_ms[4];
  out->prep_upload_ms = S.prep_ms[5];
  return SBR_OK;
}

sbr_status sbr_scene_mesh_order(const sbr_scene* scene, int* out) {
  if (!scene || !out) {
    set_err("NULL argument");
    return SBR_ERR_INVALID_ARG;
  }
  std::copy(scene->impl.host.mesh_order.begin(), scene->impl.host.mesh_order.end(), out);
  return SBR_OK;
}

sbr_status sbr_scene_set_mesh_order(sbr_scene* scene, const int* order) {
  if (!scene || !order) {
    set_err("NULL argument");
    return SBR_ERR_INVALID_ARG;
  }
  const int nt = int(scene->impl.host.tris.size());
  std::vector<int> o(order, order + nt), seen(nt, 0);
  for (int v : o) {
    if (v < 0 || v >= nt || seen[v]++) {
      set_err("mesh order is not a permutation of the triangle ids");
      return SBR_ERR_INVALID_ARG;
    }
  }
  ABI_GUARD({
    // not to be called while solves on this scene are in flight
    std::lock_guard<std::mutex> lock(scene->impl.pool_mu);
    scene->impl.host.mesh_order = o;
    upload_mesh_order(scene->impl, o);
    return SBR_OK;
  })
}

sbr_status sbr_scene_set_materials(sbr_scene* scene, const int* material_ids,
                                   const sbr_material* materials, int n_materials) {
  if (!scene || !materials || n_materials <= 0) {
    set_err("sbr_scene_set_materials: need a scene and at least one material");
    return SBR_ERR_INVALID_ARG;
  }
  if (!material_error(materials, n_materials).empty()) {
    set_err("sbr_scene_set_materials: " + material_error(materials, n_materials));
    return SBR_ERR_INVALID_ARG;
  }
  SceneImpl& S = scene->impl;
  const int nt = int(S.host.tris.size());
  for (int i = 0; material_ids && i < nt; ++i)
    if (material_ids[i] < 0 || material_ids[i] >= n_materials) {
      set_err("material id out of range at triangle " + std::to_string(i));
      return SBR_ERR_INVALID_ARG;
    }
  ABI_GUARD({
    // not to be called while solves on this scene are in flight
    std::lock_guard<std::mutex> lock(S.pool_mu);
    for (int i = 0; i < nt; ++i) S.host.tris[i].mat = material_ids ? material_ids[i] : 0;
    S.materials.assign(materials, materials + n_materials);
    upload_scene(S);
    upload_mesh_order(S, S.host.mesh_order);
    return SBR_OK;
  })
}

sbr_status sbr_stl_read(const char* path, int* n_triangles, float* vertices, float* normals) {
  if (!path || !n_triangles) {
    set_err("sbr_stl_read: NULL argument");
    return SBR_ERR_INVALID_ARG;
  }
  std::vector<float> v, n;
  std::string err;
  if (!read_stl(path, v, n, err)) {
    set_err(err);
    return SBR_ERR_IO;
  }
  const int nt = int(n.size() / 3);
  if (vertices && normals) {
    if (*n_triangles < nt) {
      set_err("sbr_stl_read: buffers hold " + std::to_string(*n_triangles) + " facets, file has " +
              std::to_string(nt));
      *n_triangles = nt;
      return SBR_ERR_CAPACITY;
    }
    std::copy(v.begin(), v.end(), vertices);
    std::copy(n.begin(), n.end(), normals);
  }
  *n_triangles = nt;
  return SBR_OK;
}

sbr_status sbr_scene_coplanar_ids(const sbr_scene* scene, int* out) {
  if (!scene || !out) {
    set_err("NULL argument");
    return SBR_ERR_INVALID_ARG;
  }
  for (size_t i = 0; i < scene->impl.host.tris.size(); ++i) out[i] = scene->impl.host.tris[i].cop;
  return SBR_OK;
}

sbr_status sbr_scene_destroy(sbr_scene* scene) {
  if (!scene) return SBR_OK;
  // solves hold a workspace until they return; destroying a scene while a
  // solve on it is running is the caller's error
  if (scene->impl.stream) cudaStreamSynchronize(scene->impl.stream);
  cudaStream_t st = scene->impl.stream;
  delete scene;
  if (st) cudaStreamDestroy(st);
  return SBR_OK;
}

sbr_status sbr_solve_batch(sbr_scene* scene, const sbr_request* requests, int n_requests,
                           sbr_result** out) {
  if (!scene || !requests || n_requests <= 0 || !out) {
    set_err("sbr_solve_batch: NULL argument or empty batch");
    return SBR_ERR_INVALID_ARG;
  }
  *out = nullptr;
  ABI_GUARD({
    SceneImpl& S = scene->impl;
    CK(cudaSetDevice(S.device));
    WorkspacePool& pool = ws_pool();
    const int dev = S.device & 63;
    std::unique_ptr<Workspace> W;
    {
      std::lock_guard<std::mutex> lock(pool.mu);
      if (!pool.idle[dev].empty()) {
        W = std::move(pool.idle[dev].back());
        pool.idle[dev].pop_back();
      }
    }
    if (!W) W = std::make_unique<Workspace>();
    struct Return {
      WorkspacePool& pool;
      int dev;
      std::unique_ptr<Workspace>& W;
      ~Return() {
        std::lock_guard<std::mutex> lock(pool.mu);
        pool.idle[dev].push_back(std::move(W));
      }
    } give_back{pool, dev, W};
    // Split the batch into device passes whose estimated footprint (node
    // records, queues, receivers) fits in 60% of the free device memory.
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const double budget = std::max(2e9, 0.45 * double(free_b));
    auto est = [](const sbr_request& q) { return request_bytes(q); };
    bool batch_check = false;  // every pass carries the FP64 shadow if any request wants it
    for (int r = 0; r < n_requests; ++r)
      batch_check |= requests[r].field_check && requests[r].field_precision != SBR_FIELD_FP64;
    const Tuning tu = tuning_for(S, requests, n_requests);
    auto res = std::make_unique<sbr_result>();
    int first = 0;
    while (first < n_requests) {
      int last = first + 1;
      double acc = est(requests[first]);
      while (last < n_requests && acc + est(requests[last]) <= budget) acc += est(requests[last++]);
      if (first == 0 && last == n_requests) {
        solve_impl(S, *W, requests, n_requests, *res, tu);
        break;
      }
      sbr_result part;
      solve_impl(S, *W, requests + first, last - first, part, tu, batch_check);
      const long long ray_base = (long long)res->tri.size();
      for (sbr_path p : part.paths) {
        p.request += first;
        p.ray_offset += ray_base;
        res->paths.push_back(p);
      }
      res->segments_per_request.insert(res->segments_per_request.end(),
                                       part.segments_per_request.begin(),
                                       part.segments_per_request.end());
      res->rx_per_request.insert(res->rx_per_request.end(), part.rx_per_request.begin(),
                                 part.rx_per_request.end());
      res->launches_per_request.insert(res->launches_per_request.end(),
                                       part.launches_per_request.begin(),
                                       part.launches_per_request.end());
      res->field.insert(res->field.end(), part.field.begin(), part.field.end());
      res->field64.insert(res->field64.end(), part.field64.begin(), part.field64.end());
      res->field_bound.insert(res->field_bound.end(), part.field_bound.begin(),
                              part.field_bound.end());
      res->tri.insert(res->tri.end(), part.tri.begin(), part.tri.end());
      res->cop.insert(res->cop.end(), part.cop.begin(), part.cop.end());
      res->kind.insert(res->kind.end(), part.kind.begin(), part.kind.end());
      res->points.insert(res->points.end(), part.points.begin(), part.points.end());
      long long* a = &res->counts.segments;
      const long long* b = &part.counts.segments;
      for (size_t k = 0; k < sizeof(sbr_counts) / sizeof(long long); ++k)
        a[k] = (first == 0 || a[k] < 0 || b[k] < 0) ? (first == 0 ? b[k] : -1) : a[k] + b[k];
      double* ta = &res->timing.total_ms;
      const double* tb = &part.timing.total_ms;
      for (size_t k = 0; k < sizeof(sbr_timing) / sizeof(double); ++k) ta[k] += tb[k];
      first = last;
    }
    *out = res.release();
    return SBR_OK;
  })
}

sbr_status sbr_solve(sbr_scene* scene, const sbr_request* request, sbr_result** out) {
  return sbr_solve_batch(scene, request, 1, out);
}

static void tuning_to_c(const Tuning& t, sbr_tuning* o) {
  o->trace_kernel = t.trace_kernel;
  o->find_steps = t.find_steps;
  o->find_refill = t.find_refill;
  o->find_blocks_per_sm = t.find_bps;
  o->trace_blocks_per_sm = t.trace_bps;
  o->capture_blocks_per_sm = t.capture_bps;
  o->trace_chunk_log2 = t.chunk_log2;
  o->pipeline_graph = t.graph;
  o->find_tris_per_step = t.find_tris;
}

sbr_status sbr_scene_set_tuning(sbr_scene* scene, const sbr_tuning* t) {
  if (!scene || !t) {
    set_err("sbr_scene_set_tuning: NULL argument");
    return SBR_ERR_INVALID_ARG;
  }
  if (t->find_steps < 0 || t->find_refill < 0 || t->find_refill > 32 ||
      t->find_blocks_per_sm < 0 || t->trace_blocks_per_sm < 0 || t->capture_blocks_per_sm < 0 ||
      (t->trace_chunk_log2 != 0 && (t->trace_chunk_log2 < 16 || t->trace_chunk_log2 > 26)) ||
      t->trace_kernel < 0 || t->trace_kernel > 2 || t->pipeline_graph < -1 ||
      t->pipeline_graph > 1 || t->find_tris_per_step < 0 || t->find_tris_per_step > 2) {
    set_err("sbr_scene_set_tuning: fields must be >= 0, find_refill <= 32, trace_chunk_log2 "
            "0 or 16..26, trace_kernel 0..2, pipeline_graph -1..1 and find_tris_per_step "
            "0..2");
    return SBR_ERR_INVALID_ARG;
  }
  SceneImpl& S = scene->impl;
  std::lock_guard<std::mutex> lock(S.tune_mu);
  S.tuning.find_steps = t->find_steps;
  S.tuning.find_refill = t->find_refill;
  S.tuning.find_bps = t->find_blocks_per_sm;
  S.tuning.trace_bps = t->trace_blocks_per_sm;
  S.tuning.capture_bps = t->capture_blocks_per_sm;
  S.tuning.chunk_log2 = t->trace_chunk_log2;
  S.tuning.trace_kernel = t->trace_kernel;
  S.tuning.graph = t->pipeline_graph;
  S.tuning.find_tris = t->find_tris_per_step;
  return SBR_OK;
}

sbr_status sbr_scene_get_tuning(sbr_scene* scene, const sbr_request* requests, int n_requests,
                                sbr_tuning* out) {
  if (!scene || !out || n_requests < 0 || (n_requests > 0 && !requests)) {
    set_err("sbr_scene_get_tuning: bad arguments");
    return SBR_ERR_INVALID_ARG;
  }
  ABI_GUARD({
    CK(cudaSetDevice(scene->impl.device));
    tuning_to_c(resolved(tuning_for(scene->impl, requests, n_requests)), out);
    return SBR_OK;
  })
}

sbr_status sbr_autotune(sbr_scene* scene, const sbr_request* requests, int n_requests, int rounds,
                        sbr_tuning* out, double* best_ms) {
  if (!scene || !requests || n_requests <= 0 || rounds < 1 || rounds > 8) {
    set_err("sbr_autotune: need a scene, a non-empty batch and 1..8 rounds");
    return SBR_ERR_INVALID_ARG;
  }
  SceneImpl& S = scene->impl;
  const std::string key = mix_key(requests, n_requests);
  Tuning cur;
  {
    std::lock_guard<std::mutex> lock(S.tune_mu);
    auto it = S.tuned.find(key);
    cur = it != S.tuned.end() ? it->second : S.tuning;
  }
  sbr_status st = SBR_OK;
  ABI_GUARD({
    CK(cudaSetDevice(S.device));
    cur = resolved(cur);
  })
  // device time of the batch under tuning t: the better of two solves
  auto time_of = [&](const Tuning& t, double& ms) -> sbr_status {
    {
      std::lock_guard<std::mutex> lock(S.tune_mu);
      S.tuned[key] = t;
    }
    ms = 1e300;
    for (int k = 0; k < 2; ++k) {
      sbr_result* r = nullptr;
      const sbr_status s = sbr_solve_batch(scene, requests, n_requests, &r);
      if (s != SBR_OK) return s;
      ms = std::min(ms, r->timing.device_ms);
      sbr_result_destroy(r);
    }
    return SBR_OK;
  };
  double best = 0, ms = 0;
  if ((st = time_of(cur, best)) != SBR_OK) return st;  // also sizes the workspace
  if ((st = time_of(cur, best)) != SBR_OK) return st;
  const int ff = find_fit(), tf = trace_fit(), cf = capture_fit();
  auto span = [](int fit) {
    std::vector<int> v;
    for (int b = std::max(1, fit / 2); b <= fit; ++b) v.push_back(b);
    return v;
  };
  const std::vector<int> steps{8, 16, 32, 64, 128}, refill{4, 8, 16, 24, 32},
      chunk{20, 22, 24, 25, 26},
      kernels{1, 2}, tris{1, 2};
  for (int round = 0; round < rounds; ++round) {
    bool moved = false;
    for (int p = 0; p < 8; ++p) {
      const std::vector<int> cand = p == 0   ? kernels
                                    : p == 1 ? steps
                                    : p == 2 ? refill
                                    : p == 3 ? span(ff)
                                    : p == 4 ? span(tf)
                                    : p == 5 ? span(cf)
                                    : p == 6 ? chunk
                                             : tris;
      for (int v : cand) {
        Tuning t = cur;
        int* f[8] = {&t.trace_kernel, &t.find_steps, &t.find_refill, &t.find_bps, &t.trace_bps,
                     &t.capture_bps, &t.chunk_log2, &t.find_tris};
        if (*f[p] == v) continue;
        *f[p] = v;
        if ((st = time_of(t, ms)) != SBR_OK) return st;
        if (ms < 0.99 * best) {  // a change must gain at least 1 %
          best = ms;
          cur = t;
          moved = true;
        }
      }
    }
    if (!moved) break;
  }
  {
    std::lock_guard<std::mutex> lock(S.tune_mu);
    S.tuned[key] = cur;
  }
  if (out) tuning_to_c(cur, out);
  if (best_ms) *best_ms = best;
  return SBR_OK;
}

sbr_status sbr_result_counts(const sbr_result* r, sbr_counts* out) {
  if (!r || !out) {
    set_err("NULL argument");
    return SBR_ERR_INVALID_ARG;
  }
  *out = r->counts;
  return SBR_OK;
}

sbr_status sbr_result_field(const sbr_result* r, double* out) {
  if (!r || !out) {
    set_err("NULL argument");
    return SBR_ERR_INVALID_ARG;
  }
  std::copy(r->field.begin(), r->field.end(), out);
  return SBR_OK;
}

sbr_status sbr_result_field_bound(const sbr_result* r, double* out) {
  if (!r || !out) {
    set_err("NULL argument");
    return SBR_ERR_INVALID_ARG;
  }
  if (r->field_bound.size() * 6 != r->field.size()) {
    set_err("sbr_result_field_bound: no bounds in this result");
    return SBR_ERR_NOT_READY;
  }
  std::copy(r->field_bound.begin(), r->field_bound.end(), out);
  return SBR_OK;
}

sbr_status sbr_result_field_fp64(const sbr_result* r, double* out) {
  if (!r || !out) {
    set_err("NULL argument");
    return SBR_ERR_INVALID_ARG;
  }
  if (r->field64.size() != r->field.size()) {
    set_err("sbr_result_field_fp64: the request did not set field_check with an FP32 precision");
    return SBR_ERR_NOT_READY;
  }
  std::copy(r->field64.begin(), r->field64.end(), out);
  return SBR_OK;
}

sbr_status sbr_result_field_error(const sbr_result* r, sbr_field_error* out) {
  if (!r || !out) {
    set_err("NULL argument");
    return SBR_ERR_INVALID_ARG;
  }
  if (r->field64.size() != r->field.size()) {
    set_err("sbr_result_field_error: the request did not set field_check with an FP32 precision");
    return SBR_ERR_NOT_READY;
  }
  sbr_field_error e{};
  const size_t n_rx = r->field.size() / 6;
  for (size_t k = 0; k < n_rx; ++k) {
    const double* a = &r->field[6 * k];
    const double* b = &r->field64[6 * k];
    double scale = 0;
    for (int j = 0; j < 3; ++j) scale = std::max(scale, std::hypot(b[2 * j], b[2 * j + 1]));
    if (scale == 0) continue;
    for (int j = 0; j < 3; ++j) {
      const double ar = a[2 * j], ai = a[2 * j + 1], br = b[2 * j], bi = b[2 * j + 1];
      const double mb = std::hypot(br, bi);
      if (!(mb > 1e-6 * scale)) continue;
      const double ma = std::hypot(ar, ai);
      const double rel_mag = std::fabs(ma - mb) / mb;
      // arg(a * conj(b))
      const double ph = std::fabs(std::atan2(ai * br - ar * bi, ar * br + ai * bi));
      const double rel_vec = std::hypot(ar - br, ai - bi) / mb;
      ++e.components;
      if (rel_mag > 1e-4 || ph > 1e-3) ++e.over_tolerance;
      e.max_rel_mag = std::max(e.max_rel_mag, rel_mag);
      e.max_phase_rad = std::max(e.max_phase_rad, ph);
      e.max_rel_vec = std::max(e.max_rel_vec, rel_vec);
    }
  }
  *out = e;
  return SBR_OK;
}

sbr_status sbr_result_paths(const sbr_result* r, sbr_path* paths, int* tri, int* cop, int* kind,
                            double* points) {
  if (!r) {
    set_err("NULL argument");
    return SBR_ERR_INVALID_ARG;
  }
  if (paths) std::copy(r->paths.begin(), r->paths.end(), paths);
  if (tri) std::copy(r->tri.begin(), r->tri.end(), tri);
  if (cop) std::copy(r->cop.begin(), r->cop.end(), cop);
  if (kind) std::copy(r->kind.begin(), r->kind.end(), kind);
  if (points) std::copy(r->points.begin(), r->points.end(), points);
  return SBR_OK;
}

sbr_status sbr_result_timing(const sbr_result* r, sbr_timing* out) {
  if (!r || !out) {
    set_err("NULL argument");
    return SBR_ERR_INVALID_ARG;
  }
  *out = r->timing;
  return SBR_OK;
}

sbr_status sbr_result_destroy(sbr_result* r) {
  delete r;
  return SBR_OK;
}

}  // extern "C"
