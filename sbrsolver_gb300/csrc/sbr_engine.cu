// GB300 SBR engine: device-resident scene, wavefront ray tracing, reception
// capture, image correction, duplicate removal and the received field, behind
// the C ABI declared in include/sbr.h.
//
// Pipeline per solve (one CUDA stream, no host round trip between stages):
//   grid     receivers -> uniform grid (bbox, count, scan, scatter)
//   trace    one kernel per bounce depth over a compacted wavefront queue;
//            each ray runs the closest-hit query, writes its tree node and
//            spawns its reflected / transmitted children (RTSolver.cpp:128-257)
//   capture  every node tests the receivers near its segment against its
//            reception sphere (RTSolver.cpp:805-863); a capture counts unless an
//            ancestor captured the same receiver (RayCapture deletes the
//            subtree, RTSolver.cpp:277-284).  Captures are grouped by
//            (receiver, path class) with the minimum (launch, BFS) rank
//   correct  one image-method correction per group (RTSolver.cpp:299-433)
//   dedup    minimum rank per (receiver, coplanar key) over corrected groups
//            (RTSolver.cpp:435-459); the minimum is the reference's survivor
//   field    per survivor (FieldCompute.cpp:71-151), summed per receiver in
//            (launch, BFS) order (FieldCompute.cpp:11-25)
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sbr.h"
#include "sbr_device.h"
#include "sbr_field.cuh"
#include "sbr_host.h"
#include "sbr_kernels.cuh"

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
    cudaError_t e = cudaMalloc(&q, want * sizeof(T));
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

static uint32_t next_pow2(uint64_t x) {
  uint64_t p = 1;
  while (p < x) p <<= 1;
  return uint32_t(std::min<uint64_t>(p, 1ull << 31));
}

// ============================================================ kernels

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Warp-aggregated slot reservation: every active lane asks for `cnt` (0..2)
// entries; one atomicAdd per warp.
__device__ __forceinline__ unsigned long long warp_reserve(unsigned long long* ctr, unsigned cnt) {
  const unsigned mask = __activemask();
  const unsigned b1 = __ballot_sync(mask, cnt >= 1);
  const unsigned b2 = __ballot_sync(mask, cnt >= 2);
  const unsigned lt = (1u << lane_id()) - 1u;
  const unsigned before = __popc(b1 & lt) + __popc(b2 & lt);
  const unsigned total = __popc(b1) + __popc(b2);
  const int leader = __ffs(mask) - 1;
  unsigned long long base = 0;
  if (lane_id() == unsigned(leader) && total) base = atomicAdd(ctr, (unsigned long long)total);
  base = __shfl_sync(mask, base, leader);
  return base + before;
}

// Open addressing with linear probing.  Tables are kept at most half full
// (the host grows them between solves from the occupancy counters), so a
// probe run longer than kMaxProbe means the table is too small: the insert
// reports overflow and the solve is repeated with a larger table.
constexpr uint32_t kMaxProbe = 256;

__device__ __forceinline__ uint32_t ht_insert(HashTable t, unsigned long long key, unsigned* ov,
                                              unsigned bit, unsigned long long* used,
                                              unsigned long long* lost, bool* fresh = nullptr) {
  uint32_t h = uint32_t(mix64(key)) & t.mask;
  const uint32_t lim = min(kMaxProbe, t.mask + 1);
  for (uint32_t i = 0; i < lim; ++i) {
    unsigned long long k = *reinterpret_cast<volatile unsigned long long*>(&t.keys[h]);
    if (k == key) return h;
    if (k == kEmptyKey) {
      unsigned long long old = atomicCAS(&t.keys[h], kEmptyKey, key);
      if (old == kEmptyKey) {
        atomicAdd(used, 1ull);
        if (fresh) *fresh = true;
        return h;
      }
      if (old == key) return h;
    }
    h = (h + 1) & t.mask;
  }
  atomicOr(ov, bit);
  atomicAdd(lost, 1ull);
  return 0xFFFFFFFFu;
}

__device__ __forceinline__ uint32_t ht_find(HashTable t, unsigned long long key) {
  uint32_t h = uint32_t(mix64(key)) & t.mask;
  const uint32_t lim = min(kMaxProbe, t.mask + 1);
  for (uint32_t i = 0; i < lim; ++i) {
    unsigned long long k = t.keys[h];
    if (k == key) return h;
    if (k == kEmptyKey) return 0xFFFFFFFFu;
    h = (h + 1) & t.mask;
  }
  return 0xFFFFFFFFu;
}

__global__ void k_fill_u64(unsigned long long* p, size_t n, unsigned long long v) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
       i += size_t(gridDim.x) * blockDim.x)
    p[i] = v;
}

// ---- receiver grid ------------------------------------------------------

// Order-preserving float <-> int mapping for atomicMin/Max on floats.
__device__ __forceinline__ int f2o(float f) {
  int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float o2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }

struct GridBuild {
  int bmin[3], bmax[3];  // ordered ints
  float cmax;            // max |rx| (as float, atomicMax on ordered int below)
  int cmax_o;
  int ncell;
};

__global__ void k_rx_bounds(const double* rx, const TxParams* txp, int n_tx, GridBuild* gb) {
  const int r = blockIdx.y;  // request
  if (r >= n_tx) return;
  const TxParams& P = txp[r];
  int mn[3] = {INT_MAX, INT_MAX, INT_MAX}, mx[3] = {INT_MIN, INT_MIN, INT_MIN}, cm = INT_MIN;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n_rx; i += gridDim.x * blockDim.x) {
    const double* c = rx + 3 * size_t(P.rx_first + i);
    float c32[3] = {float(c[0]), float(c[1]), float(c[2])};
    for (int a = 0; a < 3; ++a) {
      mn[a] = min(mn[a], f2o(c32[a]));
      mx[a] = max(mx[a], f2o(c32[a]));
    }
    cm = max(cm, f2o(float(sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]))));
  }
  for (int a = 0; a < 3; ++a) {
    for (int o = 16; o; o >>= 1) {
      mn[a] = min(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
      mx[a] = max(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
    }
  }
  for (int o = 16; o; o >>= 1) cm = max(cm, __shfl_xor_sync(0xffffffffu, cm, o));
  if (lane_id() == 0) {
    for (int a = 0; a < 3; ++a) {
      atomicMin(&gb[r].bmin[a], mn[a]);
      atomicMax(&gb[r].bmax[a], mx[a]);
    }
    atomicMax(&gb[r].cmax_o, cm);
  }
}

// Grid shape: cells of equal size sized for ~4 receivers per cell over the
// axes with extent, at most max_cells cells.
__global__ void k_grid_shape(GridBuild* gb, RxGrid* grids, const TxParams* txp, int n_tx,
                             int max_cells, int* cell_base) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int base = 0;
  for (int r = 0; r < n_tx; ++r) {
    RxGrid& g = grids[r];
    float lo[3], hi[3], ext[3];
    float emax = 0;
    for (int a = 0; a < 3; ++a) {
      lo[a] = o2f(gb[r].bmin[a]);
      hi[a] = o2f(gb[r].bmax[a]);
      if (txp[r].n_rx == 0) lo[a] = hi[a] = 0;
      ext[a] = hi[a] - lo[a];
      emax = fmaxf(emax, ext[a]);
    }
    int k = 0;
    double vol = 1;
    for (int a = 0; a < 3; ++a)
      if (ext[a] > 1e-6f * emax && ext[a] > 0) {
        ++k;
        vol *= ext[a];
      }
    float cell = 1.0f;
    if (k > 0) {
      double target = fmax(1.0, txp[r].n_rx / 2.0);
      cell = float(pow(vol / target, 1.0 / k));
    }
    if (cell <= 0) cell = 1.0f;
    int dim[3];
    long long tot;
    for (;;) {
      tot = 1;
      for (int a = 0; a < 3; ++a) {
        dim[a] = max(1, min(1 << 20, int(ext[a] / cell) + 1));
        tot *= dim[a];
      }
      if (tot <= max_cells) break;
      cell *= 1.25f;
    }
    for (int a = 0; a < 3; ++a) {
      g.org[a] = lo[a];
      g.dim[a] = dim[a];
      g.bmin[a] = lo[a];
      g.bmax[a] = hi[a];
    }
    g.cell = cell;
    g.inv_cell = 1.0f / cell;
    gb[r].ncell = int(tot);
    gb[r].cmax = o2f(gb[r].cmax_o);
    cell_base[r] = base;
    base += int(tot) + 1;
  }
  cell_base[n_tx] = base;
}

__device__ __forceinline__ int cell_of(const RxGrid& g, float x, float y, float z) {
  int ix = min(g.dim[0] - 1, max(0, int((x - g.org[0]) / g.cell)));
  int iy = min(g.dim[1] - 1, max(0, int((y - g.org[1]) / g.cell)));
  int iz = min(g.dim[2] - 1, max(0, int((z - g.org[2]) / g.cell)));
  return (iz * g.dim[1] + iy) * g.dim[0] + ix;
}

__global__ void k_rx_count(const double* rx, const TxParams* txp, int n_tx, const RxGrid* grids,
                           const int* cell_base, int* counts) {
  const int r = blockIdx.y;
  if (r >= n_tx) return;
  const RxGrid g = grids[r];
  const TxParams& P = txp[r];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n_rx; i += gridDim.x * blockDim.x) {
    const double* c = rx + 3 * size_t(P.rx_first + i);
    atomicAdd(&counts[cell_base[r] + cell_of(g, float(c[0]), float(c[1]), float(c[2]))], 1);
  }
}

// Single-block exclusive scan (n up to a few million): each thread scans a
// contiguous chunk, then the chunk totals are scanned across the block.
__global__ void k_scan_exclusive(const int* in, int* out, int n) {
  __shared__ int part[1024];
  const int t = threadIdx.x, T = blockDim.x;
  const int chunk = (n + T - 1) / T;
  const int b = min(n, t * chunk), e = min(n, b + chunk);
  int s = 0;
  for (int i = b; i < e; ++i) s += in[i];
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < T; off <<= 1) {
    int v = t >= off ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int run = t ? part[t - 1] : 0;
  for (int i = b; i < e; ++i) {
    int v = in[i];
    out[i] = run;
    run += v;
  }
  if (t == T - 1) out[n] = part[T - 1];
}

__global__ void k_rx_scatter(const double* rx, const TxParams* txp, int n_tx, const RxGrid* grids,
                             const int* cell_base, const int* starts, int* cursor, float4* rx32) {
  const int r = blockIdx.y;
  if (r >= n_tx) return;
  const RxGrid g = grids[r];
  const TxParams& P = txp[r];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n_rx; i += gridDim.x * blockDim.x) {
    const int gi = P.rx_first + i;
    const double* c = rx + 3 * size_t(gi);
    const int cid = cell_base[r] + cell_of(g, float(c[0]), float(c[1]), float(c[2]));
    const int pos = starts[cid] + atomicAdd(&cursor[cid], 1);
    rx32[pos] = make_float4(float(c[0]), float(c[1]), float(c[2]), __int_as_float(gi));
  }
}

__global__ void k_grid_finish(RxGrid* grids, const int* starts, const int* cell_base,
                              const float4* rx32, int n_tx) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_tx) return;
  grids[r].cell_start = starts + cell_base[r];
  grids[r].rx32 = rx32;
}

// ---- trace ------------------------------------------------------------------

struct TraceArgs {
  DevScene sc;
  const TxParams* txp;
  int n_tx;
  const double* const* dirs;  // per level
  const RayRec* in;
  RayRec* out;
  unsigned long long out_cap;
  NodeHot* nodes;
  NodeCold* nodes_cold;
  unsigned long long node_cap;
  HashTable cls_tab, cop_tab;
  ClassInfo* cls_info;
  ClassCap* cls_cap;
  const int* tri_cop;  // coplanar id by rank
  Counters* ctr;
  unsigned long long* seg_per_tx;  // executed segments per request
  int depth;
  long long n_root;    // total launches (depth 0)
  long long lo, hi;    // this launch covers rays [lo, hi) of the depth
  const uint2* cand;   // contenders of those rays (k_find)
  const unsigned char* ncand;
};

__device__ __forceinline__ int find_request(const TxParams* txp, int n_tx, long long g) {
  int lo = 0, hi = n_tx - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (txp[mid].launch_first <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// The capture-stage record of a class with image source img (FP64) whose
// last ray starts on the triangle at mesh position tpos.
__device__ void write_class_cap(const DevScene& sc, const double* img, int tpos, ClassCap& cc) {
  const Tri32 T = sc.corr32[tpos];
  const float3 o = make_float3(float(img[0]), float(img[1]), float(img[2]));
  const float no = sqrtf(o.x * o.x + o.y * o.y + o.z * o.z);
  const TriFrom F = tri_from(T, o, no);
  cc.img[0] = o.x;
  cc.img[1] = o.y;
  cc.img[2] = o.z;
  cc.tpos = tpos;
  cc.F[0] = F.sx; cc.F[1] = F.sy; cc.F[2] = F.sz;
  cc.F[3] = F.qx; cc.F[4] = F.qy; cc.F[5] = F.qz;
  cc.F[6] = F.W; cc.F[7] = F.ns;
  float v[3][3];
  for (int a = 0; a < 3; ++a) {
    v[0][a] = T.v1[a];
    v[1][a] = T.v1[a] + T.e1[a];
    v[2][a] = T.v1[a] + T.e2[a];
  }
  const float im[3] = {o.x, o.y, o.z};
  const float g[3] = {(v[0][0] + v[1][0] + v[2][0]) / 3.0f, (v[0][1] + v[1][1] + v[2][1]) / 3.0f,
                      (v[0][2] + v[1][2] + v[2][2]) / 3.0f};
  const float tmag = no + T.nv1 + T.ne1 + T.ne2 + 1.0f;
  for (int k = 0; k < 3; ++k) {
    const float* p = v[k];
    const float* q = v[k == 2 ? 0 : k + 1];
    const float a[3] = {p[0] - im[0], p[1] - im[1], p[2] - im[2]};
    const float b[3] = {q[0] - im[0], q[1] - im[1], q[2] - im[2]};
    const float n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                        a[0] * b[1] - a[1] * b[0]};
    const float nn = sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    // orient towards the triangle's centroid, which lies inside the cone
    const float gc = n[0] * (g[0] - im[0]) + n[1] * (g[1] - im[1]) + n[2] * (g[2] - im[2]);
    const float sg = gc > 0.0f ? 1.0f : -1.0f;
    for (int c = 0; c < 3; ++c) cc.n[k][c] = sg * n[c];
    cc.n[k][3] = sg * (n[0] * im[0] + n[1] * im[1] + n[2] * im[2]);
    cc.nn[k] = nn;
    cc.w[k] = nn * tmag;
    cc.gc[k] = fabsf(gc);
    cc.inv_nx[k] = 1.0f / (sg * n[0]);
  }
}

// Every thread that interns a class writes the same values (they depend
// only on the key), so concurrent writers agree.
__device__ __forceinline__ void write_class(ClassInfo& ci, const double* img, uint32_t parent,
                                            int tri, uint32_t cop, int kind, int depth) {
  ci.img[0] = img[0];
  ci.img[1] = img[1];
  ci.img[2] = img[2];
  ci.img32[0] = float(img[0]);
  ci.img32[1] = float(img[1]);
  ci.img32[2] = float(img[2]);
  ci.parent = parent;
  ci.tri = tri;
  ci.cop = cop;
  ci.kind = uint8_t(kind);
  ci.depth = uint8_t(depth);
  ci.pad0 = ci.pad1 = 0;
  ci.pad2 = 0;
}

// Number of rays entering bounce depth `depth` (known on the device only).
__device__ __forceinline__ long long rays_at_depth(const Counters* ctr, int depth, long long n_root,
                                                   unsigned long long cap) {
  return depth == 0 ? n_root : (long long)min(ctr->queue[depth], cap);
}

// Launch ray g of the batch: origin and direction (FP64).
__device__ __forceinline__ void root_ray(const TxParams* txp, int n_tx, const double* const* dirs,
                                         long long g, double* o, double* d, int& q, long long& li) {
  q = find_request(txp, n_tx, g);
  const TxParams& P = txp[q];
  li = g - P.launch_first;
  const double* dd = dirs[P.level] + 3 * li;
  for (int a = 0; a < 3; ++a) {
    o[a] = P.tx[a];
    d[a] = dd[a];
  }
}

// ---- FP32 candidate search (persistent, rays refilled per warp) ----------
//
// Each lane traverses one ray at a time.  Lanes whose ray is finished take a
// new one from the chunk's work counter (one atomic per warp, when at least
// a quarter of the warp is idle or nobody is busy), so warps stay full while
// rays of very different lengths finish at different times.
struct FindArgs {
  DevScene sc;
  const TxParams* txp;
  int n_tx;
  const double* const* dirs;
  const RayRec* in;
  const Counters* ctr;
  unsigned long long in_cap;
  long long n_root;
  int depth;
  long long lo, hi;            // this launch covers rays [lo, hi) of the depth
  unsigned long long* work;    // rays of the chunk handed out (zero at launch)
  uint2* cand;                 // kCand per ray of the chunk
  unsigned char* ncand;        // contenders per ray, kFindFallback = exact traversal
};

constexpr int kFindSteps = 16;  // traversal steps between refills

__global__ void __launch_bounds__(128, 8) k_find(FindArgs A) {
  if (A.ctr->overflow & kOvTrace) return;  // this solve will be repeated
  const long long n_all = rays_at_depth(A.ctr, A.depth, A.n_root, A.in_cap);
  const long long n = min(n_all, A.hi) - A.lo;
  if (n <= 0) return;
  const unsigned lane = lane_id();
  long long ray = -1;
  bool exhausted = false;
  float3 o32 = make_float3(0, 0, 0), d32 = o32, inv = o32;
  float no = 0.0f, nd = 0.0f, m = 0.0f, tcut = INFINITY;
  int stack[kStack];
  int sp = 0, pending = -1, nc = 0;
  bool fail = false;
  uint2* out = nullptr;
  while (true) {
    const bool idle = ray < 0 && !exhausted;
    const unsigned im = __ballot_sync(0xffffffffu, idle);
    const unsigned busy = __ballot_sync(0xffffffffu, ray >= 0);
    if (im && (__popc(im) >= 8 || busy == 0)) {
      const int leader = __ffs(im) - 1;
      unsigned long long base = 0;
      if (int(lane) == leader) base = atomicAdd(A.work, (unsigned long long)__popc(im));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (idle) {
        const long long k = (long long)base + __popc(im & ((1u << lane) - 1u));
        if (k < n) {
          ray = k;
          double o[3], d[3];
          if (A.depth == 0) {
            int q;
            long long li;
            root_ray(A.txp, A.n_tx, A.dirs, A.lo + k, o, d, q, li);
          } else {
            const RayRec& r = A.in[A.lo + k];
            for (int a = 0; a < 3; ++a) {
              o[a] = r.o[a];
              d[a] = r.d[a];
            }
          }
          o32 = make_float3(float(o[0]), float(o[1]), float(o[2]));
          d32 = make_float3(float(d[0]), float(d[1]), float(d[2]));
          inv = make_float3(1.0f / d32.x, 1.0f / d32.y, 1.0f / d32.z);
          no = sqrtf(o32.x * o32.x + o32.y * o32.y + o32.z * o32.z);
          nd = sqrtf(d32.x * d32.x + d32.y * d32.y + d32.z * d32.z);
          m = A.sc.box_margin + kFiltK * no;
          tcut = INFINITY;
          sp = 0;
          pending = -1;
          nc = 0;
          fail = false;
          stack[sp++] = 0;  // the search root is always a node
          out = A.cand + size_t(k) * kCand;
        } else {
          exhausted = true;
        }
      }
    }
    if (__ballot_sync(0xffffffffu, ray >= 0) == 0) {
      if (__all_sync(0xffffffffu, exhausted)) break;
      continue;
    }
    if (ray < 0) continue;
    bool done = false;
    for (int it = 0; it < kFindSteps && !done; ++it) {
      if (pending >= 0) {
        const int first = pending >> 3, last = first + (pending & 7);
        for (int j = first; j < last; ++j) {
          float tlo, thi;
          const int k = tri_classify(A.sc.stri[j], o32, d32, no, nd, tlo, thi);
          if (k == 0 || tlo > tcut) continue;
          if (nc == kCand) {
            fail = true;
            break;
          }
          out[nc++] = make_uint2(unsigned(__ldg(A.sc.srank + j)), __float_as_uint(tlo));
          if (k == 2) tcut = fminf(tcut, thi * (1.0f + 1.0f / 4096.0f) + 1e-30f);
        }
        pending = -1;
        if (fail) done = true;
        continue;
      }
      if (sp == 0) {
        done = true;
        break;
      }
      const int ni = stack[--sp];
      if (ni < 0) {  // a leaf deferred as the farther child
        pending = ~ni;
        continue;
      }
      float4 f0, f1, f2;
      int2 ch;
      load_node(A.sc.snode, ni, f0, f1, f2, ch);
      float tn0, tf0, tn1, tf1;
      slab32(f0.x, f0.y, f0.z, f0.w, f1.x, f1.y, o32, inv, m, tn0, tf0);
      slab32(f1.z, f1.w, f2.x, f2.y, f2.z, f2.w, o32, inv, m, tn1, tf1);
      const bool h0 = tn0 <= tf0 && tf0 >= 0.0f && tn0 <= tcut;
      const bool h1 = tn1 <= tf1 && tf1 >= 0.0f && tn1 <= tcut;
      int first = 0, second = 0;
      bool has_first = false, has_second = false;
      if (h0 && h1) {
        has_first = has_second = true;
        if (tn1 < tn0) {
          first = ch.y;
          second = ch.x;
        } else {
          first = ch.x;
          second = ch.y;
        }
      } else if (h0) {
        has_first = true;
        first = ch.x;
      } else if (h1) {
        has_first = true;
        first = ch.y;
      }
      if (has_second) {
        if (sp >= kStack) {
          fail = done = true;
          break;
        }
        stack[sp++] = second;  // node, or ~leaf code
      }
      if (has_first) {
        if (first < 0) {
          pending = ~first;
        } else {
          if (sp >= kStack) {
            fail = done = true;
            break;
          }
          stack[sp++] = first;
        }
      }
    }
    if (done) {
      A.ncand[ray] = fail ? kFindFallback : (unsigned char)nc;
      ray = -1;
    }
  }
}

// Resident blocks of k_trace per SM (register budget 65536 / (128 x this)).
#ifndef SBR_TRACE_BLOCKS
#define SBR_TRACE_BLOCKS 4
#endif
__global__ void __launch_bounds__(128, SBR_TRACE_BLOCKS) k_trace(TraceArgs A) {
  if (A.ctr->overflow & kOvTrace) return;  // this solve will be repeated
  const long long n_all = rays_at_depth(A.ctr, A.depth, A.n_root, A.out_cap);
  const long long n_in = min(n_all, A.hi);
  TraceStats st{0, 0};
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = A.lo + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_in;
       i += stride) {
    RayRec r;
    if (A.depth == 0) {
      int q;
      long long li;
      root_ray(A.txp, A.n_tx, A.dirs, i, r.o, r.d, q, li);
      r.total = 0.0;
      r.S = 0.0;
      r.parent = 0xFFFFFFFFu;
      r.cls = kRootBase + uint32_t(q);
      r.cop = kRootClass;
      r.launch = uint32_t(li);
      r.heap = 1;
      r.rc = r.tc = 0;
      r.tx = uint32_t(q);
    } else {
      r = A.in[i];
    }
    const TxParams& P = A.txp[r.tx];
    Hit h;
    const long long c = i - A.lo;
    const bool hit = resolve_hit(A.sc, r.o, r.d, A.cand + size_t(c) * kCand, A.ncand[c], h, st,
                                 &A.ctr->overflow);
    const unsigned long long ni = warp_reserve(&A.ctr->nodes, 1);
    {  // per-request segment count, one atomic per request present in the warp
      const unsigned peers = __match_any_sync(__activemask(), r.tx);
      if (int(lane_id()) == __ffs(peers) - 1)
        atomicAdd(&A.seg_per_tx[r.tx], (unsigned long long)__popc(peers));
    }
    const bool root = A.depth == 0;
    if (ni < A.node_cap) {
      NodeCold n;
      NodeHot m;
      n.s[0] = r.o[0]; n.s[1] = r.o[1]; n.s[2] = r.o[2];
      if (hit) {
        n.t[0] = h.p[0]; n.t[1] = h.p[1]; n.t[2] = h.p[2];
        m.len = float(h.dist);
      } else {
        const double sc = root ? 1E10 : 1E2;  // RTSolver.cpp:231,249
        n.t[0] = x64::add(r.o[0], x64::mul(r.d[0], sc));
        n.t[1] = x64::add(r.o[1], x64::mul(r.d[1], sc));
        n.t[2] = x64::add(r.o[2], x64::mul(r.d[2], sc));
        m.len = float(sc);
      }
      n.S = r.S;
      n.pad = 0.0;
      m.s[0] = float(r.o[0]); m.s[1] = float(r.o[1]); m.s[2] = float(r.o[2]);
      m.S = float(r.S);
      m.u[0] = float(r.d[0]); m.u[1] = float(r.d[1]); m.u[2] = float(r.d[2]);
      m.parent = r.parent;
      m.cls = r.cls;
      m.launch = r.launch;
      m.heap = r.heap;
      m.tx = r.tx;
      m.pad0 = m.pad1 = m.pad2 = 0;
      A.nodes_cold[ni] = n;
      A.nodes[ni] = m;
    } else {
      atomicOr(&A.ctr->overflow, kOvNodes);
    }
    // children (RTSolver.cpp:186-221)
    unsigned nch = 0;
    bool do_r = false, do_t = false;
    if (hit) {
      do_r = r.rc < P.R;
      do_t = r.tc < P.T;
      nch = unsigned(do_r) + unsigned(do_t);
    }
    const unsigned long long base = warp_reserve(&A.ctr->queue[A.depth + 1], nch);
    if (nch) {
      const Tri64& T = A.sc.tri64[h.rank];
      const double cum = x64::add(r.total, h.dist);  // node pathLength
      RayRec c;
      c.o[0] = h.p[0]; c.o[1] = h.p[1]; c.o[2] = h.p[2];
      c.total = cum;
      c.S = x64::add(r.S, cum);
      c.parent = uint32_t(ni);
      c.launch = r.launch;
      c.tx = r.tx;
      c.pad = 0;
      const int cop = A.tri_cop[h.rank];
      const unsigned long long ck = (unsigned long long)r.cop << 32 | uint32_t(cop);
      const uint32_t cop_cls = ht_insert(A.cop_tab, ck, &A.ctr->overflow, kOvCop, &A.ctr->used_cop,
                                           &A.ctr->lost_cop);
      // image source of the parent ray's class (the transmitter for a launch)
      const double* pimg = is_root_class(r.cls) ? P.tx : A.cls_info[r.cls].img;
      unsigned long long slot = base;
      if (do_t) {  // transmitted: same direction, heap 2h, same image source
        c.d[0] = r.d[0]; c.d[1] = r.d[1]; c.d[2] = r.d[2];
        c.heap = r.heap * 2;
        c.rc = r.rc;
        c.tc = r.tc + 1;
        const unsigned long long key = (unsigned long long)r.cls << 32 | (uint32_t(h.rank) << 1 | 1u);
        bool fresh = false;
        c.cls = ht_insert(A.cls_tab, key, &A.ctr->overflow, kOvClass, &A.ctr->used_cls,
                          &A.ctr->lost_cls, &fresh);
        c.cop = cop_cls;
        if (fresh) {  // only the thread that interned the class writes its records
          write_class(A.cls_info[c.cls], pimg, r.cls, h.rank, cop_cls, 2, A.depth + 1);
          write_class_cap(A.sc, pimg, A.sc.rank_to_id[h.rank], A.cls_cap[c.cls]);
        }
        if (slot < A.out_cap) A.out[slot] = c;
        else atomicOr(&A.ctr->overflow, kOvQueue);
        ++slot;
      }
      if (do_r) {  // reflected: Reflect(d, n).normalized(), heap 2h+1
        const double dn = x64::dot(T.n, r.d);
        double v[3];
        for (int a = 0; a < 3; ++a) v[a] = x64::sub(r.d[a], x64::mul(x64::mul(2.0, T.n[a]), dn));
        x64::normalize(v, c.d);
        c.heap = r.heap * 2 + 1;
        c.rc = r.rc + 1;
        c.tc = r.tc;
        const unsigned long long key = (unsigned long long)r.cls << 32 | (uint32_t(h.rank) << 1);
        bool fresh = false;
        c.cls = ht_insert(A.cls_tab, key, &A.ctr->overflow, kOvClass, &A.ctr->used_cls,
                          &A.ctr->lost_cls, &fresh);
        c.cop = cop_cls;
        if (fresh) {  // only the thread that interned the class writes its records
          // ImagePoint (RTSolver.cpp:910-924) across the triangle the
          // reference finds at this id's position of its mesh vector
          const CorrTri& M = A.sc.corr[A.sc.rank_to_id[h.rank]];
          double w[3], img[3];
          x64::sub3(pimg, M.v1, w);
          const double dist = x64::dot(M.n, w);
          for (int a = 0; a < 3; ++a) img[a] = x64::sub(pimg[a], x64::mul(x64::mul(2.0, dist), M.n[a]));
          write_class(A.cls_info[c.cls], img, r.cls, h.rank, cop_cls, 1, A.depth + 1);
          write_class_cap(A.sc, img, A.sc.rank_to_id[h.rank], A.cls_cap[c.cls]);
        }
        if (slot < A.out_cap) A.out[slot] = c;
        else atomicOr(&A.ctr->overflow, kOvQueue);
      }
    }
  }
  if (st.fp64_tri) atomicAdd(&A.ctr->fp64_tri, (unsigned long long)st.fp64_tri);
  if (st.fallback) atomicAdd(&A.ctr->fallback, (unsigned long long)st.fallback);
}

// ---- capture ----------------------------------------------------------------

struct CaptureArgs {
  DevScene sc;
  const NodeHot* nodes;
  const NodeCold* nodes_cold;
  const TxParams* txp;
  const RxGrid* grids;
  const GridBuild* gb;
  const double* rx;
  const ClassInfo* cls_info;
  const ClassCap* cls_cap;
  const unsigned char* direct_ok;
  Corrected* corr_list;
  unsigned long long corr_cap;
  Counters* ctr;
  unsigned long long node_cap;
  int stage_counts;
  uint2* pairs;                // (node, receiver | unsure << 31) for k_capture_finish
  unsigned long long pair_cap;
};

// MultiPathCorrection (RTSolver.cpp:330-373) for one capture, walking the
// path class from the receiver back to the transmitter: the line from each
// ray's image source to its current target must cross the triangle at that
// id's mesh position.  FP32 filter first (nearly every correction fails at
// its first test); the FP64 test in the reference's order decides the rest
// and yields the exact intersection that becomes the next target.
__device__ __forceinline__ bool correct_event(const DevScene& sc, const ClassInfo* info,
                                             uint32_t cls, const float3& c32, const double* c64,
                                             unsigned& n64) {
  double tgt[3] = {c64[0], c64[1], c64[2]};
  float3 t32 = c32;
  for (uint32_t c = cls; !is_root_class(c);) {
    const ClassInfo& ci = info[c];
    const int mpos = sc.rank_to_id[ci.tri];
    const float3 o = make_float3(ci.img32[0], ci.img32[1], ci.img32[2]);
    const float3 d = make_float3(t32.x - o.x, t32.y - o.y, t32.z - o.z);
    const float no = sqrtf(o.x * o.x + o.y * o.y + o.z * o.z);
    const float nd = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
    float tlo;
    if (!tri_filter(sc.corr32[mpos], o, d, no, nd, tlo)) return false;
    ++n64;
    double dd[3], P3[3];
    x64::sub3(tgt, ci.img, dd);
    if (!mt64c(sc.corr[mpos], ci.img, dd, P3)) return false;
    tgt[0] = P3[0];
    tgt[1] = P3[1];
    tgt[2] = P3[2];
    t32 = make_float3(float(P3[0]), float(P3[1]), float(P3[2]));
    c = ci.parent;
  }
  return true;
}

// Exact decision for a test inside the FP32 margin (reception64 on the
// node's FP64 record).
__device__ __noinline__ int capture_exact(const NodeCold* cold, uint32_t idx, const double* c64,
                                          double tanb) {
  const NodeCold& n = cold[idx];
  return reception64(n.s, n.t, c64, n.S, tanb) ? 1 : 0;
}

// One warp per tree node.  The receivers that can fall inside the node's
// reception spheres lie within rb of its segment (rb bounds the sphere radius
// (S + |P|) tan(beta), with |P| <= (cmax + S tan b) / (1 - tan b) for any
// capturing point); the segment is clipped to that region and cut into
// chunks (each receiver is owned by the chunk its projection falls in).  Each
// chunk's capsule is rasterised over the receiver grid one row of cells per
// lane; a row is one contiguous run of receivers, and the lanes stride over
// the concatenation of the rows' runs.  A capture counts unless an ancestor
// of the node captures the same receiver (RTSolver.cpp:277-284); ancestors
// come from shared memory.
constexpr int kCapWarps = 4;
// Minimum chunk length along a segment, in receiver-grid cells.
#ifndef SBR_CAP_CHUNK_CELLS
#define SBR_CAP_CHUNK_CELLS 16
#endif
constexpr float kCapChunkCells = SBR_CAP_CHUNK_CELLS;
// Nodes staged per warp at a time (at most 32: one per lane; 16 leaves more
// of the SM's shared memory to L1 for the receiver grid).
#ifndef SBR_CAP_BATCH
#define SBR_CAP_BATCH 16
#endif
constexpr int kCapBatch = SBR_CAP_BATCH;

// Upper bound on sqrt(x) from the hardware reciprocal square root (relative
// error below 2^-21), for the capture stage's conservative ranges and
// margins, which all carry slack far beyond that.
__device__ __forceinline__ float sqrt_up(float x) {
  if (!(x > 0.0f)) return 0.0f;
  if (isinf(x)) return x;
  return x * rsqrtf(x) * 1.00000095367431640625f;  // 1 + 2^-20
}

// Correction cone of a class: the points c for which the line from the
// image source img towards c crosses the class's last triangle T
// (MultiPathCorrection's first test for a capture at c; RTSolver.cpp:356).
// Three planes through img and T's edges, n_k . p >= n_k . img, formed once
// per class (write_class_cap); k_capture loosens each by 2 m_k, m_k =
// 2^-12 |n_k| (cmax + |img| + |T| + 1) bounding the FP32 error of the test
// for receivers |p| <= cmax (four times the FP32 filter margin), and uses
// no cone when a plane is ill-conditioned.  The reference's FP64 test accepts
// only points inside the exact cone, so receivers outside the loosened one
// are skipped without changing a result.

// Whether the box [lo, hi] may hold a point of the cone.
__device__ __forceinline__ bool cone_meets_box(const float* cone, const float* lo, const float* hi) {
  for (int k = 0; k < 3; ++k) {
    float mx = 0.0f, mag = fabsf(cone[4 * k + 3]) + 1.0f;
    for (int a = 0; a < 3; ++a) {
      mx += fmaxf(cone[4 * k + a] * lo[a], cone[4 * k + a] * hi[a]);
      mag += fabsf(cone[4 * k + a]) * fmaxf(fabsf(lo[a]), fabsf(hi[a]));
    }
    if (mx < cone[4 * k + 3] - 1e-3f * mag) return false;  // slack >> FP32 error of mx
  }
  return true;
}

// Narrows the cell range [x0, x1] of grid row (iy, iz) to the cells whose
// box can hold a point inside the cone; an empty row gets x0 > x1.
__device__ __forceinline__ void cone_cells(const float* cone, const RxGrid& g, float inv_cell,
                                           int iy, int iz, int& x0, int& x1) {
  const float y0 = g.org[1] + iy * g.cell, y1 = y0 + g.cell;
  const float z0 = g.org[2] + iz * g.cell, z1 = z0 + g.cell;
  for (int k = 0; k < 3; ++k) {
    const float nx = cone[4 * k], ny = cone[4 * k + 1], nz = cone[4 * k + 2], off = cone[4 * k + 3];
    // need nx*x >= off - max over the row's y/z band of (ny*y + nz*z)
    const float r = off - fmaxf(ny * y0, ny * y1) - fmaxf(nz * z0, nz * z1);
    const float slack = 1e-3f * g.cell;
    if (nx > 0.0f) {
      const float xl = r * cone[12 + k];  // x >= xl
      if (isfinite(xl)) x0 = max(x0, int(floorf((xl - g.org[0] - slack) * inv_cell)));
    } else if (nx < 0.0f) {
      const float xh = r * cone[12 + k];  // x <= xh
      if (isfinite(xh)) x1 = min(x1, int(floorf((xh - g.org[0] + slack) * inv_cell)));
    } else if (r > 0.0f) {
      x1 = x0 - 1;
    }
  }
}

struct AncRec {
  float s[3], S, u[3], len;
  uint32_t idx, pad[3];
};

// A node's segment clipped to the region that can hold a capture of this
// request's receivers, cut into chunks (nchunk = 0: nothing to test).
struct NodeSpan {
  float lo, hi, step, ns;  // ns = |segment start|
  int nchunk, use_cone;
};

// The receivers that can fall inside the node's reception spheres lie within
// rb of its segment (rb bounds the sphere radius (S + |P|) tan(beta), with
// |P| <= (cmax + S tan b) / (1 - tan b) for any capturing point).  All
// ranges are widened well beyond their FP32 rounding.
__device__ __forceinline__ NodeSpan node_span(const NodeHot& nd, const TxParams& P,
                                              const RxGrid& g, float cmax, int use_cone) {
  NodeSpan sp{0.0f, -1.0f, 0.0f, 0.0f, 0, use_cone};
  if (P.n_rx <= 0) return sp;
  const float3 s = make_float3(nd.s[0], nd.s[1], nd.s[2]);
  const float3 u = make_float3(nd.u[0], nd.u[1], nd.u[2]);
  const float len = nd.len, S = nd.S;
  const float tanb = float(P.tan_beta);
  const float pmax = __fdividef(cmax + S * tanb, fmaxf(1e-6f, 1.0f - tanb)) * 1.0001f + 1.0f;
  const float su = s.x * u.x + s.y * u.y + s.z * u.z;
  const float ss = s.x * s.x + s.y * s.y + s.z * s.z;
  sp.ns = sqrt_up(ss);
  const float disc = su * su - (ss - pmax * pmax);
  float lo = 0.0f, hi = -1.0f;
  if (disc >= 0.0f) {
    const float sq = sqrt_up(disc);
    lo = fmaxf(0.0f, -su - sq);
    hi = fminf(len, -su + sq);
  }
  const float rbg = (S + pmax) * tanb * 1.0001f + 1e-3f;  // bound over the whole segment
  for (int a = 0; a < 3 && lo <= hi; ++a) {
    const float sa = a == 0 ? s.x : (a == 1 ? s.y : s.z);
    const float ua = a == 0 ? u.x : (a == 1 ? u.y : u.z);
    const float bl = g.bmin[a] - rbg, bh = g.bmax[a] + rbg;
    if (fabsf(ua) < 1e-20f) {
      if (sa < bl || sa > bh) hi = -1.0f;
    } else {
      // slack: 1 mm plus 2^-20 relative, beyond the reciprocal's rounding
      const float ia = __frcp_rn(ua);
      const float t1 = (bl - sa) * ia, t2 = (bh - sa) * ia;
      const float tn = fminf(t1, t2), tf = fmaxf(t1, t2);
      lo = fmaxf(lo, tn - 1e-3f - 9.5367431640625e-07f * fabsf(tn));
      hi = fminf(hi, tf + 1e-3f + 9.5367431640625e-07f * fabsf(tf));
    }
  }
  if (!(lo <= hi)) return sp;
  const float r0 = (S + sqrt_up(ss + 2.0f * lo * su + lo * lo)) * tanb;
  const float lc = fmaxf(kCapChunkCells * g.cell, r0);
  int nchunk = int(ceilf(__fdividef(hi - lo, lc)));
  nchunk = max(1, min(nchunk, 4096));
  sp.lo = lo;
  sp.hi = hi;
  sp.nchunk = nchunk;
  sp.step = __fdividef(hi - lo, float(nchunk));
  return sp;
}

// Chunk ch of a node's span: its parameter range [a, b], the radius rb
// around it that can hold a capture, the reception test's error margin mr,
// and the receiver-grid cell box around it (nrows = 0: nothing to test,
// including a box wholly outside the correction cone).
struct ChunkBox {
  float a, b, rb, mr;
  int c0[3], c1[3];
  int nrows;
};

__device__ __forceinline__ ChunkBox chunk_box(const NodeHot& nd, const RxGrid& g,
                                              const NodeSpan& sp, int ch, float cmax, float tanb,
                                              bool use_cone, const float* cone) {
  ChunkBox cb;
  const float3 s = make_float3(nd.s[0], nd.s[1], nd.s[2]);
  const float3 u = make_float3(nd.u[0], nd.u[1], nd.u[2]);
  const float S = nd.S;
  cb.a = sp.lo + ch * sp.step;
  cb.b = (ch == sp.nchunk - 1) ? sp.hi : sp.lo + (ch + 1) * sp.step;
  const float pa[3] = {s.x + cb.a * u.x, s.y + cb.a * u.y, s.z + cb.a * u.z};
  const float pb[3] = {s.x + cb.b * u.x, s.y + cb.b * u.y, s.z + cb.b * u.z};
  const float npmax = fmaxf(sqrt_up(pa[0] * pa[0] + pa[1] * pa[1] + pa[2] * pa[2]),
                            sqrt_up(pb[0] * pb[0] + pb[1] * pb[1] + pb[2] * pb[2]));
  cb.mr = kFiltK * (sp.ns + cmax + S + npmax + 1.0f);
  // |P| is convex along the chunk: the larger end bounds it
  cb.rb = (S + npmax) * tanb * 1.0002f + g.cell * 0.01f + 2e-3f + cb.mr;
  for (int k = 0; k < 3; ++k) {
    cb.c0[k] = max(0, int(floorf((fminf(pa[k], pb[k]) - cb.rb - g.org[k]) * g.inv_cell)));
    cb.c1[k] = min(g.dim[k] - 1, int(floorf((fmaxf(pa[k], pb[k]) + cb.rb - g.org[k]) * g.inv_cell)));
  }
  const int ny = cb.c1[1] - cb.c0[1] + 1, nz = cb.c1[2] - cb.c0[2] + 1;
  cb.nrows = (cb.c0[0] <= cb.c1[0] && ny > 0 && nz > 0) ? ny * nz : 0;
  if (use_cone && cb.nrows) {  // the chunk's cells all outside the cone: skip it
    float blo[3], bhi[3];
    for (int k = 0; k < 3; ++k) {
      blo[k] = g.org[k] + cb.c0[k] * g.cell;
      bhi[k] = g.org[k] + (cb.c1[k] + 1) * g.cell;
    }
    if (!cone_meets_box(cone, blo, bhi)) cb.nrows = 0;
  }
  return cb;
}

// kStage: stage counts requested (every capture counted, the plain order of
// tests); otherwise the fast path with the correction prefilter and the
// deferred FP64 pass.
template <bool kStage>
__global__ void __launch_bounds__(32 * kCapWarps, kStage ? 4 : 5) k_capture(CaptureArgs A) {
  __shared__ AncRec anc[kCapWarps][kMaxDepth];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned FULL = 0xffffffffu;
  if (A.ctr->overflow & kOvTrace) return;  // this solve will be repeated
  const unsigned long long n_nodes = min(A.ctr->nodes, A.node_cap);
  unsigned long long events = 0, cand = 0, anc_tests = 0;
  unsigned n64 = 0;
  const unsigned long long nw = (unsigned long long)gridDim.x * kCapWarps;
  // Nodes are taken 32 at a time: each lane loads one node's record, its
  // class record and last triangle, so the three dependent loads are paid
  // once per 32 nodes; the warp then works through the 32 from shared memory.
  constexpr int B = kCapBatch;
  __shared__ NodeHot s_nh[kCapWarps][B];
  __shared__ Tri32 s_tl[kCapWarps][B];      // the class's last triangle
  __shared__ float s_fl[kCapWarps][B][12];  // image source + correction filter terms
  __shared__ float s_cn[kCapWarps][B][16];  // loosened correction cone
  __shared__ NodeSpan s_sp[kCapWarps][B];   // clipped span and chunking
  __shared__ ChunkBox s_ck[kCapWarps][B];   // the span's first chunk
  for (unsigned long long base = ((unsigned long long)blockIdx.x * kCapWarps + warp) * B;
       base < n_nodes; base += nw * B) {
    {
      const unsigned long long my = base + lane;
      if (lane < B && my < n_nodes) {
        const NodeHot h = A.nodes[my];
        s_nh[warp][lane] = h;
        const float cmax = A.gb[h.tx].cmax;
        int cone_ok = 0;
        if (!is_root_class(h.cls)) {
          const ClassCap c = A.cls_cap[h.cls];
          s_tl[warp][lane] = A.sc.corr32[c.tpos];
          float* fl = s_fl[warp][lane];
          for (int q = 0; q < 3; ++q) fl[q] = c.img[q];
          for (int q = 0; q < 8; ++q) fl[3 + q] = c.F[q];
          // the cone's planes loosened by 2 m, m = 2^-12 |n| (cmax + |img| + |T| + 1)
          float* cn = s_cn[warp][lane];
          cone_ok = !kStage;
          for (int k = 0; k < 3; ++k) {
            const float m = 2.44140625e-04f * (c.nn[k] * cmax + c.w[k]);
            cone_ok &= (c.gc[k] > 4.0f * m && isfinite(m)) ? 1 : 0;
            cn[4 * k + 0] = c.n[k][0];
            cn[4 * k + 1] = c.n[k][1];
            cn[4 * k + 2] = c.n[k][2];
            cn[4 * k + 3] = c.n[k][3] - 2.0f * m;
            cn[12 + k] = c.inv_nx[k];
          }
        }
        const NodeSpan sp = node_span(h, A.txp[h.tx], A.grids[h.tx], cmax, cone_ok);
        s_sp[warp][lane] = sp;
        if (sp.nchunk > 0)
          s_ck[warp][lane] = chunk_box(h, A.grids[h.tx], sp, 0, cmax, float(A.txp[h.tx].tan_beta),
                                       cone_ok != 0, s_cn[warp][lane]);
      }
      __syncwarp();
    }
    const int n_here = int(min((unsigned long long)B, n_nodes - base));
    for (int jj = 0; jj < n_here; ++jj) {
      const unsigned long long i = base + jj;
      const NodeHot nd = s_nh[warp][jj];
      const TxParams& P = A.txp[nd.tx];
      const RxGrid& g = A.grids[nd.tx];
      const float3 s = make_float3(nd.s[0], nd.s[1], nd.s[2]);
      const float3 u = make_float3(nd.u[0], nd.u[1], nd.u[2]);
      const float len = nd.len, S = nd.S;
      // Reciprocals for the cell-range arithmetic below.  Every range there is
      // widened by at least 2e-3 m + cell/100, far more than the few ulps a
      // product with a reciprocal differs from the quotient.
      const float inv_uy = __frcp_rn(u.y), inv_uz = __frcp_rn(u.z);
      const float inv_cell = g.inv_cell;
      // Stage the ancestor chain when every capture is checked against it
      // (stage counts); otherwise only corrected captures (~0.1% of captures)
      // need it and they walk the chain themselves.
      int na = 0;
      if (kStage && lane == 0) {
        for (uint32_t p = nd.parent; p != 0xFFFFFFFFu && p < A.node_cap && na < kMaxDepth;) {
          const NodeHot a = A.nodes[p];
          AncRec& r = anc[warp][na++];
          r.s[0] = a.s[0]; r.s[1] = a.s[1]; r.s[2] = a.s[2]; r.S = a.S;
          r.u[0] = a.u[0]; r.u[1] = a.u[1]; r.u[2] = a.u[2]; r.len = a.len;
          r.idx = p;
          p = a.parent;
        }
      }
      na = __shfl_sync(FULL, na, 0);
      __syncwarp();
      // Image correction of this node's class must first cross the triangle
      // the last ray reflected or passed on (MultiPathCorrection's last step):
      // an FP32 filter from the class's image source towards each receiver
      // rejects ~99.9% of receivers before the reception test.  Stage counts
      // need every capture, so they keep the reception test first.
      const bool root = is_root_class(nd.cls);
      Tri32 Tl;
      TriFrom Fl;
      float3 img = make_float3(0.0f, 0.0f, 0.0f);
      const NodeSpan sp = s_sp[warp][jj];
      const bool use_cone = sp.use_cone != 0;
      const float* cone_w = s_cn[warp][jj];
      if (!root) {
        const float* fl = s_fl[warp][jj];
        img = make_float3(fl[0], fl[1], fl[2]);
        Tl = s_tl[warp][jj];
        Fl = TriFrom{fl[3], fl[4], fl[5], fl[6], fl[7], fl[8], fl[9], fl[10]};
      }
      if (sp.nchunk > 0) {
        const float tanb = float(P.tan_beta);
        const float cmax = A.gb[nd.tx].cmax;
        const float lo = sp.lo, hi = sp.hi, ns = sp.ns;
        const int nchunk = sp.nchunk;
        const float step = sp.step;
        // error margins of the FP32 reception test, from per-node bounds
        const float ml = kFiltK * (ns + cmax + 1.0f);
        {
          for (int ch = 0; ch < nchunk; ++ch) {
            const ChunkBox cb = ch == 0 ? s_ck[warp][jj]
                                        : chunk_box(nd, g, sp, ch, cmax, tanb, use_cone, cone_w);
            const float a = cb.a, b = cb.b, rb = cb.rb, mr = cb.mr;
            const int c0[3] = {cb.c0[0], cb.c0[1], cb.c0[2]};
            const int c1[3] = {cb.c1[0], cb.c1[1], cb.c1[2]};
            const int ny = c1[1] - c0[1] + 1;
            const int nrows = cb.nrows;
            for (int rbase = 0; rbase < nrows; rbase += 32) {
              // this lane's row: the part of the chunk within rb of its y/z band
              int beg = 0, cnt = 0;
              const int ridx = rbase + lane;
              if (ridx < nrows) {
                // one layer of cells (receivers on a plane) needs no division
                const bool flat = c1[2] == c0[2];
                const int iy = c0[1] + (flat ? ridx : ridx % ny);
                const int iz = c0[2] + (flat ? 0 : ridx / ny);
                const float y0 = g.org[1] + iy * g.cell - rb, y1 = g.org[1] + (iy + 1) * g.cell + rb;
                const float z0 = g.org[2] + iz * g.cell - rb, z1 = g.org[2] + (iz + 1) * g.cell + rb;
                float la = a, lb = b;
                bool ok = true;
                if (fabsf(u.y) > 1e-20f) {
                  const float t1 = (y0 - s.y) * inv_uy, t2 = (y1 - s.y) * inv_uy;
                  la = fmaxf(la, fminf(t1, t2));
                  lb = fminf(lb, fmaxf(t1, t2));
                } else if (s.y < y0 || s.y > y1) {
                  ok = false;
                }
                if (fabsf(u.z) > 1e-20f) {
                  const float t1 = (z0 - s.z) * inv_uz, t2 = (z1 - s.z) * inv_uz;
                  la = fmaxf(la, fminf(t1, t2));
                  lb = fminf(lb, fmaxf(t1, t2));
                } else if (s.z < z0 || s.z > z1) {
                  ok = false;
                }
                if (ok && la <= lb) {
                  const float xa = s.x + la * u.x, xb = s.x + lb * u.x;
                  int x0 = max(c0[0], int(floorf((fminf(xa, xb) - rb - g.org[0]) * inv_cell)));
                  int x1 = min(c1[0], int(floorf((fmaxf(xa, xb) + rb - g.org[0]) * inv_cell)));
                  if (use_cone && x0 <= x1)
                    cone_cells(cone_w, g, inv_cell, iy, iz, x0, x1);
                  if (x0 <= x1) {
                    const int row = (iz * g.dim[1] + iy) * g.dim[0];
                    beg = g.cell_start[row + x0];
                    cnt = g.cell_start[row + x1 + 1] - beg;
                  }
                }
              }
              // concatenate the 32 rows' receiver runs
              int incl = cnt;
              for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += v;
              }
              const int total = __shfl_sync(FULL, incl, 31);
              for (int kb = 0; kb < total; kb += 32) {
                const int k = kb + lane;
                // row holding item k: first lane whose inclusive count exceeds k
                int rl = 0;
                for (int step2 = 16; step2; step2 >>= 1) {
                  const int v = __shfl_sync(FULL, incl, rl + step2 - 1);
                  if (v <= k) rl += step2;
                }
                const int rincl = __shfl_sync(FULL, incl, rl);
                const int rcnt = __shfl_sync(FULL, cnt, rl);
                const int rbeg = __shfl_sync(FULL, beg, rl);
                if (k >= total) continue;
                const int j = rbeg + (k - (rincl - rcnt));
                const float4 c4 = g.rx32[j];
                const float3 c = make_float3(c4.x, c4.y, c4.z);
                const float wx = c.x - s.x, wy = c.y - s.y, wz = c.z - s.z;
                const float lam = u.x * wx + u.y * wy + u.z * wz;
                if (ch > 0 && lam < a) continue;            // owned by an earlier chunk
                if (ch < nchunk - 1 && lam >= b) continue;  // owned by a later chunk
                const int gi = __float_as_int(c4.w);
                const double* c64 = A.rx + 3 * size_t(gi);
                ++cand;
                if (!kStage) {
                  if (root) {
                    if (!A.direct_ok[gi]) continue;
                  } else {
                    const float3 dd = make_float3(c.x - img.x, c.y - img.y, c.z - img.z);
                    if (!tri_filter_from(Tl, Fl, dd,
                                         sqrt_up(dd.x * dd.x + dd.y * dd.y + dd.z * dd.z)))
                      continue;
                  }
                }
                int v;
                if (lam < a || lam > b) {
                  // outside the chunk's own range: full-margin test
                  v = reception32(s, u, len, S, c, tanb);
                } else if (lam < -ml) {
                  v = 0;
                } else if (lam <= ml) {
                  v = -1;
                } else {
                  const float lcl = fminf(lam, len);
                  const float px = s.x + lcl * u.x, py = s.y + lcl * u.y, pz = s.z + lcl * u.z;
                  const float np = sqrt_up(px * px + py * py + pz * pz);
                  const float ex = c.x - px, ey = c.y - py, ez = c.z - pz;
                  const float d2 = ex * ex + ey * ey + ez * ez;
                  const float rad = (S + np) * tanb;
                  const float rh = rad + mr, rl2 = rad - mr;
                  v = d2 > rh * rh ? 0 : ((rl2 > 0.0f && d2 < rl2 * rl2) ? 1 : -1);
                }
                if (!kStage) {
                  // everything after the FP32 tests (exact reception test,
                  // image correction, ancestor suppression) runs densely in
                  // k_capture_finish
                  if (v == 0) continue;
                  const unsigned long long slot = warp_reserve(&A.ctr->pairs, 1);
                  if (slot < A.pair_cap)
                    A.pairs[slot] = make_uint2(uint32_t(i), uint32_t(gi) | (v < 0 ? 0x80000000u : 0u));
                  else
                    atomicOr(&A.ctr->overflow, kOvPairs);
                  continue;
                }
                if (v < 0) {
                  ++n64;
                  v = capture_exact(A.nodes_cold, uint32_t(i), c64, P.tan_beta);
                }
                if (!v) continue;
                // RayCapture deletes a captured node's subtree, so an ancestor
                // capturing the same receiver suppresses this one.
                auto suppressed = [&]() {
                  if (kStage) {
                    for (int q = 0; q < na; ++q) {
                      const AncRec& r = anc[warp][q];
                      ++anc_tests;
                      int w = reception32(make_float3(r.s[0], r.s[1], r.s[2]),
                                          make_float3(r.u[0], r.u[1], r.u[2]), r.len, r.S, c, tanb);
                      if (w < 0) {
                        ++n64;
                        w = capture_exact(A.nodes_cold, r.idx, c64, P.tan_beta);
                      }
                      if (w) return true;
                    }
                    return false;
                  }
                  for (uint32_t p = nd.parent; p != 0xFFFFFFFFu && p < A.node_cap;) {
                    const NodeHot a = A.nodes[p];
                    ++anc_tests;
                    int w = reception32(make_float3(a.s[0], a.s[1], a.s[2]),
                                        make_float3(a.u[0], a.u[1], a.u[2]), a.len, a.S, c, tanb);
                    if (w < 0) {
                      ++n64;
                      w = capture_exact(A.nodes_cold, p, c64, P.tan_beta);
                    }
                    if (w) return true;
                    p = a.parent;
                  }
                  return false;
                };
                if (kStage) {
                  if (suppressed()) continue;
                  ++events;
                }
                const bool ok = is_root_class(nd.cls)
                                    ? A.direct_ok[gi] != 0
                                    : correct_event(A.sc, A.cls_info, nd.cls, c, c64, n64);
                if (!ok) continue;
                if (!kStage && suppressed()) continue;
                const unsigned long long kk = atomicAdd(&A.ctr->corrected, 1ull);
                if (kk < A.corr_cap)
                  A.corr_list[kk] = Corrected{uint32_t(gi), nd.cls,
                                              (unsigned long long)nd.launch << kHeapBits | nd.heap};
                else
                  atomicOr(&A.ctr->overflow, kOvCorr);
              }
            }
          }
        }
      }
      __syncwarp();
    }
    __syncwarp();  // the next batch overwrites the staged records
  }
  for (int o = 16; o; o >>= 1) {
    events += __shfl_xor_sync(FULL, events, o);
    cand += __shfl_xor_sync(FULL, cand, o);
    anc_tests += __shfl_xor_sync(FULL, anc_tests, o);
    n64 += __shfl_xor_sync(FULL, n64, o);
  }
  if (lane == 0) {
    if (events) atomicAdd(&A.ctr->events, events);
    if (cand) atomicAdd(&A.ctr->cand, cand);
    if (anc_tests) atomicAdd(&A.ctr->anc, anc_tests);
    if (n64) atomicAdd(&A.ctr->fp64_capture, (unsigned long long)n64);
  }
}

// The FP64 part of capture for the pairs k_capture could not settle in FP32:
// the exact reception test where the FP32 one was unsure, then image
// correction (MultiPathCorrection / DirectPathCorrection) and suppression by
// an ancestor capturing the same receiver (RTSolver.cpp:277-284), as in
// k_capture.  One thread per pair keeps the FP64 pipe busy with full warps.
__global__ void __launch_bounds__(128) k_capture_finish(CaptureArgs A) {
  if (A.ctr->overflow & (kOvTrace | kOvPairs)) return;  // this solve will be repeated
  const unsigned long long n = min(A.ctr->pairs, A.pair_cap);
  unsigned n64 = 0;
  unsigned long long anc_tests = 0;
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    const uint2 pr = A.pairs[k];
    const uint32_t i = pr.x;
    const int gi = int(pr.y & 0x7fffffffu);
    const NodeHot nd = A.nodes[i];
    const TxParams& P = A.txp[nd.tx];
    const double* c64 = A.rx + 3 * size_t(gi);
    if (pr.y >> 31) {
      ++n64;
      if (!capture_exact(A.nodes_cold, i, c64, P.tan_beta)) continue;
    }
    const float3 c = make_float3(float(c64[0]), float(c64[1]), float(c64[2]));
    const bool ok = is_root_class(nd.cls) ? A.direct_ok[gi] != 0
                                          : correct_event(A.sc, A.cls_info, nd.cls, c, c64, n64);
    if (!ok) continue;
    const float tanb = float(P.tan_beta);
    bool sup = false;
    for (uint32_t p = nd.parent; p != 0xFFFFFFFFu && p < A.node_cap;) {
      const NodeHot a = A.nodes[p];
      ++anc_tests;
      int w = reception32(make_float3(a.s[0], a.s[1], a.s[2]), make_float3(a.u[0], a.u[1], a.u[2]),
                          a.len, a.S, c, tanb);
      if (w < 0) {
        ++n64;
        w = capture_exact(A.nodes_cold, p, c64, P.tan_beta);
      }
      if (w) {
        sup = true;
        break;
      }
      p = a.parent;
    }
    if (sup) continue;
    const unsigned long long kk = atomicAdd(&A.ctr->corrected, 1ull);
    if (kk < A.corr_cap)
      A.corr_list[kk] =
          Corrected{uint32_t(gi), nd.cls, (unsigned long long)nd.launch << kHeapBits | nd.heap};
    else
      atomicOr(&A.ctr->overflow, kOvCorr);
  }
  for (int o = 16; o; o >>= 1) {
    anc_tests += __shfl_xor_sync(0xffffffffu, anc_tests, o);
    n64 += __shfl_xor_sync(0xffffffffu, n64, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (anc_tests) atomicAdd(&A.ctr->anc, anc_tests);
    if (n64) atomicAdd(&A.ctr->fp64_capture, (unsigned long long)n64);
  }
}

// ---- correction / dedup -----------------------------------------------------

struct PathBuf {
  int n;            // rays
  int tri[kMaxDepth + 1];
  int kind[kMaxDepth + 1];
  double pts[kMaxDepth + 2][3];
};

// Path of a class: tri of each ray (ray i ends on tri[i]; the last ray ends at
// the receiver) and kind of each ray's start.
__device__ __forceinline__ bool class_path(const ClassInfo* info, uint32_t cls, PathBuf& pb) {
  int depth = 0;
  int tri_rev[kMaxDepth], kind_rev[kMaxDepth];
  for (uint32_t c = cls; !is_root_class(c); c = info[c].parent) {
    if (depth >= kMaxDepth) return false;
    tri_rev[depth] = info[c].tri;
    kind_rev[depth] = info[c].kind;
    ++depth;
  }
  pb.n = depth + 1;
  pb.kind[0] = 0;
  for (int i = 0; i < depth; ++i) {
    pb.tri[i] = tri_rev[depth - 1 - i];   // rank of the triangle hit by ray i
    pb.kind[i + 1] = kind_rev[depth - 1 - i];
  }
  pb.tri[depth] = -1;
  return true;
}

// GetImageSources + MultiPathCorrection / DirectPathCorrection
// (RTSolver.cpp:330-433).  Fills pb.pts with the corrected points.
__device__ bool correct_path(const DevScene& sc, const int* rank_to_id, const TxParams& P,
                             const double* rxp, PathBuf& pb, unsigned* overflow) {
  using namespace x64;
  const double* tx = P.tx;
  if (pb.n == 1) {
    double d[3];
    sub3(rxp, tx, d);
    Hit h;
    const bool has = exact_closest(sc, tx, d, h, overflow);
    if (has && !(norm(d) < h.dist)) return false;
    for (int a = 0; a < 3; ++a) {
      pb.pts[0][a] = tx[a];
      pb.pts[1][a] = rxp[a];
    }
    return true;
  }
  const int n = pb.n;
  double img[kMaxDepth + 1][3];
  for (int a = 0; a < 3; ++a) img[0][a] = tx[a];
  for (int i = 0; i + 1 < n; ++i) {
    const CorrTri& T = sc.corr[rank_to_id[pb.tri[i]]];
    if (pb.kind[i + 1] == 1) {  // ImagePoint (RTSolver.cpp:910-924)
      double w[3];
      sub3(img[i], T.v1, w);
      const double dist = dot(T.n, w);
      for (int a = 0; a < 3; ++a) img[i + 1][a] = sub(img[i][a], mul(mul(2.0, dist), T.n[a]));
    } else {
      for (int a = 0; a < 3; ++a) img[i + 1][a] = img[i][a];
    }
  }
  double target[3] = {rxp[0], rxp[1], rxp[2]};
  for (int a = 0; a < 3; ++a) pb.pts[n][a] = rxp[a];
  for (int i = n - 1; i >= 1; --i) {
    const CorrTri& T = sc.corr[rank_to_id[pb.tri[i - 1]]];
    double d[3], P3[3];
    sub3(target, img[i], d);
    if (!mt64c(T, img[i], d, P3)) return false;
    for (int a = 0; a < 3; ++a) {
      pb.pts[i][a] = P3[a];
      target[a] = P3[a];
    }
  }
  for (int a = 0; a < 3; ++a) pb.pts[0][a] = tx[a];
  return true;
}

// DirectPathCorrection (RTSolver.cpp:375-394) once per receiver: the direct
// path survives iff the reference-order BVH query from the transmitter along
// (rx - tx) finds nothing closer than the receiver.
__global__ void k_direct(DevScene sc, const TxParams* txp, const double* rx, const int* rx_req,
                         int n_rx, unsigned char* ok, Counters* ctr) {
  for (int gi = blockIdx.x * blockDim.x + threadIdx.x; gi < n_rx; gi += gridDim.x * blockDim.x) {
    const double* tx = txp[rx_req[gi]].tx;
    const double* c = rx + 3 * size_t(gi);
    double d[3];
    x64::sub3(c, tx, d);
    Hit h;
    TraceStats st{0, 0};
    const bool has = closest_hit(sc, tx, d, h, st, &ctr->overflow);
    ok[gi] = (!has || x64::norm(d) < h.dist) ? 1 : 0;
  }
}

// RemoveDuplicatePath (RTSolver.cpp:435-459): the first corrected path in
// (launch, BFS) order wins each (receiver, coplanar key).
__device__ __forceinline__ unsigned long long dedup_key(const ClassInfo* info, const Corrected& e) {
  const uint32_t cop = is_root_class(e.cls) ? kRootClass : info[e.cls].cop;
  return (unsigned long long)e.rx << 32 | cop;
}

__global__ void k_dedup(const Corrected* list, unsigned long long cap, const ClassInfo* info,
                        HashTable dedup, unsigned long long* dedup_rank, Counters* ctr) {
  const unsigned long long n = min(ctr->corrected, cap);
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const Corrected e = list[i];
    const uint32_t ds = ht_insert(dedup, dedup_key(info, e), &ctr->overflow, kOvDedup, &ctr->used_dd,
                                &ctr->lost_dd);
    if (ds != 0xFFFFFFFFu) atomicMin(&dedup_rank[ds], e.rank);
  }
}

struct Survivor {
  uint32_t cls, rx;
  unsigned long long rank;
};

__global__ void k_select(const Corrected* list, unsigned long long cap, const ClassInfo* info,
                         HashTable dedup, const unsigned long long* dedup_rank, Survivor* surv,
                         unsigned long long surv_cap, Counters* ctr) {
  const unsigned long long n = min(ctr->corrected, cap);
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const Corrected e = list[i];
    const uint32_t ds = ht_find(dedup, dedup_key(info, e));
    if (ds == 0xFFFFFFFFu || dedup_rank[ds] != e.rank) continue;
    const unsigned long long k = atomicAdd(&ctr->survivors, 1ull);
    if (k < surv_cap) surv[k] = Survivor{e.cls, e.rx, e.rank};
    else atomicOr(&ctr->overflow, kOvSurv);
  }
}

// ---- field ---------------------------------------------------------------

struct FieldArgs {
  DevScene sc;
  const TxParams* txp;
  const double* rx;
  const int* rx_req;
  const ClassInfo* cls_info;
  const int* rank_to_id;
  const Survivor* surv;
  Counters* ctr;
  unsigned long long cap;
  FieldConsts K;
  int precision;        // -1: each request's own; 0: FP64 for all (the FP64 shadow)
  double* path_field;   // 6 per survivor
  int* path_nray;
  int* path_tri;        // (kMaxDepth + 1) per survivor: triangle id
  int* path_cop;
  int* path_kind;
  int* path_near_edge;  // 1 if an interaction point is within 1e-6 of its triangle's edge
  double* path_pts;     // (kMaxDepth + 2) * 3 per survivor
};

// Barycentric distance of a point (on the triangle's plane) from the
// triangle's edges is below tol: min(u, v, 1-u-v) < tol.
__device__ __forceinline__ int near_edge(const CorrTri& T, const double* p, double tol) {
  double w[3] = {p[0] - T.v1[0], p[1] - T.v1[1], p[2] - T.v1[2]};
  const double d00 = T.e1[0] * T.e1[0] + T.e1[1] * T.e1[1] + T.e1[2] * T.e1[2];
  const double d01 = T.e1[0] * T.e2[0] + T.e1[1] * T.e2[1] + T.e1[2] * T.e2[2];
  const double d11 = T.e2[0] * T.e2[0] + T.e2[1] * T.e2[1] + T.e2[2] * T.e2[2];
  const double d20 = w[0] * T.e1[0] + w[1] * T.e1[1] + w[2] * T.e1[2];
  const double d21 = w[0] * T.e2[0] + w[1] * T.e2[1] + w[2] * T.e2[2];
  const double den = d00 * d11 - d01 * d01;
  if (!(den > 0)) return 1;
  const double u = (d11 * d20 - d01 * d21) / den, v = (d00 * d21 - d01 * d20) / den;
  return fmin(fmin(u, v), 1.0 - u - v) < tol ? 1 : 0;
}

__global__ void k_field(FieldArgs A) {
  const unsigned long long ns = min(A.ctr->survivors, A.cap);
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < ns;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const Survivor sv = A.surv[i];
    const uint32_t cls = sv.cls;
    const TxParams& P = A.txp[A.rx_req[sv.rx]];
    PathBuf pb;
    class_path(A.cls_info, cls, pb);
    correct_path(A.sc, A.rank_to_id, P, A.rx + 3 * size_t(sv.rx), pb, &A.ctr->overflow);
    const double* frames[kMaxDepth + 1];
    int mat[kMaxDepth + 1];
    mat[0] = 0;
    for (int r = 0; r < pb.n; ++r) {
      frames[r] = pb.tri[r] >= 0 ? A.sc.corr[A.rank_to_id[pb.tri[r]]].cs : nullptr;
      if (r + 1 < pb.n) mat[r + 1] = A.sc.tri64[pb.tri[r]].mat;
    }
    Cx<double> e[3];
    const PatternTab pat{P.pat, P.pat_nt, P.pat_np, P.pat_dt, P.pat_dp};
    const int prec = A.precision < 0 ? P.precision : A.precision;
    if (prec == 2)
      path_field<float, true>(pb.n, pb.pts, frames, pb.kind, mat, A.sc.mats, P.txcs, P.freq,
                              P.pt, P.antenna, P.fresnel != 0, A.K, e, &pat);
    else if (prec == 1)
      path_field<float>(pb.n, pb.pts, frames, pb.kind, mat, A.sc.mats, P.txcs, P.freq, P.pt,
                        P.antenna, P.fresnel != 0, A.K, e, &pat);
    else
      path_field<double>(pb.n, pb.pts, frames, pb.kind, mat, A.sc.mats, P.txcs, P.freq, P.pt,
                         P.antenna, P.fresnel != 0, A.K, e, &pat);
    for (int j = 0; j < 3; ++j) {
      A.path_field[6 * i + 2 * j] = e[j].re;
      A.path_field[6 * i + 2 * j + 1] = e[j].im;
    }
    A.path_nray[i] = pb.n;
    const size_t b = size_t(i) * (kMaxDepth + 1);
    for (int r = 0; r < pb.n; ++r) {
      const int t = pb.tri[r];
      A.path_tri[b + r] = t >= 0 ? A.rank_to_id[t] : -1;
      A.path_cop[b + r] = t >= 0 ? A.sc.tri64[t].cop : -1;
      A.path_kind[b + r] = pb.kind[r];
    }
    const size_t bp = size_t(i) * (kMaxDepth + 2) * 3;
    for (int r = 0; r <= pb.n; ++r)
      for (int a = 0; a < 3; ++a) A.path_pts[bp + 3 * r + a] = pb.pts[r][a];
    // interaction point r+1 lies on the triangle the correction intersected
    int near = 0;
    for (int r = 0; r + 1 < pb.n; ++r)
      near |= near_edge(A.sc.corr[A.rank_to_id[pb.tri[r]]], pb.pts[r + 1], 1e-6);
    A.path_near_edge[i] = near;
  }
}

// ---- per-receiver ordered sum -------------------------------------------

__global__ void k_surv_hist(const Survivor* surv, const Counters* ctr, unsigned long long cap,
                            int* counts) {
  const unsigned long long ns = min(ctr->survivors, cap);
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < ns;
       i += (unsigned long long)gridDim.x * blockDim.x)
    atomicAdd(&counts[surv[i].rx], 1);
}

__global__ void k_surv_scatter(const Survivor* surv, const Counters* ctr, unsigned long long cap,
                               const int* starts, int* cursor, int* order) {
  const unsigned long long ns = min(ctr->survivors, cap);
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < ns;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const uint32_t r = surv[i].rx;
    order[starts[r] + atomicAdd(&cursor[r], 1)] = int(i);
  }
}

// Sort each receiver's survivors by (launch, BFS) rank and sum their fields in
// that order: FP64, or compensated FP32 (Neumaier) for the FP32 precisions.
// precision -1 takes each receiver's request precision, 0 forces FP64.
__global__ void k_rx_sum(const Survivor* surv, const int* starts, int* order, int n_rx,
                         const double* path_field, int force_precision, const int* rx_req,
                         const TxParams* txp, double* field) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rx; r += gridDim.x * blockDim.x) {
    const int precision = force_precision < 0 ? txp[rx_req[r]].precision : force_precision;
    const int b = starts[r], e = starts[r + 1];
    for (int i = b + 1; i < e; ++i) {
      const int v = order[i];
      const unsigned long long key = surv[v].rank;
      int j = i - 1;
      while (j >= b && surv[order[j]].rank > key) {
        order[j + 1] = order[j];
        --j;
      }
      order[j + 1] = v;
    }
    if (precision != 0) {  // both FP32 modes: compensated FP32 sum
      float s[6] = {0, 0, 0, 0, 0, 0}, c[6] = {0, 0, 0, 0, 0, 0};
      for (int i = b; i < e; ++i)
        for (int k = 0; k < 6; ++k) {
          const float x = float(path_field[6 * size_t(order[i]) + k]);
          const float t = s[k] + x;
          c[k] += fabsf(s[k]) >= fabsf(x) ? (s[k] - t) + x : (x - t) + s[k];
          s[k] = t;
        }
      for (int k = 0; k < 6; ++k) field[6 * size_t(r) + k] = double(s[k]) + double(c[k]);
    } else {
      double s[6] = {0, 0, 0, 0, 0, 0};
      for (int i = b; i < e; ++i)
        for (int k = 0; k < 6; ++k) s[k] = __dadd_rn(s[k], path_field[6 * size_t(order[i]) + k]);
      for (int k = 0; k < 6; ++k) field[6 * size_t(r) + k] = s[k];
    }
  }
}

// ============================================================ host side

// Buffers, stream and capacities of one solve in flight.  A scene keeps a
// pool of these so that solves issued from several host threads run on
// separate streams and overlap on the GPU.
struct Workspace {
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[8] = {};
  DBuf<TxParams> txp;
  DBuf<double> rx;
  DBuf<int> rx_req;
  DBuf<GridBuild> gb;
  DBuf<RxGrid> grids;
  DBuf<int> cell_base, cell_counts, cell_starts, cell_cursor;
  DBuf<float4> rx32;
  DBuf<RayRec> q0, q1;
  DBuf<NodeHot> nodes;
  DBuf<NodeCold> nodes_cold;
  DBuf<unsigned long long> cls_keys, cop_keys, dd_keys, dd_rank;
  DBuf<ClassInfo> cls_info;
  DBuf<ClassCap> cls_cap;
  DBuf<Corrected> corr_list;
  DBuf<uint2> pairs;  // capture pairs left to the FP64 pass
  DBuf<unsigned char> direct_ok;
  DBuf<Survivor> surv;
  DBuf<int> s_counts, s_starts, s_cursor, s_order;
  DBuf<double> path_field, path_pts, field;
  DBuf<double> path_field64, field64;  // FP64 shadow of an FP32 field (field_check)
  DBuf<int> path_nray, path_tri, path_cop, path_kind, path_near;
  DBuf<Counters> ctr;
  DBuf<unsigned long long> seg_tx;
  DBuf<uint2> cand;                    // FP32 search contenders, kCand per ray of a chunk
  DBuf<unsigned char> ncand;
  DBuf<unsigned long long> find_work;  // work counter of the running search launch
  // capacities (grown from occupancy and on overflow)
  unsigned long long cap_nodes = 1 << 20, cap_queue = 1 << 19, cap_surv = 1 << 14;
  unsigned long long cap_corr = 1 << 16, cap_pairs = 1 << 20;
  uint32_t cap_cls = 1 << 16, cap_cop = 1 << 14, cap_dd = 1 << 14;
  // occupancy seen per executed segment in earlier solves, used to size the
  // tables of the next solve before it runs
  // (first solve: values typical of the urban canyon, so most first solves
  // need no retry)
  double r_cls = 0.01, r_cop = 0.004, r_corr = 0.01, r_dd = 5e-4, r_surv = 5e-4, r_pairs = 0.1;
  ~Workspace() {
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
  }
};

struct SceneImpl {
  HostScene host;
  std::vector<sbr_material> materials;
  int device = 0;
  cudaStream_t stream = nullptr;  // scene uploads
  DBuf<Node32> node32;
  DBuf<RefNode> ref;
  DBuf<Tri32> tri32;
  DBuf<Tri64> tri64;
  DBuf<Node32> snode;
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

static void upload_scene(SceneImpl& S) {
  const HostScene& H = S.host;
  const int nt = int(H.tris.size()), nn = int(H.nodes.size());
  std::vector<Node32> n32(nn);
  std::vector<RefNode> ref(nn);
  const double margin_m = std::ldexp(H.extent + 1.0, -14);
  for (int i = 0; i < nn; ++i) {
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
  std::vector<Tri32> t32(nt);
  std::vector<Tri64> t64(nt);
  std::vector<int> cop(nt), r2i(nt);
  for (int r = 0; r < nt; ++r) {
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
  for (int i = 0; i < nn; ++i)
    if (H.nodes[i].c0 < 0)
      for (int r = H.nodes[i].first; r < H.nodes[i].first + H.nodes[i].count; ++r) t64[r].node = i;
  S.n_cop = 0;
  for (auto& t : H.tris) S.n_cop = std::max(S.n_cop, t.cop + 1);
  std::vector<Material> mats(S.materials.size());
  for (size_t i = 0; i < mats.size(); ++i)
    mats[i] = Material{S.materials[i].rel_permittivity_re, S.materials[i].rel_conductivity};
  cudaStream_t st = S.stream;
  S.node32.upload(n32.data(), n32.size(), st);
  S.ref.upload(ref.data(), ref.size(), st);
  S.tri32.upload(t32.data(), t32.size(), st);
  S.tri64.upload(t64.data(), t64.size(), st);
  S.mats.upload(mats.data(), mats.size(), st);
  {  // search BVH
    const SearchBVH& B = H.search;
    std::vector<Node32> sn(B.nodes.size());
    for (size_t i = 0; i < B.nodes.size(); ++i) {
      Node32& m = sn[i];
      std::memset(&m, 0, sizeof m);
      for (int a = 0; a < 3; ++a) {
        m.lo0[a] = B.nodes[i].lo[0][a];
        m.hi0[a] = B.nodes[i].hi[0][a];
        m.lo1[a] = B.nodes[i].lo[1][a];
        m.hi1[a] = B.nodes[i].hi[1][a];
      }
      m.child[0] = B.nodes[i].child[0];
      m.child[1] = B.nodes[i].child[1];
    }
    std::vector<Tri32> st32(B.order.size());
    for (size_t j = 0; j < B.order.size(); ++j) st32[j] = t32[B.order[j]];
    S.snode.upload(sn.data(), sn.size(), st);
    S.stri.upload(st32.data(), st32.size(), st);
    S.srank.upload(B.order.data(), B.order.size(), st);
    S.dev.snode = S.snode.p;
    S.dev.stri = S.stri.p;
    S.dev.srank = S.srank.p;
    CK(cudaStreamSynchronize(st));  // the host vectors above go out of scope
  }
  {  // every reference leaf's boxes up to the root, one run per leaf
    std::vector<AncBox> ab;
    std::vector<int> off(nn, -1);
    for (int i = 0; i < nn; ++i) {
      if (H.nodes[i].c0 >= 0) continue;
      off[i] = int(ab.size());
      for (int n = i; n >= 0; n = H.nodes[n].parent) {
        AncBox b;
        std::memcpy(b.fb, ref[n].fb, sizeof b.fb);
        b.flat = ref[n].flat;
        b.node = n;
        ab.push_back(b);
      }
      AncBox end;
      std::memset(&end, 0, sizeof end);
      end.node = -1;
      ab.push_back(end);
    }
    S.anc.upload(ab.data(), ab.size(), st);
    S.anc_off.upload(off.data(), off.size(), st);
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
                            S.snode.n * sizeof(Node32) + S.stri.n * sizeof(Tri32) +
                            S.srank.n * sizeof(int) + S.anc.n * sizeof(AncBox) +
                            S.anc_off.n * sizeof(int));
  CK(cudaStreamSynchronize(st));
}

// corr[id] = the triangle at mesh position id (what triangleMesh[id] returns).
static void upload_mesh_order(SceneImpl& S, const std::vector<int>& order) {
  const HostScene& H = S.host;
  const int nt = int(H.tris.size());
  std::vector<CorrTri> c(nt);
  for (int i = 0; i < nt; ++i) {
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
  std::vector<Tri32> c32(nt);
  for (int i = 0; i < nt; ++i) {
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

// Persistent grid of the FP32 search: as many blocks as fit on the device.
static int find_grid() {
  static int g = [] {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_find, 128, 0);
    return std::max(1, sms) * std::max(1, per_sm);
  }();
  return g;
}

static int grid_for(long long n, int block) {
  int dev_sms = 152;
  long long g = (n + block - 1) / block;
  return int(std::max<long long>(1, std::min<long long>(g, (long long)dev_sms * 32)));
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

// force_check: compute the FP64 shadow field even if no request here asks for
// it (another pass of the same batch did).
static void solve_impl(SceneImpl& S, Workspace& W, const sbr_request* reqs, int n_req,
                       sbr_result& out, bool force_check = false) {
  long long nl = 0;  // kernel launches of this solve (all attempts)
  cudaStream_t st = W.stream;
  if (S.host.mesh_order.empty()) throw std::string("scene is not initialised");
  CK(cudaSetDevice(S.device));
  if (!W.stream) CK(cudaStreamCreateWithFlags(&W.stream, cudaStreamNonBlocking));
  if (!W.ev[0])
    for (auto& e : W.ev) CK(cudaEventCreate(&e));
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
    if (!(q.frequency > 0)) throw std::string("frequency must be > 0");
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
  CK(cudaEventRecord(W.ev[0], st));
  W.txp.upload(tp.data(), tp.size(), st);
  // receivers
  W.rx.ensure(std::max(1, 3 * rx_total));
  W.direct_ok.ensure(std::max(1, rx_total));
  {
    std::vector<int> req_of(std::max(1, rx_total));
    for (int r = 0; r < n_req; ++r) {
      const sbr_request& q = reqs[r];
      if (q.n_rx)
        CK(cudaMemcpyAsync(W.rx.p + 3 * size_t(tp[r].rx_first), q.rx, 3 * sizeof(double) * q.n_rx,
                           q.rx_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
      for (int i = 0; i < q.n_rx; ++i) req_of[tp[r].rx_first + i] = r;
    }
    W.rx_req.upload(req_of.data(), req_of.size(), st);
  }
  CK(cudaEventRecord(W.ev[1], st));
  // ---- receiver grid
  // cells per request: the grid aims at ~2 receivers per cell
  int max_cells = 64;
  for (auto& p : tp) max_cells = std::max(max_cells, 2 * p.n_rx + 64);
  max_cells = std::min(max_cells, 1 << 21);
  W.gb.ensure(n_req);
  {
    std::vector<GridBuild> g0(n_req);
    for (auto& g : g0) {
      for (int a = 0; a < 3; ++a) {
        g.bmin[a] = INT_MAX;
        g.bmax[a] = INT_MIN;
      }
      g.cmax_o = INT_MIN;
      g.cmax = 0;
      g.ncell = 0;
    }
    CK(cudaMemcpyAsync(W.gb.p, g0.data(), sizeof(GridBuild) * n_req, cudaMemcpyHostToDevice, st));
  }
  W.grids.ensure(n_req);
  W.cell_base.ensure(n_req + 1);
  const size_t cell_cap = size_t(n_req) * (max_cells + 1) + 1;
  W.cell_counts.ensure(cell_cap);
  W.cell_starts.ensure(cell_cap + 1);
  W.cell_cursor.ensure(cell_cap);
  W.rx32.ensure(std::max(1, rx_total));
  CK(cudaMemsetAsync(W.cell_counts.p, 0, sizeof(int) * cell_cap, st));
  CK(cudaMemsetAsync(W.cell_cursor.p, 0, sizeof(int) * cell_cap, st));
  int max_rx = 1;
  for (auto& p : tp) max_rx = std::max(max_rx, p.n_rx);
  dim3 rg(std::min(1024, (max_rx + 255) / 256), n_req);
  ++nl, k_rx_bounds<<<rg, 256, 0, st>>>(W.rx.p, W.txp.p, n_req, W.gb.p);
  ++nl, k_grid_shape<<<1, 1, 0, st>>>(W.gb.p, W.grids.p, W.txp.p, n_req, max_cells, W.cell_base.p);
  ++nl, k_rx_count<<<rg, 256, 0, st>>>(W.rx.p, W.txp.p, n_req, W.grids.p, W.cell_base.p, W.cell_counts.p);
  ++nl, k_scan_exclusive<<<1, 1024, 0, st>>>(W.cell_counts.p, W.cell_starts.p, int(cell_cap));
  ++nl, k_rx_scatter<<<rg, 256, 0, st>>>(W.rx.p, W.txp.p, n_req, W.grids.p, W.cell_base.p,
                                   W.cell_starts.p, W.cell_cursor.p, W.rx32.p);
  ++nl, k_grid_finish<<<(n_req + 127) / 128, 128, 0, st>>>(W.grids.p, W.cell_starts.p, W.cell_base.p,
                                                    W.rx32.p, n_req);
  CK(cudaGetLastError());

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
    W.cop_keys.ensure(W.cap_cop);
    W.corr_list.ensure(W.cap_corr);
    W.pairs.ensure(W.cap_pairs);
    W.dd_keys.ensure(W.cap_dd);
    W.dd_rank.ensure(W.cap_dd);
    W.surv.ensure(W.cap_surv);
    CK(cudaMemsetAsync(W.ctr.p, 0, sizeof(Counters), st));
    W.seg_tx.ensure(n_req);
    CK(cudaMemsetAsync(W.seg_tx.p, 0, sizeof(unsigned long long) * n_req, st));
    const int fb = 256;
    ++nl, k_fill_u64<<<grid_for(W.cap_cls, fb), fb, 0, st>>>(W.cls_keys.p, W.cap_cls, kEmptyKey);
    ++nl, k_fill_u64<<<grid_for(W.cap_cop, fb), fb, 0, st>>>(W.cop_keys.p, W.cap_cop, kEmptyKey);
    ++nl, k_fill_u64<<<grid_for(W.cap_dd, fb), fb, 0, st>>>(W.dd_keys.p, W.cap_dd, kEmptyKey);
    ++nl, k_fill_u64<<<grid_for(W.cap_dd, fb), fb, 0, st>>>(W.dd_rank.p, W.cap_dd, kEmptyKey);
    CK(cudaEventRecord(W.ev[2], st));
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
    ta.tri_cop = S.tri_cop.p;
    ta.ctr = W.ctr.p;
    ta.seg_per_tx = W.seg_tx.p;
    ta.n_root = launches;
    // Each depth runs in chunks of at most kTraceChunk rays: the FP32
    // search (k_find) stores the chunk's contenders, then k_trace resolves
    // them in FP64 and spawns the next depth.  The ray count of a depth > 0
    // is on the device; chunks past it return at once.
    constexpr long long kTraceChunk = 1LL << 24;
    const long long max_width = std::max<long long>(launches, (long long)W.cap_queue);
    const long long chunk = std::max<long long>(1, std::min(kTraceChunk, max_width));
    W.cand.ensure(size_t(chunk) * kCand);
    W.ncand.ensure(size_t(chunk));
    W.find_work.ensure(1);
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
    ta.cand = W.cand.p;
    ta.ncand = W.ncand.p;
    for (int d = 0; d <= max_depth; ++d) {
      ta.depth = fnd.depth = d;
      ta.in = fnd.in = (d % 2 == 0) ? W.q1.p : W.q0.p;
      ta.out = (d % 2 == 0) ? W.q0.p : W.q1.p;
      const long long bound = d == 0 ? launches : (long long)W.cap_queue;
      for (long long lo = 0; lo < bound; lo += chunk) {
        ta.lo = fnd.lo = lo;
        ta.hi = fnd.hi = std::min(bound, lo + chunk);
        CK(cudaMemsetAsync(W.find_work.p, 0, sizeof(unsigned long long), st));
        ++nl, k_find<<<find_grid(), 128, 0, st>>>(fnd);
        ++nl, k_trace<<<grid_for(ta.hi - lo, 128), 128, 0, st>>>(ta);
      }
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(W.ev[3], st));
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
    if (rx_total)
      ++nl, k_direct<<<grid_for(rx_total, 64), 64, 0, st>>>(S.dev, W.txp.p, W.rx.p, W.rx_req.p, rx_total,
                                                      W.direct_ok.p, W.ctr.p);
    if (stage_counts) {
      ++nl, k_capture<true><<<152 * 32, 32 * kCapWarps, 0, st>>>(ca);
    } else {
      ++nl, k_capture<false><<<152 * 32, 32 * kCapWarps, 0, st>>>(ca);
      ++nl, k_capture_finish<<<152 * 16, 128, 0, st>>>(ca);
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(W.ev[4], st));
    // ---- duplicate removal over the corrected captures
    const HashTable dd{W.dd_keys.p, W.cap_dd - 1};
    ++nl, k_dedup<<<grid_for(W.cap_corr, 256), 256, 0, st>>>(W.corr_list.p, W.cap_corr, W.cls_info.p,
                                                       dd, W.dd_rank.p, W.ctr.p);
    ++nl, k_select<<<grid_for(W.cap_corr, 256), 256, 0, st>>>(W.corr_list.p, W.cap_corr, W.cls_info.p,
                                                        dd, W.dd_rank.p, W.surv.p, W.cap_surv,
                                                        W.ctr.p);
    CK(cudaGetLastError());
    CK(cudaEventRecord(W.ev[5], st));
    Counters c;
    CK(cudaMemcpyAsync(&c, W.ctr.p, sizeof c, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (c.overflow & kOvStack) throw std::string("BVH deeper than the traversal stack");
    // keep every hash table at most half full for the next solve
    auto grow = [](uint32_t& cap, unsigned long long used) {
      while (used * 2 > cap && cap < (1u << 30)) cap *= 2;
    };
    grow(W.cap_cls, c.used_cls);
    grow(W.cap_cop, c.used_cop);
    grow(W.cap_dd, c.used_dd);
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
      upd(W.r_corr, c.corrected / n);
      upd(W.r_surv, c.survivors / n);
      upd(W.r_pairs, c.pairs / n);
    }
    // ---- field + ordered per-receiver sum
    const unsigned long long ns = c.survivors;
    const size_t nsa = std::max<size_t>(1, ns);
    W.path_field.ensure(6 * nsa);
    W.path_nray.ensure(nsa);
    W.path_tri.ensure(nsa * (kMaxDepth + 1));
    W.path_cop.ensure(nsa * (kMaxDepth + 1));
    W.path_kind.ensure(nsa * (kMaxDepth + 1));
    W.path_near.ensure(nsa);
    W.path_pts.ensure(nsa * (kMaxDepth + 2) * 3);
    W.field.ensure(std::max(1, 6 * rx_total));
    W.s_counts.ensure(rx_total + 1);
    W.s_starts.ensure(rx_total + 2);
    W.s_cursor.ensure(rx_total + 1);
    W.s_order.ensure(nsa);
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
    if (ns) ++nl, k_field<<<grid_for(ns, 64), 64, 0, st>>>(fa);
    CK(cudaMemsetAsync(W.s_counts.p, 0, sizeof(int) * (rx_total + 1), st));
    CK(cudaMemsetAsync(W.s_cursor.p, 0, sizeof(int) * (rx_total + 1), st));
    if (ns) ++nl, k_surv_hist<<<grid_for(ns, 256), 256, 0, st>>>(W.surv.p, W.ctr.p, W.cap_surv, W.s_counts.p);
    ++nl, k_scan_exclusive<<<1, 1024, 0, st>>>(W.s_counts.p, W.s_starts.p, rx_total);
    if (ns)
      ++nl, k_surv_scatter<<<grid_for(ns, 256), 256, 0, st>>>(W.surv.p, W.ctr.p, W.cap_surv,
                                                        W.s_starts.p, W.s_cursor.p, W.s_order.p);
    if (rx_total)
      ++nl, k_rx_sum<<<grid_for(rx_total, 128), 128, 0, st>>>(W.surv.p, W.s_starts.p, W.s_order.p,
                                                        rx_total, W.path_field.p, -1, W.rx_req.p,
                                                        W.txp.p, W.field.p);
    CK(cudaGetLastError());
    CK(cudaEventRecord(W.ev[6], st));
    if (field_check) {  // FP64 shadow of the same paths, outside the timed stages
      W.path_field64.ensure(nsa * 6);
      W.field64.ensure(std::max(1, 6 * rx_total));
      FieldArgs f64 = fa;
      f64.precision = 0;
      f64.path_field = W.path_field64.p;
      if (ns) ++nl, k_field<<<grid_for(ns, 64), 64, 0, st>>>(f64);
      if (rx_total)
        ++nl, k_rx_sum<<<grid_for(rx_total, 128), 128, 0, st>>>(W.surv.p, W.s_starts.p, W.s_order.p,
                                                          rx_total, W.path_field64.p, 0,
                                                          W.rx_req.p, W.txp.p, W.field64.p);
      CK(cudaGetLastError());
    }
    // ---- results to the host
    out.field.resize(6 * size_t(rx_total));
    if (rx_total)
      CK(cudaMemcpyAsync(out.field.data(), W.field.p, sizeof(double) * 6 * rx_total,
                         cudaMemcpyDeviceToHost, st));
    out.field64.clear();
    if (field_check) {
      out.field64.resize(6 * size_t(rx_total));
      if (rx_total)
        CK(cudaMemcpyAsync(out.field64.data(), W.field64.p, sizeof(double) * 6 * rx_total,
                           cudaMemcpyDeviceToHost, st));
    }
    std::vector<int> order(ns), nray(ns), starts(rx_total + 1), pnear(ns);
    std::vector<Survivor> sv(ns);
    std::vector<double> pf(6 * ns), pts(ns * (kMaxDepth + 2) * 3);
    std::vector<int> ptri(ns * (kMaxDepth + 1)), pcop(ns * (kMaxDepth + 1)),
        pkind(ns * (kMaxDepth + 1));
    if (ns) {
      CK(cudaMemcpyAsync(order.data(), W.s_order.p, sizeof(int) * ns, cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(nray.data(), W.path_nray.p, sizeof(int) * ns, cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(pnear.data(), W.path_near.p, sizeof(int) * ns, cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(sv.data(), W.surv.p, sizeof(Survivor) * ns, cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(pf.data(), W.path_field.p, sizeof(double) * 6 * ns, cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(ptri.data(), W.path_tri.p, sizeof(int) * ptri.size(), cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(pcop.data(), W.path_cop.p, sizeof(int) * pcop.size(), cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(pkind.data(), W.path_kind.p, sizeof(int) * pkind.size(), cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(pts.data(), W.path_pts.p, sizeof(double) * pts.size(), cudaMemcpyDeviceToHost, st));
    }
    CK(cudaEventRecord(W.ev[7], st));
    CK(cudaStreamSynchronize(st));
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
    float ms[8] = {};
    for (int i = 1; i < 8; ++i) CK(cudaEventElapsedTime(&ms[i], W.ev[i - 1], W.ev[i]));
    out.timing.h2d_ms = ms[1];
    out.timing.trace_ms = ms[3];
    out.timing.capture_ms = ms[4];
    out.timing.correct_ms = ms[5];
    out.timing.field_ms = ms[6];
    out.timing.d2h_ms = ms[7];
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
const char* sbr_version(void) { return "sbr-gb300 0.1 (sm_103a)"; }

static sbr_status scene_common(std::vector<float>& v, std::vector<float>& n, const int* mat_ids,
                               const sbr_material* materials, int n_materials, sbr_scene** out) {
  ABI_GUARD({
    if (!out) throw std::string("out is NULL");
    *out = nullptr;
    if (n_materials <= 0 || !materials) throw std::string("at least one material is required");
    const int nt = int(n.size() / 3);
    if (mat_ids)
      for (int i = 0; i < nt; ++i)
        if (mat_ids[i] < 0 || mat_ids[i] >= n_materials)
          throw std::string("material id out of range at triangle ") + std::to_string(i);
    auto sc = std::make_unique<sbr_scene>();
    SceneImpl& S = sc->impl;
    std::string err;
    if (!prepare_scene(nt, v.data(), n.data(), mat_ids, S.host, err)) throw err;
    if (S.host.max_depth + 4 > kStack)
      throw std::string("BVH depth ") + std::to_string(S.host.max_depth) +
          " exceeds the traversal stack (" + std::to_string(kStack) + ")";
    S.materials.assign(materials, materials + n_materials);
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
      cudaGetLastError();
      throw CudaError{cudaErrorNoDevice, "no CUDA device"};
    }
    CK(cudaGetDevice(&S.device));
    CK(cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking));
    upload_scene(S);
    upload_mesh_order(S, S.host.mesh_order);
    *out = sc.release();
    return SBR_OK;
  })
}

sbr_status sbr_scene_create(int n_triangles, const float* vertices, const float* normals,
                            const int* material_ids, const sbr_material* materials,
                            int n_materials, sbr_scene** out) {
  if (n_triangles <= 0 || !vertices || !normals) {
    set_err("sbr_scene_create: empty triangle list");
    return SBR_ERR_INVALID_ARG;
  }
  std::vector<float> v(vertices, vertices + 9 * size_t(n_triangles));
  std::vector<float> n(normals, normals + 3 * size_t(n_triangles));
  return scene_common(v, n, material_ids, materials, n_materials, out);
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
  return scene_common(v, n, material_ids, materials, n_materials, out);
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
    auto res = std::make_unique<sbr_result>();
    int first = 0;
    while (first < n_requests) {
      int last = first + 1;
      double acc = est(requests[first]);
      while (last < n_requests && acc + est(requests[last]) <= budget) acc += est(requests[last++]);
      if (first == 0 && last == n_requests) {
        solve_impl(S, *W, requests, n_requests, *res);
        break;
      }
      sbr_result part;
      solve_impl(S, *W, requests + first, last - first, part, batch_check);
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
