// Trace stage: the reference's RayLaunch (RTSolver.cpp:128-257) as a
// wavefront, one bounce depth per launch pair: k_find (FP32 candidate search
// on the search BVH) and k_trace (FP64 resolution against the reference BVH,
// tree node, children, path-class interning).
#pragma once

#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "sbr_device.h"
#include "sbr_field.cuh"
#include "sbr_kernels.cuh"
#include "sbr_common.cuh"

namespace sbr {

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
  uint32_t* cls_list;  // slots of the classes interned, in interning order
  const int* tri_cop;  // coplanar id by rank
  Counters* ctr;
  unsigned long long* seg_per_tx;  // executed segments per request
  int depth;
  long long n_root;    // total launches (depth 0)
  long long lo, hi;    // this launch covers rays [lo, hi) of the depth
  const uint2* cand;   // contenders of those rays (k_find)
  const unsigned char* ncand;
  const RayF32* ray32; // FP32 copies of those rays (k_find)
  unsigned long long* work;  // rays of the chunk handed out (zero at launch)
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
// last ray starts on the triangle at mesh position tpos: the FP32 image source
// and correction-filter terms (the cone follows in k_class_cones).
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
}

// Correction cones of the interned classes (one thread per class-table
// slot, after the trace): three planes through the image source and the
// last triangle's edges, formed in FP64 and rounded to FP32, so a plane's
// error is its FP32 rounding alone.
__global__ void k_class_cones(const uint32_t* list, const Counters* ctr, uint32_t cap,
                              const ClassInfo* info, DevScene sc, ClassCap* caps) {
  if (ctr->overflow & kOvTrace) return;  // this solve will be repeated
  const unsigned long long n = min(ctr->cls_listed, (unsigned long long)cap);
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    const uint32_t s = list[k];
    const ClassInfo& ci = info[s];
    const CorrTri& T = sc.corr[sc.rank_to_id[ci.tri]];
    ClassCap& cc = caps[s];
    double v[3][3];
    for (int a = 0; a < 3; ++a) {
      v[0][a] = T.v1[a];
      v[1][a] = T.v1[a] + T.e1[a];
      v[2][a] = T.v1[a] + T.e2[a];
    }
    const double* im = ci.img;
    const double g[3] = {(v[0][0] + v[1][0] + v[2][0]) / 3.0, (v[0][1] + v[1][1] + v[2][1]) / 3.0,
                         (v[0][2] + v[1][2] + v[2][2]) / 3.0};
    auto norm3 = [](const double* x) { return sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]); };
    const float tmag =
        float((norm3(im) + norm3(T.v1) + norm3(T.e1) + norm3(T.e2)) * (1.0 + 1e-6)) + 1.0f;
    for (int k = 0; k < 3; ++k) {
      const double* p = v[k];
      const double* q = v[k == 2 ? 0 : k + 1];
      const double a[3] = {p[0] - im[0], p[1] - im[1], p[2] - im[2]};
      const double b[3] = {q[0] - im[0], q[1] - im[1], q[2] - im[2]};
      const double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                           a[0] * b[1] - a[1] * b[0]};
      const double nn = norm3(n);
      // orient towards the triangle's centroid, which lies inside the cone
      const double gc = n[0] * (g[0] - im[0]) + n[1] * (g[1] - im[1]) + n[2] * (g[2] - im[2]);
      const double sg = gc > 0.0 ? 1.0 : -1.0;
      for (int c = 0; c < 3; ++c) cc.n[k][c] = float(sg * n[c]);
      cc.n[k][3] = float(sg * (n[0] * im[0] + n[1] * im[1] + n[2] * im[2]));
      cc.nn[k] = float(nn * (1.0 + 1e-6));
      cc.w[k] = cc.nn[k] * tmag;
      cc.gc[k] = float(fabs(gc));
      cc.inv_nx[k] = 1.0f / cc.n[k][0];
    }
  }
}

// Records an interned class's slot for k_class_cones (the list has the class
// table's capacity, which bounds the classes).
__device__ __forceinline__ void list_class(const TraceArgs& A, uint32_t cls) {
  const unsigned long long k = atomicAdd(&A.ctr->cls_listed, 1ull);
  if (k <= A.cls_tab.mask) A.cls_list[k] = cls;
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

// Ray i of bounce depth `depth`: a launch ray (depth 0) or a queued child.
__device__ __forceinline__ void load_ray(const TxParams* txp, int n_tx, const double* const* dirs,
                                         const RayRec* in, int depth, long long i, RayRec& r) {
  if (depth == 0) {
    int q;
    long long li;
    root_ray(txp, n_tx, dirs, i, r.o, r.d, q, li);
    r.total = 0.0;
    r.S = 0.0;
    r.parent = 0xFFFFFFFFu;
    r.orank = -1;
    r.cls = kRootBase + uint32_t(q);
    r.cop = kRootClass;
    r.launch = uint32_t(li);
    r.heap = 1;
    r.rc = r.tc = 0;
    r.tx = uint32_t(q);
  } else {
    r = in[i];
  }
}

// The tree node of a resolved ray (RTSolver.cpp:142-257): its record (hot
// FP32 part and cold FP64 part), the segment counted for its request.  A
// ray that hits nothing ends at src + 1e10 d (a launch) or src + 100 d
// (RTSolver.cpp:231,249).  Returns the node index.
__device__ __forceinline__ unsigned long long emit_node(NodeHot* nodes, NodeCold* cold,
                                                        unsigned long long cap, Counters* ctr,
                                                        unsigned long long* seg_per_tx,
                                                        const RayRec& r, bool root,
                                                        const float3& o32, const float3& d32,
                                                        bool hit, const Hit& h) {
  const unsigned long long ni = warp_reserve(&ctr->nodes, 1);
  {  // per-request segment count, one atomic per request present in the warp
    const unsigned peers = __match_any_sync(__activemask(), r.tx);
    if (int(lane_id()) == __ffs(peers) - 1)
      atomicAdd(&seg_per_tx[r.tx], (unsigned long long)__popc(peers));
  }
  if (ni < cap) {
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
    m.s[0] = o32.x; m.s[1] = o32.y; m.s[2] = o32.z;
    m.S = float(r.S);
    m.u[0] = d32.x; m.u[1] = d32.y; m.u[2] = d32.z;
    m.parent = r.parent;
    m.cls = r.cls;
    m.launch = r.launch;
    m.heap = r.heap;
    m.tx = r.tx;
    m.pad0 = m.pad1 = m.pad2 = 0;
    cold[ni] = n;
    nodes[ni] = m;
  } else {
    atomicOr(&ctr->overflow, kOvNodes);
  }
  return ni;
}

// The position of the j-th (0-based) set bit of m (j < popc(m)).
__device__ __forceinline__ int nth_set_bit(unsigned m, int j) {
  int p = 0;
  for (int w = 16; w >= 1; w >>= 1) {
    const int c = __popc(m & (((1u << w) - 1u) << p));  // set bits in [p, p + w)
    if (c <= j) {
      j -= c;
      p += w;
    }
  }
  return p;
}

// ---- FP32 candidate search (persistent, rays refilled per warp) ----------
//
// Each lane traverses one ray at a time.  Lanes whose ray is finished take a
// new one from the chunk's work counter (one atomic per warp, when at least
// half the warp is idle or nobody is busy), so warps stay full while rays of
// very different lengths finish at different times.  The search tree is
// four-wide; a step is one node visit (four child boxes) or up to
// tris_per_step triangle tests, so lanes in a leaf and lanes between nodes
// advance at a similar pace.  The FP32 copy of each ray it loads is kept for
// k_trace (ray32).
struct FindArgs {
  DevScene sc;
  const TxParams* txp;
  int n_tx;
  const double* const* dirs;
  RayRec* in;  // reflected rays get their direction normalised here
  const Counters* ctr;
  unsigned long long in_cap;
  long long n_root;
  int depth;
  long long lo, hi;            // this launch covers rays [lo, hi) of the depth
  unsigned long long* work;    // rays of the chunk handed out (zero at launch)
  uint2* cand;                 // kCand per ray of the chunk
  unsigned char* ncand;        // contenders per ray, kFindFallback = exact traversal
  RayF32* ray32;               // FP32 copy per ray of the chunk
  int steps;                   // traversal steps between refills
  int refill;                  // idle lanes that trigger a refill
  int tris_per_step;           // triangles of a leaf tested per step (1 or 2)
};

// Defaults of the search's tunables (the autotuner may choose others).
constexpr int kFindSteps = 32;
constexpr int kFindRefill = 16;

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
  int sp = 0, pending = -1, nc = 0, orank = -1;
  bool fail = false;
  uint2* out = nullptr;
  while (true) {
    const bool idle = ray < 0 && !exhausted;
    const unsigned im = __ballot_sync(0xffffffffu, idle);
    const unsigned busy = __ballot_sync(0xffffffffu, ray >= 0);
    if (im && (__popc(im) >= A.refill || busy == 0)) {
      const int leader = __ffs(im) - 1;
      unsigned long long base = 0;
      if (int(lane) == leader) base = atomicAdd(A.work, (unsigned long long)__popc(im));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (idle) {
        const long long k = (long long)base + __popc(im & ((1u << lane) - 1u));
        if (k < n) {
          ray = k;
          double o[3], d[3];
          orank = -1;
          if (A.depth == 0) {
            int q;
            long long li;
            root_ray(A.txp, A.n_tx, A.dirs, A.lo + k, o, d, q, li);
          } else {
            RayRec& r = A.in[A.lo + k];
            for (int a = 0; a < 3; ++a) {
              o[a] = r.o[a];
              d[a] = r.d[a];
            }
            if (r.heap & 1) {
              // a reflected ray (heap 2h+1) arrives with Reflect(d, n) not yet
              // normalised: normalise it here, where a refill runs on at least
              // half the warp's lanes, and store it for k_trace
              double v[3] = {d[0], d[1], d[2]};
              x64::normalize(v, d);
              for (int a = 0; a < 3; ++a) r.d[a] = d[a];
            }
            orank = r.orank;
          }
          o32 = make_float3(float(o[0]), float(o[1]), float(o[2]));
          d32 = make_float3(float(d[0]), float(d[1]), float(d[2]));
          {
            float4* f = reinterpret_cast<float4*>(A.ray32 + k);
            f[0] = make_float4(o32.x, o32.y, o32.z, 0.0f);
            f[1] = make_float4(d32.x, d32.y, d32.z, 0.0f);
          }
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
    for (int it = 0; it < A.steps && !done; ++it) {
      if (pending >= 0) {
        // up to tris_per_step triangles of the pending leaf per step (a node
        // visit tests two child boxes), so lanes testing triangles and lanes
        // stepping through nodes take steps of comparable cost
        for (int q = 0; q < A.tris_per_step && pending >= 0; ++q) {
          const int j = pending >> 3, left = (pending & 7) - 1;
          pending = left > 0 ? ((j + 1) << 3 | left) : -1;
          float tlo, thi;
          const Tri32 T = A.sc.stri[j];
          const int k = tri_classify(T, o32, d32, no, nd, tlo, thi);
          if (k == 0 || tlo > tcut) continue;
          const int rk = __ldg(A.sc.srank + j);
          // the triangle the ray starts on, left at a clear angle: the
          // reference's test of it certainly fails (origin_rejected); such a
          // contender is never certain (k == 2), so dropping it changes no cut
          if (rk == orank && origin_rejected(T, o32, d32)) continue;
          if (nc == kCand) {
            fail = done = true;
            break;
          }
          out[nc++] = make_uint2(unsigned(rk), __float_as_uint(tlo));
          if (k == 2) tcut = fminf(tcut, thi * (1.0f + kTieSlack) + 1e-30f);
        }
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
      // a four-wide node: the children the ray's slab test keeps (within
      // tcut), nearest first; the farther ones go on the stack, the nearest
      // on top (a leaf as the nearest becomes the pending leaf at once)
      const float4* p = reinterpret_cast<const float4*>(A.sc.snode4 + ni);
      const float4 lx = __ldg(p), ly = __ldg(p + 1), lz = __ldg(p + 2);
      const float4 hx = __ldg(p + 3), hy = __ldg(p + 4), hz = __ldg(p + 5);
      const int4 cr = __ldg(reinterpret_cast<const int4*>(p + 6));
      auto visit = [&](float ax, float ay, float az, float bx, float by, float bz, int c,
                       float& t) -> int {
        float tn, tf;
        slab32(ax, ay, az, bx, by, bz, o32, inv, m, tn, tf);
        const bool h = c != kEmptyChild && tn <= tf && tf >= 0.0f && tn <= tcut;
        t = h ? tn : INFINITY;
        return h ? c : kEmptyChild;
      };
      float t0, t1, t2, t3;
      int c0 = visit(lx.x, ly.x, lz.x, hx.x, hy.x, hz.x, cr.x, t0);
      int c1 = visit(lx.y, ly.y, lz.y, hx.y, hy.y, hz.y, cr.y, t1);
      int c2 = visit(lx.z, ly.z, lz.z, hx.z, hy.z, hz.z, cr.z, t2);
      int c3 = visit(lx.w, ly.w, lz.w, hx.w, hy.w, hz.w, cr.w, t3);
      auto order = [](float& ta, int& ca, float& tb, int& cb) {
        if (tb < ta) {
          const float t = ta;
          ta = tb;
          tb = t;
          const int c = ca;
          ca = cb;
          cb = c;
        }
      };
      order(t0, c0, t1, c1);  // sorting network for four
      order(t2, c2, t3, c3);
      order(t0, c0, t2, c2);
      order(t1, c1, t3, c3);
      order(t1, c1, t2, c2);
      const int need = int(c0 != kEmptyChild) + int(c1 != kEmptyChild) +
                       int(c2 != kEmptyChild) + int(c3 != kEmptyChild);
      if (sp + need > kStack) {
        fail = done = true;
        break;
      }
      if (c3 != kEmptyChild) stack[sp++] = c3;  // node, or ~leaf code
      if (c2 != kEmptyChild) stack[sp++] = c2;
      if (c1 != kEmptyChild) stack[sp++] = c1;
      if (c0 != kEmptyChild) {
        if (c0 < 0) pending = ~c0;
        else stack[sp++] = c0;
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

// The tree node of a resolved ray and its children (RTSolver.cpp:142-257):
// node record, reflected and transmitted rays, path-class interning.
__device__ __forceinline__ void finish_ray(const TraceArgs& A, const RayRec& r, const float3& o32,
                                           const float3& d32, bool hit, const Hit& h) {
  const TxParams& P = A.txp[r.tx];
  const unsigned long long ni = emit_node(A.nodes, A.nodes_cold, A.node_cap, A.ctr, A.seg_per_tx,
                                          r, A.depth == 0, o32, d32, hit, h);
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
    c.orank = h.rank;
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
        list_class(A, c.cls);
      }
      if (slot < A.out_cap) A.out[slot] = c;
      else atomicOr(&A.ctr->overflow, kOvQueue);
      ++slot;
    }
    if (do_r) {  // reflected: Reflect(d, n), heap 2h+1; k_find normalises it
      const double dn = x64::dot(T.n, r.d);
      for (int a = 0; a < 3; ++a) c.d[a] = x64::sub(r.d[a], x64::mul(x64::mul(2.0, T.n[a]), dn));
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
        list_class(A, c.cls);
      }
      if (slot < A.out_cap) A.out[slot] = c;
      else atomicOr(&A.ctr->overflow, kOvQueue);
    }
  }
}

// Every ancestor box of the winner's leaf in the reference BVH must pass the
// reference's slab test, else the ray takes the reference-order traversal.
__device__ __forceinline__ bool reachable_or_exact(const DevScene& sc, const RayRec& r,
                                                   const float3& o32, const float3& d32, Hit& best,
                                                   TraceStats& st, unsigned* overflow) {
  best.leaf = sc.tri64[best.rank].node;
  const float3 i32 = make_float3(1.0f / d32.x, 1.0f / d32.y, 1.0f / d32.z);
  for (const AncBox* a = sc.anc + sc.anc_off[best.leaf];; ++a) {
    const AncBox b = *a;
    if (b.node < 0) break;
    int v = slab_certain(b.fb, b.flat, o32, d32, i32);
    if (v < 0) v = slab64(sc.ref[b.node].bb, r.o, r.d) ? 1 : 0;
    if (!v) {
      ++st.fallback;
      return exact_closest(sc, r.o, r.d, best, overflow);
    }
  }
  return true;
}

// FP64 resolution of the contenders k_find left: they are tested in
// ascending order of their FP32 lower bound on t until none can reach the
// best exact distance; the answer is the lexicographic minimum (distance,
// depth-first rank), the reference's strict '<' in visit order, accepted if
// its leaf is reachable in the reference BVH (reachable_or_exact).  The kernel
// is persistent: each lane holds one ray and runs at most one
// FP64 triangle test per round, so the warp's FP64 instructions serve every
// lane that has a test due, whether it is a ray's first contender or a later
// one.  A lane whose ray is resolved writes the node and children in the
// same round and takes a new ray (one atomic per warp); a ray needing a
// second test no longer holds the whole warp through a second pass of the
// test with a few lanes.
__global__ void __launch_bounds__(128, SBR_TRACE_BLOCKS) k_trace(TraceArgs A) {
  if (A.ctr->overflow & kOvTrace) return;  // this solve will be repeated
  const long long n_all = rays_at_depth(A.ctr, A.depth, A.n_root, A.out_cap);
  const long long n = min(n_all, A.hi) - A.lo;
  if (n <= 0) return;
  const unsigned lane = lane_id();
  TraceStats st{0, 0};
  long long c = -1;  // the lane's ray (index in the chunk), -1 = none
  bool exhausted = false;
  RayRec r;
  float3 o32 = make_float3(0.0f, 0.0f, 0.0f), d32 = o32;
  int cr[kCand];
  float ct[kCand];
  int nc = 0, next = 0;
  Hit best;
  best.rank = INT_MAX;
  while (true) {
    // Refill: the idle lanes take the next window of rays (the j-th idle
    // lane the window's j-th ray, so the loads stay in order).  A ray k_find
    // left without a contender hits nothing: its lane writes the node at once
    // and stays idle, so such rays never hold a lane through a round of FP64
    // tests.  Windows repeat until no lane is idle or the chunk is done;
    // `exhausted` is the same on every lane.
    unsigned im = __ballot_sync(0xffffffffu, c < 0);
    while (im && !exhausted) {
      const int want = __popc(im);
      const int leader = __ffs(im) - 1;
      unsigned long long base = 0;
      if (int(lane) == leader) base = atomicAdd(A.work, (unsigned long long)want);
      base = __shfl_sync(0xffffffffu, base, leader);
      if ((long long)base + want >= n) exhausted = true;
      const long long k = (long long)base + __popc(im & ((1u << lane) - 1u));
      if (c < 0 && k < n) {
        load_ray(A.txp, A.n_tx, A.dirs, A.in, A.depth, A.lo + k, r);
        const float4* f = reinterpret_cast<const float4*>(A.ray32 + k);
        const float4 fo = f[0], fd = f[1];
        o32 = make_float3(fo.x, fo.y, fo.z);
        d32 = make_float3(fd.x, fd.y, fd.z);
        nc = A.ncand[k];
        if (nc == 0) {
          Hit none;
          emit_node(A.nodes, A.nodes_cold, A.node_cap, A.ctr, A.seg_per_tx, r, A.depth == 0,
                    o32, d32, false, none);
        } else {
          c = k;
          if (nc != kFindFallback) {
            const uint2* cand = A.cand + size_t(k) * kCand;
            for (int j = 0; j < nc; ++j) {
              const uint2 e = cand[j];
              const float t = __uint_as_float(e.y);
              int m = j - 1;
              while (m >= 0 && ct[m] > t) {  // insertion by lower bound (stable)
                ct[m + 1] = ct[m];
                cr[m + 1] = cr[m];
                --m;
              }
              ct[m + 1] = t;
              cr[m + 1] = int(e.x);
            }
          }
          next = 0;
          best.rank = INT_MAX;
          best.dist = __longlong_as_double(0x7ff0000000000000ll);
          best.t = best.dist;
        }
      }
      im = __ballot_sync(0xffffffffu, c < 0);
    }
    if (__ballot_sync(0xffffffffu, c >= 0) == 0) break;  // every lane is out of rays
    if (c < 0) continue;
    bool done, hit;
    if (nc == kFindFallback) {  // more contenders than kept, or a deep stack: one-pass search
      hit = closest_hit(A.sc, r.o, r.d, best, st, &A.ctr->overflow);
      done = true;
    } else {
      if (next < nc) {  // the next contender, nearest lower bound first
        const int rk = cr[next++];
        ++st.fp64_tri;
        double t, P[3], dist;
        if (mt64(A.sc.tri64[rk], r.o, r.d, t, P, dist) &&
            (dist < best.dist || (dist == best.dist && rk < best.rank))) {
          best.dist = dist;
          best.t = t;
          best.p[0] = P[0];
          best.p[1] = P[1];
          best.p[2] = P[2];
          best.rank = rk;
        }
      }
      // resolved when no further contender can reach the best exact distance
      done = !(next < nc &&
               (best.rank == INT_MAX || ct[next] <= float(best.t) * (1.0f + kTieSlack) + 1e-30f));
      hit = false;
      if (done && best.rank != INT_MAX)
        hit = reachable_or_exact(A.sc, r, o32, d32, best, st, &A.ctr->overflow);
    }
    if (done) {
      finish_ray(A, r, o32, d32, hit, best);
      c = -1;
    }
  }
  if (st.fp64_tri) atomicAdd(&A.ctr->fp64_tri, (unsigned long long)st.fp64_tri);
  if (st.fallback) atomicAdd(&A.ctr->fallback, (unsigned long long)st.fallback);
}

}  // namespace sbr

namespace sbr {

// ---- FP64 resolution with the rays in shared memory ----------------------
//
// The same resolution as k_trace, scheduled so the FP64 work runs on full
// warps.  k_trace keeps one ray per lane, so a warp's FP64 instructions
// serve only the lanes whose ray has a test (or a node to write) due that
// round: about a third of the lanes, measured.  Here each warp keeps
// kPoolSlots rays in shared memory, more than its lanes; every round it lists
// the slots with a test due and hands them out to its lanes in order (the
// n-th lane takes the n-th listed slot), then lists the resolved slots and
// hands those out for the node record and children, then refills the empty
// slots (one atomic per warp).  A ray's tests still run one at a time in
// ascending order of their lower bounds, so every decision is k_trace's.
constexpr int kPoolSlots = 48;  // at most 64 (two ballot words)
constexpr int kPoolWarps = 4;   // warps per block

struct PoolSlots {  // one warp's slots, structure of arrays
  double o[3][kPoolSlots], d[3][kPoolSlots];
  double total[kPoolSlots], S[kPoolSlots];
  double bt[kPoolSlots], bdist[kPoolSlots], bp[3][kPoolSlots];
  float o32[3][kPoolSlots], d32[3][kPoolSlots];
  float ct[kCand][kPoolSlots];
  int cr[kCand][kPoolSlots];
  int brank[kPoolSlots], orank[kPoolSlots];
  uint32_t parent[kPoolSlots], cls[kPoolSlots], cop[kPoolSlots], launch[kPoolSlots];
  uint32_t heap[kPoolSlots], tx[kPoolSlots];
  uint16_t rc[kPoolSlots], tc[kPoolSlots];
  uint8_t nc[kPoolSlots], nx[kPoolSlots], active[kPoolSlots], pad[kPoolSlots];
};

// The position of the j-th (0-based) set bit of the 64-slot mask (m0, m1).
__device__ __forceinline__ int nth_slot(unsigned m0, unsigned m1, int j) {
  const int c0 = __popc(m0);
  return j < c0 ? nth_set_bit(m0, j) : 32 + nth_set_bit(m1, j - c0);
}

__global__ void __launch_bounds__(32 * kPoolWarps, 4) k_trace_pool(TraceArgs A) {
  if (A.ctr->overflow & kOvTrace) return;  // this solve will be repeated
  const long long n_all = rays_at_depth(A.ctr, A.depth, A.n_root, A.out_cap);
  const long long n = min(n_all, A.hi) - A.lo;
  if (n <= 0) return;
  extern __shared__ __align__(16) unsigned char pool_smem[];
  PoolSlots& P = reinterpret_cast<PoolSlots*>(pool_smem)[threadIdx.x >> 5];
  const unsigned lane = lane_id();
  TraceStats st{0, 0};
  const bool hi_slot = lane + 32 < unsigned(kPoolSlots);  // this lane's second slot exists
  P.active[lane] = 0;
  if (hi_slot) P.active[lane + 32] = 0;
  bool exhausted = false;
  __syncwarp();
  while (true) {
    // ---- refill the empty slots
    const unsigned e0 = __ballot_sync(0xffffffffu, !P.active[lane]);
    const unsigned e1 = __ballot_sync(0xffffffffu, hi_slot && !P.active[lane + 32]);
    const int n_empty = __popc(e0) + __popc(e1);
    if (!exhausted && n_empty > 0) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(A.work, (unsigned long long)n_empty);
      base = __shfl_sync(0xffffffffu, base, 0);
      if ((long long)base + n_empty >= n) exhausted = true;
      for (int j = int(lane); j < n_empty; j += 32) {
        const long long k = (long long)base + j;
        if (k >= n) break;
        const int s = nth_slot(e0, e1, j);
        RayRec r;
        load_ray(A.txp, A.n_tx, A.dirs, A.in, A.depth, A.lo + k, r);
        if (A.ncand[k] == 0) {  // no contender: it hits nothing; its slot stays empty
          const float4* f = reinterpret_cast<const float4*>(A.ray32 + k);
          const float4 fo = f[0], fd = f[1];
          Hit none;
          emit_node(A.nodes, A.nodes_cold, A.node_cap, A.ctr, A.seg_per_tx, r, A.depth == 0,
                    make_float3(fo.x, fo.y, fo.z), make_float3(fd.x, fd.y, fd.z), false, none);
          continue;
        }
        for (int a = 0; a < 3; ++a) {
          P.o[a][s] = r.o[a];
          P.d[a][s] = r.d[a];
        }
        P.total[s] = r.total;
        P.S[s] = r.S;
        P.parent[s] = r.parent;
        P.cls[s] = r.cls;
        P.cop[s] = r.cop;
        P.launch[s] = r.launch;
        P.heap[s] = r.heap;
        P.rc[s] = r.rc;
        P.tc[s] = r.tc;
        P.tx[s] = r.tx;
        P.orank[s] = r.orank;
        const float4* f = reinterpret_cast<const float4*>(A.ray32 + k);
        const float4 fo = f[0], fd = f[1];
        P.o32[0][s] = fo.x;
        P.o32[1][s] = fo.y;
        P.o32[2][s] = fo.z;
        P.d32[0][s] = fd.x;
        P.d32[1][s] = fd.y;
        P.d32[2][s] = fd.z;
        const int nc = A.ncand[k];
        P.nc[s] = uint8_t(nc);
        if (nc != kFindFallback) {
          // contenders by ascending lower bound (stable insertion)
          float ct[kCand];
          int cr[kCand];
          const uint2* cand = A.cand + size_t(k) * kCand;
          for (int c = 0; c < nc; ++c) {
            const uint2 e = cand[c];
            const float t = __uint_as_float(e.y);
            int m = c - 1;
            while (m >= 0 && ct[m] > t) {
              ct[m + 1] = ct[m];
              cr[m + 1] = cr[m];
              --m;
            }
            ct[m + 1] = t;
            cr[m + 1] = int(e.x);
          }
          for (int c = 0; c < nc; ++c) {
            P.ct[c][s] = ct[c];
            P.cr[c][s] = cr[c];
          }
        }
        P.nx[s] = 0;
        P.brank[s] = INT_MAX;
        P.bdist[s] = __longlong_as_double(0x7ff0000000000000ll);
        P.bt[s] = P.bdist[s];
        P.active[s] = 1;
      }
    }
    __syncwarp();
    const unsigned a0 = __ballot_sync(0xffffffffu, P.active[lane]);
    const unsigned a1 = __ballot_sync(0xffffffffu, hi_slot && P.active[lane + 32]);
    if (!(a0 | a1) && exhausted) break;
    // ---- one FP64 test for every slot with one due, slots handed out in order
    auto due = [&](int s) {
      return P.active[s] && P.nc[s] != kFindFallback && P.nx[s] < P.nc[s];
    };
    const unsigned t0 = __ballot_sync(0xffffffffu, due(int(lane)));
    const unsigned t1 = __ballot_sync(0xffffffffu, hi_slot && due(int(lane) + 32));
    const int n_test = __popc(t0) + __popc(t1);
    for (int j = int(lane); j < n_test; j += 32) {
      const int s = nth_slot(t0, t1, j);
      const int rk = P.cr[P.nx[s]][s];
      P.nx[s] = uint8_t(P.nx[s] + 1);
      ++st.fp64_tri;
      const double o[3] = {P.o[0][s], P.o[1][s], P.o[2][s]};
      const double d[3] = {P.d[0][s], P.d[1][s], P.d[2][s]};
      double t, Q[3], dist;
      if (mt64(A.sc.tri64[rk], o, d, t, Q, dist) &&
          (dist < P.bdist[s] || (dist == P.bdist[s] && rk < P.brank[s]))) {
        P.bdist[s] = dist;
        P.bt[s] = t;
        P.bp[0][s] = Q[0];
        P.bp[1][s] = Q[1];
        P.bp[2][s] = Q[2];
        P.brank[s] = rk;
      }
    }
    __syncwarp();
    // ---- resolved slots: no further contender can reach the best distance
    auto resolved = [&](int s) {
      if (!P.active[s]) return false;
      if (P.nc[s] == kFindFallback) return true;
      const int nx = P.nx[s];
      return !(nx < P.nc[s] &&
               (P.brank[s] == INT_MAX || P.ct[nx][s] <= float(P.bt[s]) * (1.0f + kTieSlack) + 1e-30f));
    };
    const unsigned r0 = __ballot_sync(0xffffffffu, resolved(int(lane)));
    const unsigned r1 = __ballot_sync(0xffffffffu, hi_slot && resolved(int(lane) + 32));
    const int n_res = __popc(r0) + __popc(r1);
    for (int j0 = 0; j0 < n_res; j0 += 32) {
      const int j = j0 + int(lane);
      if (j < n_res) {
        const int s = nth_slot(r0, r1, j);
        RayRec r;
        for (int a = 0; a < 3; ++a) {
          r.o[a] = P.o[a][s];
          r.d[a] = P.d[a][s];
        }
        r.total = P.total[s];
        r.S = P.S[s];
        r.parent = P.parent[s];
        r.cls = P.cls[s];
        r.cop = P.cop[s];
        r.launch = P.launch[s];
        r.heap = P.heap[s];
        r.rc = P.rc[s];
        r.tc = P.tc[s];
        r.tx = P.tx[s];
        r.orank = P.orank[s];
        const float3 o32 = make_float3(P.o32[0][s], P.o32[1][s], P.o32[2][s]);
        const float3 d32 = make_float3(P.d32[0][s], P.d32[1][s], P.d32[2][s]);
        Hit best;
        best.rank = P.brank[s];
        best.dist = P.bdist[s];
        best.t = P.bt[s];
        best.p[0] = P.bp[0][s];
        best.p[1] = P.bp[1][s];
        best.p[2] = P.bp[2][s];
        bool hit;
        if (P.nc[s] == kFindFallback) {  // more contenders than kept: one-pass search
          hit = closest_hit(A.sc, r.o, r.d, best, st, &A.ctr->overflow);
        } else {
          hit = best.rank != INT_MAX && reachable_or_exact(A.sc, r, o32, d32, best, st,
                                                            &A.ctr->overflow);
        }
        finish_ray(A, r, o32, d32, hit, best);
        P.active[s] = 0;
      }
      // finish_ray's warp-wide reservations need every lane: the loop bound is uniform
    }
    __syncwarp();
  }
  if (st.fp64_tri) atomicAdd(&A.ctr->fp64_tri, (unsigned long long)st.fp64_tri);
  if (st.fallback) atomicAdd(&A.ctr->fallback, (unsigned long long)st.fallback);
}

}  // namespace sbr
