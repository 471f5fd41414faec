// Scene preparation on the device: the parts of the reference's scene set-up
// whose results do not depend on the order std::sort leaves equal keys in,
// so that the GPU can build them exactly as the host does:
//
//   * exact vertex merge (StlReader.h:448-508: equal float triples are one
//     vertex) and coplanar grouping (Preprocessor.cpp:116-246: triangles
//     sharing an edge of merged vertices, with facet normals exactly equal or
//     opposite, are one coplanar group), numbered by each group's smallest
//     triangle index, as the host numbers them;
//   * per-triangle surface frames and boxes (Triangle.cpp:37-70), FP64 with
//     every operation rounded separately, in the host's order;
//   * this project's search BVH (32-bin SAH over FP32 centroids, leaves of at
//     most 7 triangles), node for node and in the same depth-first numbering
//     as the host build.
//
// The reference BVH, whose shape depends on the order std::sort leaves
// equal centroids in, is built by sbr_refbvh.cuh.
#pragma once

#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "sbr_common.cuh"
#include "sbr_device.h"

namespace sbr {
namespace prep {

// ---- stable radix sort of a permutation, one key bit per pass ------------
//
// perm is reordered by the bit `bit` of word[perm[i]] (zeros first), stably;
// a full LSD sort calls this for every bit that varies, least significant
// first.  f = 1 - bit, scanned, gives each zero its place; ones follow.
__global__ void k_bit_flags(const uint32_t* word, const int* perm, int n, int bit, int* f) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    f[i] = ((word[perm[i]] >> bit) & 1u) ? 0 : 1;
}

__global__ void k_bit_scatter(const uint32_t* word, const int* perm, int n, int bit,
                              const int* scan, int* out) {
  const int zeros = scan[n];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int p = perm[i];
    const int d = ((word[p] >> bit) & 1u) ? zeros + (i - scan[i]) : scan[i];
    out[d] = p;
  }
}

// OR of (word[i] xor word[0]): the bits that vary.
__global__ void k_varying_bits(const uint32_t* word, int n, unsigned* out) {
  unsigned acc = 0;
  const uint32_t w0 = n ? word[0] : 0u;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    acc |= word[i] ^ w0;
  for (int o = 16; o; o >>= 1) acc |= __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane_id() == 0 && acc) atomicOr(out, acc);
}

// ---- vertex merge and coplanar groups -------------------------------------

// Float bits of each vertex coordinate, -0 read as +0 (they compare equal).
__global__ void k_vertex_words(const float* v, int nv, uint32_t* wx, uint32_t* wy, uint32_t* wz,
                               int* perm) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) {
    const float x = v[3 * i], y = v[3 * i + 1], z = v[3 * i + 2];
    wx[i] = __float_as_uint(x == 0.0f ? 0.0f : x);
    wy[i] = __float_as_uint(y == 0.0f ? 0.0f : y);
    wz[i] = __float_as_uint(z == 0.0f ? 0.0f : z);
    perm[i] = i;
  }
}

// Start flags of runs of equal (a, b[, c]) words along the sorted permutation.
__global__ void k_run_starts(const uint32_t* a, const uint32_t* b, const uint32_t* c,
                             const int* perm, int n, int* f) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int s = 1;
    if (i > 0) {
      const int p = perm[i], q = perm[i - 1];
      s = a[p] != a[q] || b[p] != b[q] || (c && c[p] != c[q]);
    }
    f[i] = s;
  }
}

// Merged vertex id of every vertex: the index of its run.
__global__ void k_vertex_ids(const int* perm, const int* f, const int* scan, int n, int* uid) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    uid[perm[i]] = scan[i] + f[i] - 1;
}

// The three edges of every triangle as (smaller id, larger id) words, in
// the host's order: (v1, v2), (v2, v3), (v1, v3).  Triangles whose merged
// vertices coincide are counted (the reference reader drops them; the
// library refuses such input).
__global__ void k_edges(const int* uid, int nt, uint32_t* hi, uint32_t* lo, int* perm,
                        int* degenerate) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
    const int a = uid[3 * t], b = uid[3 * t + 1], c = uid[3 * t + 2];
    if (a == b || a == c || b == c) atomicAdd(degenerate, 1);
    const int e[3][2] = {{min(a, b), max(a, b)}, {min(b, c), max(b, c)}, {min(a, c), max(a, c)}};
    for (int k = 0; k < 3; ++k) {
      hi[3 * t + k] = uint32_t(e[k][0]);
      lo[3 * t + k] = uint32_t(e[k][1]);
      perm[3 * t + k] = 3 * t + k;
    }
  }
}

__device__ __forceinline__ bool same_or_opposite(const float* nrm, int a, int b) {
  const float* p = nrm + 3 * a;
  const float* q = nrm + 3 * b;
  return (p[0] == q[0] && p[1] == q[1] && p[2] == q[2]) ||
         (p[0] == -q[0] && p[1] == -q[1] && p[2] == -q[2]);
}

__device__ __forceinline__ int root_of(const int* parent, int a) {
  while (true) {
    const int p = __ldcg(parent + a);
    if (p == a) return a;
    a = p;
  }
}

// One hooking round: for every pair of triangles on a shared edge whose
// normals are equal or opposite, the larger of their two roots is linked
// to the smaller one.  Links only ever point to smaller indices, so a
// component's root is its smallest triangle once no pair has two roots.
__global__ void k_hook(const uint32_t* hi, const uint32_t* lo, const int* perm, const int* start,
                       int ne, const float* nrm, int* parent, int* changed) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ne; i += gridDim.x * blockDim.x) {
    if (!start[i]) continue;
    const int p0 = perm[i];
    int j = i + 1;
    while (j < ne && hi[perm[j]] == hi[p0] && lo[perm[j]] == lo[p0]) ++j;
    for (int x = i; x < j; ++x)
      for (int y = x + 1; y < j; ++y) {
        const int a = perm[x] / 3, b = perm[y] / 3;
        if (!same_or_opposite(nrm, a, b)) continue;
        const int ra = root_of(parent, a), rb = root_of(parent, b);
        if (ra == rb) continue;
        atomicMin(&parent[max(ra, rb)], min(ra, rb));
        *changed = 1;
      }
  }
}

__global__ void k_compress(int* parent, int n, int* is_root) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int r = root_of(parent, t);
    parent[t] = r;
    if (is_root) is_root[t] = r == t;
  }
}

__global__ void k_group_ids(const int* parent, const int* scan, int n, int* cop) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
    cop[t] = scan[parent[t]];
}

// ---- triangle frames and boxes (FP64, the host's operation order) ---------

// rows x = y cross n, y = (v2 - v1) / |v2 - v1|, z = n (Triangle.cpp:37-49);
// box min / max of the vertices and its centre.
__global__ void k_frames(const float* v, const float* nrm, int nt, double* cs, double* bb,
                         double* center) {
  using namespace x64;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
    const float* p = v + 9 * size_t(t);
    double v1[3], v2[3], v3[3], n[3];
    for (int a = 0; a < 3; ++a) {
      v1[a] = p[a];
      v2[a] = p[3 + a];
      v3[a] = p[6 + a];
      n[a] = nrm[3 * t + a];
    }
    double e[3], y[3], x[3];
    sub3(v2, v1, e);
    normalize(e, y);
    cross(y, n, x);
    double* c = cs + 9 * size_t(t);
    for (int j = 0; j < 3; ++j) {
      c[j] = x[j];
      c[3 + j] = y[j];
      c[6 + j] = n[j];
    }
    double* b = bb + 6 * size_t(t);
    for (int a = 0; a < 3; ++a) {
      // std::min / std::max over (v1, v2, v3): the first smallest / largest
      double lo = v1[a], hi = v1[a];
      if (v2[a] < lo) lo = v2[a];
      if (v3[a] < lo) lo = v3[a];
      if (hi < v2[a]) hi = v2[a];
      if (hi < v3[a]) hi = v3[a];
      b[a] = lo;
      b[3 + a] = hi;
      center[3 * size_t(t) + a] = div(add(lo, hi), 2.0);
    }
  }
}

// ---- search BVH --------------------------------------------------------

constexpr int kBins = 32;

struct FBox32 {
  float lo[3], hi[3];
};

// Surface area as the host computes it: 2 (dx dy + dy dz + dz dx), each
// product and sum rounded separately, 0 for an empty box.
__device__ __forceinline__ float area32(const float* lo, const float* hi) {
  const float dx = __fsub_rn(hi[0], lo[0]), dy = __fsub_rn(hi[1], lo[1]),
              dz = __fsub_rn(hi[2], lo[2]);
  if (dx < 0.0f) return 0.0f;
  return __fmul_rn(2.0f, __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dy, dz)), __fmul_rn(dz, dx)));
}

// Per-triangle box and centroid (FP32), as the host's search build forms them.
__global__ void k_tri_boxes(const float* v, int nt, float* blo, float* bhi, float* cen, int* ord) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
    const float* p = v + 9 * size_t(t);
    for (int a = 0; a < 3; ++a) {
      // -0 read as +0, as the host build reads it
      const float x = p[a] == 0.0f ? 0.0f : p[a], y = p[3 + a] == 0.0f ? 0.0f : p[3 + a],
                  z = p[6 + a] == 0.0f ? 0.0f : p[6 + a];
      const float l = fminf(fminf(x, y), z), h = fmaxf(fmaxf(x, y), z);
      blo[3 * t + a] = l;
      bhi[3 * t + a] = h;
      cen[3 * t + a] = __fmul_rn(0.5f, __fadd_rn(l, h));
    }
    ord[t] = t;
  }
}

// A segment [b, e) of the triangle order, to become a node or a leaf.
struct Seg {
  int b, e, depth;
  int parent;  // BFS node id of the parent, -1 for the root
  int which;   // 0 left, 1 right child of the parent
};

// What the per-segment step decided.
struct SegPlan {
  int kind;    // 0 leaf, 1 binned split, 2 median split
  int node;    // BFS node id (splits)
  int axis, best;
  float lo, k;  // bin_of(p) = clamp(int((cen - lo) * k))
  int mid;
};

struct BNode {  // node in breadth-first order; children: BFS id, or ~(first << 3 | count)
  float lo[2][3], hi[2][3];
  int child[2];
};

__device__ __forceinline__ int bin_of(float c, float lo, float k) {
  return min(kBins - 1, max(0, int(__fmul_rn(__fsub_rn(c, lo), k))));
}

// One block per segment: its box and centroid box, the host's split choice
// (largest centroid extent; 32 bins; the first cheapest bin boundary; the
// leaf rule), and the record in its parent.
__global__ void k_plan(const Seg* segs, int n_segs, const int* ord, const float* blo,
                       const float* bhi, const float* cen, BNode* nodes, int* n_nodes,
                       SegPlan* plans, int* max_depth, int* root_ref, float* root_box) {
  const int s = blockIdx.x;
  if (s >= n_segs) return;
  const Seg S = segs[s];
  __shared__ int sbox[12], scb[6];
  __shared__ int bcnt[kBins];
  __shared__ int bbox[kBins][6];
  if (threadIdx.x < 6) {
    sbox[threadIdx.x] = threadIdx.x < 3 ? INT_MAX : INT_MIN;
    scb[threadIdx.x] = threadIdx.x < 3 ? INT_MAX : INT_MIN;
  }
  for (int i = threadIdx.x; i < kBins; i += blockDim.x) {
    bcnt[i] = 0;
    for (int a = 0; a < 3; ++a) {
      bbox[i][a] = INT_MAX;
      bbox[i][3 + a] = INT_MIN;
    }
  }
  __syncthreads();
  for (int i = S.b + threadIdx.x; i < S.e; i += blockDim.x) {
    const int p = ord[i];
    for (int a = 0; a < 3; ++a) {
      atomicMin(&sbox[a], f2o(blo[3 * p + a]));
      atomicMax(&sbox[3 + a], f2o(bhi[3 * p + a]));
      atomicMin(&scb[a], f2o(cen[3 * p + a]));
      atomicMax(&scb[3 + a], f2o(cen[3 * p + a]));
    }
  }
  __syncthreads();
  const int n = S.e - S.b;
  float box_lo[3], box_hi[3], cb_lo[3], cb_hi[3];
  for (int a = 0; a < 3; ++a) {
    box_lo[a] = o2f(sbox[a]);
    box_hi[a] = o2f(sbox[3 + a]);
    cb_lo[a] = o2f(scb[a]);
    cb_hi[a] = o2f(scb[3 + a]);
  }
  int ax = 0;
  for (int a = 1; a < 3; ++a)
    if (__fsub_rn(cb_hi[a], cb_lo[a]) > __fsub_rn(cb_hi[ax], cb_lo[ax])) ax = a;
  const float ext = __fsub_rn(cb_hi[ax], cb_lo[ax]);
  const float k = ext > 0.0f ? __fdiv_rn(float(kBins), ext) : 0.0f;
  const bool binned = n > 2 && ext > 0.0f;
  if (binned) {
    for (int i = S.b + threadIdx.x; i < S.e; i += blockDim.x) {
      const int p = ord[i], q = bin_of(cen[3 * p + ax], cb_lo[ax], k);
      atomicAdd(&bcnt[q], 1);
      for (int a = 0; a < 3; ++a) {
        atomicMin(&bbox[q][a], f2o(blo[3 * p + a]));
        atomicMax(&bbox[q][3 + a], f2o(bhi[3 * p + a]));
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    SegPlan P;
    P.kind = 0;
    P.node = -1;
    P.axis = ax;
    P.best = -1;
    P.lo = cb_lo[ax];
    P.k = k;
    P.mid = -1;
    if (n > 2) {
      int mid_kind = -1;  // -1: none yet
      if (ext > 0.0f) {
        float right_area[kBins];
        int right_cnt[kBins];
        float alo[3] = {INFINITY, INFINITY, INFINITY}, ahi[3] = {-INFINITY, -INFINITY, -INFINITY};
        int c = 0;
        for (int i = kBins - 1; i > 0; --i) {
          for (int a = 0; a < 3; ++a) {
            if (bcnt[i]) {
              alo[a] = fminf(alo[a], o2f(bbox[i][a]));
              ahi[a] = fmaxf(ahi[a], o2f(bbox[i][3 + a]));
            }
          }
          c += bcnt[i];
          right_area[i] = area32(alo, ahi);
          right_cnt[i] = c;
        }
        float llo[3] = {INFINITY, INFINITY, INFINITY}, lhi[3] = {-INFINITY, -INFINITY, -INFINITY};
        int lc = 0, best = -1;
        float best_cost = INFINITY;
        for (int i = 0; i < kBins - 1; ++i) {
          for (int a = 0; a < 3; ++a) {
            if (bcnt[i]) {
              llo[a] = fminf(llo[a], o2f(bbox[i][a]));
              lhi[a] = fmaxf(lhi[a], o2f(bbox[i][3 + a]));
            }
          }
          lc += bcnt[i];
          if (lc == 0 || right_cnt[i + 1] == 0) continue;
          const float cost = __fadd_rn(__fmul_rn(area32(llo, lhi), float(lc)),
                                       __fmul_rn(right_area[i + 1], float(right_cnt[i + 1])));
          if (cost < best_cost) {
            best_cost = cost;
            best = i;
          }
        }
        const float barea = area32(box_lo, box_hi);
        const float leaf_cost = __fmul_rn(barea, float(n));
        if (best >= 0 && (n > 7 || __fadd_rn(best_cost, barea) < leaf_cost)) {
          mid_kind = 1;
          P.best = best;
        } else if (n <= 7) {
          mid_kind = 0;
        }
      } else if (n <= 7) {
        mid_kind = 0;
      }
      if (mid_kind != 0) {
        // a binned split empties no side (best has triangles on both); past
        // depth 48, or without a usable split, the median of the axis
        P.kind = (mid_kind == 1 && S.depth <= 48) ? 1 : 2;
        if (P.kind == 2) P.mid = S.b + n / 2;
        P.node = atomicAdd(n_nodes, 1);
      }
    }
    atomicMax(max_depth, S.depth);
    // the segment's box and reference in its parent
    const int ref = P.kind == 0 ? ~((S.b << 3) | n) : P.node;
    if (S.parent >= 0) {
      BNode& pn = nodes[S.parent];
      for (int a = 0; a < 3; ++a) {
        pn.lo[S.which][a] = box_lo[a];
        pn.hi[S.which][a] = box_hi[a];
      }
      pn.child[S.which] = ref;
    } else {
      *root_ref = ref;
      for (int a = 0; a < 3; ++a) {
        root_box[a] = box_lo[a];
        root_box[3 + a] = box_hi[a];
      }
    }
    plans[s] = P;
  }
}

// One block per binned split: stable partition of the segment (bin <= best
// first), through tmp; writes the split point.
__global__ void k_partition(const Seg* segs, int n_segs, SegPlan* plans, int* ord, int* tmp,
                            const float* cen) {
  const int s = blockIdx.x;
  if (s >= n_segs) return;
  SegPlan& P = plans[s];
  if (P.kind != 1) return;
  const Seg S = segs[s];
  __shared__ int warp_sum[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // pass 1: left side in order
  for (int base = S.b; base < S.e; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const int p = i < S.e ? ord[i] : 0;
    const int f = i < S.e && bin_of(cen[3 * p + P.axis], P.lo, P.k) <= P.best;
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    if (lane == 0) warp_sum[wid] = __popc(bal);
    __syncthreads();
    int before = carry;
    for (int w = 0; w < wid; ++w) before += warp_sum[w];
    before += __popc(bal & ((1u << lane) - 1u));
    if (f) tmp[S.b + before] = p;
    __syncthreads();
    if (threadIdx.x == 0)
      for (int w = 0; w < nw; ++w) carry += warp_sum[w];
    __syncthreads();
  }
  const int n_left = carry;
  __syncthreads();
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  // pass 2: right side in order
  for (int base = S.b; base < S.e; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const int p = i < S.e ? ord[i] : 0;
    const int f = i < S.e && !(bin_of(cen[3 * p + P.axis], P.lo, P.k) <= P.best);
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    if (lane == 0) warp_sum[wid] = __popc(bal);
    __syncthreads();
    int before = carry;
    for (int w = 0; w < wid; ++w) before += warp_sum[w];
    before += __popc(bal & ((1u << lane) - 1u));
    if (f) tmp[S.b + n_left + before] = p;
    __syncthreads();
    if (threadIdx.x == 0)
      for (int w = 0; w < nw; ++w) carry += warp_sum[w];
    __syncthreads();
  }
  for (int i = S.b + threadIdx.x; i < S.e; i += blockDim.x) ord[i] = tmp[i];
  if (threadIdx.x == 0) P.mid = S.b + n_left;
}

// Median splits: the segment ordered by (centroid on the axis, triangle id),
// one block per segment, by rank counting (segments here are small: the
// median is taken only when no binned split helps, which needs at least 8
// triangles with coincident centroids, or past depth 48).
__global__ void k_median(const Seg* segs, int n_segs, const SegPlan* plans, int* ord, int* tmp,
                         const float* cen, int* too_big) {
  const int s = blockIdx.x;
  if (s >= n_segs) return;
  const SegPlan P = plans[s];
  if (P.kind != 2) return;
  const Seg S = segs[s];
  const int n = S.e - S.b;
  if (n > 8192) {
    if (threadIdx.x == 0) atomicAdd(too_big, 1);
    return;
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int p = ord[S.b + i];
    const float c = cen[3 * p + P.axis];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const int q = ord[S.b + j];
      const float d = cen[3 * q + P.axis];
      rank += (d < c || (d == c && q < p)) ? 1 : 0;
    }
    tmp[S.b + rank] = p;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) ord[S.b + i] = tmp[S.b + i];
}

// The children of every split become the next level's segments.
__global__ void k_children(const Seg* segs, int n_segs, const SegPlan* plans, Seg* next,
                           int* n_next) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n_segs; s += gridDim.x * blockDim.x) {
    const SegPlan P = plans[s];
    if (P.kind == 0) continue;
    const Seg S = segs[s];
    const int k = atomicAdd(n_next, 2);
    next[k] = Seg{S.b, P.mid, S.depth + 1, P.node, 0};
    next[k + 1] = Seg{P.mid, S.e, S.depth + 1, P.node, 1};
  }
}

// ---- ancestor boxes of the reference leaves --------------------------------

// Per reference leaf, its box and its ancestors' up to the root as AncBox
// records (the FP32 copy, the flat-axis mask, the node) from off[leaf], then
// an end marker; k_trace's reachability check walks one run per hit.
__global__ void k_anc_fill(const RefNode* ref, int nn, const int* off, AncBox* anc) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
    if (ref[i].c0 >= 0) continue;
    AncBox* o = anc + off[i];
    for (int n = i; n >= 0; n = ref[n].parent, ++o) {
      AncBox b;
      for (int a = 0; a < 6; ++a) b.fb[a] = ref[n].fb[a];
      b.flat = ref[n].flat;
      b.node = n;
      *o = b;
    }
    AncBox end;
    for (int a = 0; a < 6; ++a) end.fb[a] = 0.0f;
    end.flat = 0;
    end.node = -1;
    *o = end;
  }
}

}  // namespace prep
}  // namespace sbr
