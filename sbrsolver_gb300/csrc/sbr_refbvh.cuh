// The reference BVH (BVH/BVH.h:135-230) built on the device, node for node
// and leaf order for leaf order equal to the host build (sbr_host.cpp).
//
// The reference splits a node by sorting its object list with std::sort
// along x, then y, then z (keys: triangle box centres, many of them equal),
// sweeping box surface areas over each order for the cheapest split, and
// sorting once more along the best axis.  Objects with equal keys end up in
// the order std::sort's introsort leaves them in, and that order shapes the
// tree (which objects go left, the leaf order, hence the closest-hit ties).
// This file restates that introsort so that every comparison, exchange and
// move is the one std::sort (libstdc++) makes:
//   * segments longer than 16 with depth budget left: the median of
//     (f + 1, middle, l - 1) is exchanged to the front, then an unguarded
//     Hoare partition of [f + 1, l) around it; both parts continue with one
//     unit of depth budget less (initially 2 floor(log2 n));
//   * a segment out of depth budget is heap sorted (heap built over the
//     whole segment, then popped), as std::partial_sort(f, l, l) does;
//   * segments of at most 16 are left for a final insertion sort.
// Three facts make it parallel without changing any of those steps:
//   * the two parts of a partition are sorted independently, so the
//     segments of all nodes of a tree level are processed together;
//   * a partition is the sequence of exchanges of the k-th left stop (the
//     k-th position, left to right, whose key is not less than the pivot)
//     with the k-th right stop (right to left, key not greater than the
//     pivot) for as long as the left stop lies left of the right stop; those
//     exchanges touch distinct positions, and the cut is the first left stop
//     that does not (or the last right stop exchanged, if that is smaller);
//   * the final insertion sort never moves an element past a partition
//     boundary (everything left of one is not greater than everything right
//     of it), so it is an insertion sort of each segment of at most 16 alone.
// A CPU restatement of these steps reproduced std::sort on 20,000 random
// inputs with many equal keys; the GPU tests compare the device tree with
// the host tree on every test scene.
#pragma once

#include <cstdint>

namespace sbr {
namespace refbvh {

constexpr int kTile = 2048;        // elements per block of the partition rounds
constexpr int kTileThreads = 256;  // 8 consecutive elements per thread
constexpr int kSmallMax = 2048;    // longest segment one warp sorts in shared memory
constexpr int kShortMax = 256;     // segments up to this long use the lighter warp sort
constexpr int kInsertion = 16;     // segments this short wait for insertion sort

struct __align__(16) SortSeg {
  int f, l, d, tile0;  // range [f, l), depth budget, first tile (partition rounds)
};

// Node of the tree, in the order levels create them.
struct __align__(16) RNode {
  double bb[6];      // box, as the host forms it (min xyz, max xyz)
  int f, l;          // objects [f, l) of the build order
  int c0, c1;        // children, -1 for a leaf
};

// What one level decides for each of its nodes.
struct __align__(16) NodeBest {
  double cost;  // best split cost so far (starts at the leaf cost n)
  int axis;     // -1: no split beats the leaf
  int split;    // objects left of the split
};

// Control words: sort list counts and the next level's sizes.
enum Ctl {
  kBig = 0, kBigNext, kSmall, kShort, kTiny, kHeap, kTiles, kTilesNext, kNodes, kActiveNext,
  kSweepTiles, kTiledNodes, kSmallNodes, kError, kCtlWords
};

__device__ __forceinline__ int floor_log2(int n) { return 31 - __clz(n); }


// Box centre along axis a exactly as the reference computes it from the
// box of float vertices: (min + max) / 2 in FP64.
__device__ __forceinline__ double centre(const float4& lo, const float4& hi, int a) {
  const float l = a == 0 ? lo.x : (a == 1 ? lo.y : lo.z);
  const float h = a == 0 ? hi.x : (a == 1 ? hi.y : hi.z);
  return __ddiv_rn(__dadd_rn(double(l), double(h)), 2.0);
}

// Surface area of a box as the host computes it (sbr_host.cpp
// surface_area): 0 for a box that is flat or empty along any axis, else
// 2 (dx dy + dy dz + dz dx) with every operation rounded on its own.
__device__ __forceinline__ double surface_area(float lx, float ly, float lz, float hx, float hy,
                                               float hz) {
  if (hx <= lx || hy <= ly || hz <= lz) return 0.0;
  const double dx = __dsub_rn(double(hx), double(lx));
  const double dy = __dsub_rn(double(hy), double(ly));
  const double dz = __dsub_rn(double(hz), double(lz));
  const double s = __dadd_rn(__dadd_rn(__dmul_rn(dx, dy), __dmul_rn(dy, dz)), __dmul_rn(dz, dx));
  return __dmul_rn(2.0, s);
}

// ---- per-triangle boxes ----------------------------------------------------

// Box of each triangle's float vertices, as std::min / std::max over the
// three (the first of equal values wins, which fixes the sign of a zero);
// lo.w carries the triangle id.
__global__ void k_boxes(const float* v, int nt, float4* lo, float4* hi) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const float* p = v + 9 * size_t(t);
  float l[3], h[3];
  for (int a = 0; a < 3; ++a) {
    l[a] = p[a];
    h[a] = p[a];
    if (p[3 + a] < l[a]) l[a] = p[3 + a];
    if (p[6 + a] < l[a]) l[a] = p[6 + a];
    if (h[a] < p[3 + a]) h[a] = p[3 + a];
    if (h[a] < p[6 + a]) h[a] = p[6 + a];
  }
  lo[t] = make_float4(l[0], l[1], l[2], __int_as_float(t));
  hi[t] = make_float4(h[0], h[1], h[2], 0.0f);
}

// ---- the sort --------------------------------------------------------------

template <class K, class I>
__device__ __forceinline__ void swap_pair(K* key, I* idx, int a, int b) {
  const double k = key[a];
  key[a] = key[b];
  key[b] = k;
  const int i = idx[a];
  idx[a] = idx[b];
  idx[b] = i;
}

// Exchanges the median of (a, b, c) into r, with the reference sort's
// comparisons in its order.
template <class K, class I>
__device__ __forceinline__ void median_to_first(K* key, I* idx, int r, int a, int b, int c) {
  if (key[a] < key[b]) {
    if (key[b] < key[c]) swap_pair(key, idx, r, b);
    else if (key[a] < key[c]) swap_pair(key, idx, r, c);
    else swap_pair(key, idx, r, a);
  } else if (key[a] < key[c]) {
    swap_pair(key, idx, r, a);
  } else if (key[b] < key[c]) {
    swap_pair(key, idx, r, c);
  } else {
    swap_pair(key, idx, r, b);
  }
}

// Insertion sort of [f, l): each element moves left past strictly greater
// ones (the final pass of std::sort restricted to one segment).
template <class K, class I>
__device__ void insertion_sort(K* key, I* idx, int f, int l) {
  for (int i = f + 1; i < l; ++i) {
    const double k = key[i];
    const int x = idx[i];
    int j = i;
    while (j > f && k < key[j - 1]) {
      key[j] = key[j - 1];
      idx[j] = idx[j - 1];
      --j;
    }
    key[j] = k;
    idx[j] = x;
  }
}

// Heap sort of [0, n) in the steps std::partial_sort(f, l, l) takes: the
// heap is built by sifting each parent from the last down to the root
// (the hole goes down to the larger child, the right one on ties, to the
// bottom, then the value climbs back), then the root is popped n - 1 times.
template <class K, class I>
__device__ void heap_push(K* key, I* idx, long hole, long top, double v, int vi) {
  long parent = (hole - 1) / 2;
  while (hole > top && key[parent] < v) {
    key[hole] = key[parent];
    idx[hole] = idx[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  key[hole] = v;
  idx[hole] = vi;
}
template <class K, class I>
__device__ void heap_adjust(K* key, I* idx, long hole, long len, double v, int vi) {
  const long top = hole;
  long child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (key[child] < key[child - 1]) child--;
    key[hole] = key[child];
    idx[hole] = idx[child];
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    key[hole] = key[child - 1];
    idx[hole] = idx[child - 1];
    hole = child - 1;
  }
  heap_push(key, idx, hole, top, v, vi);
}
template <class K, class I>
__device__ void heap_sort(K* key, I* idx, long n) {
  if (n >= 2)
    for (long parent = (n - 2) / 2;; --parent) {
      heap_adjust(key, idx, parent, n, key[parent], idx[parent]);
      if (parent == 0) break;
    }
  for (long last = n; last > 1;) {
    --last;
    const double v = key[last];
    const int vi = idx[last];
    key[last] = key[0];
    idx[last] = idx[0];
    heap_adjust(key, idx, 0, last, v, vi);
  }
}

// Files a segment of the sort: nothing to do (<= 1), insertion list (<= 16),
// heap list (no depth budget left), a warp's list (<= kSmallMax), else the
// partition rounds (with its tiles reserved).
// small: capacity small_cap; segments of at most kShortMax are filed from
// its end, longer ones from its start.
__device__ __forceinline__ void file_segment(int f, int l, int d, SortSeg* big, SortSeg* small,
                                             int small_cap, SortSeg* tiny, SortSeg* heap, int* ctl,
                                             int big_slot, int tiles_slot) {
  const int n = l - f;
  if (n <= 1) return;
  if (n <= kInsertion) {
    tiny[atomicAdd(ctl + kTiny, 1)] = SortSeg{f, l, d, 0};
  } else if (d == 0) {
    heap[atomicAdd(ctl + kHeap, 1)] = SortSeg{f, l, d, 0};
  } else if (n <= kShortMax) {  // the short ones fill the small list from its end
    small[small_cap - 1 - atomicAdd(ctl + kShort, 1)] = SortSeg{f, l, d, 0};
  } else if (n <= kSmallMax) {
    small[atomicAdd(ctl + kSmall, 1)] = SortSeg{f, l, d, 0};
  } else {
    const int tiles = (n + kTile - 1) / kTile;
    const int t0 = atomicAdd(ctl + tiles_slot, tiles);
    big[atomicAdd(ctl + big_slot, 1)] = SortSeg{f, l, d, t0};
  }
}

// Initial segments: the objects of each listed node (a split node only,
// for the final sort along its best axis).
__global__ void k_file_nodes(const RNode* nodes, const int* active, int m, const NodeBest* best,
                             SortSeg* big, SortSeg* small, int small_cap, SortSeg* tiny,
                             SortSeg* heap, int* ctl) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= m) return;
  if (best && best[a].axis < 0) return;
  const RNode& nd = nodes[active[a]];
  const int n = nd.l - nd.f;
  if (n < 2) return;
  file_segment(nd.f, nd.l, 2 * floor_log2(n), big, small, small_cap, tiny, heap, ctl, kBig,
               kTiles);
}

// Tile -> segment map of the partition rounds.
__global__ void k_tile_map(const SortSeg* big, const int* n_big, int* tile_seg) {
  const int s = blockIdx.x;
  if (s >= *n_big) return;
  const SortSeg g = big[s];
  const int tiles = (g.l - g.f + kTile - 1) / kTile;
  for (int t = threadIdx.x; t < tiles; t += blockDim.x) tile_seg[g.tile0 + t] = s;
}

// Round step 1: the median of three to the front of every big segment.
__global__ void k_pivot(const SortSeg* big, int n_big, double* key, int* idx) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_big) return;
  const SortSeg g = big[s];
  median_to_first(key, idx, g.f, g.f + 1, g.f + (g.l - g.f) / 2, g.l - 1);
}

// Stop flags of position p of segment g around pivot key pk: left stops in
// [f + 1, l), right stops in [f, l).
__device__ __forceinline__ void stop_flags(const double* key, const SortSeg& g, double pk, int p,
                                           int& lf, int& rf) {
  lf = rf = 0;
  if (p >= g.l) return;
  const double k = key[p];
  lf = p > g.f && !(k < pk);
  rf = !(pk < k);
}

// Block-wide exclusive sum of one value per thread; returns the total.
__device__ __forceinline__ int block_exclusive(int v, int& excl, int* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = lane < int(blockDim.x >> 5) ? sh[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    sh[32 + lane] = t;  // inclusive over warps
  }
  __syncthreads();
  const int before = w ? sh[32 + w - 1] : 0;
  excl = before + x - v;
  const int total = sh[32 + (blockDim.x >> 5) - 1];
  __syncthreads();
  return total;
}

// Round step 2: stop counts per tile.
__global__ void __launch_bounds__(kTileThreads) k_count(const SortSeg* big, const int* tile_seg,
                                                        const double* key, int* cnt_l,
                                                        int* cnt_r) {
  __shared__ int sh[64];
  const int tile = blockIdx.x;
  const SortSeg g = big[tile_seg[tile]];
  const double pk = key[g.f];
  const int base = g.f + (tile - g.tile0) * kTile + threadIdx.x * (kTile / kTileThreads);
  int nl = 0, nr = 0;
  for (int j = 0; j < kTile / kTileThreads; ++j) {
    int lf, rf;
    stop_flags(key, g, pk, base + j, lf, rf);
    nl += lf;
    nr += rf;
  }
  int ex;
  const int tl = block_exclusive(nl, ex, sh);
  const int tr = block_exclusive(nr, ex, sh);
  if (threadIdx.x == 0) {
    cnt_l[tile] = tl;
    cnt_r[tile] = tr;
  }
}

// Round step 3: tile offsets and stop totals per segment.
__global__ void k_tile_offsets(const SortSeg* big, int n_big, const int* cnt_l, const int* cnt_r,
                               int* off_l, int* off_r, int2* totals) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_big) return;
  const SortSeg g = big[s];
  const int tiles = (g.l - g.f + kTile - 1) / kTile;
  int al = 0, ar = 0;
  for (int t = 0; t < tiles; ++t) {
    off_l[g.tile0 + t] = al;
    off_r[g.tile0 + t] = ar;
    al += cnt_l[g.tile0 + t];
    ar += cnt_r[g.tile0 + t];
  }
  totals[s] = make_int2(al, ar);
}

// Round step 4: the stops' positions, left stops ascending in lpos[f ..],
// right stops descending in rpos[f ..].
__global__ void __launch_bounds__(kTileThreads) k_stops(const SortSeg* big, const int* tile_seg,
                                                        const double* key, const int* off_l,
                                                        const int* off_r, const int2* totals,
                                                        int* lpos, int* rpos) {
  __shared__ int sh[64];
  const int tile = blockIdx.x;
  const int s = tile_seg[tile];
  const SortSeg g = big[s];
  const double pk = key[g.f];
  const int base = g.f + (tile - g.tile0) * kTile + threadIdx.x * (kTile / kTileThreads);
  int lf[kTile / kTileThreads], rf[kTile / kTileThreads];
  int nl = 0, nr = 0;
  for (int j = 0; j < kTile / kTileThreads; ++j) {
    stop_flags(key, g, pk, base + j, lf[j], rf[j]);
    nl += lf[j];
    nr += rf[j];
  }
  int el, er;
  block_exclusive(nl, el, sh);
  block_exclusive(nr, er, sh);
  int rl = off_l[tile] + el, rr = off_r[tile] + er;
  const int n_r = totals[s].y;
  for (int j = 0; j < kTile / kTileThreads; ++j) {
    if (lf[j]) lpos[g.f + rl++] = base + j;
    if (rf[j]) rpos[g.f + (n_r - 1 - rr++)] = base + j;
  }
}

// Round step 5: the exchanges (k-th left stop with k-th right stop while
// the left one lies left of the right one).
__global__ void __launch_bounds__(kTileThreads) k_exchange(const SortSeg* big,
                                                           const int* tile_seg,
                                                           const int2* totals, const int* lpos,
                                                           const int* rpos, double* key,
                                                           int* idx) {
  const int tile = blockIdx.x;
  const int s = tile_seg[tile];
  const SortSeg g = big[s];
  const int m = min(totals[s].x, totals[s].y);
  const int k0 = (tile - g.tile0) * kTile;
  for (int k = k0 + threadIdx.x; k < min(m, k0 + kTile); k += blockDim.x) {
    const int a = lpos[g.f + k], b = rpos[g.f + k];
    if (a < b) swap_pair(key, idx, a, b);
  }
}

// Round step 6: the cut of every big segment and its two parts filed.
__global__ void k_cut(const SortSeg* big, int n_big, const int2* totals, const int* lpos,
                      const int* rpos, SortSeg* big_next, SortSeg* small, int small_cap,
                      SortSeg* tiny, SortSeg* heap, int* ctl) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_big) return;
  const SortSeg g = big[s];
  const int nl = totals[s].x, nr = totals[s].y;
  int lo = 0, hi = min(nl, nr);  // first k whose left stop is not left of its right stop
  while (lo < hi) {
    const int mid = (lo + hi) / 2;
    if (lpos[g.f + mid] < rpos[g.f + mid]) lo = mid + 1;
    else hi = mid;
  }
  const int K = lo;
  int cut = K < nl ? lpos[g.f + K] : g.l;
  if (K >= 1) cut = min(cut, rpos[g.f + K - 1]);
  if (cut <= g.f || cut >= g.l) {  // the sentinel argument guarantees both parts
    atomicOr(ctl + kError, 1);
    return;
  }
  file_segment(g.f, cut, g.d - 1, big_next, small, small_cap, tiny, heap, ctl, kBigNext,
               kTilesNext);
  file_segment(cut, g.l, g.d - 1, big_next, small, small_cap, tiny, heap, ctl, kBigNext,
               kTilesNext);
}

// A warp per segment of at most kSmallMax: the segment is sorted in shared
// memory (partition by the warp, exchanges spread over its lanes), then the
// leftover segments of at most 16 are insertion sorted, one per lane.
template <int kCap>
constexpr size_t small_smem() {
  return size_t(kCap) * (8 + 4 + 2 + 2 + 4);
}

// segs: the list; n_segs: its count; from_end > 0: the list is read from
// its end (entry from_end - 1 - s, from_end being the list's capacity).
template <int kCap>
__global__ void __launch_bounds__(32) k_small(const SortSeg* segs, const int* n_segs,
                                              int from_end, double* key, int* idx, int* ctl) {
  extern __shared__ __align__(16) unsigned char smem[];
  double* sk = reinterpret_cast<double*>(smem);
  int* si = reinterpret_cast<int*>(sk + kCap);
  short* lp = reinterpret_cast<short*>(si + kCap);
  short* rp = lp + kCap;
  int* tiny = reinterpret_cast<int*>(rp + kCap);
  __shared__ int3 stack[64];
  const int lane = threadIdx.x;
  const unsigned below = (1u << lane) - 1u;
  const int n = *n_segs;
  for (int s = blockIdx.x; s < n; s += gridDim.x) {
    const SortSeg g = segs[from_end > 0 ? from_end - 1 - s : s];
    const int len = g.l - g.f;
    for (int i = lane; i < len; i += 32) {
      sk[i] = key[g.f + i];
      si[i] = idx[g.f + i];
    }
    if (lane == 0) stack[0] = make_int3(0, len, g.d);
    int sp = 1, n_tiny = 0;
    __syncwarp();
    while (sp > 0) {
      const int3 t = stack[--sp];
      __syncwarp();
      const int f = t.x, l = t.y, d = t.z;
      if (l - f <= kInsertion) {
        if (l - f >= 2) {
          if (lane == 0) tiny[n_tiny] = f | ((l - f) << 16);
          ++n_tiny;
        }
        continue;
      }
      if (d == 0) {
        if (lane == 0) heap_sort(sk + f, si + f, l - f);
        __syncwarp();
        continue;
      }
      if (lane == 0) median_to_first(sk, si, f, f + 1, f + (l - f) / 2, l - 1);
      __syncwarp();
      const double pk = sk[f];
      int nl = 0, nr = 0;
      for (int b = f + 1; b < l; b += 32) {
        const int p = b + lane;
        const bool fl = p < l && !(sk[p] < pk);
        const unsigned m = __ballot_sync(0xffffffffu, fl);
        if (fl) lp[nl + __popc(m & below)] = short(p);
        nl += __popc(m);
      }
      for (int b = l - 1; b >= f; b -= 32) {
        const int p = b - lane;
        const bool fr = p >= f && !(pk < sk[p]);
        const unsigned m = __ballot_sync(0xffffffffu, fr);
        if (fr) rp[nr + __popc(m & below)] = short(p);
        nr += __popc(m);
      }
      __syncwarp();
      const int mk = min(nl, nr);
      int K = 0;
      for (int b = 0; b < mk; b += 32) {
        const int k = b + lane;
        const unsigned m = __ballot_sync(0xffffffffu, k < mk && lp[k] < rp[k]);
        K += __popc(m);
        if (m != 0xffffffffu) break;
      }
      for (int k = lane; k < K; k += 32) swap_pair(sk, si, lp[k], rp[k]);
      int cut = K < nl ? int(lp[K]) : l;
      if (K >= 1) cut = min(cut, int(rp[K - 1]));
      __syncwarp();
      if (cut <= f || cut >= l || sp + 2 > 64) {
        if (lane == 0) atomicOr(ctl + kError, 2);
        sp = 0;
        n_tiny = 0;
        break;
      }
      if (lane == 0) {
        stack[sp] = make_int3(f, cut, d - 1);
        stack[sp + 1] = make_int3(cut, l, d - 1);
      }
      sp += 2;
      __syncwarp();
    }
    __syncwarp();
    for (int j = lane; j < n_tiny; j += 32) {
      const int f = tiny[j] & 0xffff, c = tiny[j] >> 16;
      insertion_sort(sk, si, f, f + c);
    }
    __syncwarp();
    for (int i = lane; i < len; i += 32) {
      key[g.f + i] = sk[i];
      idx[g.f + i] = si[i];
    }
    __syncwarp();
  }
}

// Insertion sort of the short segments the partition rounds left.
__global__ void k_tiny(const SortSeg* segs, const int* n_segs, double* key, int* idx) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= *n_segs) return;
  insertion_sort(key, idx, segs[s].f, segs[s].l);
}

// Heap sort of the segments the partition rounds ran out of depth on.
__global__ void k_heap(const SortSeg* segs, const int* n_segs, double* key, int* idx) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= *n_segs) return;
  heap_sort(key + segs[s].f, idx + segs[s].f, segs[s].l - segs[s].f);
}

// ---- one tree level ------------------------------------------------------

// Sort keys: position p of an active node (of a split node, for the final
// sort) gets its box centre along the axis; every position starts as itself
// in the permutation.
__global__ void k_keys(const float4* lo, const float4* hi, const int* node_of,
                       const NodeBest* best, int axis, int n, double* key, int* idx) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  idx[p] = p;
  const int a = node_of[p];
  if (a < 0) return;
  const int ax = best ? best[a].axis : axis;
  if (ax < 0) return;
  key[p] = centre(lo[p], hi[p], ax);
}

// The build order after a sort: records moved along the permutation.
__global__ void k_gather(const float4* lo, const float4* hi, const int* idx, int n, float4* lo2,
                         float4* hi2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int q = idx[p];
  lo2[p] = lo[q];
  hi2[p] = hi[q];
}

// ---- per-level node work on warp tiles ------------------------------------
//
// A node's objects [f, l) are cut into tiles of kWarpTile consecutive
// objects (a node has at least one tile, a tile never spans two nodes); a
// warp works on a tile, 8 consecutive objects per lane.
constexpr int kSweepItems = 8;
constexpr int kWarpTile = 32 * kSweepItems;

struct BoxF {
  float l[3], h[3];
};

__device__ __forceinline__ BoxF box_merge(const BoxF& a, const BoxF& b) {
  BoxF r;
  for (int c = 0; c < 3; ++c) {
    r.l[c] = fminf(a.l[c], b.l[c]);
    r.h[c] = fmaxf(a.h[c], b.h[c]);
  }
  return r;
}

__device__ __forceinline__ BoxF box_empty() {
  BoxF r;
  for (int c = 0; c < 3; ++c) {
    r.l[c] = INFINITY;
    r.h[c] = -INFINITY;
  }
  return r;
}

__device__ __forceinline__ BoxF box_shfl_up(const BoxF& x, int o) {
  BoxF y;
  for (int c = 0; c < 3; ++c) {
    y.l[c] = __shfl_up_sync(0xffffffffu, x.l[c], o);
    y.h[c] = __shfl_up_sync(0xffffffffu, x.h[c], o);
  }
  return y;
}

__device__ __forceinline__ BoxF box_shfl_down(const BoxF& x, int o) {
  BoxF y;
  for (int c = 0; c < 3; ++c) {
    y.l[c] = __shfl_down_sync(0xffffffffu, x.l[c], o);
    y.h[c] = __shfl_down_sync(0xffffffffu, x.h[c], o);
  }
  return y;
}

__device__ __forceinline__ BoxF rec_box(const float4& L, const float4& H) {
  return BoxF{{L.x, L.y, L.z}, {H.x, H.y, H.z}};
}

// The box bounds as the host's node box takes them: the least lower bound
// (greatest upper bound), the later object winning between equal values, so
// that the sign of a zero is the host's.
struct ExactBox {
  float v[6];
  int p[6];  // object position the value came from, -1: none yet
};

__device__ __forceinline__ bool exact_better(int c, float v, int p, float bv, int bp) {
  if (p < 0) return false;
  if (bp < 0) return true;
  return c < 3 ? (v < bv || (v == bv && p > bp)) : (v > bv || (v == bv && p > bp));
}

__device__ __forceinline__ void exact_add(ExactBox& b, int c, float v, int p) {
  if (exact_better(c, v, p, b.v[c], b.p[c])) {
    b.v[c] = v;
    b.p[c] = p;
  }
}

__device__ __forceinline__ void exact_warp_reduce(ExactBox& b) {
  for (int o = 16; o; o >>= 1)
    for (int c = 0; c < 6; ++c) {
      const float v = __shfl_down_sync(0xffffffffu, b.v[c], o);
      const int p = __shfl_down_sync(0xffffffffu, b.p[c], o);
      exact_add(b, c, v, p);
    }
}

struct __align__(16) TileBest {
  double cost;
  int i, pad;
};

constexpr int kNodeSmall = 16;  // nodes this small are handled by one thread each

// Tiles of every active node of more than kNodeSmall objects (per node its
// first tile and tile count, per tile its node), and the lists of those
// nodes and of the small ones.
__global__ void k_level_tiles(const RNode* nodes, const int* active, int m, int2* node_tiles,
                              int* tile_node, int* tiled, int* small_nodes, int* ctl) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= m) return;
  const RNode& nd = nodes[active[a]];
  const int n = nd.l - nd.f;
  if (n <= kNodeSmall) {
    small_nodes[atomicAdd(ctl + kSmallNodes, 1)] = a;
    node_tiles[a] = make_int2(0, 0);
    return;
  }
  const int nt = (n + kWarpTile - 1) / kWarpTile;
  const int t0 = atomicAdd(ctl + kSweepTiles, nt);
  node_tiles[a] = make_int2(t0, nt);
  tiled[atomicAdd(ctl + kTiledNodes, 1)] = a;
  for (int t = 0; t < nt; ++t) tile_node[t0 + t] = a;
}

// A small node's set-up, one thread each: its positions marked, its box
// formed object by object as the host forms it (box = std::min(object, box),
// std::max(object, box)), the surface area and the leaf cost as the best.
__global__ void k_small_node_box(RNode* nodes, const int* active, const int* small_nodes, int k,
                                 const float4* lo, const float4* hi, int* node_of,
                                 double* sa_root, NodeBest* best) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k) return;
  const int a = small_nodes[j];
  RNode& nd = nodes[active[a]];
  float b[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int p = nd.f; p < nd.l; ++p) {
    node_of[p] = a;
    const float4 L = lo[p], H = hi[p];
    const float x[6] = {L.x, L.y, L.z, H.x, H.y, H.z};
    for (int c = 0; c < 3; ++c) {
      if (!(b[c] < x[c])) b[c] = x[c];
      if (!(x[3 + c] < b[3 + c])) b[3 + c] = x[3 + c];
    }
  }
  for (int c = 0; c < 6; ++c) nd.bb[c] = double(b[c]);
  sa_root[a] = surface_area(b[0], b[1], b[2], b[3], b[4], b[5]);
  best[a] = NodeBest{double(nd.l - nd.f), -1, -1};
}

// A small node's sweep over one axis order, one thread each, in the
// reference loop's order: prefix areas, then suffix areas with the costs,
// a cost kept when it is below the best so far.
__global__ void k_small_node_sweep(const RNode* nodes, const int* active, const int* small_nodes,
                                   int k, const float4* lo, const float4* hi,
                                   const double* sa_root, int axis, NodeBest* best) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k) return;
  const int a = small_nodes[j];
  const RNode& nd = nodes[active[a]];
  const int n = nd.l - nd.f;
  if (n < 3) return;
  double sa1[kNodeSmall];
  BoxF run = box_empty();
  for (int i = 0; i < n; ++i) {
    run = box_merge(run, rec_box(lo[nd.f + i], hi[nd.f + i]));
    sa1[i] = surface_area(run.l[0], run.l[1], run.l[2], run.h[0], run.h[1], run.h[2]);
  }
  double sa2[kNodeSmall];
  run = box_empty();
  for (int i = n - 1; i >= 0; --i) {
    run = box_merge(run, rec_box(lo[nd.f + i], hi[nd.f + i]));
    sa2[i] = surface_area(run.l[0], run.l[1], run.l[2], run.h[0], run.h[1], run.h[2]);
  }
  NodeBest b = best[a];
  const double sr = sa_root[a];
  for (int i = 1; i < n - 1; ++i) {
    const double num = __dadd_rn(__dmul_rn(double(i), sa1[i]), __dmul_rn(double(n - i), sa2[i]));
    const double cost = __dadd_rn(2.0, __ddiv_rn(__dmul_rn(num, 1.0), sr));
    if (cost < b.cost) b = NodeBest{cost, axis, i};
  }
  best[a] = b;
}

// Level set-up per tile: positions marked with their node, and the tile's
// share of the node box (taken in the order the objects arrive in).
__global__ void k_tile_exact_box(const RNode* nodes, const int* active, const int2* node_tiles,
                                 const int* tile_node, int n_tiles, const float4* lo,
                                 const float4* hi, int* node_of, ExactBox* tbox) {
  const int tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (tile >= n_tiles) return;
  const int a = tile_node[tile];
  const RNode& nd = nodes[active[a]];
  const int b = nd.f + (tile - node_tiles[a].x) * kWarpTile + lane * kSweepItems;
  ExactBox e;
  for (int c = 0; c < 6; ++c) {
    e.v[c] = 0.0f;
    e.p[c] = -1;
  }
  for (int j = 0; j < kSweepItems; ++j) {
    const int p = b + j;
    if (p >= nd.l) break;
    node_of[p] = a;
    const float4 L = lo[p], H = hi[p];
    const float x[6] = {L.x, L.y, L.z, H.x, H.y, H.z};
    for (int c = 0; c < 6; ++c) exact_add(e, c, x[c], p);
  }
  exact_warp_reduce(e);
  if (lane == 0) tbox[tile] = e;
}

// Node box from its tiles, its surface area, and the leaf cost as the best
// so far; a warp per node.
__global__ void k_node_box(RNode* nodes, const int* active, const int* tiled, int k,
                           const int2* node_tiles, const ExactBox* tbox, double* sa_root,
                           NodeBest* best) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= k) return;
  const int a = tiled[w];
  const int2 nt = node_tiles[a];
  ExactBox e;
  for (int c = 0; c < 6; ++c) {
    e.v[c] = 0.0f;
    e.p[c] = -1;
  }
  for (int t = lane; t < nt.y; t += 32) {
    const ExactBox& x = tbox[nt.x + t];
    for (int c = 0; c < 6; ++c) exact_add(e, c, x.v[c], x.p[c]);
  }
  exact_warp_reduce(e);
  if (lane == 0) {
    RNode& nd = nodes[active[a]];
    for (int c = 0; c < 6; ++c) nd.bb[c] = double(e.v[c]);
    sa_root[a] = surface_area(e.v[0], e.v[1], e.v[2], e.v[3], e.v[4], e.v[5]);
    best[a] = NodeBest{double(nd.l - nd.f), -1, -1};
  }
}

// Box of each tile's objects (in the current order).
__global__ void k_tile_boxes(const RNode* nodes, const int* active, const int2* node_tiles,
                             const int* tile_node, int n_tiles, const float4* lo,
                             const float4* hi, BoxF* tagg) {
  const int tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (tile >= n_tiles) return;
  const int a = tile_node[tile];
  const RNode& nd = nodes[active[a]];
  const int b = nd.f + (tile - node_tiles[a].x) * kWarpTile + lane * kSweepItems;
  BoxF x = box_empty();
  for (int j = 0; j < kSweepItems && b + j < nd.l; ++j) x = box_merge(x, rec_box(lo[b + j], hi[b + j]));
  for (int o = 16; o; o >>= 1) x = box_merge(x, box_shfl_down(x, o));
  if (lane == 0) tagg[tile] = x;
}

// Per node, the box of the objects before each of its tiles (pre) and
// after it (post); a warp per node, 32 tiles at a time.
__global__ void k_tile_carries(const int* tiled, int k, const int2* node_tiles, const BoxF* tagg,
                               BoxF* pre, BoxF* post) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= k) return;
  const int a = tiled[w];
  const int2 nt = node_tiles[a];
  BoxF run = box_empty();
  for (int c = 0; c < nt.y; c += 32) {
    const int t = c + lane;
    BoxF x = t < nt.y ? tagg[nt.x + t] : box_empty();
    for (int o = 1; o < 32; o <<= 1) {
      const BoxF y = box_shfl_up(x, o);
      if (lane >= o) x = box_merge(y, x);
    }
    BoxF ex = box_shfl_up(x, 1);
    if (lane == 0) ex = box_empty();
    if (t < nt.y) pre[nt.x + t] = box_merge(run, ex);
    BoxF last;
    for (int k = 0; k < 3; ++k) {
      last.l[k] = __shfl_sync(0xffffffffu, x.l[k], 31);
      last.h[k] = __shfl_sync(0xffffffffu, x.h[k], 31);
    }
    run = box_merge(run, last);
  }
  run = box_empty();
  for (int c = 0; c < nt.y; c += 32) {  // from the last tile backwards
    const int t = nt.y - 1 - (c + lane);
    BoxF x = t >= 0 ? tagg[nt.x + t] : box_empty();
    for (int o = 1; o < 32; o <<= 1) {
      const BoxF y = box_shfl_up(x, o);
      if (lane >= o) x = box_merge(y, x);
    }
    BoxF ex = box_shfl_up(x, 1);
    if (lane == 0) ex = box_empty();
    if (t >= 0) post[nt.x + t] = box_merge(run, ex);
    BoxF last;
    for (int k = 0; k < 3; ++k) {
      last.l[k] = __shfl_sync(0xffffffffu, x.l[k], 31);
      last.h[k] = __shfl_sync(0xffffffffu, x.h[k], 31);
    }
    run = box_merge(run, last);
  }
}

// The reference's sweep over one axis order (BVH.h:135-230), a warp per
// tile: for object i of the node, the surface area of the box of objects
// 0..i (sa1) and of objects i..n-1 (sa2), the cost
// 2 + (i sa1 + (n - i) sa2) / SA(node box) for 1 <= i <= n - 2 (each operation
// rounded on its own), and the tile's cheapest split below the leaf cost,
// the first one among equal costs.
__global__ void k_tile_sweep(const RNode* nodes, const int* active, const int2* node_tiles,
                             const int* tile_node, int n_tiles, const float4* lo,
                             const float4* hi, const BoxF* pre, const BoxF* post,
                             const double* sa_root, TileBest* tbest) {
  const int tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (tile >= n_tiles) return;
  const int a = tile_node[tile];
  const RNode& nd = nodes[active[a]];
  const int n = nd.l - nd.f;
  const int i0 = (tile - node_tiles[a].x) * kWarpTile + lane * kSweepItems;  // object index
  BoxF bx[kSweepItems];
  BoxF mine = box_empty();
  for (int j = 0; j < kSweepItems; ++j) {
    bx[j] = i0 + j < n ? rec_box(lo[nd.f + i0 + j], hi[nd.f + i0 + j]) : box_empty();
    mine = box_merge(mine, bx[j]);
  }
  // boxes of the lanes before / after this one
  BoxF up = mine, down = mine;
  for (int o = 1; o < 32; o <<= 1) {
    const BoxF y = box_shfl_up(up, o);
    if (lane >= o) up = box_merge(y, up);
    const BoxF z = box_shfl_down(down, o);
    if (lane + o < 32) down = box_merge(down, z);
  }
  BoxF before = box_shfl_up(up, 1), after = box_shfl_down(down, 1);
  if (lane == 0) before = box_empty();
  if (lane == 31) after = box_empty();
  double sa1[kSweepItems];
  BoxF run = box_merge(pre[tile], before);
  for (int j = 0; j < kSweepItems; ++j) {
    run = box_merge(run, bx[j]);
    sa1[j] = surface_area(run.l[0], run.l[1], run.l[2], run.h[0], run.h[1], run.h[2]);
  }
  const double sr = sa_root[a], leaf = double(n);
  double bc = INFINITY;
  int bi = INT_MAX;
  run = box_merge(post[tile], after);
  for (int j = kSweepItems - 1; j >= 0; --j) {
    run = box_merge(run, bx[j]);
    const int i = i0 + j;
    if (i >= 1 && i <= n - 2) {
      const double sa2 = surface_area(run.l[0], run.l[1], run.l[2], run.h[0], run.h[1], run.h[2]);
      const double num = __dadd_rn(__dmul_rn(double(i), sa1[j]), __dmul_rn(double(n - i), sa2));
      const double cost = __dadd_rn(2.0, __ddiv_rn(__dmul_rn(num, 1.0), sr));
      if (cost < leaf && (cost < bc || (cost == bc && i < bi))) {
        bc = cost;
        bi = i;
      }
    }
  }
  for (int o = 16; o; o >>= 1) {
    const double oc = __shfl_down_sync(0xffffffffu, bc, o);
    const int oi = __shfl_down_sync(0xffffffffu, bi, o);
    if (oc < bc || (oc == bc && oi < bi)) {
      bc = oc;
      bi = oi;
    }
  }
  if (lane == 0) tbest[tile] = TileBest{bc, bi, 0};
}

// The node's cheapest split of this axis, kept if it beats the best so far
// (earlier axes win ties, as the strict < of the reference's loop decides);
// a warp per node.
__global__ void k_node_best(const int* tiled, int k, const int2* node_tiles, const TileBest* tbest,
                            int axis, NodeBest* best) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= k) return;
  const int a = tiled[w];
  const int2 nt = node_tiles[a];
  double bc = INFINITY;
  int bi = INT_MAX;
  for (int t = lane; t < nt.y; t += 32) {
    const TileBest x = tbest[nt.x + t];
    if (x.cost < bc || (x.cost == bc && x.i < bi)) {
      bc = x.cost;
      bi = x.i;
    }
  }
  for (int o = 16; o; o >>= 1) {
    const double oc = __shfl_down_sync(0xffffffffu, bc, o);
    const int oi = __shfl_down_sync(0xffffffffu, bi, o);
    if (oc < bc || (oc == bc && oi < bi)) {
      bc = oc;
      bi = oi;
    }
  }
  if (lane == 0 && bi != INT_MAX && bc < best[a].cost) best[a] = NodeBest{bc, axis, bi};
}

// Children of the split nodes (after the final sort), and the next level's
// active list.
__global__ void k_children(RNode* nodes, const int* active, int m, const NodeBest* best,
                           int* next, int* ctl) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= m) return;
  if (best[a].axis < 0) return;
  RNode& nd = nodes[active[a]];
  const int c = atomicAdd(ctl + kNodes, 2);
  nodes[c].f = nd.f;
  nodes[c].l = nd.f + best[a].split;
  nodes[c].c0 = nodes[c].c1 = -1;
  nodes[c + 1].f = nd.f + best[a].split;
  nodes[c + 1].l = nd.l;
  nodes[c + 1].c0 = nodes[c + 1].c1 = -1;
  nd.c0 = c;
  nd.c1 = c + 1;
  const int k = atomicAdd(ctl + kActiveNext, 2);
  next[k] = c;
  next[k + 1] = c + 1;
}

// Triangle ids in build order.
__global__ void k_ids(const float4* lo, int n, int* ids) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) ids[p] = __float_as_int(lo[p].w);
}

}  // namespace refbvh
}  // namespace sbr
