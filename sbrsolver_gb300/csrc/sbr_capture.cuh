// Capture stage: RayCapture's reception-sphere test (RTSolver.cpp:259-297,
// 805-863) for every tree node against the receivers near its segment, with
// the first step of image correction as a prefilter; k_capture_finish makes
// the FP64 decisions (exact reception test, MultiPathCorrection, suppression
// by a capturing ancestor) for what the FP32 tests could not settle.
#pragma once

#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "sbr_device.h"
#include "sbr_field.cuh"
#include "sbr_kernels.cuh"
#include "sbr_common.cuh"
#include "sbr_trace.cuh"

namespace sbr {

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
  HashTable corr_cache;        // (class, receiver) -> its image correction's outcome
  unsigned char* corr_val;     // per slot: 0 not known yet, 1 fails, 2 succeeds
  unsigned long long* work;    // nodes handed out to warps (zero at launch)
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

// A warp works through batches of nodes.  Each node's segment is clipped to
// the region that can hold its captures and cut into chunks (each receiver is
// owned by the chunk its projection falls in); each chunk's capsule is
// rasterised over the receiver grid one row of cells per lane; a row is one
// contiguous run of receivers, and the lanes stride over the concatenation of
// the rows' runs.  A capture counts unless an ancestor of the node captures
// the same receiver (RTSolver.cpp:277-284).
constexpr int kCapWarps = 4;
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
// per class in FP64 and rounded to FP32 (k_class_cones); k_capture loosens
// each by 2 m_k, m_k = 2^-19 |n_k| (cmax + |img| + |T| + 1).  The FP32 test
// of a point p (|p| <= cmax) or of a cell corner errs by under
// 10 * 2^-24 |n_k| (cmax + |img| + |T|): the plane's rounding, the rounding
// of p, and the dot product.  No cone is used when a plane is
// ill-conditioned (the centroid within 4 m_k of it).  The reference's FP64 test accepts
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
  const float tanb = P.tan_beta32;
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
  const float lc = fmaxf(g.chunk_len, r0);
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
  cb.mr = kRecK * (sp.ns + cmax + S + npmax + 1.0f);
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

// Next batch of `b` nodes for the calling warp (all lanes get the same base).
__device__ __forceinline__ unsigned long long next_batch(unsigned long long* work, int lane,
                                                         int b) {
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(work, (unsigned long long)b);
  return __shfl_sync(0xffffffffu, base, 0);
}

// kStage: stage counts requested (every capture counted, the plain order of
// tests); otherwise the fast path with the correction prefilter and the
// deferred FP64 pass.
// Resident blocks per SM of the fast path (register budget 65536 / (128 x this)).
#ifndef SBR_CAP_BLOCKS
#define SBR_CAP_BLOCKS 6
#endif
template <bool kStage>
__global__ void __launch_bounds__(32 * kCapWarps, kStage ? 4 : SBR_CAP_BLOCKS) k_capture(CaptureArgs A) {
  __shared__ AncRec anc[kCapWarps][kMaxDepth];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned FULL = 0xffffffffu;
  if (A.ctr->overflow & kOvTrace) return;  // this solve will be repeated
  const unsigned long long n_nodes = min(A.ctr->nodes, A.node_cap);
  unsigned long long events = 0, cand = 0, anc_tests = 0;
  unsigned n64 = 0;
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
  // Batches of B nodes are handed out by a work counter, one atomic per warp
  // and batch, so warps that drew short segments take more batches.
  for (unsigned long long base = next_batch(A.work, lane, B); base < n_nodes;
       base = next_batch(A.work, lane, B)) {
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
          // the cone's planes loosened by 2 m, m = 2^-19 |n| (cmax + |img| + |T| + 1)
          float* cn = s_cn[warp][lane];
          cone_ok = !kStage;
          for (int k = 0; k < 3; ++k) {
            const float m = 1.9073486328125e-06f * (c.nn[k] * cmax + c.w[k]);
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
          s_ck[warp][lane] = chunk_box(h, A.grids[h.tx], sp, 0, cmax, A.txp[h.tx].tan_beta32,
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
        const float tanb = P.tan_beta32;
        const float cmax = A.gb[nd.tx].cmax;
        const float ns = sp.ns;
        const int nchunk = sp.nchunk;
        // error margins of the FP32 reception test, from per-node bounds
        const float ml = kRecK * (ns + cmax + 1.0f);
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
                  if constexpr (kStage) {
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
                  } else {
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
                  }
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

// ---- fast path, flattened over the nodes of a batch ------------------------
//
// The same tests as k_capture's fast path with the same chunks, cell boxes
// and margins, so the same (node, receiver) pairs reach k_capture_finish.
// The warp stages B nodes (one lane each: node record, class record, last
// triangle, loosened correction cone, clipped span), then works through the
// whole batch at three flattened levels instead of node by node: the batch's
// (node, chunk) items with one lane per item (cell box, cone test), those
// items' rows of cells with one lane per row (the row's receiver run), and
// those rows' receivers with one lane per receiver (correction prefilter,
// FP32 reception test).  Each level is an inclusive prefix count over the
// lanes; an item finds its parent by a binary search over the counts.  A
// node with a handful of candidates (about six per node at level 9) thus no
// longer holds all 32 lanes through its own chunk, row and receiver passes.

__device__ __forceinline__ int warp_incl_scan(int v, int lane) {
  for (int o = 1; o < 32; o <<= 1) {
    const int x = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += x;
  }
  return v;
}

// The first lane whose inclusive count exceeds k (0 <= k < the total).
__device__ __forceinline__ int warp_find(int incl, int k) {
  int rl = 0;
  for (int step = 16; step; step >>= 1) {
    const int v = __shfl_sync(0xffffffffu, incl, rl + step - 1);
    if (v <= k) rl += step;
  }
  return rl;
}

constexpr int kFastB = 32;  // nodes staged per warp and batch (one per lane)

__global__ void __launch_bounds__(32 * kCapWarps, SBR_CAP_BLOCKS) k_capture_fast(CaptureArgs A) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned FULL = 0xffffffffu;
  if (A.ctr->overflow & kOvTrace) return;  // this solve will be repeated
  const unsigned long long n_nodes = min(A.ctr->nodes, A.node_cap);
  unsigned long long cand = 0;
  constexpr int B = kFastB;
  __shared__ NodeHot s_nh[kCapWarps][B];
  __shared__ Tri32 s_tl[kCapWarps][B];      // the class's last triangle
  __shared__ float s_fl[kCapWarps][B][12];  // image source + correction filter terms
  __shared__ float s_cn[kCapWarps][B][16];  // loosened correction cone
  __shared__ NodeSpan s_sp[kCapWarps][B];   // clipped span and chunking
  __shared__ ChunkBox s_ck[kCapWarps][32];  // the current 32 (node, chunk) items
  __shared__ int s_ckn[kCapWarps][32];      // their node (batch index) | chunk << 8
  for (unsigned long long base = next_batch(A.work, lane, B); base < n_nodes;
       base = next_batch(A.work, lane, B)) {
    int nck = 0;  // chunks of this lane's node
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
          // the cone's planes loosened by 2 m, m = 2^-19 |n| (cmax + |img| + |T| + 1)
          float* cn = s_cn[warp][lane];
          cone_ok = 1;
          for (int k = 0; k < 3; ++k) {
            const float m = 1.9073486328125e-06f * (c.nn[k] * cmax + c.w[k]);
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
        nck = sp.nchunk;
      }
      __syncwarp();
    }
    const int ck_incl = warp_incl_scan(nck, lane);
    const int n_ck = __shfl_sync(FULL, ck_incl, 31);
    for (int k0 = 0; k0 < n_ck; k0 += 32) {
      // level 1: one lane per (node, chunk) item
      const int k = k0 + lane;
      const int j = warp_find(ck_incl, min(k, n_ck - 1));
      const int j_incl = __shfl_sync(FULL, ck_incl, j), j_n = __shfl_sync(FULL, nck, j);
      int nrows = 0;
      if (k < n_ck) {
        const int ch = k - (j_incl - j_n);
        const NodeHot& nd = s_nh[warp][j];
        const NodeSpan& sp = s_sp[warp][j];
        const ChunkBox cb = chunk_box(nd, A.grids[nd.tx], sp, ch, A.gb[nd.tx].cmax,
                                      A.txp[nd.tx].tan_beta32, sp.use_cone != 0, s_cn[warp][j]);
        s_ck[warp][lane] = cb;
        s_ckn[warp][lane] = j | ch << 8;
        nrows = cb.nrows;
      }
      __syncwarp();
      const int r_incl = warp_incl_scan(nrows, lane);
      const int n_r = __shfl_sync(FULL, r_incl, 31);
      for (int r0 = 0; r0 < n_r; r0 += 32) {
        // level 2: one lane per row of cells: the part of its chunk within rb
        // of the row's y/z band, cut to the cone, as a run of receivers
        const int r = r0 + lane;
        const int ci = warp_find(r_incl, min(r, n_r - 1));
        const int ci_incl = __shfl_sync(FULL, r_incl, ci), ci_n = __shfl_sync(FULL, nrows, ci);
        int beg = 0, cnt = 0;
        if (r < n_r) {
          const int ridx = r - (ci_incl - ci_n);
          const ChunkBox& cb = s_ck[warp][ci];
          const int jn = s_ckn[warp][ci] & 0xff;
          const NodeHot& nd = s_nh[warp][jn];
          const RxGrid& g = A.grids[nd.tx];
          const float3 s = make_float3(nd.s[0], nd.s[1], nd.s[2]);
          const float3 u = make_float3(nd.u[0], nd.u[1], nd.u[2]);
          // Reciprocals for the cell-range arithmetic: every range is widened
          // by at least 2e-3 m + cell/100, far more than the few ulps a product
          // with a reciprocal differs from the quotient.
          const float inv_uy = __frcp_rn(u.y), inv_uz = __frcp_rn(u.z);
          const float rb = cb.rb;
          const int ny = cb.c1[1] - cb.c0[1] + 1;
          // one layer of cells (receivers on a plane) needs no division
          const bool flat = cb.c1[2] == cb.c0[2];
          const int iy = cb.c0[1] + (flat ? ridx : ridx % ny);
          const int iz = cb.c0[2] + (flat ? 0 : ridx / ny);
          const float y0 = g.org[1] + iy * g.cell - rb, y1 = g.org[1] + (iy + 1) * g.cell + rb;
          const float z0 = g.org[2] + iz * g.cell - rb, z1 = g.org[2] + (iz + 1) * g.cell + rb;
          float la = cb.a, lb = cb.b;
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
            const float inv_cell = g.inv_cell;
            const float xa = s.x + la * u.x, xb = s.x + lb * u.x;
            int x0 = max(cb.c0[0], int(floorf((fminf(xa, xb) - rb - g.org[0]) * inv_cell)));
            int x1 = min(cb.c1[0], int(floorf((fmaxf(xa, xb) + rb - g.org[0]) * inv_cell)));
            if (s_sp[warp][jn].use_cone && x0 <= x1)
              cone_cells(s_cn[warp][jn], g, inv_cell, iy, iz, x0, x1);
            if (x0 <= x1) {
              const int row = (iz * g.dim[1] + iy) * g.dim[0];
              beg = g.cell_start[row + x0];
              cnt = g.cell_start[row + x1 + 1] - beg;
            }
          }
        }
        const int c_incl = warp_incl_scan(cnt, lane);
        const int n_c = __shfl_sync(FULL, c_incl, 31);
        for (int q0 = 0; q0 < n_c; q0 += 32) {
          // level 3: one lane per candidate receiver
          const int q = q0 + lane;
          const int rl = warp_find(c_incl, min(q, n_c - 1));
          const int rincl = __shfl_sync(FULL, c_incl, rl);
          const int rcnt = __shfl_sync(FULL, cnt, rl);
          const int rbeg = __shfl_sync(FULL, beg, rl);
          const int rci = __shfl_sync(FULL, ci, rl);
          if (q >= n_c) continue;
          const int ckn = s_ckn[warp][rci];
          const int jn = ckn & 0xff, ch = ckn >> 8;
          const NodeHot& nd = s_nh[warp][jn];
          const NodeSpan& sp = s_sp[warp][jn];
          const float a = s_ck[warp][rci].a, b = s_ck[warp][rci].b, mr = s_ck[warp][rci].mr;
          const RxGrid& g = A.grids[nd.tx];
          const float3 s = make_float3(nd.s[0], nd.s[1], nd.s[2]);
          const float3 u = make_float3(nd.u[0], nd.u[1], nd.u[2]);
          const float4 c4 = g.rx32[rbeg + (q - (rincl - rcnt))];
          const float3 c = make_float3(c4.x, c4.y, c4.z);
          const float wx = c.x - s.x, wy = c.y - s.y, wz = c.z - s.z;
          const float lam = u.x * wx + u.y * wy + u.z * wz;
          if (ch > 0 && lam < a) continue;                 // owned by an earlier chunk
          if (ch < sp.nchunk - 1 && lam >= b) continue;    // owned by a later chunk
          const int gi = __float_as_int(c4.w);
          ++cand;
          if (is_root_class(nd.cls)) {
            if (!A.direct_ok[gi]) continue;
          } else {
            // MultiPathCorrection's last step must cross the class's last
            // triangle: FP32 filter from the image source towards the receiver
            const float* fl = s_fl[warp][jn];
            const TriFrom Fl{fl[3], fl[4], fl[5], fl[6], fl[7], fl[8], fl[9], fl[10]};
            const float3 dd = make_float3(c.x - fl[0], c.y - fl[1], c.z - fl[2]);
            if (!tri_filter_from(s_tl[warp][jn], Fl, dd,
                                 sqrt_up(dd.x * dd.x + dd.y * dd.y + dd.z * dd.z)))
              continue;
          }
          const float tanb = A.txp[nd.tx].tan_beta32;
          const float len = nd.len, S = nd.S;
          int v;
          if (lam < a || lam > b) {
            // outside the chunk's own range: full-margin test
            v = reception32(s, u, len, S, c, tanb);
          } else {
            const float ml = kRecK * (sp.ns + A.gb[nd.tx].cmax + 1.0f);
            if (lam < -ml) {
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
          }
          // the exact reception test, image correction and ancestor
          // suppression run densely in k_capture_finish
          if (v == 0) continue;
          const unsigned long long slot = warp_reserve(&A.ctr->pairs, 1);
          if (slot < A.pair_cap)
            A.pairs[slot] =
                make_uint2(uint32_t(base + jn), uint32_t(gi) | (v < 0 ? 0x80000000u : 0u));
          else
            atomicOr(&A.ctr->overflow, kOvPairs);
        }
      }
      __syncwarp();  // the next group of items overwrites s_ck
    }
    __syncwarp();  // the next batch overwrites the staged records
  }
  for (int o = 16; o; o >>= 1) cand += __shfl_xor_sync(FULL, cand, o);
  if (lane == 0 && cand) atomicAdd(&A.ctr->cand, cand);
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
    bool ok;
    if (is_root_class(nd.cls)) {
      ok = A.direct_ok[gi] != 0;
    } else {
      // The correction depends only on the class and the receiver, and the
      // reception spheres are wide (beta = acos(-1/sqrt 5) / (3 (L + 1))), so
      // many nodes of one class capture the same receiver: the outcome is
      // kept per (class, receiver) and each is computed about once.
      const unsigned long long key = (unsigned long long)nd.cls << 32 | uint32_t(gi);
      bool fresh = false;
      const uint32_t slot = ht_claim(A.corr_cache, key, 32, fresh);
      unsigned char known = 0;
      if (slot != 0xFFFFFFFFu && !fresh)
        known = *reinterpret_cast<volatile unsigned char*>(&A.corr_val[slot]);
      if (known) {
        ok = known == 2;
      } else {
        ok = correct_event(A.sc, A.cls_info, nd.cls, c, c64, n64);
        if (slot != 0xFFFFFFFFu) {
          A.corr_val[slot] = ok ? 2 : 1;
          if (fresh) atomicAdd(&A.ctr->used_cc, 1ull);
        }
      }
    }
    if (!ok) continue;
    const float tanb = P.tan_beta32;
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

}  // namespace sbr
