// Path stage: duplicate removal by coplanar key (RTSolver.cpp:435-459), the
// corrected geometry and field of each survivor (FieldCompute.cpp:71-151)
// and the per-receiver sum in (launch, BFS) order (FieldCompute.cpp:11-25).
#pragma once

#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "sbr_device.h"
#include "sbr_field.cuh"
#include "sbr_kernels.cuh"
#include "sbr_common.cuh"
#include "sbr_trace.cuh"
#include "sbr_capture.cuh"

namespace sbr {

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
// (RTSolver.cpp:330-433) for a path whose correction succeeded when it was
// captured (correct_event; k_direct for the direct path): fills pb.pts with
// the corrected points.
__device__ bool correct_path(const DevScene& sc, const int* rank_to_id, const TxParams& P,
                             const double* rxp, PathBuf& pb) {
  using namespace x64;
  const double* tx = P.tx;
  if (pb.n == 1) {  // the exact segment Tx -> Rx (RTSolver.cpp:385-387)
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
  SegTerms* seg;        // (kMaxDepth + 1) per survivor
  int* path_mat;        // (kMaxDepth + 1) per survivor: material of each ray's start
  // FP32 field mode: bound on each component's absolute error per survivor
  // (0: computed in FP64; -1: no bound, the FP32-phase study mode)
  double* path_bound;
  const int* rx_flag;   // receivers whose paths k_escalate recomputes in FP64
  unsigned long long* fstat;  // [0] paths whose field FP32 mode took in FP64, [1] receivers
};

// FP32 field mode: a path whose condition number (path_combine's kappa)
// exceeds this is computed in FP64.
constexpr float kKappaMax32 = 32.0f;

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

// Field stage, one kernel per part: k_path corrects each survivor's path
// (FP64 image correction, sequential along the path) and writes its points,
// triangles and kinds; k_seg computes every segment's terms (one thread per
// segment); k_combine carries each path's field along it.
__global__ void k_path(FieldArgs A) {
  const unsigned long long ns = min(A.ctr->survivors, A.cap);
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < ns;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const Survivor sv = A.surv[i];
    const TxParams& P = A.txp[A.rx_req[sv.rx]];
    PathBuf pb;
    class_path(A.cls_info, sv.cls, pb);
    correct_path(A.sc, A.rank_to_id, P, A.rx + 3 * size_t(sv.rx), pb);
    A.path_nray[i] = pb.n;
    const size_t b = size_t(i) * (kMaxDepth + 1);
    for (int r = 0; r < pb.n; ++r) {
      const int t = pb.tri[r];
      A.path_tri[b + r] = t >= 0 ? A.rank_to_id[t] : -1;
      A.path_cop[b + r] = t >= 0 ? A.sc.tri64[t].cop : -1;
      A.path_kind[b + r] = pb.kind[r];
      // the hit triangle's own material (the ray's hit record carries it)
      A.path_mat[b + r] = r > 0 ? A.sc.tri64[pb.tri[r - 1]].mat : 0;
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

// The path inputs of path i for the field functions: points, frames of the
// triangles each ray ends on, kinds and materials of each ray's start.
struct PathView {
  int n;
  const double (*pts)[3];
  const double* frames[kMaxDepth + 1];
  int kind[kMaxDepth + 1];
  int mat[kMaxDepth + 1];
};

__device__ __forceinline__ void path_view(const FieldArgs& A, unsigned long long i, PathView& v) {
  v.n = A.path_nray[i];
  v.pts = reinterpret_cast<const double(*)[3]>(A.path_pts + size_t(i) * (kMaxDepth + 2) * 3);
  const size_t b = size_t(i) * (kMaxDepth + 1);
  for (int r = 0; r < v.n; ++r) {
    // frames by the id's position in the caller's mesh vector, as the
    // reference looks them up (FieldCompute.cpp:107)
    const int id = A.path_tri[b + r];
    v.frames[r] = id >= 0 ? A.sc.corr[id].cs : nullptr;
    v.kind[r] = A.path_kind[b + r];
    v.mat[r] = A.path_mat[b + r];
  }
}

__global__ void k_seg(FieldArgs A) {
  const unsigned long long ns = min(A.ctr->survivors, A.cap);
  const unsigned long long n_slots = ns * (kMaxDepth + 1);
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
       k < n_slots; k += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long i = k / (kMaxDepth + 1);
    const int r = int(k % (kMaxDepth + 1));
    if (r >= A.path_nray[i]) continue;
    const Survivor sv = A.surv[i];
    const TxParams& P = A.txp[A.rx_req[sv.rx]];
    PathView v;
    path_view(A, i, v);
    const PatternTab pat{P.pat, P.pat_nt, P.pat_np, P.pat_dt, P.pat_dp};
    const int prec = A.precision < 0 ? P.precision : A.precision;
    SegTerms t;
    if (prec != 0)
      seg_terms<float>(r, v.pts, v.frames, v.kind, v.mat, A.sc.mats, P.txcs, P.freq, P.pt,
                       P.antenna, P.fresnel != 0, A.K, t, &pat);
    else
      seg_terms<double>(r, v.pts, v.frames, v.kind, v.mat, A.sc.mats, P.txcs, P.freq, P.pt,
                        P.antenna, P.fresnel != 0, A.K, t, &pat);
    A.seg[k] = t;
  }
}

__global__ void k_combine(FieldArgs A) {
  const unsigned long long ns = min(A.ctr->survivors, A.cap);
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < ns;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const Survivor sv = A.surv[i];
    const TxParams& P = A.txp[A.rx_req[sv.rx]];
    PathView v;
    path_view(A, i, v);
    SegTerms* seg = A.seg + size_t(i) * (kMaxDepth + 1);
    Cx<double> e[3];
    const int prec = A.precision < 0 ? P.precision : A.precision;
    double bound = 0.0;
    if (prec == 2) {
      path_combine<float, true>(v.n, seg, v.pts, v.frames, v.kind, P.txcs, P.freq, A.K, e);
      bound = -1.0;
    } else if (prec == 1) {
      float kappa = 0.0f;
      path_combine<float>(v.n, seg, v.pts, v.frames, v.kind, P.txcs, P.freq, A.K, e, &kappa);
      bool pole = false;
      for (int r = 0; r < v.n; ++r) pole |= seg[r].fp64_fresnel != 0;
      if (pole || !(kappa <= kKappaMax32)) {
        // an ill-conditioned path: its terms and field again, in FP64
        const PatternTab pat{P.pat, P.pat_nt, P.pat_np, P.pat_dt, P.pat_dp};
        for (int r = 0; r < v.n; ++r)
          seg_terms<double>(r, v.pts, v.frames, v.kind, v.mat, A.sc.mats, P.txcs, P.freq, P.pt,
                            P.antenna, P.fresnel != 0, A.K, seg[r], &pat);
        path_combine<double>(v.n, seg, v.pts, v.frames, v.kind, P.txcs, P.freq, A.K, e);
        atomicAdd(&A.fstat[0], 1ull);
      } else {
        // each component errs by at most (7 kappa) ulps of |E| (measured on
        // every path of the urban canyon); the bound takes 16 kappa, plus
        // the FP32 rounding of the path field when the sum reads it
        const double mag = sqrt(e[0].re * e[0].re + e[0].im * e[0].im + e[1].re * e[1].re +
                                e[1].im * e[1].im + e[2].re * e[2].re + e[2].im * e[2].im);
        bound = (16.0 * double(kappa) + 1.0) * 0x1p-24 * mag;
      }
    } else {
      path_combine<double>(v.n, seg, v.pts, v.frames, v.kind, P.txcs, P.freq, A.K, e);
    }
    if (A.path_bound) A.path_bound[i] = bound;
    for (int j = 0; j < 3; ++j) {
      A.path_field[6 * i + 2 * j] = e[j].re;
      A.path_field[6 * i + 2 * j + 1] = e[j].im;
    }
  }
}

// FP32 field mode, receivers k_rx_sum could not certify: every path of such
// a receiver gets its terms and field again in FP64 (k_rx_sum then sums the
// receiver in FP64).
__global__ void k_escalate(FieldArgs A) {
  const unsigned long long ns = min(A.ctr->survivors, A.cap);
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < ns;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const Survivor sv = A.surv[i];
    if (!A.rx_flag[sv.rx] || A.path_bound[i] == 0.0) continue;  // taken in FP64 already
    const TxParams& P = A.txp[A.rx_req[sv.rx]];
    PathView v;
    path_view(A, i, v);
    SegTerms* seg = A.seg + size_t(i) * (kMaxDepth + 1);
    const PatternTab pat{P.pat, P.pat_nt, P.pat_np, P.pat_dt, P.pat_dp};
    for (int r = 0; r < v.n; ++r)
      seg_terms<double>(r, v.pts, v.frames, v.kind, v.mat, A.sc.mats, P.txcs, P.freq, P.pt,
                        P.antenna, P.fresnel != 0, A.K, seg[r], &pat);
    Cx<double> e[3];
    path_combine<double>(v.n, seg, v.pts, v.frames, v.kind, P.txcs, P.freq, A.K, e);
    for (int j = 0; j < 3; ++j) {
      A.path_field[6 * i + 2 * j] = e[j].re;
      A.path_field[6 * i + 2 * j + 1] = e[j].im;
    }
    A.path_bound[i] = 0.0;
    atomicAdd(&A.fstat[0], 1ull);
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
//
// FP32 field mode (precision 1, with path_bound): the receiver's error bound
// is the sum of its paths' bounds plus the compensated sum's own rounding
// (2 ulps of the result).  The receiver is certified when that bound is
// within half the field tolerance (1e-4 relative magnitude) of each
// component, or, for a component below 1e-9 of the receiver's largest, of
// that largest one; bound[r] then states it.  Otherwise rx_flag[r] is set:
// k_escalate recomputes its paths in FP64 and a second call (only = rx_flag,
// force_precision 0) sums it in FP64, with bound 0.
__global__ void k_rx_sum(const Survivor* surv, const int* starts, int* order, int n_rx,
                         const double* path_field, int force_precision, const int* rx_req,
                         const TxParams* txp, double* field, const double* path_bound = nullptr,
                         double* bound = nullptr, int* rx_flag = nullptr,
                         unsigned long long* fstat = nullptr, const int* only = nullptr) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rx; r += gridDim.x * blockDim.x) {
    if (only && !only[r]) continue;
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
      double B = 0.0;
      for (int i = b; i < e; ++i) {
        for (int k = 0; k < 6; ++k) {
          const float x = float(path_field[6 * size_t(order[i]) + k]);
          const float t = s[k] + x;
          c[k] += fabsf(s[k]) >= fabsf(x) ? (s[k] - t) + x : (x - t) + s[k];
          s[k] = t;
        }
        if (path_bound) {
          const double pb = path_bound[order[i]];
          B = (pb < 0.0 || B < 0.0) ? -1.0 : B + pb;
        }
      }
      double f[6];
      for (int k = 0; k < 6; ++k) f[k] = field[6 * size_t(r) + k] = double(s[k]) + double(c[k]);
      if (path_bound && bound) {
        if (precision != 1 || B < 0.0) {
          bound[r] = -1.0;  // FP32-phase study mode: no bound
        } else {
          double mag[3], big = 0.0;
          for (int j = 0; j < 3; ++j) {
            mag[j] = sqrt(f[2 * j] * f[2 * j] + f[2 * j + 1] * f[2 * j + 1]);
            big = fmax(big, mag[j]);
          }
          B = B * (1.0 + 1e-6) + 0x1p-23 * big;
          bool ok = true;
          for (int j = 0; j < 3; ++j)
            ok &= B <= 0.5e-4 * (mag[j] > 1e-9 * big ? mag[j] : big);
          bound[r] = B;
          if (!ok) {
            rx_flag[r] = 1;
            atomicAdd(&fstat[1], 1ull);
          }
        }
      }
    } else {
      double s[6] = {0, 0, 0, 0, 0, 0};
      for (int i = b; i < e; ++i)
        for (int k = 0; k < 6; ++k) s[k] = __dadd_rn(s[k], path_field[6 * size_t(order[i]) + k]);
      for (int k = 0; k < 6; ++k) field[6 * size_t(r) + k] = s[k];
      if (bound) bound[r] = 0.0;
    }
  }
}

}  // namespace sbr
