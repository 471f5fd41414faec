// Device functions of the SBR path: closest hit, reception sphere, image
// correction and the received field.  Reference behaviour is cited per
// function (paths relative to SBRSolver_rev2/).
#pragma once

#include <cfloat>
#include <climits>
#include <cuda_runtime.h>

#include "sbr_device.h"

namespace sbr {

constexpr double kEps64 = 1.1920928955078125e-07;  // FLT_EPSILON as double, Constants.h:13
constexpr float kEps32 = 1.1920928955078125e-07f;
constexpr float kFiltK = 6.103515625e-05f;         // 2^-14: FP32 filter margin factor
// Margin factor of the FP32 reception test: |dist - radius| and the
// projection are decided in FP32 only when they clear this times the
// magnitudes involved (|segment start| + |receiver| + 1 + unfolded length).
// Bounding every rounding of the FP32 evaluation and of its rounded inputs
// against the FP64 test gives under 30 * 2^-24 of the same magnitudes.
#ifndef SBR_REC_K
#define SBR_REC_K 1.52587890625e-05f  // 2^-16
#endif
constexpr float kRecK = SBR_REC_K;
// Relative slack when a bound on a contender's t is compared with another
// hit's t: a contender whose lower bound exceeds t * (1 + kTieSlack) lies
// farther along the ray, so its FP64 distance is larger (distances of one ray
// are t |d| to within a few FP64 ulps); the slack covers that and the FP32
// rounding of the product.
#ifndef SBR_TIE_SLACK
#define SBR_TIE_SLACK 9.5367431640625e-07f  // 2^-20
#endif
constexpr float kTieSlack = SBR_TIE_SLACK;

struct Hit {
  double t, dist;
  double p[3];
  int rank;  // index in depth-first triangle order, INT_MAX = no hit
  int leaf;
};

// Triangle::RayIntersects (Triangle.cpp:80-124), FP64, reference operation order.
__device__ __forceinline__ bool mt64(const Tri64& T, const double* o, const double* d, double& t,
                                     double* P, double& dist) {
  using namespace x64;
  double h[3];
  cross(d, T.e2, h);
  const double a = dot(T.e1, h);
  if (a > -kEps64 && a < kEps64) return false;
  // 1.0 / a (Triangle.cpp): the correctly rounded reciprocal is the same
  // double as the correctly rounded quotient 1.0 / a
  const double f = __drcp_rn(a);
  double s[3];
  sub3(o, T.v1, s);
  const double u = mul(f, dot(s, h));
  if (u < 0.0 || u > 1.0) return false;
  double q[3];
  cross(s, T.e1, q);
  const double v = mul(f, dot(d, q));
  if (v < 0.0 || add(u, v) > 1.0) return false;
  const double tt = mul(f, dot(T.e2, q));
  if (!(tt > kEps64)) return false;
  P[0] = add(o[0], mul(d[0], tt));
  P[1] = add(o[1], mul(d[1], tt));
  P[2] = add(o[2], mul(d[2], tt));
  double w[3];
  sub3(P, o, w);
  dist = norm(w);
  t = tt;
  return true;
}

// Same test on a CorrTri (image correction looks triangles up by mesh position).
__device__ __forceinline__ bool mt64c(const CorrTri& T, const double* o, const double* d,
                                      double* P) {
  Tri64 t;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    t.v1[i] = T.v1[i];
    t.e1[i] = T.e1[i];
    t.e2[i] = T.e2[i];
  }
  double tt, dist;
  return mt64(t, o, d, tt, P, dist);
}

// BVHNode::IntersectsAABB (BVH/BVHNode.h:64-85), FP64, with std::min/std::max
// argument order so NaN slabs are ignored exactly as the reference ignores them.
__device__ __forceinline__ bool slab64(const double* bb, const double* o, const double* d) {
  using namespace x64;
  double tmax = __longlong_as_double(0x7ff0000000000000ll);
  double tmin = -tmax;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const double t1 = div(sub(bb[i], o[i]), d[i]);
    const double t2 = div(sub(bb[3 + i], o[i]), d[i]);
    const double tn = (t2 < t1) ? t2 : t1;
    const double tf = (t1 < t2) ? t2 : t1;
    tmax = (tf < tmax) ? tf : tmax;
    tmin = (tmin < tn) ? tn : tmin;
    if (tmin > tmax) return false;
  }
  return true;
}

// BVH::RayIntersects (BVH/BVH.h:276-328) exactly: depth-first, both children,
// children[0] first, strict '<' on distance so the first visited wins ties.
__device__ __noinline__ bool exact_closest(const DevScene& sc, const double* o, const double* d,
                                           Hit& best, unsigned* overflow) {
  int stack[kStack];
  int sp = 0;
  stack[sp++] = 0;
  best.rank = INT_MAX;
  best.dist = __longlong_as_double(0x7ff0000000000000ll);
  while (sp > 0) {
    const int n = stack[--sp];
    const RefNode& nd = sc.ref[n];
    if (!slab64(nd.bb, o, d)) continue;
    if (nd.c0 >= 0) {
      if (sp + 2 > kStack) {
        atomicOr(overflow, kOvStack);
        return false;
      }
      stack[sp++] = nd.c1;
      stack[sp++] = nd.c0;
    } else {
      for (int r = nd.first; r < nd.first + nd.count; ++r) {
        double t, P[3], dist;
        if (mt64(sc.tri64[r], o, d, t, P, dist) && dist < best.dist) {
          best.dist = dist;
          best.t = t;
          best.p[0] = P[0];
          best.p[1] = P[1];
          best.p[2] = P[2];
          best.rank = r;
          best.leaf = n;
        }
      }
    }
  }
  return best.rank != INT_MAX;
}

// FP32 Moller-Trumbore filter with error margins.  Returns false only when
// the FP64 test certainly rejects; otherwise tlo is a lower bound on t.
__device__ __forceinline__ bool tri_filter(const Tri32& T, const float3& o, const float3& d,
                                           float no, float nd, float& tlo) {
  const float hx = d.y * T.e2[2] - d.z * T.e2[1];
  const float hy = d.z * T.e2[0] - d.x * T.e2[2];
  const float hz = d.x * T.e2[1] - d.y * T.e2[0];
  const float a = T.e1[0] * hx + T.e1[1] * hy + T.e1[2] * hz;
  const float sx = o.x - T.v1[0], sy = o.y - T.v1[1], sz = o.z - T.v1[2];
  float U = sx * hx + sy * hy + sz * hz;
  const float qx = sy * T.e1[2] - sz * T.e1[1];
  const float qy = sz * T.e1[0] - sx * T.e1[2];
  const float qz = sx * T.e1[1] - sy * T.e1[0];
  float V = d.x * qx + d.y * qy + d.z * qz;
  float W = T.e2[0] * qx + T.e2[1] * qy + T.e2[2] * qz;
  const float ns = no + T.nv1;
  const float ea = kFiltK * T.ne1 * T.ne2 * nd;
  const float eU = kFiltK * ns * nd * T.ne2;
  const float eV = kFiltK * ns * T.ne1 * nd;
  const float eW = kFiltK * ns * T.ne1 * T.ne2;
  const float A = fabsf(a);
  if (A <= kEps32 + ea) {  // near-parallel: the FP64 test decides
    tlo = 0.0f;
    return true;
  }
  if (a < 0.0f) {
    U = -U;
    V = -V;
    W = -W;
  }
  if (U < -eU || V < -eV) return false;
  if (U > A + ea + eU) return false;
  if (U + V > A + ea + eU + eV) return false;
  const float thi = (W + eW) / (A - ea);
  if (thi <= kEps32 * 0.5f) return false;
  tlo = (W - eW) / (A + ea);
  return true;
}

// tri_filter for many rays from one origin o (an image source towards many
// receivers): the terms that depend only on o and the triangle are formed
// once.  Same arithmetic and margins as tri_filter.
struct TriFrom {
  float sx, sy, sz;  // o - v1
  float qx, qy, qz;  // (o - v1) x e1
  float W;           // e2 . q
  float ns;          // |o| + |v1|
};

__device__ __forceinline__ TriFrom tri_from(const Tri32& T, const float3& o, float no) {
  TriFrom F;
  F.sx = o.x - T.v1[0];
  F.sy = o.y - T.v1[1];
  F.sz = o.z - T.v1[2];
  F.qx = F.sy * T.e1[2] - F.sz * T.e1[1];
  F.qy = F.sz * T.e1[0] - F.sx * T.e1[2];
  F.qz = F.sx * T.e1[1] - F.sy * T.e1[0];
  F.W = T.e2[0] * F.qx + T.e2[1] * F.qy + T.e2[2] * F.qz;
  F.ns = no + T.nv1;
  return F;
}

__device__ __forceinline__ bool tri_filter_from(const Tri32& T, const TriFrom& F,
                                                const float3& d, float nd) {
  const float hx = d.y * T.e2[2] - d.z * T.e2[1];
  const float hy = d.z * T.e2[0] - d.x * T.e2[2];
  const float hz = d.x * T.e2[1] - d.y * T.e2[0];
  const float a = T.e1[0] * hx + T.e1[1] * hy + T.e1[2] * hz;
  float U = F.sx * hx + F.sy * hy + F.sz * hz;
  float V = d.x * F.qx + d.y * F.qy + d.z * F.qz;
  float W = F.W;
  const float ea = kFiltK * T.ne1 * T.ne2 * nd;
  const float eU = kFiltK * F.ns * nd * T.ne2;
  const float eV = kFiltK * F.ns * T.ne1 * nd;
  const float eW = kFiltK * F.ns * T.ne1 * T.ne2;
  const float A = fabsf(a);
  if (A <= kEps32 + ea) return true;  // near-parallel: the FP64 test decides
  if (a < 0.0f) {
    U = -U;
    V = -V;
    W = -W;
  }
  if (U < -eU || V < -eV) return false;
  if (U > A + ea + eU) return false;
  if (U + V > A + ea + eU + eV) return false;
  // thi = (W + eW) / (A - ea) > eps/2 with A - ea > 0, without the division
  return W + eW > (kEps32 * 0.5f) * (A - ea);
}

// As tri_filter, also telling whether the FP64 test certainly hits (2) or
// may go either way (1); 0 = certainly misses.  [tlo, thi] bounds t.
__device__ __forceinline__ int tri_classify(const Tri32& T, const float3& o, const float3& d,
                                            float no, float nd, float& tlo, float& thi) {
  const float hx = d.y * T.e2[2] - d.z * T.e2[1];
  const float hy = d.z * T.e2[0] - d.x * T.e2[2];
  const float hz = d.x * T.e2[1] - d.y * T.e2[0];
  const float a = T.e1[0] * hx + T.e1[1] * hy + T.e1[2] * hz;
  const float sx = o.x - T.v1[0], sy = o.y - T.v1[1], sz = o.z - T.v1[2];
  float U = sx * hx + sy * hy + sz * hz;
  const float qx = sy * T.e1[2] - sz * T.e1[1];
  const float qy = sz * T.e1[0] - sx * T.e1[2];
  const float qz = sx * T.e1[1] - sy * T.e1[0];
  float V = d.x * qx + d.y * qy + d.z * qz;
  float W = T.e2[0] * qx + T.e2[1] * qy + T.e2[2] * qz;
  const float ns = no + T.nv1;
  const float ea = kFiltK * T.ne1 * T.ne2 * nd;
  const float eU = kFiltK * ns * nd * T.ne2;
  const float eV = kFiltK * ns * T.ne1 * nd;
  const float eW = kFiltK * ns * T.ne1 * T.ne2;
  const float A = fabsf(a);
  if (A <= kEps32 + ea) {
    tlo = 0.0f;
    thi = INFINITY;
    return 1;
  }
  if (a < 0.0f) {
    U = -U;
    V = -V;
    W = -W;
  }
  if (U < -eU || V < -eV) return 0;
  if (U > A + ea + eU) return 0;
  if (U + V > A + ea + eU + eV) return 0;
  thi = (W + eW) / (A - ea);
  if (thi <= kEps32 * 0.5f) return 0;
  tlo = (W - eW) / (A + ea);
  const bool sure = U > eU && V > eV && U + V < A - ea - eU - eV && tlo > 2.0f * kEps32;
  return sure ? 2 : 1;
}

__device__ __forceinline__ void load_node(const Node32* nodes, int i, float4& f0, float4& f1,
                                          float4& f2, int2& ch) {
  const float4* p = reinterpret_cast<const float4*>(nodes + i);
  f0 = __ldg(p);
  f1 = __ldg(p + 1);
  f2 = __ldg(p + 2);
  const float4 f3 = __ldg(p + 3);
  ch = make_int2(__float_as_int(f3.x), __float_as_int(f3.y));
}

__device__ __forceinline__ void slab32(float lx, float ly, float lz, float hx, float hy, float hz,
                                       const float3& o, const float3& inv, float m, float& tn,
                                       float& tf) {
  const float ax = ((lx - m) - o.x) * inv.x, bx = ((hx + m) - o.x) * inv.x;
  const float ay = ((ly - m) - o.y) * inv.y, by = ((hy + m) - o.y) * inv.y;
  const float az = ((lz - m) - o.z) * inv.z, bz = ((hz + m) - o.z) * inv.z;
  tn = fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fminf(az, bz));
  tf = fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fmaxf(az, bz));
}

struct TraceStats {
  unsigned fp64_tri, fallback;
};

// The reference's slab test (slab64) decided in FP32 where the error bounds
// allow: 1 = accepted, 0 = rejected, -1 = within the error bounds (run
// slab64).  Box bounds are float values (they come from float vertices), so
// only the origin, direction and the arithmetic carry FP32 error; each
// slab parameter t = (b - o) / d is within
//   e = 2^-20 (|lo| + |hi| + 2|o|) / |d|
// of its FP64 value.  A flat axis (lo == hi) gives one FP64 value t for both
// planes, so the FP64 test accepts iff the other axes' intervals contain it.
// inv = 1/d in FP32: a product with it differs from the quotient by a few
// ulps, far inside e.
__device__ __forceinline__ int slab_certain(const float* bb, int flatmask, const float3& o,
                                            const float3& d, const float3& inv) {
  const float K = 9.5367431640625e-07f;  // 2^-20
  float A_lo = -INFINITY, A_hi = -INFINITY, B_lo = INFINITY, B_hi = INFINITY;
  float v = 0.0f, ev = 0.0f;
  int flat = 0;
  if (flatmask & 8) return -1;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float da = a == 0 ? d.x : (a == 1 ? d.y : d.z);
    const float oa = a == 0 ? o.x : (a == 1 ? o.y : o.z);
    const float ia = a == 0 ? inv.x : (a == 1 ? inv.y : inv.z);
    if (da == 0.0f) return -1;
    const float lo = bb[a], hi = bb[3 + a];
    const float t1 = (lo - oa) * ia, t2 = (hi - oa) * ia;
    const float e = K * (fabsf(lo) + fabsf(hi) + 2.0f * fabsf(oa)) * fabsf(ia);
    if (!isfinite(t1) || !isfinite(t2) || !isfinite(e)) return -1;
    if (flatmask & (1 << a)) {
      if (flat++) return -1;
      v = t1;
      ev = e;
      continue;
    }
    const float tn = fminf(t1, t2), tf = fmaxf(t1, t2);
    A_lo = fmaxf(A_lo, tn - e);
    A_hi = fmaxf(A_hi, tn + e);
    B_lo = fminf(B_lo, tf - e);
    B_hi = fminf(B_hi, tf + e);
  }
  if (flat) {
    if (A_hi < v - ev && v + ev < B_lo) return 1;
    if (v + ev < A_lo || v - ev > B_hi || A_lo > B_hi) return 0;
    return -1;
  }
  if (A_hi < B_lo) return 1;
  if (A_lo > B_hi) return 0;
  return -1;
}

// Closest hit with the reference's result.  FP32 ordered traversal over the
// reference BVH (boxes widened by box_margin so no box the FP64 test accepts
// is missed), FP32 triangle filter, FP64 test for every triangle the filter
// cannot rule out, lexicographic (distance, depth-first rank) minimum - the
// reference's strict '<' in visit order.  The winner is accepted only if every
// ancestor box of its leaf passes the reference's FP64 slab test; otherwise
// the ray is re-run with the reference-order traversal.
__device__ __noinline__ bool closest_hit(const DevScene& sc, const double* o, const double* d,
                                         Hit& best, TraceStats& st, unsigned* overflow) {
  const float3 o32 = make_float3(float(o[0]), float(o[1]), float(o[2]));
  const float3 d32 = make_float3(float(d[0]), float(d[1]), float(d[2]));
  const float3 inv = make_float3(1.0f / d32.x, 1.0f / d32.y, 1.0f / d32.z);
  const float no = sqrtf(o32.x * o32.x + o32.y * o32.y + o32.z * o32.z);
  const float nd = sqrtf(d32.x * d32.x + d32.y * d32.y + d32.z * d32.z);
  const float m = sc.box_margin + kFiltK * no;
  best.rank = INT_MAX;
  best.dist = __longlong_as_double(0x7ff0000000000000ll);
  best.t = best.dist;
  float tcut = INFINITY;  // boxes entered beyond this cannot hold a better hit

  int stack[kStack];
  int sp = 0;
  int pending_leaf = -1;
  constexpr int kCand = 8;
  int cand_r[kCand], cand_leaf[kCand];
  float cand_t[kCand];
  int ncand = 0;
  if (sc.root_leaf) pending_leaf = 0;
  else stack[sp++] = 0;
  bool stack_overflow = false;

  while (true) {
    if (pending_leaf >= 0) {
      const RefNode& L = sc.ref[pending_leaf];
      for (int r = L.first; r < L.first + L.count; ++r) {
        float tlo, thi;
        const int k = tri_classify(sc.tri32[r], o32, d32, no, nd, tlo, thi);
        if (k == 0 || tlo > tcut) continue;
        if (ncand < kCand) {
          cand_r[ncand] = r;
          cand_leaf[ncand] = pending_leaf;
          cand_t[ncand] = tlo;
          ++ncand;
          if (k == 2) tcut = fminf(tcut, thi * (1.0f + kTieSlack) + 1e-30f);
        } else {
          // too many contenders: resolve this one now
          ++st.fp64_tri;
          double t, P[3], dist;
          if (mt64(sc.tri64[r], o, d, t, P, dist) &&
              (dist < best.dist || (dist == best.dist && r < best.rank))) {
            best.dist = dist;
            best.t = t;
            best.p[0] = P[0];
            best.p[1] = P[1];
            best.p[2] = P[2];
            best.rank = r;
            best.leaf = pending_leaf;
            tcut = fminf(tcut, float(t) * (1.0f + kTieSlack) + 1e-30f);
          }
        }
      }
      pending_leaf = -1;
    }
    if (sp == 0) break;
    const int ni = stack[--sp];
    if (ni < 0) {  // a leaf deferred as the farther child
      pending_leaf = ~ni;
      continue;
    }
    float4 f0, f1, f2;
    int2 ch;
    load_node(sc.node32, ni, f0, f1, f2, ch);
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
        stack_overflow = true;
        break;
      }
      stack[sp++] = second;  // internal node or ~leaf
    }
    if (has_first) {
      if (first < 0) {
        pending_leaf = ~first;
      } else {
        if (sp >= kStack) {
          stack_overflow = true;
          break;
        }
        stack[sp++] = first;
      }
    }
  }

  // Resolve the contenders exactly, nearest lower bound first, until none
  // can reach the best exact distance.
  for (int i = 1; i < ncand; ++i) {  // insertion sort by tlo (ncand <= kCand)
    const float kt = cand_t[i];
    const int kr = cand_r[i], kl = cand_leaf[i];
    int j = i - 1;
    while (j >= 0 && cand_t[j] > kt) {
      cand_t[j + 1] = cand_t[j];
      cand_r[j + 1] = cand_r[j];
      cand_leaf[j + 1] = cand_leaf[j];
      --j;
    }
    cand_t[j + 1] = kt;
    cand_r[j + 1] = kr;
    cand_leaf[j + 1] = kl;
  }
  for (int i = 0; i < ncand; ++i) {
    if (best.rank != INT_MAX && cand_t[i] > float(best.t) * (1.0f + kTieSlack) + 1e-30f) break;
    const int r = cand_r[i];
    ++st.fp64_tri;
    double t, P[3], dist;
    if (mt64(sc.tri64[r], o, d, t, P, dist) &&
        (dist < best.dist || (dist == best.dist && r < best.rank))) {
      best.dist = dist;
      best.t = t;
      best.p[0] = P[0];
      best.p[1] = P[1];
      best.p[2] = P[2];
      best.rank = r;
      best.leaf = cand_leaf[i];
    }
  }
  bool ok = !stack_overflow;
  if (ok && best.rank != INT_MAX) {
    // every ancestor of the winner's leaf must pass the FP64 slab test
    for (int n = best.leaf; n >= 0; n = sc.ref[n].parent) {
      int v = slab_certain(sc.ref[n].fb, sc.ref[n].flat, o32, d32, inv);
      if (v < 0) v = slab64(sc.ref[n].bb, o, d) ? 1 : 0;
      if (!v) {
        ok = false;
        break;
      }
    }
  }
  if (!ok) {
    ++st.fallback;
    return exact_closest(sc, o, d, best, overflow);
  }
  return best.rank != INT_MAX;
}

// ---- split closest hit: FP32 candidate search, then FP64 resolution -------
//
// The same decision as closest_hit, cut in two so that the FP32 traversal
// (divergent: rays visit very different numbers of nodes) and the FP64
// resolution (dense FP64 work) run in separate kernels.  The search keeps up
// to kCand contender triangles per ray (depth-first rank, FP32 lower bound on
// t); more contenders, or a stack overflow, send the ray to the
// reference-order FP64 traversal.
constexpr int kCand = 8;
constexpr unsigned char kFindFallback = 0xFF;

// Whether the reference's test of the triangle a ray starts on certainly
// fails (so its FP64 test can be skipped).  The ray's origin is the hit
// point the parent ray's FP64 test produced on that triangle, within about
// 1e-15 |P| of its plane; leaving at |cos| >= 1e-2 the reference's t for it
// is then below 1e-10 for |P| < 1e5, far under the t > FLT_EPSILON it
// requires (Triangle.cpp:113).
// o32, d32: the ray's origin and direction rounded to FP32 (conversions from
// FP64 occupy the FP64 pipe like an FP64 add, so a ray's are made once).
__device__ __forceinline__ bool origin_rejected(const Tri32& T, const float3& o32,
                                                const float3& d32) {
  const float ox = o32.x, oy = o32.y, oz = o32.z;
  if (!(fabsf(ox) < 1e5f && fabsf(oy) < 1e5f && fabsf(oz) < 1e5f)) return false;
  const float nx = T.e1[1] * T.e2[2] - T.e1[2] * T.e2[1];
  const float ny = T.e1[2] * T.e2[0] - T.e1[0] * T.e2[2];
  const float nz = T.e1[0] * T.e2[1] - T.e1[1] * T.e2[0];
  const float dx = d32.x, dy = d32.y, dz = d32.z;
  const float dn = dx * nx + dy * ny + dz * nz;
  const float nn = sqrtf(nx * nx + ny * ny + nz * nz), dd = sqrtf(dx * dx + dy * dy + dz * dz);
  return fabsf(dn) >= 1e-2f * nn * dd;
}

// HitReceptionSphere (RTSolver.cpp:805-863), FP64 in the reference's order.
__device__ __forceinline__ bool reception64(const double* s, const double* t, const double* c,
                                            double path_len, double tan_beta) {
  using namespace x64;
  double rd[3], w[3];
  sub3(t, s, rd);
  sub3(c, s, w);
  double t0 = div(dot(rd, w), sqn(rd));
  if (t0 < 0) return false;
  if (t0 >= 1) t0 = 1;
  double P[3] = {add(s[0], mul(t0, rd[0])), add(s[1], mul(t0, rd[1])), add(s[2], mul(t0, rd[2]))};
  const double unfolded = add(path_len, norm(P));
  const double radius = mul(unfolded, tan_beta);
  double e[3];
  sub3(c, P, e);
  return norm(e) <= radius;
}

// FP32 reception filter: 1 = captured, 0 = not captured, -1 = within the
// error margin (decide with reception64).
__device__ __forceinline__ int reception32(const float3& s, const float3& u, float len, float S,
                                           const float3& c, float tanb) {
  const float wx = c.x - s.x, wy = c.y - s.y, wz = c.z - s.z;
  const float lam = u.x * wx + u.y * wy + u.z * wz;
  const float ns = sqrtf(s.x * s.x + s.y * s.y + s.z * s.z);
  const float nc = sqrtf(c.x * c.x + c.y * c.y + c.z * c.z);
  const float mag = ns + nc + 1.0f;
  const float ml = kRecK * mag;
  if (lam < -ml) return 0;
  if (lam <= ml) return -1;
  const float lc = fminf(lam, len);
  const float px = s.x + lc * u.x, py = s.y + lc * u.y, pz = s.z + lc * u.z;
  const float np = sqrtf(px * px + py * py + pz * pz);
  const float ex = c.x - px, ey = c.y - py, ez = c.z - pz;
  const float dist = sqrtf(ex * ex + ey * ey + ez * ez);
  const float rad = (S + np) * tanb;
  const float mr = kRecK * (mag + S + np);
  if (dist > rad + mr) return 0;
  if (dist < rad - mr) return 1;
  return -1;
}

}  // namespace sbr
