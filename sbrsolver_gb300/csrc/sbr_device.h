// Device data layout and arithmetic shared by the SBR kernels.
//
// Precision scheme.  Every decision that selects a path (which triangle a
// ray hits, whether a receiver is inside a reception sphere, whether an image
// correction finds its facet) must come out exactly as the reference's FP64
// code decides it.  Two kinds of arithmetic are therefore used:
//   * x64::* — FP64 with __dadd_rn/__dmul_rn/__ddiv_rn/__dsqrt_rn, which are
//     never contracted into FMA, evaluated in the reference's operation order.
//     On IEEE hardware these give bit-identical results to the reference
//     compiled without FP contraction.  They carry the ray state (origins,
//     directions, path lengths) and settle every close decision.
//   * FP32 filters with explicit error margins.  They answer the common case
//     (a triangle clearly missed, a receiver clearly outside its sphere) and
//     hand anything within the margin to the FP64 form.
#pragma once

#include <climits>

#include <cstdint>
#include <cuda_runtime.h>

namespace sbr {

constexpr uint32_t kRootClass = 0xFFFFFFFFu;  // coplanar class of the empty path prefix
// Path classes (interned facet/interaction prefixes) of different requests
// must not merge because each class carries its request's image source:
// the empty prefix of request q is class kRootBase + q.
constexpr uint32_t kRootBase = 0xFFFF0000u;
__host__ __device__ __forceinline__ bool is_root_class(uint32_t c) { return c >= kRootBase; }
constexpr unsigned long long kEmptyKey = 0xFFFFFFFFFFFFFFFFull;
constexpr int kHeapBits = 17;                  // rank = launch << 17 | BFS heap index
constexpr int kMaxDepth = 16;                  // max interactions per path (R + T)
constexpr int kStack = 96;                     // traversal stack entries

// FP32 traversal node: the boxes of both children of one reference BVH node.
// child >= 0: internal node index; child < 0: ~(leaf node index).
struct __align__(16) Node32 {
  float lo0[3], hi0[3], lo1[3], hi1[3];
  int child[2];
  int pad[2];
};

// Four-wide node of the search BVH (128 bytes): up to four child boxes, each
// coordinate as a four-lane vector, and the child refs (>= 0: node index,
// < 0: ~(first << 3 | count) of a leaf, kEmptyChild: no child).
struct __align__(16) Node4 {
  float lo[3][4];
  float hi[3][4];
  int child[4];
  int pad[4];
};
constexpr int kEmptyChild = INT_MIN;

// FP64 reference node (depth-first numbering), with its box also as floats
// (exact: box bounds are float vertex coordinates) and a mask of its flat
// axes (lo == hi), so FP32 tests need no FP64 conversions.
struct RefNode {
  double bb[6];
  float fb[6];
  int c0, c1, first, count, parent, flat;
};

// One box on a reference leaf's path to the root (leaf first), stored
// contiguously per leaf so the reachability check of a hit reads one run
// instead of chasing parent links.  node < 0 ends a leaf's run.
struct __align__(16) AncBox {
  float fb[6];
  int flat;  // RefNode::flat
  int node;  // RefNode index (its FP64 box decides cases the FP32 test cannot)
};

// Triangle, depth-first leaf order (index == closest-hit tie rank).
struct __align__(16) Tri32 {
  float v1[3], nv1;  // |v1|
  float e1[3], ne1;  // |e1|
  float e2[3], ne2;  // |e2|
};
struct Tri64 {
  double v1[3], e1[3], e2[3], n[3];
  int id, cop, mat, node;  // node: leaf that holds it
};

// What the reference's triangleMesh[i] holds for position i of the caller's
// vector (after ConstructBVH reordered it): used by image correction and the
// field stage, which index the mesh by triangle id.
struct CorrTri {
  double v1[3], e1[3], e2[3], n[3], cs[9];
  int mat, pad;
};

struct Material {
  double eps_re, sigma, width;  // width: slab thickness (m), 0 in the reference
};

struct DevScene {
  const Node32* node32;
  const RefNode* ref;
  const Tri32* tri32;
  const Tri64* tri64;
  const CorrTri* corr;
  const Tri32* corr32;     // FP32 filter copy of corr
  const int* rank_to_id;   // triangle id of each depth-first rank
  const Material* mats;
  // search BVH of the FP32 candidate search, four-wide (child < 0:
  // ~(first << 3 | count))
  const Node4* snode4;
  const Tri32* stri;    // triangles in search leaf order
  const int* srank;     // their depth-first ranks
  const AncBox* anc;    // per reference leaf: its boxes up to the root
  const int* anc_off;   // start of a leaf's run in anc (by node index)
  int n_tri, n_nodes, n_mats;
  int root_leaf;
  float box_margin;  // absolute FP32 box expansion (metres)
};

// One ray of the wavefront: the RayLaunch call that will create one tree node.
struct __align__(16) RayRec {
  double o[3], d[3];
  double total;    // totalPathLength argument of RayLaunch (RTSolver.cpp:137)
  double S;        // pathLength argument RayCapture will give the node (RTSolver.cpp:288)
  uint32_t parent; // node index of the parent, 0xFFFFFFFF for a root
  uint32_t cls;    // class (interned tri/kind prefix) of the node
  uint32_t cop;    // coplanar-prefix class of the node
  uint32_t launch;
  uint32_t heap;   // BFS heap index (root 1, transmit child 2h, reflect child 2h+1)
  uint16_t rc, tc;
  uint32_t tx;     // transmitter (request) index
  int orank;       // depth-first rank of the triangle the ray starts on, -1 for a launch
};

// FP32 copy of a ray, made by the candidate search when it loads the ray
// (it converts the FP64 origin and direction anyway), for the FP32 checks and
// the node record of the ray's resolution, which then convert nothing (an
// FP64 -> FP32 conversion costs an FP64 pipe slot): origin (o.w unused) and
// unit direction (d.w unused).
struct __align__(16) RayF32 {
  float4 o, d;
};

// One executed segment (tree node), split in two arrays: the FP32 part the
// capture stage reads for every node and ancestor, and the FP64 part it
// reads only for the rare tests inside the FP32 error margin.
struct __align__(16) NodeHot {
  float s[3], S;    // source point, RayCapture's pathLength argument
  float u[3], len;  // unit direction and segment length
  uint32_t parent, cls, launch, heap;
  uint32_t tx, pad0, pad1, pad2;
};
struct __align__(16) NodeCold {
  double s[3], t[3];  // source and target points (RTSolver.cpp:156-183, 228-255)
  double S, pad;
};

// Per transmitter (one request of a batch).
struct TxParams {
  double tx[3];
  double txcs[9];
  double freq, pt, tan_beta, k;
  double cmax;       // max |receiver| of this request's receivers
  int R, T, antenna, fresnel;
  int n_launch, level;
  int rx_first, n_rx;          // receivers of this request in the batch arrays
  long long launch_first;      // first global launch index
  int grid;                    // receiver grid index
  int precision;               // field precision: 0 FP64, 1 FP32, 2 FP32 with FP32 phase
  float tan_beta32;            // tan_beta rounded to FP32 on the host (a device
                               // conversion would take an FP64 pipe slot per use)
  // tabulated pattern (antenna 3): per (theta, phi) grid point the complex
  // relative amplitudes of E_theta and E_phi (re, im, re, im)
  const float4* pat;
  int pat_nt, pat_np;
  double pat_dt, pat_dp;       // grid steps (degrees)
};

struct RxGrid {
  float org[3], cell;
  int dim[3];
  float inv_cell;  // 1 / cell
  float chunk_len; // minimum chunk length along a node's segment in capture (m)
  const int* cell_start;  // ncell + 1
  const float4* rx32;     // sorted by cell: xyz, w = receiver index (int bits)
  float bmin[3], bmax[3];
};

struct HashTable {
  unsigned long long* keys;
  uint32_t mask;
};

// One path class: the path's last ray starts on `tri` (depth-first rank),
// reached by interaction `kind` (1 reflect, 2 transmit) from class `parent`.
// img is the image source of that ray (GetImageSources, RTSolver.cpp:396-433,
// FP64 in the reference's order), img32 its FP32 copy.
struct __align__(16) ClassInfo {
  double img[3];
  float img32[3];
  uint32_t parent;
  int tri;
  uint32_t cop;
  uint8_t kind, depth, pad0, pad1;
  uint32_t pad2;
};

// What the capture stage needs of a class: the FP32 image source and the
// FP32 image-correction filter terms from it to the class's last triangle
// (mesh position tpos), written when the class is interned, and that
// triangle's correction cone without the request-dependent margin, formed in
// FP64 after the trace (k_class_cones).
struct __align__(16) ClassCap {
  float img[3];
  int tpos;        // corr32 index of the last triangle
  float F[8];      // TriFrom: o - v1, (o - v1) x e1, e2 . q, |o| + |v1|
  float n[3][4];   // cone plane k: oriented normal, n . img
  float nn[3];     // |n_k|
  float w[3];      // |n_k| (|img| + |T| + 1)
  float gc[3];     // |n_k . (centroid - img)|
  float inv_nx[3]; // 1 / n_k.x
};

// A capture whose image correction succeeded (one reference path before
// duplicate removal).
struct Corrected {
  uint32_t rx, cls;
  unsigned long long rank;
};

struct Counters {
  unsigned long long nodes;      // executed segments
  unsigned long long queue[kMaxDepth + 2];
  unsigned long long events;     // captured paths (before correction)
  unsigned long long corrected;  // captured paths whose correction succeeded
  unsigned long long survivors;
  unsigned long long fp64_tri;   // exact triangle tests run
  unsigned long long fallback;   // rays that needed the reference-order traversal
  unsigned long long fp64_capture;
  unsigned long long used_cls, used_cop, used_dd;  // occupied hash slots
  unsigned long long lost_cls, lost_cop, lost_dd;  // inserts refused by a full table
  unsigned long long pairs;      // (node, receiver) pairs handed to the FP64 capture pass
  unsigned long long cand;       // receiver candidates tested by the capture stage
  unsigned long long anc;        // ancestor re-tests for suppression
  unsigned long long used_cc;    // (class, receiver) corrections cached
  unsigned long long cls_listed; // classes listed for their correction cones
  unsigned int overflow;         // bit mask of capacity overflows
  unsigned int pad;
};

enum OverflowBits : unsigned {
  kOvNodes = 1, kOvQueue = 2, kOvClass = 4, kOvCop = 8, kOvCorr = 16, kOvDedup = 32,
  kOvSurv = 64, kOvStack = 128, kOvPairs = 256
};
// Overflows of the trace stage: the solve will be repeated, so the stages
// after it skip their work.
constexpr unsigned kOvTrace = kOvNodes | kOvQueue | kOvClass | kOvCop;

// ------------------------------------------------------------------ FP64
namespace x64 {
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double sqrt_(double a) { return __dsqrt_rn(a); }
// ((a0 b0 + a1 b1) + a2 b2): Eigen's reduction order for 3-vectors
__device__ __forceinline__ double dot(const double* a, const double* b) {
  return add(add(mul(a[0], b[0]), mul(a[1], b[1])), mul(a[2], b[2]));
}
__device__ __forceinline__ double sqn(const double* a) { return dot(a, a); }
__device__ __forceinline__ double norm(const double* a) { return sqrt_(sqn(a)); }
__device__ __forceinline__ void cross(const double* a, const double* b, double* r) {
  r[0] = sub(mul(a[1], b[2]), mul(a[2], b[1]));
  r[1] = sub(mul(a[2], b[0]), mul(a[0], b[2]));
  r[2] = sub(mul(a[0], b[1]), mul(a[1], b[0]));
}
__device__ __forceinline__ void sub3(const double* a, const double* b, double* r) {
  r[0] = sub(a[0], b[0]);
  r[1] = sub(a[1], b[1]);
  r[2] = sub(a[2], b[2]);
}
__device__ __forceinline__ void normalize(const double* a, double* r) {
  double z = sqn(a);
  if (z > 0) {
    double s = sqrt_(z);
    r[0] = div(a[0], s);
    r[1] = div(a[1], s);
    r[2] = div(a[2], s);
  } else {
    r[0] = a[0];
    r[1] = a[1];
    r[2] = a[2];
  }
}
}  // namespace x64

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

}  // namespace sbr
