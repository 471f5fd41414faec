// Host-side scene preparation for the SBR GPU path.
//
// The reference prepares a scene once on the host: STL read with exact
// vertex merging (SBRSolver_rev2/StlReader.h:448-700), coplanar grouping
// (Preprocessor.cpp:116-246), per-triangle frame/box (Triangle.cpp:37-70),
// and a SAH BVH (BVH/BVH.h:135-274).  This library does the same work in
// C++ with the same FP64 operation order (built with -ffp-contract=off), so
// the BVH topology, the depth-first triangle order that decides closest-hit
// ties, and the permutation ConstructBVH leaves in the caller's triangle
// vector all match the reference.  The GPU kernels consume the flattened
// result (sbr_device.h).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace sbr {

struct HostTri {
  double v1[3], v2[3], v3[3], n[3];
  double cs[9];      // surface frame rows: x = y cross n, y = (v2-v1)/|v2-v1|, z = n
  double bb[6];      // min xyz, max xyz
  double center[3];  // box centre
  int id = -1, cop = -1, mat = 0;
};

// Reference BVH node, numbered in depth-first order (children[0] subtree
// first) so the leaf triangle order equals the reference's visit order.
struct HostNode {
  double bb[6];
  int c0 = -1, c1 = -1;      // child node indices, -1 for a leaf
  int first = 0, count = 0;  // leaf: range in dfs_tris
  int parent = -1;
  int depth = 0;
};

// Search BVH of the FP32 candidate search: a binned-SAH binary BVH over the
// triangles (any topology finds the same candidates; the reference BVH
// above still decides ties and reachability), leaves of at most 7
// triangles.  Node child ref: >= 0 node index, < 0 ~(first << 3 | count)
// into `order` (depth-first ranks in leaf order).
struct SearchNode {
  float lo[2][3], hi[2][3];
  int child[2];
};
struct SearchBVH {
  std::vector<SearchNode> nodes;  // node 0 is the root
  std::vector<int> order;
  int max_depth = 0;
};

struct HostScene {
  std::vector<HostTri> tris;    // by triangle id (file order after merge)
  std::vector<int> mesh_order;  // reference caller vector after ConstructBVH: position -> id
  std::vector<HostNode> nodes;  // depth-first
  std::vector<int> dfs_tris;    // triangle ids in depth-first leaf order
  int max_depth = 0;
  double extent = 0;            // max |coordinate| of any vertex
  SearchBVH search;
};

// Binary or ASCII STL (format chosen as StlReader.h:703-718 does).  Returns
// float coordinates (9 per facet, file order) and facet normals (3 per facet).
bool read_stl(const std::string& path, std::vector<float>& v, std::vector<float>& n,
              std::string& err);

// Triangle soup -> prepared scene.  mat may be null (all 0).  The merge drops
// facets whose vertices collapse, exactly like the reference reader.
// host_tables = false leaves the coplanar ids (HostTri::cop) and the search
// BVH to the caller (the device builds them), and skips the vertex merge
// they need.
bool prepare_scene(int n_tri, const float* v, const float* nrm, const int* mat, HostScene& out,
                   std::string& err, bool host_tables = true, bool ref_bvh = true);

// The search BVH's triangle ids -> depth-first ranks of the reference BVH.
void map_search_order(HostScene& H);

// Builds H.search from the triangles in depth-first rank order.
void build_search_bvh(HostScene& H);

// Icosahedron launch directions at a subdivision level, in the reference's
// vertex order (Icosahedron.cpp:3-109), 3 doubles per direction.
void icosphere(int level, std::vector<double>& dirs);

}  // namespace sbr
