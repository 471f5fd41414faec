// C++ drop-in for SBRSolver's hot-path interface, over the C ABI (sbr.h).
//
// Mirrors the names, arguments and call order of the reference's host API so
// that a caller like SBRSolver_rev2.cpp:53-142 (main) compiles against this
// header with its namespace imported:
//
//   Preprocessor::StlToGeometry   Preprocessor.h:25-32, Preprocessor.cpp:69-114
//   Preprocessor::GenerateRxPlane Preprocessor.cpp:254-268
//   Preprocessor::GenerateRXLine  Preprocessor.cpp:270-284
//   Preprocessor::ReadLocationFile Preprocessor.h:21
//   Preprocessor::ReadPatternFile Preprocessor.cpp:3-35 (+ AntennaPattern, antenna type 3)
//   GenerateRaysOnIcosahedron     Icosahedron.h:8, Icosahedron.cpp:80-109
//   BVH<Triangle>::ConstructBVH   BVH/BVH.h:25,135-230
//   RTSolver::Init / ExecuteRayTracing / Save*   RTSolver.h:18-45
//   FieldCompute::FieldAtReceiver FieldCompute.h:39
//   GlobalConfig                  GlobalConfig.h:5-7 (empty there; here it holds
//                                 the settings the reference hard-codes)
//
// Differences a caller sees:
//   * Vec3 / Mat3 / VecVec3 are small value types of this header, not Eigen
//     types; they offer x()/y()/z(), operator[] / operator() access and
//     brace initialisation like the reference's uses of them.
//   * BVH<Triangle>::ConstructBVH builds the scene on the GPU (SAH BVH,
//     coplanar ids, device upload) and reorders the caller's vector exactly
//     as the reference's build sorts it; it also fills Triangle::coplanarId.
//   * RTSolver::Init binds the materials to that scene, reading each
//     Triangle::materialId at that moment.
//   * Errors throw sbrgb::Error (status + message) instead of failing silently.
//
// Link with libsbr.so (-lsbr).  Header-only; needs C++17.
#pragma once

#include <array>
#include <cmath>
#include <complex>
#include <cstdio>
#include <fstream>
#include <initializer_list>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "sbr.h"

namespace sbrgb {

class Error : public std::runtime_error {
 public:
  Error(sbr_status s, const std::string& msg) : std::runtime_error(msg), status(s) {}
  sbr_status status;
};

inline void check(sbr_status s) {
  if (s != SBR_OK) throw Error(s, sbr_last_error());
}

// ---------------------------------------------------------------- values

struct Vec3 {
  double v[3] = {0, 0, 0};
  Vec3() = default;
  Vec3(double x, double y, double z) : v{x, y, z} {}
  double& operator[](int i) { return v[i]; }
  double operator[](int i) const { return v[i]; }
  double& operator()(int i) { return v[i]; }
  double operator()(int i) const { return v[i]; }
  double x() const { return v[0]; }
  double y() const { return v[1]; }
  double z() const { return v[2]; }
  const double* data() const { return v; }
};

// Row-major 3x3; Mat3{{r0}, {r1}, {r2}} as in SBRSolver_rev2.cpp:119.
struct Mat3 {
  double m[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  Mat3() = default;
  Mat3(std::initializer_list<std::initializer_list<double>> rows) {
    int i = 0;
    for (auto& r : rows) {
      int j = 0;
      for (double x : r)
        if (i < 3 && j < 3) m[i][j++] = x;
      ++i;
    }
  }
  static Mat3 Identity() { return Mat3{{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}; }
  double& operator()(int i, int j) { return m[i][j]; }
  double operator()(int i, int j) const { return m[i][j]; }
};

using VecVec3 = std::vector<Vec3>;
using cdouble = std::complex<double>;
using Vec3c = std::array<cdouble, 3>;

// DataStructures.h:20-28, same fields and order as sbr_material.
struct MaterialProperties {
  double frequency = 0;
  double transmissionLoss = 0;
  double reflectionLoss = 0;
  double relPermittivityRe = 1;
  double relPermittivityIm = 0;
  double relConductivity = 0;
  // Not in the reference: wall thickness (m) for the slab coefficients used
  // when useFresnelCoeff is false; 0 is what the reference always passes.
  double width = 0;
};

// Triangle.h:8-46: the fields a caller reads or sets.
struct Triangle {
  Vec3 v1, v2, v3, norm;
  int triangleId = -1;
  int coplanarId = -1;
  int materialId = 0;
};

// Settings the reference fixes in code: the antenna pattern (FieldCompute.cpp:117
// uses the Hertzian dipole) and the field precision of this library.
struct GlobalConfig {
  int antennaType = SBR_ANTENNA_HERTZIAN;
  int fieldPrecision = SBR_FIELD_FP64;
  bool fieldCheck = false;                // FP32 precisions: also state the error against FP64
  const sbr_pattern* pattern = nullptr;  // antennaType SBR_ANTENNA_TABULATED
};

// DataStructures.h:32-37: antenna gain table keyed by (theta, phi) degrees.
struct GainInfo {
  float data[4];  // theta gain, theta phase, phi gain, phi phase
};
using ThetaPhiAngle = std::pair<float, float>;
using GainMap = std::map<ThetaPhiAngle, GainInfo>;

// A TXPattern.dat table on the device (sbr_pattern_read), for antenna type 3.
class AntennaPattern {
 public:
  explicit AntennaPattern(const std::string& fileName) { check(sbr_pattern_read(fileName.c_str(), &p_)); }
  AntennaPattern(const AntennaPattern&) = delete;
  AntennaPattern& operator=(const AntennaPattern&) = delete;
  ~AntennaPattern() { sbr_pattern_destroy(p_); }
  const sbr_pattern* get() const { return p_; }

 private:
  sbr_pattern* p_ = nullptr;
};

// ---------------------------------------------------------- preprocessing

namespace Preprocessor {

// The facets in file order as heap-allocated Triangles (the reference's
// std::vector<Triangle*>; the caller deletes them).  saveEdges / saveFaces /
// dataDir are accepted for signature compatibility; no debug VTK is written.
inline bool StlToGeometry(std::string fileName, std::vector<Triangle*>& output,
                          bool saveEdges = false, bool saveFaces = false,
                          std::string dataDir = "") {
  (void)saveEdges;
  (void)saveFaces;
  (void)dataDir;
  int n = 0;
  if (sbr_stl_read(fileName.c_str(), &n, nullptr, nullptr) != SBR_OK) return false;
  std::vector<float> v(9 * size_t(n)), nr(3 * size_t(n));
  if (sbr_stl_read(fileName.c_str(), &n, v.data(), nr.data()) != SBR_OK) return false;
  output.reserve(output.size() + size_t(n));
  for (int t = 0; t < n; ++t) {
    auto* tri = new Triangle();
    const float* p = &v[9 * size_t(t)];
    tri->v1 = Vec3(p[0], p[1], p[2]);
    tri->v2 = Vec3(p[3], p[4], p[5]);
    tri->v3 = Vec3(p[6], p[7], p[8]);
    tri->norm = Vec3(nr[3 * size_t(t)], nr[3 * size_t(t) + 1], nr[3 * size_t(t) + 2]);
    tri->triangleId = t;
    output.push_back(tri);
  }
  return true;
}

inline void GenerateRxPlane(double xMin, double yMin, double xMax, double yMax, double height,
                            double resolution, VecVec3& output) {
  int n = 0;
  check(sbr_generate_rx_plane(xMin, yMin, xMax, yMax, height, resolution, nullptr, 0, &n));
  std::vector<double> p(3 * size_t(n));
  check(sbr_generate_rx_plane(xMin, yMin, xMax, yMax, height, resolution, p.data(), n, &n));
  for (int i = 0; i < n; ++i) output.emplace_back(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}

inline void GenerateRXLine(Vec3 start, Vec3 end, double resolution, VecVec3& output) {
  int n = 0;
  check(sbr_generate_rx_line(start.data(), end.data(), resolution, nullptr, 0, &n));
  std::vector<double> p(3 * size_t(n));
  check(sbr_generate_rx_line(start.data(), end.data(), resolution, p.data(), n, &n));
  for (int i = 0; i < n; ++i) output.emplace_back(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}

// Preprocessor.cpp:3-35: lines of six numbers (theta phi g_theta arg_theta
// g_phi arg_phi) into the map; other lines are skipped.
inline bool ReadPatternFile(std::string fileName, GainMap& output) {
  std::ifstream in(fileName);
  if (!in) return false;
  std::string line;
  while (std::getline(in, line)) {
    float v[6];
    char extra;
    if (std::sscanf(line.c_str(), " %f %f %f %f %f %f %c", &v[0], &v[1], &v[2], &v[3], &v[4],
                    &v[5], &extra) != 6)
      continue;
    output[{v[0], v[1]}] = GainInfo{{v[2], v[3], v[4], v[5]}};
  }
  return true;
}

// Whitespace-separated x y z per line; lines that do not parse are skipped.
inline bool ReadLocationFile(std::string fileName, VecVec3& output) {
  std::ifstream in(fileName);
  if (!in) return false;
  std::string line;
  while (std::getline(in, line)) {
    double x, y, z;
    char extra;
    if (std::sscanf(line.c_str(), " %lf %lf %lf %c", &x, &y, &z, &extra) == 3)
      output.emplace_back(x, y, z);
  }
  return true;
}

}  // namespace Preprocessor

// Icosahedron.cpp:80-109: the unit launch directions of a subdivision level in
// the reference's vertex order, heap-allocated like the reference's (the
// caller deletes the vector); the origin does not change them there either.
inline std::vector<Vec3>* GenerateRaysOnIcosahedron(int tessellation, Vec3 origin) {
  (void)origin;
  long long n = 0;
  check(sbr_launch_directions(tessellation, nullptr, 0, &n));
  std::vector<double> d(3 * size_t(n));
  check(sbr_launch_directions(tessellation, d.data(), n, &n));
  auto* out = new std::vector<Vec3>;
  out->reserve(size_t(n));
  for (long long i = 0; i < n; ++i) out->emplace_back(d[3 * i], d[3 * i + 1], d[3 * i + 2]);
  return out;
}

// ------------------------------------------------------------------ scene

template <class T>
class BVH;

template <>
class BVH<Triangle> {
 public:
  BVH() = default;
  BVH(const BVH&) = delete;
  BVH& operator=(const BVH&) = delete;
  ~BVH() { sbr_scene_destroy(scene_); }

  // Builds the device scene from the triangles (ids 0..n-1 in any order) and
  // leaves `objects` sorted the way the reference's SAH build leaves it.
  void ConstructBVH(std::vector<Triangle*>& objects) {
    const int n = int(objects.size());
    by_id_.assign(size_t(n), nullptr);
    for (Triangle* t : objects) {
      if (!t || t->triangleId < 0 || t->triangleId >= n || by_id_[size_t(t->triangleId)])
        throw Error(SBR_ERR_INVALID_ARG, "ConstructBVH: triangle ids must be 0..n-1, once each");
      by_id_[size_t(t->triangleId)] = t;
    }
    std::vector<float> v(9 * size_t(n)), nr(3 * size_t(n));
    std::vector<int> mat(static_cast<size_t>(n));
    int n_mat = 1;
    for (int i = 0; i < n; ++i) {
      const Triangle& t = *by_id_[size_t(i)];
      const Vec3* p[3] = {&t.v1, &t.v2, &t.v3};
      for (int k = 0; k < 3; ++k)
        for (int a = 0; a < 3; ++a) v[9 * size_t(i) + 3 * k + a] = float((*p[k])[a]);
      for (int a = 0; a < 3; ++a) nr[3 * size_t(i) + a] = float(t.norm[a]);
      mat[size_t(i)] = t.materialId;
      if (t.materialId >= n_mat) n_mat = t.materialId + 1;
    }
    // placeholder materials until RTSolver::Init binds the real table
    std::vector<sbr_material> placeholder(size_t(n_mat), sbr_material{0, 0, 0, 1, 0, 0, 0});
    sbr_scene_destroy(scene_);
    scene_ = nullptr;
    check(sbr_scene_create(n, v.data(), nr.data(), mat.data(), placeholder.data(), n_mat,
                           &scene_));
    std::vector<int> order(static_cast<size_t>(n)), cop(static_cast<size_t>(n));
    check(sbr_scene_mesh_order(scene_, order.data()));
    check(sbr_scene_coplanar_ids(scene_, cop.data()));
    for (int i = 0; i < n; ++i) {
      objects[size_t(i)] = by_id_[size_t(order[size_t(i)])];
      by_id_[size_t(i)]->coplanarId = cop[size_t(i)];
    }
  }

  sbr_scene* scene() const { return scene_; }
  const std::vector<Triangle*>& triangles_by_id() const { return by_id_; }

 private:
  sbr_scene* scene_ = nullptr;
  std::vector<Triangle*> by_id_;
};

// ------------------------------------------------------------------ solve

class FieldCompute {
 public:
  FieldCompute() = default;
  explicit FieldCompute(std::vector<double> field) : field_(std::move(field)) {}
  // The received field at a receiver (global Cartesian Ex, Ey, Ez).
  Vec3c FieldAtReceiver(int receiverId) const {
    if (receiverId < 0 || 6 * size_t(receiverId) + 6 > field_.size())
      throw Error(SBR_ERR_INVALID_ARG, "FieldAtReceiver: receiver id out of range");
    const double* f = &field_[6 * size_t(receiverId)];
    return Vec3c{cdouble(f[0], f[1]), cdouble(f[2], f[3]), cdouble(f[4], f[5])};
  }
  const std::vector<double>& raw() const { return field_; }

 private:
  std::vector<double> field_;
};

class RTSolver {
 public:
  explicit RTSolver(GlobalConfig config = GlobalConfig()) : config_(config) {}
  RTSolver(const RTSolver&) = delete;
  RTSolver& operator=(const RTSolver&) = delete;
  virtual ~RTSolver() { Cleanup(); }

  int Init(MaterialProperties materialProperties[], int materialPropertiesCount,
           BVH<Triangle>& triangles) {
    Cleanup();
    if (!triangles.scene()) throw Error(SBR_ERR_INVALID_ARG, "Init: ConstructBVH was not called");
    std::vector<sbr_material> m(static_cast<size_t>(materialPropertiesCount));
    for (int i = 0; i < materialPropertiesCount; ++i) {
      const MaterialProperties& p = materialProperties[i];
      m[size_t(i)] = sbr_material{p.frequency,         p.transmissionLoss,  p.reflectionLoss,
                                  p.relPermittivityRe, p.relPermittivityIm, p.relConductivity,
                                  p.width};
    }
    const auto& tris = triangles.triangles_by_id();
    std::vector<int> ids(tris.size());
    for (size_t i = 0; i < tris.size(); ++i) ids[i] = tris[i]->materialId;
    check(sbr_scene_set_materials(triangles.scene(), ids.data(), m.data(),
                                  materialPropertiesCount));
    bvh_ = &triangles;
    return 0;
  }

  void Cleanup() {
    if (result_) sbr_result_destroy(result_);
    result_ = nullptr;
    receivers_.clear();
    field_ = FieldCompute();
    bvh_ = nullptr;
  }

  // Returns launches x receivers, as the reference does (RTSolver.cpp:125).
  int ExecuteRayTracing(Vec3 sourcePoint, const Mat3& txCoordSys, int maxReflectionCount,
                        int maxTransmissionCount, double frequency, double pt,
                        bool useFresnelCoeff, VecVec3& receivers,
                        std::vector<Triangle*>& triangleMesh, int txTesslation) {
    (void)triangleMesh;  // the scene holds the mesh in the order ConstructBVH left it
    if (!bvh_) throw Error(SBR_ERR_INVALID_ARG, "ExecuteRayTracing: Init was not called");
    receivers_.resize(3 * receivers.size());
    for (size_t i = 0; i < receivers.size(); ++i)
      for (int a = 0; a < 3; ++a) receivers_[3 * i + a] = receivers[i][a];
    sbr_request q{};
    for (int a = 0; a < 3; ++a) q.tx[a] = sourcePoint[a];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) q.tx_coord_sys[3 * i + j] = txCoordSys(i, j);
    q.max_reflection = maxReflectionCount;
    q.max_transmission = maxTransmissionCount;
    q.frequency = frequency;
    q.pt = pt;
    q.use_fresnel = useFresnelCoeff ? 1 : 0;
    q.tessellation = txTesslation;
    q.antenna = config_.antennaType;
    q.field_precision = config_.fieldPrecision;
    q.field_check = config_.fieldCheck ? 1 : 0;
    q.pattern = config_.pattern;
    q.n_rx = int(receivers.size());
    q.rx = receivers_.data();
    if (result_) sbr_result_destroy(result_);
    result_ = nullptr;
    check(sbr_solve(bvh_->scene(), &q, &result_));
    std::vector<double> f(receivers_.size() * 2);
    check(sbr_result_field(result_, f.data()));
    field_ = FieldCompute(std::move(f));
    check(sbr_result_counts(result_, &counts_));
    return int(counts_.launches * (long long)receivers.size());
  }

  bool SavePathsAsVtk(std::string fname) {
    need_result();
    std::vector<sbr_path> p(size_t(counts_.paths));
    std::vector<int> tri(size_t(counts_.rays)), cop(tri.size()), kind(tri.size());
    std::vector<double> pts(6 * tri.size());
    check(sbr_result_paths(result_, p.data(), tri.data(), cop.data(), kind.data(), pts.data()));
    return sbr_write_paths_vtk(fname.c_str(), p.data(), int(p.size()), pts.data(),
                               field_.raw().data(), n_rx()) == SBR_OK;
  }
  bool SaveReceiversAsVtk(std::string fname) {
    need_result();
    return sbr_write_receivers_vtk(fname.c_str(), receivers_.data(), n_rx(),
                                   field_.raw().data()) == SBR_OK;
  }
  bool SaveFieldAsCsv(std::string fname) {
    need_result();
    return sbr_write_field_csv(fname.c_str(), receivers_.data(), n_rx(), field_.raw().data()) ==
           SBR_OK;
  }
  bool SaveIcosahedronAsVtk(std::string fname, Vec3 rayOrg, int tessellation) {
    return sbr_write_launch_rays_vtk(fname.c_str(), rayOrg.data(), tessellation) == SBR_OK;
  }

  // The field stage's output (FieldCompute is built inside ExecuteRayTracing
  // in the reference; here it is the result's field).
  const FieldCompute& fieldCompute() const { return field_; }
  const sbr_counts& counts() const { return counts_; }
  const sbr_result* result() const { return result_; }
  // FP32 precisions with GlobalConfig::fieldCheck: error against FP64.
  sbr_field_error fieldError() const {
    need_result();
    sbr_field_error e{};
    check(sbr_result_field_error(result_, &e));
    return e;
  }

 private:
  void need_result() const {
    if (!result_) throw Error(SBR_ERR_NOT_READY, "ExecuteRayTracing has not run");
  }
  int n_rx() const { return int(receivers_.size() / 3); }

  GlobalConfig config_;
  BVH<Triangle>* bvh_ = nullptr;
  sbr_result* result_ = nullptr;
  sbr_counts counts_{};
  std::vector<double> receivers_;
  FieldCompute field_;
};

}  // namespace sbrgb
