// Harness around the compiled reference (test infrastructure, oracle side).
//
// Links the reference's own translation units (SBRSolver_rev2/*.cpp, built
// unmodified against oracle/compat/Eigen) and drives them the way the
// reference's main() does (SBRSolver_rev2/SBRSolver_rev2.cpp:53-142), with
// the scene, materials, transmitter and receivers read from a case file
// instead of being hard-coded.  It writes every surviving path per receiver
// and the received field so the CPU restatement (oracle/sbr_oracle.cpp) and
// the GPU path can be pinned against the reference itself.
//
// Access to RTSolver/FieldCompute internals: this translation unit alone
// compiles the reference headers with private/protected opened so it can
// read _rayPaths after ExecuteRayTracing and call the Fresnel/pattern
// building blocks.  The reference hard-codes the Hertzian pattern in
// FieldForPath (FieldCompute.cpp:117); for other antenna types the harness
// re-runs the same per-segment loop (FieldCompute.cpp:71-151) over the
// reference's own helpers with the chosen pattern, and checks that its loop
// reproduces FieldForPath bit-for-bit when the pattern is the Hertzian one.
// Every standard header the reference pulls in is included before the
// access specifiers are opened below, so only the reference's own classes
// see the change.
#include <algorithm>
#include <atomic>
#include <cassert>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <fstream>
#include <iostream>
#include <iterator>
#include <limits>
#include <list>
#include <map>
#include <mutex>
#include <new>
#include <queue>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>
#include <Eigen/Dense>
#include <Eigen/StdVector>

#define private public
#define protected public
#include "RTSolver.h"
#include "FieldCompute.h"
#include "Icosahedron.h"
#undef private
#undef protected

namespace {

struct Case {
  std::string stl, trimat, rx, out;
  std::vector<MaterialProperties> mats;
  std::vector<double> widths;  // per material; the reference passes 0
  Vec3 tx{0, 0, 0};
  Mat3 txcs = Mat3::Identity();
  int refl = 1, trans = 0, tess = 2, antenna = 1;
  double freq = 1.8e9, pt = 1.0;
  bool fresnel = true;
};

bool read_case(const char* path, Case& c) {
  std::ifstream in(path);
  if (!in) return false;
  std::string key;
  while (in >> key) {
    if (key == "stl") in >> c.stl;
    else if (key == "trimat") in >> c.trimat;
    else if (key == "rx") in >> c.rx;
    else if (key == "out") in >> c.out;
    else if (key == "materials") {
      int n;
      in >> n;
      c.mats.resize(n);
      for (auto& m : c.mats)
        in >> m.frequency >> m.transmissionLoss >> m.reflectionLoss >> m.relPermittivityRe >>
            m.relPermittivityIm >> m.relConductivity;
    } else if (key == "widths") {
      int n;
      in >> n;
      c.widths.resize(n);
      for (double& w : c.widths) in >> w;
    } else if (key == "tx") in >> c.tx(0) >> c.tx(1) >> c.tx(2);
    else if (key == "txcs") {
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) in >> c.txcs(i, j);
    } else if (key == "refl") in >> c.refl;
    else if (key == "trans") in >> c.trans;
    else if (key == "tess") in >> c.tess;
    else if (key == "antenna") in >> c.antenna;
    else if (key == "freq") in >> c.freq;
    else if (key == "pt") in >> c.pt;
    else if (key == "fresnel") { int f; in >> f; c.fresnel = f != 0; }
    else { std::fprintf(stderr, "unknown key %s\n", key.c_str()); return false; }
  }
  return true;
}

bool read_points(const std::string& path, VecVec3& out) {
  std::ifstream in(path);
  if (!in) return false;
  long n;
  in >> n;
  for (long i = 0; i < n; ++i) {
    Vec3 p;
    in >> p(0) >> p(1) >> p(2);
    out.push_back(p);
  }
  return true;
}

// FieldCompute.cpp:71-151 with the pattern type and the per-material wall
// thickness passed to ComputeRefcField/ComputeTransField as parameters (the
// reference passes width 0 at FieldCompute.cpp:131,138).
Vec3c field_for_path(FieldCompute& fc, const std::vector<Ray>& path, int antenna,
                     const std::vector<double>& widths) {
  auto width_of = [&](int m) { return m < int(widths.size()) ? widths[m] : 0.0; };
  double lamda = SPEED_OF_LIGHT / fc._frequency;
  double k = (2 * PI) / lamda;
  Mat3 globalCoordSys = Mat3::Identity();
  Mat3 currentCoordSys = globalCoordSys;
  Mat3 nextCoordSys = fc._txCoordSys;
  Vec3c incidentField{cdouble(0, 0), cdouble(0, 0), cdouble(0, 0)};
  Vec3c totalField{cdouble(0, 0), cdouble(0, 0), cdouble(0, 0)};
  double totalPathLength = 0.0;
  for (int i = 0; i < int(path.size()); i++) {
    const Ray& ray = path[i];
    Vec3 vecGlobal = ray.targetPoint - ray.sourcePoint;
    Vec3 vecLocal = RotateToNewCoordSys(vecGlobal, globalCoordSys, nextCoordSys);
    Vec3 vecSph = CartesianToSpherical(vecLocal);
    double r = vecSph(0), theta = vecSph(1), phi = vecSph(2);
    totalPathLength += r;
    currentCoordSys = nextCoordSys;
    if (ray.hitSurfaceID == -1) nextCoordSys = globalCoordSys;
    else nextCoordSys = fc._triangleMesh->at(ray.hitSurfaceID)->coordSys;
    if (i == 0) {
      incidentField = fc.GetAnalyticEfieldPattern(antenna, theta, phi, fc._txPower);
    } else {
      incidentField = RotateToNewCoordSys(totalField, currentCoordSys, globalCoordSys);
      incidentField = CartesianToSphericalVector(incidentField, theta, phi);
    }
    if (ray.reflectionMaterialId >= 0) {
      double incidentAngle =
          AngleBetween(vecGlobal, currentCoordSys(2, Eigen::indexing::all), false, true);
      double relPerm = fc._materials[ray.reflectionMaterialId].relPermittivityRe;
      double sigma = fc._materials[ray.reflectionMaterialId].relConductivity;
      totalField = fc.ComputeRefcField(incidentField, relPerm, sigma, fc._frequency,
                                       incidentAngle, width_of(ray.reflectionMaterialId),
                                       fc._useFresnelCoeff);
    } else if (ray.penetrationMaterialId >= 0) {
      double incidentAngle =
          AngleBetween(vecGlobal, currentCoordSys(2, Eigen::indexing::all), false, true);
      double relPerm = fc._materials[ray.penetrationMaterialId].relPermittivityRe;
      double sigma = fc._materials[ray.penetrationMaterialId].relConductivity;
      totalField = fc.ComputeTransField(incidentField, relPerm, sigma, fc._frequency,
                                        incidentAngle, width_of(ray.penetrationMaterialId),
                                        fc._useFresnelCoeff);
    } else {
      totalField = incidentField;
    }
    totalField = SphericalToCartesianVector(totalField, theta, phi);
    totalField = RotateToNewCoordSys(totalField, currentCoordSys, globalCoordSys);
  }
  totalField = totalField * exp(-j * k * totalPathLength) / totalPathLength;
  return totalField;
}

bool same_bits(const Vec3c& a, const Vec3c& b) {
  for (int i = 0; i < 3; ++i) {
    double x[2] = {a(i).real(), a(i).imag()}, y[2] = {b(i).real(), b(i).imag()};
    if (std::memcmp(x, y, sizeof x) != 0) return false;
  }
  return true;
}

int run_case(const Case& c) {
  VecVec3 rx;
  if (!read_points(c.rx, rx)) { std::fprintf(stderr, "cannot read %s\n", c.rx.c_str()); return 2; }
  std::vector<Triangle*> mesh;
  if (!Preprocessor::StlToGeometry(c.stl, mesh, false, false, "")) return 3;
  if (!c.trimat.empty() && c.trimat != "-") {
    std::ifstream in(c.trimat);
    for (auto* t : mesh) in >> t->materialId;
  }
  BVH<Triangle> bvh;
  bvh.ConstructBVH(mesh);

  // RTSolver's constructor runs Cleanup() on members it never initialised
  // (RTSolver.cpp:3-6,24-50); give it zeroed storage.
  void* mem = std::calloc(1, sizeof(RTSolver));
  RTSolver* solver = new (mem) RTSolver();
  std::vector<MaterialProperties> mats = c.mats;
  solver->Init(mats.data(), int(mats.size()), bvh);

  solver->ExecuteRayTracing(c.tx, c.txcs, c.refl, c.trans, c.freq, c.pt, c.fresnel, rx, mesh,
                            c.tess);
  const long segments = RayGlobalId.load();

  FieldCompute fc(solver->_rayPaths, mesh, rx, solver->_pathsCount, solver->_materialProperties,
                  c.txcs, c.freq, c.pt, c.fresnel);

  FILE* f = std::fopen(c.out.c_str(), "w");
  if (!f) return 4;
  std::fprintf(f, "segments %ld\nlaunches %d\nreceivers %d\ntriangles %zu\n", segments,
               solver->_pathsCount, solver->_receiverCount, mesh.size());
  int loop_mismatch = 0;
  bool zero_width = true;
  for (double w : c.widths) zero_width = zero_width && w == 0.0;
  const std::vector<double> no_width;
  for (int k = 0; k < solver->_receiverCount; ++k) {
    Vec3c total{cdouble(0, 0), cdouble(0, 0), cdouble(0, 0)};
    for (int i = 0; i < solver->_pathsCount; ++i) {
      for (const auto& path : solver->_rayPaths[i][k].rayPaths) {
        Vec3c e = field_for_path(fc, path, c.antenna, c.widths);
        if (!same_bits(field_for_path(fc, path, 1, no_width), fc.FieldForPath(path)))
          ++loop_mismatch;
        total += e;
        std::fprintf(f, "path %d %d %zu %.17g %.17g %.17g %.17g %.17g %.17g\n", k, i, path.size(),
                     e(0).real(), e(0).imag(), e(1).real(), e(1).imag(), e(2).real(),
                     e(2).imag());
        for (const Ray& r : path)
          std::fprintf(f, " ray %d %d %d %d %.17g %.17g %.17g %.17g %.17g %.17g\n", r.hitSurfaceID,
                       r.hitCoplanarId, r.reflectionMaterialId, r.penetrationMaterialId,
                       r.sourcePoint(0), r.sourcePoint(1), r.sourcePoint(2), r.targetPoint(0),
                       r.targetPoint(1), r.targetPoint(2));
      }
    }
    const Vec3c& ref = solver->_efield->at(k);
    if (c.antenna == 1 && zero_width && !same_bits(ref, total)) ++loop_mismatch;
    std::fprintf(f, "field %d %.17g %.17g %.17g %.17g %.17g %.17g\n", k, total(0).real(),
                 total(0).imag(), total(1).real(), total(1).imag(), total(2).real(),
                 total(2).imag());
  }
  std::fprintf(f, "loop_mismatch %d\n", loop_mismatch);
  std::fclose(f);
  return loop_mismatch == 0 ? 0 : 5;
}

// Stage counts: re-runs ExecuteRayTracing's three loops (RTSolver.cpp:82-121)
// through the solver's own private members and reports how many paths exist
// after capture, after image correction and after duplicate removal.
int run_stages(const Case& c, const char* out) {
  VecVec3 rx;
  if (!read_points(c.rx, rx)) return 2;
  std::vector<Triangle*> mesh;
  if (!Preprocessor::StlToGeometry(c.stl, mesh, false, false, "")) return 3;
  if (!c.trimat.empty() && c.trimat != "-") {
    std::ifstream in(c.trimat);
    for (auto* t : mesh) in >> t->materialId;
  }
  BVH<Triangle> bvh;
  bvh.ConstructBVH(mesh);
  void* mem = std::calloc(1, sizeof(RTSolver));
  RTSolver* s = new (mem) RTSolver();
  std::vector<MaterialProperties> mats = c.mats;
  s->Init(mats.data(), int(mats.size()), bvh);
  RayGlobalId = 0;
  s->_maxReflectionCount = c.refl;
  s->_maxTransmissionCount = c.trans;
  s->_txTesslation = c.tess + 1;
  s->_shootRayList = GenerateRaysOnIcosahedron(c.tess, c.tx);
  s->_receivers = &rx;
  s->_receiverCount = int(rx.size());
  s->_pathsCount = int(s->_shootRayList->size());
  s->_efield = new std::vector<Vec3c>;
  s->InitRayPaths();
  Vec3 src = c.tx;
  long captured = 0;
  for (int i = 0; i < s->_pathsCount; i++) {
    PathTreeNode rootNode;
    rootNode.ray.id = RayGlobalId++;
    s->RayLaunch(&rootNode, src, s->_shootRayList->at(i), -1, -1, 0, 0, 0, true, INF);
    for (int j = 0; j < s->_receiverCount; j++) {
      PathTreeNode* cloneRoot = CloneNode(&rootNode);
      CloneTree(&rootNode, cloneRoot);
      s->RayCapture(cloneRoot, rx[j], 0.0);
      s->_rayPaths[i][j] = Paths(cloneRoot);
      captured += long(s->_rayPaths[i][j].rayPaths.size());
      cloneRoot = DeleteChildNodes(cloneRoot);
      delete cloneRoot;
    }
  }
  const long segments = RayGlobalId.load();
  long corrected = 0, deduped = 0;
  for (int k = 0; k < s->_receiverCount; k++) {
    s->ImagePathCorrection(k, c.tx, mesh);
    for (int i = 0; i < s->_pathsCount; i++) corrected += long(s->_rayPaths[i][k].rayPaths.size());
    s->RemoveDuplicatePath(k);
    for (int i = 0; i < s->_pathsCount; i++) deduped += long(s->_rayPaths[i][k].rayPaths.size());
  }
  FILE* f = std::fopen(out, "w");
  if (!f) return 4;
  std::fprintf(f, "segments %ld\ncaptured %ld\ncorrected %ld\ndeduplicated %ld\n", segments,
               captured, corrected, deduped);
  std::fclose(f);
  return 0;
}

// Icosahedron launch directions (Icosahedron.cpp:80-109), full precision.
int dump_ico(int level, const char* out) {
  std::vector<Vec3>* dirs = GenerateRaysOnIcosahedron(level, Vec3(0, 0, 0));
  FILE* f = std::fopen(out, "wb");
  if (!f) return 4;
  for (const Vec3& d : *dirs) std::fwrite(d.data(), sizeof(double), 3, f);
  std::fclose(f);
  delete dirs;
  return 0;
}

// Scene preparation + BVH (Preprocessor.cpp:69-246, BVH.h:135-230): per
// triangle (id, coplanar id) and the BVH in node order.
int dump_scene(const char* stl, const char* out) {
  std::vector<Triangle*> mesh;
  if (!Preprocessor::StlToGeometry(stl, mesh, false, false, "")) return 3;
  BVH<Triangle> bvh;
  bvh.ConstructBVH(mesh);
  FILE* f = std::fopen(out, "w");
  if (!f) return 4;
  std::fprintf(f, "triangles %zu\n", mesh.size());
  for (auto* t : mesh)
    std::fprintf(f, "tri %d %d %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n",
                 t->triangleId, t->coplanarId, t->coordSys(0, 0), t->coordSys(0, 1),
                 t->coordSys(0, 2), t->coordSys(1, 0), t->coordSys(1, 1), t->coordSys(1, 2),
                 t->coordSys(2, 0), t->coordSys(2, 1), t->coordSys(2, 2));
  std::fprintf(f, "nodes %zu\n", bvh.nodes.size());
  for (auto& n : bvh.nodes) {
    std::fprintf(f, "node %d %d %.9g %.9g %.9g %.9g %.9g %.9g %zu", n.children[0], n.children[1],
                 n.bbox(0, 0), n.bbox(0, 1), n.bbox(0, 2), n.bbox(1, 0), n.bbox(1, 1),
                 n.bbox(1, 2), n.objects.size());
    for (auto* t : n.objects) std::fprintf(f, " %d", t->triangleId);
    std::fprintf(f, "\n");
  }
  std::fclose(f);
  return 0;
}

// Fresnel sweep exactly as FieldCompute::RefCoeffTest (FieldCompute.cpp:27-47).
int dump_coeff(int n, double freq, double e1r, double e1i, double e2r, double e2i, const char* out) {
  FieldCompute fc;
  fc.RefCoeffTest(n, freq, cdouble(e1r, e1i), cdouble(e2r, e2i), out);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc >= 2 && std::strcmp(argv[1], "case") == 0 && argc == 3) {
    Case c;
    if (!read_case(argv[2], c)) return 2;
    std::streambuf* old = std::cout.rdbuf();
    std::ostringstream sink;
    std::cout.rdbuf(sink.rdbuf());  // the solver prints progress lines
    int rc = run_case(c);
    std::cout.rdbuf(old);
    return rc;
  }
  if (argc == 4 && std::strcmp(argv[1], "stages") == 0) {
    Case c;
    if (!read_case(argv[2], c)) return 2;
    std::streambuf* old = std::cout.rdbuf();
    std::ostringstream sink;
    std::cout.rdbuf(sink.rdbuf());
    int rc = run_stages(c, argv[3]);
    std::cout.rdbuf(old);
    return rc;
  }
  if (argc == 4 && std::strcmp(argv[1], "ico") == 0) return dump_ico(std::atoi(argv[2]), argv[3]);
  if (argc == 4 && std::strcmp(argv[1], "scene") == 0) return dump_scene(argv[2], argv[3]);
  if (argc == 9 && std::strcmp(argv[1], "coeff") == 0)
    return dump_coeff(std::atoi(argv[2]), std::atof(argv[3]), std::atof(argv[4]),
                      std::atof(argv[5]), std::atof(argv[6]), std::atof(argv[7]), argv[8]);
  std::fprintf(stderr,
               "usage: ref_harness case <file> | stages <file> <out> | ico <level> <out> | scene <stl> <out> |"
               " coeff <n> <freq> <e1r> <e1i> <e2r> <e2i> <out>\n");
  return 1;
}
