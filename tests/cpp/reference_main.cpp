// The reference's main() (SBRSolver_rev2.cpp:53-142) written against the
// C++ drop-in header: same calls, same arguments.  Usage:
//   reference_main <ground.stl> <output dir> [prep]
// Writes RayPath.vtk, RxLocations.vtk, ElectricField.csv and Icosahedron.vtk
// (level 3 from the Tx) into the output dir.  With "prep" it stops after the
// host-side preprocessing (no GPU needed) and prints what it read.
#include <cstdio>
#include <string>
#include <vector>

#include "sbr_solver.hpp"

using namespace sbrgb;

int main(int argc, char** argv) {
  if (argc != 3 && argc != 4) {
    std::fprintf(stderr, "usage: %s ground.stl outdir [prep]\n", argv[0]);
    return 2;
  }
  const std::string stlFileName = argv[1], out = argv[2];
  double freq = 1.8e9;
  double Pt = 1;
  int maxReflection = 1;
  int maxTransmission = 0;
  try {
    VecVec3 rxLocation;
    std::vector<Triangle*> triangle_mesh;
    BVH<Triangle> bvh;
    Preprocessor::GenerateRXLine(Vec3(0, 0, 3), Vec3(0, 3000, 3), 1, rxLocation);
    if (!Preprocessor::StlToGeometry(stlFileName, triangle_mesh, true, true, out)) {
      std::fprintf(stderr, "cannot read %s: %s\n", stlFileName.c_str(), sbr_last_error());
      return 1;
    }
    if (argc == 4) {
      const Triangle& t = *triangle_mesh.back();
      VecVec3 plane;
      Preprocessor::GenerateRxPlane(-5, -5, 5, 5, 7, 1, plane);
      std::printf("triangles %zu last %d (%g %g %g) receivers %zu last (%g %g %g) plane %zu\n",
                  triangle_mesh.size(), t.triangleId, t.v3.x(), t.v3.y(), t.v3.z(),
                  rxLocation.size(), rxLocation.back().x(), rxLocation.back().y(),
                  rxLocation.back().z(), plane.size());
      std::vector<Vec3>* rays = GenerateRaysOnIcosahedron(2, Vec3(0, 0, 5));
      std::printf("rays %zu last %.17g %.17g %.17g\n", rays->size(), rays->back().x(),
                  rays->back().y(), rays->back().z());
      delete rays;
      for (Triangle* p : triangle_mesh) delete p;
      return 0;
    }
    bvh.ConstructBVH(triangle_mesh);
    Vec3 rayOrig{0, 0, 5};
    MaterialProperties materials[4];
    materials[0].frequency = 1.8e9;
    materials[0].reflectionLoss = 0.05;
    materials[0].transmissionLoss = 221.13;
    materials[0].relConductivity = 1e6;
    materials[0].relPermittivityRe = 1;
    materials[0].relPermittivityIm = 0;
    materials[1] = {1.8e9, -1, -1, 2.5, 0.3, 0.03};
    materials[2] = {1.8e9, -1, -1, 1.8, 0.3, 0.03};
    materials[3] = {1.8e9, -1, -1, 6, 0.05, 0.005};
    int tessllation = 2;
    Mat3 txCoordSys{{0, 1, 0}, {0, 0, 1}, {1, 0, 0}};
    GlobalConfig cfg;  // Hertzian dipole, FP64, as the reference
    RTSolver* rayTracer = new RTSolver(cfg);
    rayTracer->Init(materials, 1, bvh);
    int total_paths = rayTracer->ExecuteRayTracing(rayOrig, txCoordSys, maxReflection,
                                                   maxTransmission, freq, Pt, true, rxLocation,
                                                   triangle_mesh, tessllation);
    bool ok = rayTracer->SavePathsAsVtk(out + "/RayPath.vtk") &&
              rayTracer->SaveIcosahedronAsVtk(out + "/Icosahedron.vtk", rayOrig, 3) &&
              rayTracer->SaveReceiversAsVtk(out + "/RxLocations.vtk") &&
              rayTracer->SaveFieldAsCsv(out + "/ElectricField.csv");
    Vec3c e = rayTracer->fieldCompute().FieldAtReceiver(0);
    std::printf("launches x receivers %d, paths %lld, |Ex(rx0)| %.6g\n", total_paths,
                rayTracer->counts().paths, std::abs(e[0]));
    delete rayTracer;
    for (Triangle* t : triangle_mesh) delete t;
    return ok ? 0 : 1;
  } catch (const Error& e) {
    std::fprintf(stderr, "error %d: %s\n", int(e.status), e.what());
    return 1;
  }
}
