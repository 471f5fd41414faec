// Command-line driver of the CPU restatement (TEST INFRASTRUCTURE).  Reads the
// same case file as the reference harness (oracle/ref_harness.cpp) and writes
// the same report format, so the two can be compared line by line.
#include "sbr_oracle.cpp"

#include <chrono>

int main(int argc, char** argv) {
  if (argc < 3 || std::strcmp(argv[1], "case") != 0) {
    std::fprintf(stderr, "usage: oracle_cli case <file> [threads]\n");
    return 1;
  }
  std::ifstream in(argv[2]);
  std::string key, stl, trimat, rxp, out;
  std::vector<MaterialProperties_c> mats;
  oracle_request rq{};
  double txcs[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  rq.max_reflection = 1; rq.tessellation = 2; rq.antenna = 1; rq.frequency = 1.8e9; rq.pt = 1;
  rq.use_fresnel = 1;
  while (in >> key) {
    if (key == "stl") in >> stl;
    else if (key == "trimat") in >> trimat;
    else if (key == "rx") in >> rxp;
    else if (key == "out") in >> out;
    else if (key == "materials") {
      int n; in >> n; mats.resize(n);
      for (auto& m : mats) in >> m.frequency >> m.transmissionLoss >> m.reflectionLoss >>
          m.relPermittivityRe >> m.relPermittivityIm >> m.relConductivity;
    } else if (key == "widths") {
      int n; in >> n;
      if (n != int(mats.size())) { std::fprintf(stderr, "widths: need one per material\n"); return 2; }
      for (auto& m : mats) in >> m.width;
    } else if (key == "tx") in >> rq.tx[0] >> rq.tx[1] >> rq.tx[2];
    else if (key == "txcs") for (double& v : txcs) in >> v;
    else if (key == "refl") in >> rq.max_reflection;
    else if (key == "trans") in >> rq.max_transmission;
    else if (key == "tess") in >> rq.tessellation;
    else if (key == "antenna") in >> rq.antenna;
    else if (key == "freq") in >> rq.frequency;
    else if (key == "pt") in >> rq.pt;
    else if (key == "fresnel") in >> rq.use_fresnel;
    else { std::fprintf(stderr, "unknown key %s\n", key.c_str()); return 2; }
  }
  std::memcpy(rq.tx_coord_sys, txcs, sizeof txcs);
  std::vector<double> rx;
  {
    std::ifstream r(rxp);
    long n; r >> n;
    rx.resize(3 * n);
    for (auto& v : rx) r >> v;
  }
  rq.n_rx = int(rx.size() / 3);
  rq.rx = rx.data();
  rq.n_materials = int(mats.size());
  rq.materials = mats.data();
  oracle_scene* sc = nullptr;
  if (oracle_scene_from_stl(stl.c_str(), &sc)) return 3;
  if (!trimat.empty() && trimat != "-") {
    std::ifstream tm(trimat);
    std::vector<int> ids(sc->s.tris.size());
    for (auto& v : ids) tm >> v;
    oracle_scene_set_materials(sc, ids.data());
  }
  const int threads = argc > 3 ? std::atoi(argv[3]) : 0;
  auto t0 = std::chrono::steady_clock::now();
  oracle_result* res = nullptr;
  oracle_solve(sc, &rq, threads, &res);
  double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  FILE* f = std::fopen(out.c_str(), "w");
  std::fprintf(f, "segments %ld\nlaunches %zu\nreceivers %d\ntriangles %zu\n", res->segments,
               orc::icosphere(rq.tessellation).size(), rq.n_rx, sc->s.tris.size());
  size_t p = 0;
  for (int k = 0; k < rq.n_rx; ++k) {
    for (; p < res->paths.size() && res->paths[p].receiver == k; ++p) {
      const oracle_path& op = res->paths[p];
      std::fprintf(f, "path %d %ld %d %.17g %.17g %.17g %.17g %.17g %.17g\n", k, op.launch,
                   op.n_rays, op.field[0], op.field[1], op.field[2], op.field[3], op.field[4],
                   op.field[5]);
      long o = res->ray_offset[p];
      for (int r = 0; r < op.n_rays; ++r) {
        int kind = res->kind[o + r];
        int mat = r == 0 ? -1 : sc->s.tris[res->tri[o + r - 1]].mat;
        const double* q = &res->pts[6 * (o + r)];
        std::fprintf(f, " ray %d %d %d %d %.17g %.17g %.17g %.17g %.17g %.17g\n", res->tri[o + r],
                     res->cop[o + r], kind == 1 ? mat : -1, kind == 2 ? mat : -1, q[0], q[1],
                     q[2], q[3], q[4], q[5]);
      }
    }
    const double* e = &res->field[6 * k];
    std::fprintf(f, "field %d %.17g %.17g %.17g %.17g %.17g %.17g\n", k, e[0], e[1], e[2], e[3],
                 e[4], e[5]);
  }
  std::fprintf(f, "loop_mismatch 0\n");
  std::fclose(f);
  std::fprintf(stderr, "oracle: %.3f s, %ld segments, %ld captured, %ld corrected, %zu kept\n", sec,
               res->segments, res->captured, res->corrected, res->paths.size());
  oracle_result_destroy(res);
  oracle_scene_destroy(sc);
  return 0;
}
