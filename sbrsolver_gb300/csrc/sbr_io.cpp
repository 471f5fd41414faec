// Result files in the reference's formats, byte for byte:
//   field CSV        RTSolver::SaveFieldAsCsv      (RTSolver.cpp:692-717)
//   ray-path VTK     RTSolver::SavePathsAsVtk      (RTSolver.cpp:510-610) + PathsToVector (:768-803)
//   receiver VTK     RTSolver::SaveReceiversAsVtk  (RTSolver.cpp:612-690)
//   launch-ray VTK   RTSolver::SaveIcosahedronAsVtk (RTSolver.cpp:719-766)
//
// The numbers go through std::ostream with its default formatting (six
// significant digits), as in the reference, including its quirks:
//   * SaveFieldAsCsv sets std::showpos on the stream and never clears it, so
//     every row after the first prints '+' on non-negative coordinates;
//   * the Phase columns hold the plain sum of the three component phases in
//     radians (the reference's conversion to degrees is an expression whose
//     value is discarded);
//   * VTK ray paths are listed launch by launch, then by receiver, then in
//     breadth-first order of the launch's ray tree.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <fstream>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/sbr.h"
#include "sbr_host.h"

namespace sbr {
void set_error_message(const std::string& s);
}

namespace {

using cd = std::complex<double>;

const char* kVtkHead = "# vtk DataFile Version 2.0";

// Field of receiver k as three complex components.
void field_at(const double* f, long long k, cd e[3]) {
  for (int j = 0; j < 3; ++j) e[j] = cd(f[6 * k + 2 * j], f[6 * k + 2 * j + 1]);
}

// Euclidean norm of a complex 3-vector: sqrt(sum |e_j|^2), summed in order.
double cnorm(const cd e[3]) {
  double s = 0;
  for (int j = 0; j < 3; ++j) s += e[j].real() * e[j].real() + e[j].imag() * e[j].imag();
  return std::sqrt(s);
}

double total_phase(const cd e[3]) {
  const double p = (std::arg(e[0]) + std::arg(e[1])) + std::arg(e[2]);
  return std::isfinite(p) ? p : 0.0;
}

sbr_status open_or_fail(std::ofstream& ofs, const char* path, const char* who) {
  if (!path) {
    sbr::set_error_message(std::string(who) + ": NULL path");
    return SBR_ERR_INVALID_ARG;
  }
  ofs.open(path);
  if (!ofs) {
    sbr::set_error_message(std::string(who) + ": cannot open " + path);
    return SBR_ERR_IO;
  }
  return SBR_OK;
}

sbr_status close_or_fail(std::ofstream& ofs, const char* path, const char* who) {
  ofs.close();
  if (ofs.fail()) {
    sbr::set_error_message(std::string(who) + ": write to " + path + " failed");
    return SBR_ERR_IO;
  }
  return SBR_OK;
}

}  // namespace

extern "C" {

sbr_status sbr_write_field_csv(const char* path, const double* rx, int n_rx, const double* field) {
  if (n_rx < 0 || (n_rx > 0 && (!rx || !field))) {
    sbr::set_error_message("sbr_write_field_csv: bad arguments");
    return SBR_ERR_INVALID_ARG;
  }
  std::ofstream ofs;
  if (sbr_status s = open_or_fail(ofs, path, "sbr_write_field_csv")) return s;
  ofs << "X,Y,Z,Ex,Ey,Ez" << '\n';
  for (int i = 0; i < n_rx; ++i) {
    cd e[3];
    field_at(field, i, e);
    ofs << rx[3 * i] << "," << rx[3 * i + 1] << "," << rx[3 * i + 2] << ",";
    ofs << std::showpos;  // stays set for the rest of the file
    for (int j = 0; j < 3; ++j) ofs << e[j].real() << e[j].imag() << "i" << (j < 2 ? "," : "\n");
  }
  return close_or_fail(ofs, path, "sbr_write_field_csv");
}

sbr_status sbr_write_receivers_vtk(const char* path, const double* rx, int n_rx,
                                   const double* field) {
  if (n_rx < 0 || (n_rx > 0 && (!rx || !field))) {
    sbr::set_error_message("sbr_write_receivers_vtk: bad arguments");
    return SBR_ERR_INVALID_ARG;
  }
  std::ofstream ofs;
  if (sbr_status s = open_or_fail(ofs, path, "sbr_write_receivers_vtk")) return s;
  ofs << kVtkHead << "\nRay Path Visualization\nASCII\nDATASET POLYDATA\n\n";
  ofs << "POINTS " << n_rx << " float\n";
  for (int i = 0; i < n_rx; ++i)
    ofs << " " << rx[3 * i] << " " << rx[3 * i + 1] << " " << rx[3 * i + 2] << "\n";
  ofs << "VERTICES 1 " << n_rx + 1 << "\n" << n_rx << "\n";
  for (int i = 0; i < n_rx; ++i) {
    ofs << " " << i;
    if (i % 5 == 4) ofs << "\n";
  }
  ofs << "\n";
  ofs << "POINT_DATA " << n_rx << "\nFIELD FieldData 4\n";
  ofs << "ReceiverID 1 " << n_rx << " int\n";
  for (int i = 0; i < n_rx; ++i) ofs << " " << i << "\n";
  ofs << "Eabs 1 " << n_rx << " double\n";
  for (int i = 0; i < n_rx; ++i) {
    cd e[3];
    field_at(field, i, e);
    const double n = cnorm(e);
    ofs << " " << (std::isfinite(n) ? n : 0.0) << "\n";
  }
  ofs << "EdB 1 " << n_rx << " double\n";
  for (int i = 0; i < n_rx; ++i) {
    cd e[3];
    field_at(field, i, e);
    const double n = cnorm(e);
    const double a = std::isfinite(n) ? n : 0.0;
    ofs << " " << (a > 0.0 ? 20 * std::log10(n * 1e6) : -300.0) << "\n";
  }
  ofs << "Phase 1 " << n_rx << " double\n";
  for (int i = 0; i < n_rx; ++i) {
    cd e[3];
    field_at(field, i, e);
    ofs << " " << total_phase(e) << "\n";
  }
  return close_or_fail(ofs, path, "sbr_write_receivers_vtk");
}

sbr_status sbr_write_paths_vtk(const char* path, const sbr_path* paths, int n_paths,
                               const double* points, const double* field, int n_rx) {
  if (n_paths < 0 || n_rx < 0 || (n_paths > 0 && (!paths || !points || !field))) {
    sbr::set_error_message("sbr_write_paths_vtk: bad arguments");
    return SBR_ERR_INVALID_ARG;
  }
  for (int i = 0; i < n_paths; ++i)
    if (paths[i].receiver < 0 || paths[i].receiver >= n_rx || paths[i].n_rays < 1 ||
        paths[i].ray_offset < 0) {
      sbr::set_error_message("sbr_write_paths_vtk: path " + std::to_string(i) +
                             " has a receiver or ray range out of bounds");
      return SBR_ERR_INVALID_ARG;
    }
  // launch-major, then receiver, then breadth-first position in the tree
  std::vector<int> order(n_paths);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    const sbr_path &p = paths[a], &q = paths[b];
    if (p.launch != q.launch) return p.launch < q.launch;
    if (p.receiver != q.receiver) return p.receiver < q.receiver;
    return p.heap < q.heap;
  });
  long long n_vert = 0, total = 0;
  for (int i = 0; i < n_paths; ++i) {
    n_vert += paths[i].n_rays + 1;
    total += paths[i].n_rays + 2;
  }
  std::ofstream ofs;
  if (sbr_status s = open_or_fail(ofs, path, "sbr_write_paths_vtk")) return s;
  ofs << kVtkHead << "\nRay Path Visualization\nASCII\nDATASET POLYDATA\n\n";
  ofs << "POINTS " << n_vert << " float\n";
  auto pt = [&](const double* p) { ofs << " " << p[0] << " " << p[1] << " " << p[2] << "\n"; };
  for (int k : order) {
    const sbr_path& p = paths[k];
    const double* r = points + 6 * p.ray_offset;  // per ray: source xyz, target xyz
    pt(r);
    for (int j = 0; j < p.n_rays; ++j) pt(r + 6 * j + 3);
  }
  ofs << "LINES " << n_paths << " " << total << "\n";
  long long v = 0;
  for (int k : order) {
    const int m = paths[k].n_rays + 1;
    ofs << " " << m << " ";
    for (int j = 0; j < m; ++j) ofs << v++ << " ";
    ofs << "\n";
  }
  ofs << "CELL_DATA " << n_paths << "\nFIELD FieldData 5\n";
  ofs << "LaunchID 1 " << n_paths << " int\n";
  for (int k : order) ofs << " " << paths[k].launch << "\n";
  ofs << "ReceiverID 1 " << n_paths << " int\n";
  for (int k : order) ofs << " " << paths[k].receiver << "\n";
  ofs << "Eabs 1 " << n_paths << " double\n";
  for (int k : order) {
    cd e[3];
    field_at(field, paths[k].receiver, e);
    const double n = cnorm(e);
    ofs << " " << (std::isfinite(n) ? n : 0.0) << "\n";
  }
  ofs << "EdB 1 " << n_paths << " double\n";
  for (int k : order) {
    cd e[3];
    field_at(field, paths[k].receiver, e);
    const double n = cnorm(e);
    double db = std::isfinite(n) ? 20 * std::log10(n * 1e6) : -300.0;
    ofs << " " << (std::isfinite(db) ? db : -300.0) << "\n";
  }
  ofs << "Phase 1 " << n_paths << " double\n";
  for (int k : order) {
    cd e[3];
    field_at(field, paths[k].receiver, e);
    ofs << " " << total_phase(e) << "\n";
  }
  return close_or_fail(ofs, path, "sbr_write_paths_vtk");
}

sbr_status sbr_generate_rx_line(const double* start, const double* end, double resolution,
                                double* out, int capacity, int* n_out) {
  if (!start || !end || !n_out || !(resolution > 0)) {
    sbr::set_error_message("sbr_generate_rx_line: need start, end, a positive resolution, n_out");
    return SBR_ERR_INVALID_ARG;
  }
  double d[3] = {end[0] - start[0], end[1] - start[1], end[2] - start[2]};
  const double len = std::sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
  const double fn = std::floor(len / resolution);
  if (!(fn < 2147483647.0)) {
    sbr::set_error_message("sbr_generate_rx_line: too many points");
    return SBR_ERR_INVALID_ARG;
  }
  const int n = std::max(0, int(fn));
  if (len > 0)
    for (double& c : d) c /= len;
  if (out) {
    if (capacity < n) {
      *n_out = n;
      sbr::set_error_message("sbr_generate_rx_line: capacity below the point count");
      return SBR_ERR_CAPACITY;
    }
    for (int i = 0; i < n; ++i) {
      const double s = double(i) * resolution;
      for (int a = 0; a < 3; ++a) {
        const double step = s * d[a];  // rounded before the add (no contraction)
        out[3 * size_t(i) + a] = start[a] + step;
      }
    }
  }
  *n_out = n;
  return SBR_OK;
}

sbr_status sbr_generate_rx_plane(double x_min, double y_min, double x_max, double y_max,
                                 double height, double resolution, double* out, int capacity,
                                 int* n_out) {
  if (!n_out || !(resolution > 0)) {
    sbr::set_error_message("sbr_generate_rx_plane: need a positive resolution and n_out");
    return SBR_ERR_INVALID_ARG;
  }
  const double fx = (x_max - x_min) / resolution, fy = (y_max - y_min) / resolution;
  if (!(fx < 1e9 && fy < 1e9)) {
    sbr::set_error_message("sbr_generate_rx_plane: too many points");
    return SBR_ERR_INVALID_ARG;
  }
  const long long nx = (long long)int(fx), ny = (long long)int(fy);
  const long long n = (nx >= 0 && ny >= 0) ? (nx + 1) * (ny + 1) : 0;
  if (n > 2147483647LL) {
    sbr::set_error_message("sbr_generate_rx_plane: too many points");
    return SBR_ERR_INVALID_ARG;
  }
  if (out) {
    if (capacity < n) {
      *n_out = int(n);
      sbr::set_error_message("sbr_generate_rx_plane: capacity below the point count");
      return SBR_ERR_CAPACITY;
    }
    size_t k = 0;
    for (long long i = 0; n && i <= nx; ++i) {
      const double x = x_min + double(i) * resolution;
      for (long long j = 0; j <= ny; ++j) {
        out[k++] = x;
        out[k++] = y_min + double(j) * resolution;
        out[k++] = height;
      }
    }
  }
  *n_out = int(n);
  return SBR_OK;
}

sbr_status sbr_write_launch_rays_vtk(const char* path, const double* origin, int tessellation) {
  if (!origin || tessellation < 0 || tessellation > 12) {
    sbr::set_error_message("sbr_write_launch_rays_vtk: need an origin and a level in 0..12");
    return SBR_ERR_INVALID_ARG;
  }
  std::vector<double> d;
  sbr::icosphere(tessellation, d);
  const size_t n = d.size() / 3;
  std::ofstream ofs;
  if (sbr_status s = open_or_fail(ofs, path, "sbr_write_launch_rays_vtk")) return s;
  ofs << kVtkHead << "\nTX Icosahedron Visualization\nASCII\nDATASET POLYDATA\n\n";
  ofs << "POINTS " << n + 1 << " float\n";
  ofs << " " << origin[0] << " " << origin[1] << " " << origin[2] << "\n";
  for (size_t i = 0; i < n; ++i)
    ofs << " " << origin[0] + 1.0 * d[3 * i] << " " << origin[1] + 1.0 * d[3 * i + 1] << " "
        << origin[2] + 1.0 * d[3 * i + 2] << "\n";
  ofs << "LINES " << n << " " << 3 * n << "\n";
  for (size_t i = 1; i <= n; ++i) ofs << " 2 0 " << i << "\n";
  ofs << "CELL_DATA " << n << "\nFIELD FieldData 1\n";
  ofs << "LaunchID 1 " << n << " int\n";
  for (size_t i = 0; i < n; ++i) ofs << " " << i << "\n";
  return close_or_fail(ofs, path, "sbr_write_launch_rays_vtk");
}

sbr_status sbr_launch_directions(int tessellation, double* directions, long long cap,
                                 long long* n_rays) {
  if (!n_rays || tessellation < 0 || tessellation > 12 || (directions && cap < 0)) {
    sbr::set_error_message("sbr_launch_directions: need n_rays, a level in 0..12 and cap >= 0");
    return SBR_ERR_INVALID_ARG;
  }
  const long long n = 10LL * (1LL << (2 * tessellation)) + 2;
  *n_rays = n;
  if (!directions) return SBR_OK;
  if (cap < n) {
    sbr::set_error_message("sbr_launch_directions: room for " + std::to_string(cap) +
                           " rays, the level has " + std::to_string(n));
    return SBR_ERR_CAPACITY;
  }
  std::vector<double> d;
  sbr::icosphere(tessellation, d);
  std::memcpy(directions, d.data(), sizeof(double) * d.size());
  return SBR_OK;
}

}  // extern "C"
