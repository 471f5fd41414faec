// Tabulated antenna patterns: the TXPattern.dat format the reference ships
// (data/TXPattern.dat) and reads with Preprocessor::ReadPatternFile into a
// GainMap of (theta, phi) -> (g_theta, arg_theta, g_phi, arg_phi)
// (Preprocessor.cpp:3-35, common/DataStructures.h:32-37).  The reference
// loads the table but never applies it; here antenna type 3 applies it to
// the launch direction as E_theta, E_phi = sqrt(60 Pt) 10^(g/20) e^(j arg),
// gains in dB and phases in degrees, bilinear on the (theta, phi) grid.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sbr.h"

namespace sbr {
void set_error_message(const std::string& s);
}

struct sbr_pattern {
  int nt = 0, np = 0;
  double dt = 1, dp = 1;
  std::vector<float> amp;  // 4 per grid point: re, im of E_theta, then E_phi
  float* dev = nullptr;    // the same on the device
  int device = -1;
  ~sbr_pattern() {
    if (dev) cudaFree(dev);
  }
};

namespace sbr {

// The device table and grid of a pattern, for the solver's request setup.
void pattern_fields(const sbr_pattern* p, const float** dev, int* nt, int* np, double* dt,
                    double* dp, int* device) {
  *dev = p->dev;
  *device = p->device;
  *nt = p->nt;
  *np = p->np;
  *dt = p->dt;
  *dp = p->dp;
}

}  // namespace sbr

namespace {

sbr_status make_pattern(int nt, int np, double dt, double dp, const float* gp, sbr_pattern** out) {
  if (!out || !gp || nt < 1 || np < 1 || !(dt > 0) || !(dp > 0) ||
      std::fabs(np * dp - 360.0) > 1e-6 * 360.0 || (nt - 1) * dt > 180.0 + 1e-9) {
    sbr::set_error_message(
        "sbr_pattern_create: need n_theta >= 1, n_phi * d_phi = 360 and (n_theta - 1) * d_theta "
        "<= 180");
    return SBR_ERR_INVALID_ARG;
  }
  auto* p = new sbr_pattern();
  p->nt = nt;
  p->np = np;
  p->dt = dt;
  p->dp = dp;
  const size_t n = size_t(nt) * size_t(np);
  p->amp.resize(4 * n);
  const double deg = 3.14159265358979323846 / 180.0;
  for (size_t k = 0; k < n; ++k) {
    for (int c = 0; c < 2; ++c) {
      const double g = std::pow(10.0, double(gp[4 * k + 2 * c]) / 20.0);
      const double a = double(gp[4 * k + 2 * c + 1]) * deg;
      p->amp[4 * k + 2 * c] = float(g * std::cos(a));
      p->amp[4 * k + 2 * c + 1] = float(g * std::sin(a));
    }
  }
  cudaGetDevice(&p->device);
  if (cudaMalloc(&p->dev, 4 * sizeof(float) * n) != cudaSuccess ||
      cudaMemcpy(p->dev, p->amp.data(), 4 * sizeof(float) * n, cudaMemcpyHostToDevice) !=
          cudaSuccess) {
    cudaGetLastError();
    delete p;
    sbr::set_error_message("sbr_pattern_create: device allocation or copy failed");
    return SBR_ERR_CUDA;
  }
  *out = p;
  return SBR_OK;
}

}  // namespace

extern "C" {

sbr_status sbr_pattern_create(int n_theta, int n_phi, double d_theta, double d_phi,
                              const float* gain_phase, sbr_pattern** out) {
  return make_pattern(n_theta, n_phi, d_theta, d_phi, gain_phase, out);
}

sbr_status sbr_pattern_read(const char* path, sbr_pattern** out) {
  if (!path || !out) {
    sbr::set_error_message("sbr_pattern_read: NULL argument");
    return SBR_ERR_INVALID_ARG;
  }
  std::ifstream in(path);
  if (!in) {
    sbr::set_error_message(std::string("sbr_pattern_read: cannot open ") + path);
    return SBR_ERR_IO;
  }
  // rows of six numbers, as ReadPatternFile keeps them; other lines are skipped
  std::map<std::pair<float, float>, std::vector<float>> rows;
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ss(line);
    std::vector<std::string> tok;
    std::string t;
    while (ss >> t) tok.push_back(t);
    if (tok.size() != 6) continue;
    float v[6];
    bool ok = true;
    for (int i = 0; i < 6 && ok; ++i) {
      char* end = nullptr;
      v[i] = std::strtof(tok[i].c_str(), &end);
      ok = end && *end == '\0';
    }
    if (!ok) continue;
    rows[{v[0], v[1]}] = {v[2], v[3], v[4], v[5]};
  }
  if (rows.size() < 2) {
    sbr::set_error_message(std::string("sbr_pattern_read: no pattern rows in ") + path);
    return SBR_ERR_IO;
  }
  // regular grid: steps from the distinct angles
  std::vector<float> th, ph;
  for (const auto& r : rows) {
    if (th.empty() || th.back() != r.first.first) th.push_back(r.first.first);
  }
  {
    std::map<float, int> ps;
    for (const auto& r : rows) ps[r.first.second] = 1;
    for (const auto& q : ps) ph.push_back(q.first);
  }
  const double dt = th.size() > 1 ? double(th[1]) - double(th[0]) : 1.0;
  const double dp = ph.size() > 1 ? double(ph[1]) - double(ph[0]) : 360.0;
  const int nt = int(th.size()), np = int(ph.size());
  if (th[0] != 0.0f || ph[0] != 0.0f) {
    sbr::set_error_message("sbr_pattern_read: the grid must start at theta = phi = 0");
    return SBR_ERR_INVALID_ARG;
  }
  std::vector<float> gp(4 * size_t(nt) * size_t(np));
  for (int i = 0; i < nt; ++i)
    for (int j = 0; j < np; ++j) {
      auto it = rows.find({float(i * dt), float(j * dp)});
      if (it == rows.end()) {
        sbr::set_error_message("sbr_pattern_read: missing grid point theta " +
                               std::to_string(i * dt) + " phi " + std::to_string(j * dp));
        return SBR_ERR_INVALID_ARG;
      }
      for (int c = 0; c < 4; ++c) gp[4 * (size_t(i) * np + j) + c] = it->second[c];
    }
  return make_pattern(nt, np, dt, dp, gp.data(), out);
}

sbr_status sbr_pattern_info(const sbr_pattern* p, int* n_theta, int* n_phi, double* d_theta,
                            double* d_phi) {
  if (!p) {
    sbr::set_error_message("sbr_pattern_info: NULL pattern");
    return SBR_ERR_INVALID_ARG;
  }
  if (n_theta) *n_theta = p->nt;
  if (n_phi) *n_phi = p->np;
  if (d_theta) *d_theta = p->dt;
  if (d_phi) *d_phi = p->dp;
  return SBR_OK;
}

sbr_status sbr_pattern_destroy(sbr_pattern* p) {
  delete p;
  return SBR_OK;
}

}  // extern "C"
