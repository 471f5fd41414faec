// Received field of one corrected path (FieldCompute::FieldForPath,
// FieldCompute.cpp:71-151, with GetAnalyticEfieldPattern :153-183,
// ComputeRefcField/ComputeTransField :185-235, GetTECoeff/GetTMCoeff/
// GetTransAngle :237-302 and the VecMatDef.h:51-155 helpers).
//
// Templated on the real type: double reproduces the reference's FP64
// arithmetic; float computes the per-segment rotations and Fresnel
// coefficients in FP32 while the path length and the phase k*L stay FP64
// (k*L reaches ~1e6 rad at 28 GHz and 1 km, far beyond FP32 resolution).
// Complex functions are written from their textbook definitions
// (principal branches), not copied from any math library.
#pragma once

#include <cuda_runtime.h>

namespace sbr {

template <class R>
struct Cx {
  R re, im;
};
template <class R>
__device__ __forceinline__ Cx<R> cx(R a, R b = R(0)) {
  return Cx<R>{a, b};
}
template <class R>
__device__ __forceinline__ Cx<R> operator+(Cx<R> a, Cx<R> b) {
  return cx(a.re + b.re, a.im + b.im);
}
template <class R>
__device__ __forceinline__ Cx<R> operator-(Cx<R> a, Cx<R> b) {
  return cx(a.re - b.re, a.im - b.im);
}
template <class R>
__device__ __forceinline__ Cx<R> operator-(Cx<R> a) {
  return cx(-a.re, -a.im);
}
template <class R>
__device__ __forceinline__ Cx<R> operator*(Cx<R> a, Cx<R> b) {
  return cx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <class R>
__device__ __forceinline__ Cx<R> operator*(R s, Cx<R> a) {
  return cx(s * a.re, s * a.im);
}
template <class R>
__device__ __forceinline__ Cx<R> operator*(Cx<R> a, R s) {
  return cx(a.re * s, a.im * s);
}
// Smith's division (Smith 1962).
template <class R>
__device__ __forceinline__ Cx<R> operator/(Cx<R> a, Cx<R> b) {
  if (fabs(b.re) >= fabs(b.im)) {
    R r = b.im / b.re, den = b.re + b.im * r;
    return cx((a.re + a.im * r) / den, (a.im - a.re * r) / den);
  }
  R r = b.re / b.im, den = b.im + b.re * r;
  return cx((a.re * r + a.im) / den, (a.im * r - a.re) / den);
}
template <class R>
__device__ __forceinline__ Cx<R> operator/(R s, Cx<R> b) {
  return cx(s) / b;
}
template <class R>
__device__ __forceinline__ Cx<R> operator/(Cx<R> a, R s) {
  return cx(a.re / s, a.im / s);
}
// Principal square root: with r = |z|, sqrt(z) = (sqrt((r+x)/2), y/(2t)) for
// x >= 0, else (|y|/(2t), sign(y) t) with t = sqrt((r-x)/2).
template <class R>
__device__ __forceinline__ Cx<R> csqrt(Cx<R> z) {
  if (z.re == R(0) && z.im == R(0)) return cx(R(0), z.im);
  R r = hypot(z.re, z.im);
  if (z.re >= R(0)) {
    R t = sqrt((r + z.re) * R(0.5));
    return cx(t, z.im / (R(2) * t));
  }
  R t = sqrt((r - z.re) * R(0.5));
  return cx(fabs(z.im) / (R(2) * t), copysign(t, z.im));
}
template <class R>
__device__ __forceinline__ Cx<R> cexp_(Cx<R> z) {
  R e = exp(z.re);
  return cx(e * cos(z.im), e * sin(z.im));
}
template <class R>
__device__ __forceinline__ Cx<R> clog_(Cx<R> z) {
  return cx(log(hypot(z.re, z.im)), atan2(z.im, z.re));
}
template <class R>
__device__ __forceinline__ Cx<R> csin_(Cx<R> z) {
  return cx(sin(z.re) * cosh(z.im), cos(z.re) * sinh(z.im));
}
template <class R>
__device__ __forceinline__ Cx<R> ccos_(Cx<R> z) {
  return cx(cos(z.re) * cosh(z.im), -(sin(z.re) * sinh(z.im)));
}
// asin z = -i log(i z + sqrt(1 - z^2))
template <class R>
__device__ __forceinline__ Cx<R> casin_(Cx<R> z) {
  Cx<R> iz = cx(-z.im, z.re);
  Cx<R> w = clog_(iz + csqrt(cx(R(1)) - z * z));
  return cx(w.im, -w.re);
}

template <class R>
struct M3 {
  R m[9];  // row-major
};
template <class R>
__device__ __forceinline__ void mv(const M3<R>& a, const R* v, R* r) {
  for (int i = 0; i < 3; ++i) r[i] = (a.m[3 * i] * v[0] + a.m[3 * i + 1] * v[1]) + a.m[3 * i + 2] * v[2];
}
template <class R>
__device__ __forceinline__ void mtv(const M3<R>& a, const Cx<R>* v, Cx<R>* r) {  // a^T v
  for (int i = 0; i < 3; ++i)
    r[i] = (a.m[i] * v[0] + a.m[3 + i] * v[1]) + a.m[6 + i] * v[2];
}
template <class R>
__device__ __forceinline__ void mcv(const M3<R>& a, const Cx<R>* v, Cx<R>* r) {  // a v
  for (int i = 0; i < 3; ++i)
    r[i] = (a.m[3 * i] * v[0] + a.m[3 * i + 1] * v[1]) + a.m[3 * i + 2] * v[2];
}

// Tabulated antenna pattern (the TXPattern.dat grid of data/TXPattern.dat,
// which Preprocessor::ReadPatternFile loads, Preprocessor.cpp:3-35): complex
// relative amplitudes of E_theta and E_phi on a regular (theta, phi) grid in
// degrees, phi periodic.  E = sqrt(60 Pt) * amplitude, as the analytic
// patterns scale with sqrt(60 Pt G).
struct PatternTab {
  const float4* a;  // nt * np entries, theta-major
  int nt, np;
  double dt, dp;
};

// Bilinear interpolation of the grid at (theta, phi) degrees; theta clamped
// to the grid, phi wrapped.  out = (re, im) of E_theta then E_phi.
__device__ __forceinline__ void pattern_at(const PatternTab& p, double th, double ph, double* out) {
  double ft = th / p.dt;
  ft = fmin(fmax(ft, 0.0), double(p.nt - 1));
  int t0 = min(int(ft), p.nt - 2 >= 0 ? p.nt - 2 : 0);
  const double wt = p.nt > 1 ? ft - t0 : 0.0;
  const int t1 = p.nt > 1 ? t0 + 1 : t0;
  double fp = ph / p.dp;
  fp -= floor(fp / p.np) * p.np;
  int p0 = int(fp);
  if (p0 >= p.np) p0 = p.np - 1;
  const double wp = fp - p0;
  const int p1 = (p0 + 1) % p.np;
  const float4 a00 = p.a[t0 * p.np + p0], a01 = p.a[t0 * p.np + p1];
  const float4 a10 = p.a[t1 * p.np + p0], a11 = p.a[t1 * p.np + p1];
  const double w00 = (1 - wt) * (1 - wp), w01 = (1 - wt) * wp, w10 = wt * (1 - wp), w11 = wt * wp;
  out[0] = w00 * a00.x + w01 * a01.x + w10 * a10.x + w11 * a11.x;
  out[1] = w00 * a00.y + w01 * a01.y + w10 * a10.y + w11 * a11.y;
  out[2] = w00 * a00.z + w01 * a01.z + w10 * a10.z + w11 * a11.z;
  out[3] = w00 * a00.w + w01 * a01.w + w10 * a10.w + w11 * a11.w;
}

struct FieldConsts {
  double e0, eta0, pi_hi, pi_lo;  // reference constants (computed on the host)
};

// The slab's round-trip phase factor ph = e^(-j 2q), q = (2 pi width / lam)
// sqrt(n_t - sin^2 theta_i) (FieldCompute.cpp:257-258,286-287; the square root
// takes the refractive index n_t, as the reference's does).  Taken in FP64 for
// every field precision: 2q reaches hundreds of radians for walls many
// wavelengths thick.  Width 0 (what the reference always passes) gives q = 0
// and ph = 1 exactly.
__device__ __forceinline__ Cx<double> slab_phase(double theta_i, Cx<double> eps_t, double lam,
                                                 double width, double two_pi) {
  if (width == 0.0) return cx(1.0, 0.0);
  const Cx<double> nt = csqrt(eps_t), si = csin_(cx(theta_i));
  const Cx<double> q = ((two_pi * width) / lam) * csqrt(nt - si * si);
  return cexp_(cx(0.0, -2.0) * q);
}

template <class R>
__device__ __forceinline__ R cabs_(Cx<R> z) {
  return hypot(z.re, z.im);
}

// GetTransAngle + GetTMCoeff/GetTECoeff for air -> eps_t; returns the
// coefficient pair (TM, TE) applied to E_theta, E_phi.  ph: slab_phase.
// cond (optional) receives the smallest ratio |denominator| / (sum of the
// magnitudes of its two terms) over the coefficients' denominators: near 0
// the coefficient sits near a pole of its formula, where the rounding of its
// inputs is amplified by about the inverse of that ratio.
template <class R>
__device__ void fresnel_pair(bool reflect, R theta_i, Cx<R> eps_t, Cx<R> ph, bool inf_wall,
                             R eta0, Cx<R>& c_tm, Cx<R>& c_te, R* cond = nullptr) {
  const Cx<R> ni = cx(R(1)), nt = csqrt(eps_t);
  const Cx<R> ti = cx(theta_i);
  const Cx<R> tt = casin_((ni / nt) * csin_(ti));
  const Cx<R> etai = eta0 / ni, etat = eta0 / nt;
  const Cx<R> ci = ccos_(ti), ct = ccos_(tt);
  const Cx<R> a_te = etat / ct, b_te = etai / ci, a_tm = etat * ct, b_tm = etai * ci;
  const Cx<R> g_te = -(a_te - b_te) / (a_te + b_te);
  const Cx<R> g_tm = (-a_tm + b_tm) / (a_tm + b_tm);
  if (cond)
    *cond = fmin(cabs_(a_te + b_te) / (cabs_(a_te) + cabs_(b_te)),
                 cabs_(a_tm + b_tm) / (cabs_(a_tm) + cabs_(b_tm)));
  if (inf_wall) {
    c_tm = reflect ? g_tm : cx(R(0));
    c_te = reflect ? g_te : cx(R(0));
    return;
  }
  // Slab of thickness width (FieldCompute.cpp:255-262,284-291); width 0
  // gives reflection 0 and transmission 1.
  const Cx<R> one = cx(R(1));
  const Cx<R> den_tm = one - g_tm * g_tm * ph, den_te = one - g_te * g_te * ph;
  if (cond)
    *cond = fmin(*cond, fmin(cabs_(den_tm) / (R(1) + cabs_(g_tm * g_tm * ph)),
                             cabs_(den_te) / (R(1) + cabs_(g_te * g_te * ph))));
  if (reflect) {
    c_tm = (g_tm * (one - ph)) / den_tm;
    c_te = (g_te * (one - ph)) / den_te;
  } else {
    c_tm = ((one - g_tm * g_tm) * ph) / den_tm;
    c_te = ((one - g_te * g_te) * ph) / den_te;
  }
}

// FieldForPath (FieldCompute.cpp:71-151) in two parts.  Everything a segment
// contributes except the field it carries depends only on the path's geometry:
// its length, the spherical angles of its direction in the frame it starts in,
// the coefficients of the interaction at its start and, for the launch
// segment, the antenna pattern.  seg_terms computes those for one segment (one
// thread per segment, so the long FP64 chains of the transcendental functions
// run side by side); path_combine then carries the field along the path with
// the same operations, in the same order, as one sequential pass would.
// R: real type of the rotation/Fresnel arithmetic.  Values of type R are
// stored as doubles, which holds floats exactly.
// FP32 field mode: interactions whose Fresnel denominators cancel below
// this fraction of their terms take the FP64 coefficients (fresnel_pair).
constexpr float kFresnelCond32 = 0.125f;

struct SegTerms {
  double r;               // segment length (FP64)
  double st, ct, sp, cp;  // sin / cos of the direction's theta and phi
  double ctm[2], cte[2];  // TM / TE coefficients of the interaction at the start
  double inc[6];          // launch segment: the pattern's field (r, theta, phi)
  int fp64_fresnel;       // FP32 mode: the coefficients came from the FP64 formula
  int pad;
};

// The frame a segment starts in: the transmitter's for the launch segment,
// else the frame of the triangle the previous segment ended on (none: global).
template <class R>
__device__ __forceinline__ M3<R> start_frame(int i, const double* const* frames,
                                             const double* txcs) {
  M3<R> f;
  const double* src = i == 0 ? txcs : frames[i - 1];
  if (src == nullptr) {
    for (int j = 0; j < 9; ++j) f.m[j] = (j % 4 == 0) ? R(1) : R(0);
  } else {
    for (int j = 0; j < 9; ++j) f.m[j] = R(src[j]);
  }
  return f;
}

// Segment i of a path with points pts (i -> i+1), triangle frames frames[k]
// of the triangle ray k ends on (null = none), and the kind / material of
// each ray's start.
template <class R>
__device__ void seg_terms(int i, const double (*pts)[3], const double* const* frames,
                          const int* kind, const int* mat, const Material* mats,
                          const double* txcs, double freq, double pt, int antenna, bool fresnel,
                          const FieldConsts& K, SegTerms& out, const PatternTab* pat = nullptr) {
  const double lam64 = 2.99792458e8 / freq;
  const M3<R> cur = start_frame<R>(i, frames, txcs);
  double vg64[3] = {pts[i + 1][0] - pts[i][0], pts[i + 1][1] - pts[i][1], pts[i + 1][2] - pts[i][2]};
  R vg[3] = {R(vg64[0]), R(vg64[1]), R(vg64[2])};
  R vl[3];
  mv(cur, vg, vl);
  // CartesianToSpherical (VecMatDef.h:132-155); r is kept in FP64, the length
  // of the vector rotated by the FP64 frame, as in the reference (the FP32
  // mode forms it the same way below).
  if constexpr (sizeof(R) == sizeof(double)) {
    double vl64[3];
    for (int j = 0; j < 3; ++j)
      vl64[j] = (cur.m[3 * j] * vg64[0] + cur.m[3 * j + 1] * vg64[1]) + cur.m[3 * j + 2] * vg64[2];
    out.r = sqrt((vl64[0] * vl64[0] + vl64[1] * vl64[1]) + vl64[2] * vl64[2]);
  }
  R th, ph;
  if (vl[0] == R(0) && vl[1] == R(0) && vl[2] == R(0)) th = R(K.pi_hi * 0.5);
  else th = atan2(sqrt(vl[0] * vl[0] + vl[1] * vl[1]), vl[2]);
  ph = atan2(vl[1], vl[0]);
  if (ph < R(0)) ph = R((double(ph) + 2.0 * K.pi_hi) + 2.0 * K.pi_lo);
  if constexpr (sizeof(R) == sizeof(double)) {
    out.st = sin(th);
    out.ct = cos(th);
    out.sp = sin(ph);
    out.cp = cos(ph);
  } else {
    // FP32 mode: the segment rotated into its frame in FP64 (a few FP64
    // operations per segment), then the basis from its components, which
    // keeps each of sin/cos theta, phi to a few FP32 ulps even for
    // directions near the frame's axis, where an FP32 rotation or sin(theta)
    // of theta near 0 or pi loses most of their relative precision
    const double* fr = i == 0 ? txcs : frames[i - 1];
    double w64[3];
    float w[3];
    for (int j = 0; j < 3; ++j) {
      const double r0 = fr ? fr[3 * j] : (j == 0 ? 1.0 : 0.0);
      const double r1 = fr ? fr[3 * j + 1] : (j == 1 ? 1.0 : 0.0);
      const double r2 = fr ? fr[3 * j + 2] : (j == 2 ? 1.0 : 0.0);
      w64[j] = (r0 * vg64[0] + r1 * vg64[1]) + r2 * vg64[2];
      w[j] = float(w64[j]);
    }
    // the segment length as the FP64 mode (and the reference) takes it: of
    // the vector rotated by the FP64 frame, which a triangle's single-
    // precision file normal leaves orthonormal only to ~1e-7, so the
    // global length would move the phase k*L of a long path by ~1e-4 rad
    out.r = sqrt((w64[0] * w64[0] + w64[1] * w64[1]) + w64[2] * w64[2]);
    const float rho = sqrtf(w[0] * w[0] + w[1] * w[1]);
    const float len = sqrtf(rho * rho + w[2] * w[2]);
    if (len > 0.0f) {
      out.st = double(rho / len);
      out.ct = double(w[2] / len);
    } else {  // the zero vector: theta = pi/2, phi = 0 (VecMatDef.h:132-155)
      out.st = 1.0;
      out.ct = 0.0;
    }
    out.sp = rho > 0.0f ? double(w[1] / rho) : 0.0;
    out.cp = rho > 0.0f ? double(w[0] / rho) : 1.0;
    th = atan2(rho, w[2]);  // the pattern's angles
    if (len == 0.0f) th = R(K.pi_hi * 0.5);
    ph = atan2(w[1], w[0]);
    if (ph < R(0)) ph = R((double(ph) + 2.0 * K.pi_hi) + 2.0 * K.pi_lo);
  }
  for (int j = 0; j < 6; ++j) out.inc[j] = 0.0;
  out.fp64_fresnel = 0;
  out.pad = 0;
  if (i == 0) {
    Cx<R> inc[3] = {cx(R(0)), cx(R(0)), cx(R(0))};
    if constexpr (sizeof(R) == sizeof(double)) {
      if (antenna == 0) inc[0] = cx(R(0), R(sqrt(60.0 * pt)));
      if (antenna == 1) inc[1] = cx(R(0), R(sqrt(60.0 * pt * 1.5)) * sin(th));
      else if (antenna == 2)
        inc[1] = cx(R(0), R(sqrt(60.0 * pt)) * (cos(R(K.pi_hi) * cos(th) / R(2)) / sin(th)));
    } else {
      // FP32: sin and cos of theta from the segment's components (accurate
      // to ulps, unlike sin(theta) near the dipole axis, where theta's own
      // FP32 rounding is most of sin(theta)).  The half-wave pattern's
      // cos(pi/2 cos th) is sin(pi s) with s = sin^2(th/2) = st^2 / (2 (1 + ct))
      // or cos^2(th/2) = st^2 / (2 (1 - ct)), whichever is at most 1/2: no
      // cancellation near the axis, where cos(pi/2 cos th) -> 0.
      const float st = float(out.st), ct = float(out.ct);
      if (antenna == 0) inc[0] = cx(R(0), R(sqrt(60.0 * pt)));
      if (antenna == 1) inc[1] = cx(R(0), R(sqrt(60.0 * pt * 1.5)) * st);
      else if (antenna == 2) {
        const float h2 = (st * st) / (2.0f * (ct >= 0.0f ? 1.0f + ct : 1.0f - ct));
        inc[1] = cx(R(0), R(sqrt(60.0 * pt)) * (sinf(float(K.pi_hi) * h2) / st));
      }
    }
    if (antenna == 3 && pat) {
      double a[4];
      pattern_at(*pat, double(th) * (180.0 / K.pi_hi), double(ph) * (180.0 / K.pi_hi), a);
      const double amp = sqrt(60.0 * pt);
      inc[1] = cx(R(amp * a[0]), R(amp * a[1]));
      inc[2] = cx(R(amp * a[2]), R(amp * a[3]));
    }
    for (int j = 0; j < 3; ++j) {
      out.inc[2 * j] = double(inc[j].re);
      out.inc[2 * j + 1] = double(inc[j].im);
    }
  }
  Cx<R> ctm = cx(R(1)), cte = cx(R(1));
  if (kind[i] != 0) {
    // AngleBetween(vecGlobal, current row 2) in radians (VecMatDef.h:56-77),
    // in FP64 for every precision: the reference's coefficients have poles
    // (its angle convention puts some reflections past 90 degrees), and near
    // one even the FP32 rounding of the angle moves a coefficient by 1e-5
    const double* fr = i == 0 ? txcs : frames[i - 1];
    double a[3] = {vg64[0], vg64[1], vg64[2]};
    double b[3] = {fr ? fr[6] : 0.0, fr ? fr[7] : 0.0, fr ? fr[8] : 1.0};
    double za = (a[0] * a[0] + a[1] * a[1]) + a[2] * a[2];
    if (za > 0.0) { double s = sqrt(za); a[0] /= s; a[1] /= s; a[2] /= s; }
    double zb = (b[0] * b[0] + b[1] * b[1]) + b[2] * b[2];
    if (zb > 0.0) { double s = sqrt(zb); b[0] /= s; b[1] /= s; b[2] /= s; }
    double ratio = (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
    double ang;
    if (ratio < 0.0) {
      double e0 = -a[0] - b[0], e1 = -a[1] - b[1], e2 = -a[2] - b[2];
      double y = 2.0 * asin(sqrt((e0 * e0 + e1 * e1) + e2 * e2) / 2.0);
      ang = (K.pi_hi - y) + K.pi_lo;
    } else {
      double e0 = a[0] - b[0], e1 = a[1] - b[1], e2 = a[2] - b[2];
      ang = 2.0 * asin(sqrt((e0 * e0 + e1 * e1) + e2 * e2) / 2.0);
    }
    const Material& m = mats[mat[i]];
    const Cx<double> eps64 = cx(m.eps_re, -1.0 * m.sigma / (K.e0 * 2.0 * K.pi_hi * freq));
    const Cx<R> eps_t = cx(R(eps64.re), R(eps64.im));
    Cx<double> p64 = cx(1.0);
    if (!fresnel) p64 = slab_phase(ang, eps64, lam64, m.width, 2.0 * K.pi_hi);
    const Cx<R> sph = cx(R(p64.re), R(p64.im));
    R cond = R(1);
    fresnel_pair<R>(kind[i] == 1, R(ang), eps_t, sph, fresnel, R(K.eta0), ctm, cte, &cond);
    if constexpr (sizeof(R) != sizeof(double)) {
      // near a pole the FP32 coefficients carry errors of ~2^-24 / cond:
      // take them from the FP64 formula there
      if (!(cond >= kFresnelCond32)) {
        Cx<double> tm64, te64;
        fresnel_pair<double>(kind[i] == 1, ang, eps64, p64, fresnel, K.eta0, tm64, te64);
        ctm = cx(R(tm64.re), R(tm64.im));
        cte = cx(R(te64.re), R(te64.im));
        out.fp64_fresnel = 1;
      }
    }
  }
  out.ctm[0] = double(ctm.re);
  out.ctm[1] = double(ctm.im);
  out.cte[0] = double(cte.re);
  out.cte[1] = double(cte.im);
}

// The field at the end of an n-ray path from its segments' terms
// (FieldCompute.cpp:99-148): E * exp(-j k L) / L, k L in FP64.
// fp32_phase: take the path length and the phase k*L in FP32 (only to measure
// what FP64 phase buys).
//
// kappa (optional, FP32 mode) receives the path's condition number for this
// arithmetic: the largest field the path could carry, |E_launch| times each
// interaction's largest coefficient magnitude (at least 1), over the field it
// ends with.  Rotations and coefficients each err by a few ulps of the field
// they act on, so the path's FP32 error is a few ulps of |E| times kappa
// (measured: at most 7 ulps x kappa); kappa >> 1 means the path's field is
// the small remainder of much larger terms.
template <class R, bool fp32_phase = false>
__device__ void path_combine(int n, const SegTerms* seg, const double (*pts)[3],
                             const double* const* frames, const int* kind, const double* txcs,
                             double freq, const FieldConsts& K, Cx<double>* out,
                             float* kappa = nullptr) {
  const double lam64 = 2.99792458e8 / freq;
  Cx<R> tot[3] = {cx(R(0)), cx(R(0)), cx(R(0))};
  double L = 0.0;
  float gain = 1.0f, in0 = 0.0f;
  for (int i = 0; i < n; ++i) {
    const SegTerms& t = seg[i];
    const M3<R> cur = start_frame<R>(i, frames, txcs);
    L += t.r;
    const R st = R(t.st), ct = R(t.ct), sp = R(t.sp), cp = R(t.cp);
    // TransformationMatrix(theta, phi, sph2Cart=true), VecMatDef.h:85-99
    const M3<R> T{{st * cp, ct * cp, -sp, st * sp, ct * sp, cp, ct, -st, R(0)}};
    Cx<R> inc[3];
    if (i == 0) {
      for (int j = 0; j < 3; ++j) {
        inc[j] = cx(R(t.inc[2 * j]), R(t.inc[2 * j + 1]));
        in0 += float(t.inc[2 * j] * t.inc[2 * j] + t.inc[2 * j + 1] * t.inc[2 * j + 1]);
      }
    } else {
      Cx<R> g[3];
      mtv(cur, tot, g);   // RotateToNewCoordSys(E, current, global) = current^T E
      mtv(T, g, inc);     // CartesianToSphericalVector = T^T
    }
    if (kind[i] != 0) {
      tot[0] = inc[0];
      tot[1] = inc[1] * cx(R(t.ctm[0]), R(t.ctm[1]));
      tot[2] = inc[2] * cx(R(t.cte[0]), R(t.cte[1]));
      if (kappa)
        gain *= fmaxf(1.0f, fmaxf(float(hypot(t.ctm[0], t.ctm[1])), float(hypot(t.cte[0], t.cte[1]))));
    } else {
      tot[0] = inc[0];
      tot[1] = inc[1];
      tot[2] = inc[2];
    }
    Cx<R> c[3];
    mcv(T, tot, c);     // SphericalToCartesianVector = T
    mtv(cur, c, tot);   // back to global: current^T
  }
  if (kappa) {
    float o = 0.0f;
    for (int j = 0; j < 3; ++j) o += float(tot[j].re) * float(tot[j].re) + float(tot[j].im) * float(tot[j].im);
    *kappa = o > 0.0f ? gain * sqrtf(in0) / sqrtf(o) : INFINITY;
  }
  // E * exp(-j k L) / L with k L in FP64 and reduced mod 2 pi before sin/cos
  if (fp32_phase) {
    const float k32 = float((2.0 * K.pi_hi) / lam64);
    float L32 = 0.0f;
    for (int i = 0; i < n; ++i) {
      const float dx = float(pts[i + 1][0] - pts[i][0]), dy = float(pts[i + 1][1] - pts[i][1]),
                  dz = float(pts[i + 1][2] - pts[i][2]);
      L32 += sqrtf(dx * dx + dy * dy + dz * dz);
    }
    const float kl = k32 * L32;
    const float s = sinf(-kl), c = cosf(-kl);
    for (int j = 0; j < 3; ++j) {
      const float re = float(tot[j].re), im = float(tot[j].im);
      out[j] = Cx<double>{double((re * c - im * s) / L32), double((re * s + im * c) / L32)};
    }
    return;
  }
  const double k = (2.0 * K.pi_hi) / lam64;
  const double kl = k * L;
  const double s = sin(-kl), c = cos(-kl);
  for (int j = 0; j < 3; ++j) {
    const double re = double(tot[j].re), im = double(tot[j].im);
    out[j] = Cx<double>{(re * c - im * s) / L, (re * s + im * c) / L};
  }
}

}  // namespace sbr
