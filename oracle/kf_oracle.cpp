// kf_oracle.cpp — CPU FP64 restatement of the reference KalmanFitter hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle the CUDA fitter is checked
// against; it is never linked into the product library.  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
//
// It restates, function by function, the reference files listed below (paths
// relative to the reference project root), in plain C++17 with dense
// fixed-size matrices in place of Eigen.  The reference cannot be built here
// (it needs Eigen3, Boost and ROOT), so parity with the reference binary is
// unpinned; the restatement is pinned by known-answer tests (analytic helix,
// finite-difference Jacobians, least-squares Kalman algebra, pull widths).
//
// Extensions beyond the reference, all off or neutral by default:
//  - chi2: sum of predicted-residual chi2 r^T (V + H C H^T)^-1 r (the
//    reference leaves chi2 at 0, Fitter/GainMatrixUpdater.hpp:90-101);
//  - holes: planes without a hit are crossed without an update (as the
//    reference does when no source link matches, KalmanFitter.hpp:292-296);
//    the fit succeeds when every supplied hit produced a state;
//  - outliers: with outlier_chi2_cut > 0 a hit whose predicted chi2 exceeds
//    the cut becomes a state with filtered = predicted and no stepper update;
//  - field: constant or trilinear 3D grid, times a global scale;
//  - faithful_jacobian = 0 rebuilds jacToGlobal after each update;
//  - outliers cross their plane's material like hits do (the reference has
//    no outliers).

#include "../include/gb300kf.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <limits>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef KFO_TRACE_ON
#include <cstdio>
#define KFO_TRACE(...) std::printf(__VA_ARGS__)
#else
#define KFO_TRACE(...)
#endif

namespace kfo {

// ---------------------------------------------------------------------------
// Small dense matrices (stand-in for the Eigen fixed-size types,
// Utilities/Definitions.hpp).  Products sum k = 0..K-1 in order.
// ---------------------------------------------------------------------------
template <int R, int C> struct Mat {
  double a[R][C];
  double &operator()(int i, int j) { return a[i][j]; }
  double operator()(int i, int j) const { return a[i][j]; }
  static Mat zero() {
    Mat m;
    for (int i = 0; i < R; ++i)
      for (int j = 0; j < C; ++j) m.a[i][j] = 0.0;
    return m;
  }
  static Mat identity() {
    Mat m = zero();
    for (int i = 0; i < R && i < C; ++i) m.a[i][i] = 1.0;
    return m;
  }
};

template <int R, int K, int C>
static Mat<R, C> mul(const Mat<R, K> &A, const Mat<K, C> &B) {
  Mat<R, C> r;
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) {
      double s = 0.0;
      for (int k = 0; k < K; ++k) s += A.a[i][k] * B.a[k][j];
      r.a[i][j] = s;
    }
  return r;
}
template <int R, int C> static Mat<C, R> tr(const Mat<R, C> &A) {
  Mat<C, R> r;
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) r.a[j][i] = A.a[i][j];
  return r;
}
template <int R, int C>
static Mat<R, C> sub(const Mat<R, C> &A, const Mat<R, C> &B) {
  Mat<R, C> r;
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) r.a[i][j] = A.a[i][j] - B.a[i][j];
  return r;
}

struct V3 {
  double x[3];
  double &operator[](int i) { return x[i]; }
  double operator[](int i) const { return x[i]; }
};
static inline V3 v3(double a, double b, double c) { return V3{{a, b, c}}; }
static inline V3 operator+(const V3 &a, const V3 &b) {
  return v3(a[0] + b[0], a[1] + b[1], a[2] + b[2]);
}
static inline V3 operator-(const V3 &a, const V3 &b) {
  return v3(a[0] - b[0], a[1] - b[1], a[2] - b[2]);
}
static inline V3 operator*(double s, const V3 &a) {
  return v3(s * a[0], s * a[1], s * a[2]);
}
static inline double dot(const V3 &a, const V3 &b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
static inline V3 cross(const V3 &a, const V3 &b) {
  return v3(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
            a[0] * b[1] - a[1] * b[0]);
}
static inline double norm(const V3 &a) { return std::sqrt(dot(a, a)); }
static inline V3 normalized(const V3 &a) {
  double n = norm(a);
  return v3(a[0] / n, a[1] / n, a[2] / n);
}
// Utilities/Helpers.hpp:43-59 (phi), :90-105 (theta), :66-82 (perp)
static inline double vphi(const V3 &v) { return std::atan2(v[1], v[0]); }
static inline double vperp(const V3 &v) {
  return std::sqrt(v[0] * v[0] + v[1] * v[1]);
}
static inline double vtheta(const V3 &v) {
  return std::atan2(std::sqrt(v[0] * v[0] + v[1] * v[1]), v[2]);
}
// Utilities/Helpers.hpp:168-177: column-wise cross product of a 3x3 matrix
static Mat<3, 3> colcross(const Mat<3, 3> &m, const V3 &v) {
  Mat<3, 3> r;
  for (int j = 0; j < 3; ++j) {
    V3 c = cross(v3(m.a[0][j], m.a[1][j], m.a[2][j]), v);
    r.a[0][j] = c[0];
    r.a[1][j] = c[1];
    r.a[2][j] = c[2];
  }
  return r;
}

enum Status { kMissed = 0, kReachable = 1, kOnSurface = 2 };
struct Intersection {
  V3 position;
  double path;
  int status;
};

// ---------------------------------------------------------------------------
// Surfaces
// ---------------------------------------------------------------------------
// PlaneSurface<InfiniteBounds>: transform = rotation R (columns U, V, T) plus
// translation c (Surfaces/detail/PlaneSurface.ipp:24-46).
struct Plane {
  V3 c;
  double R[3][3];
  // homogeneous surface material (Material.hpp, MaterialSlab.hpp): thickness
  // (mm), X0, L0 (mm), Ar, Z, molar density (mol/mm^3); thickness 0 = none
  double mat[6] = {0., 0., 0., 0., 0., 0.};
  V3 normal() const { return v3(R[0][2], R[1][2], R[2][2]); }
  // PlanarHelper::intersectionEstimate, Surfaces/detail/PlanarHelper.hpp:28-49
  Intersection intersect(const V3 &pos, const V3 &dir, double tol) const {
    V3 n = normal();
    double denom = dot(dir, n);
    if (denom != 0.0) {
      double path = dot(n, c - pos) / denom;
      int st = (path * path < tol * tol) ? kOnSurface : kReachable;
      return {pos + path * dir, path, st};
    }
    return {pos, INFINITY, kMissed};
  }
  // PlaneSurface.ipp:215-226 (the inverse transform applied as R^T (p - c))
  void globalToLocal(const V3 &pos, double loc[2]) const {
    V3 d = pos - c;
    loc[0] = R[0][0] * d[0] + R[1][0] * d[1] + R[2][0] * d[2];
    loc[1] = R[0][1] * d[0] + R[1][1] * d[1] + R[2][1] * d[2];
  }
  // PlaneSurface.ipp:206-213
  V3 localToGlobal(double l0, double l1) const {
    return v3(R[0][0] * l0 + R[0][1] * l1 + c[0],
              R[1][0] * l0 + R[1][1] * l1 + c[1],
              R[2][0] * l0 + R[2][1] * l1 + c[2]);
  }
  // PlaneSurface.ipp:122-156
  void initJacobianToGlobal(Mat<8, 6> &J, const V3 &dir) const {
    const double x = dir[0], y = dir[1], z = dir[2];
    const double cos_theta = z, sin_theta = std::sqrt(x * x + y * y);
    const double inv_sin_theta = 1. / sin_theta;
    const double cos_phi = x * inv_sin_theta, sin_phi = y * inv_sin_theta;
    for (int r = 0; r < 3; ++r) {
      J.a[r][0] = R[r][0];
      J.a[r][1] = R[r][1];
    }
    J.a[3][5] = 1;
    J.a[4][2] = (-sin_theta) * sin_phi;
    J.a[4][3] = cos_theta * cos_phi;
    J.a[5][2] = sin_theta * cos_phi;
    J.a[5][3] = cos_theta * sin_phi;
    J.a[6][3] = (-sin_theta);
    J.a[7][4] = 1;
  }
  // PlaneSurface.ipp:158-189; returns R^T in rft
  void initJacobianToLocal(Mat<6, 8> &J, const V3 &dir, double rft[3][3]) const {
    const double x = dir[0], y = dir[1], z = dir[2];
    const double cosTheta = z, sinTheta = std::sqrt(x * x + y * y);
    const double invSinTheta = 1. / sinTheta;
    const double cosPhi = x * invSinTheta, sinPhi = y * invSinTheta;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) rft[i][j] = R[j][i];
    for (int j = 0; j < 3; ++j) {
      J.a[0][j] = rft[0][j];
      J.a[1][j] = rft[1][j];
    }
    J.a[5][3] = 1;
    J.a[2][4] = -sinPhi * invSinTheta;
    J.a[2][5] = cosPhi * invSinTheta;
    J.a[3][4] = cosPhi * cosTheta;
    J.a[3][5] = sinPhi * cosTheta;
    J.a[3][6] = -sinTheta;
    J.a[4][7] = 1;
  }
  // PlaneSurface.ipp:191-204
  Mat<1, 6> derivativeFactors(const V3 &dir, const double rft[3][3],
                              const Mat<8, 6> &J) const {
    double nv[3] = {rft[2][0], rft[2][1], rft[2][2]};
    const double dp = nv[0] * dir[0] + nv[1] * dir[1] + nv[2] * dir[2];
    for (int i = 0; i < 3; ++i) nv[i] /= dp;
    Mat<1, 6> s;
    for (int j = 0; j < 6; ++j)
      s.a[0][j] = nv[0] * J.a[0][j] + nv[1] * J.a[1][j] + nv[2] * J.a[2][j];
    return s;
  }
};

// LineSurface built from a point (translation only, axis z),
// Surfaces/detail/LineSurface.ipp:19-21.
struct Line {
  V3 c;
  // LineSurface.ipp:46-61 (line direction = z)
  void referenceFrame(const V3 &mom, double F[3][3]) const {
    V3 measY = v3(0, 0, 1);
    V3 measX = normalized(cross(measY, mom));
    V3 measD = cross(measX, measY);
    for (int r = 0; r < 3; ++r) {
      F[r][0] = measX[r];
      F[r][1] = measY[r];
      F[r][2] = measD[r];
    }
  }
  // LineSurface.ipp:229-262
  Intersection intersect(const V3 &ma, const V3 &ea, double tol) const {
    V3 mb = c, eb = v3(0, 0, 1);
    V3 mab = mb - ma;
    double eaTeb = dot(ea, eb);
    double denom = 1 - eaTeb * eaTeb;
    if (denom * denom > tol * tol) {
      double u = (dot(mab, ea) - dot(mab, eb) * eaTeb) / denom;
      int st = (u * u < tol * tol) ? kOnSurface : kReachable;
      return {ma + u * ea, u, st};
    }
    return {ma, DBL_MAX, kMissed};
  }
  // LineSurface.ipp:184-198
  V3 localToGlobal(double l0, double l1, const V3 &mom) const {
    V3 radius = cross(v3(0, 0, 1), mom);
    V3 locZ = v3(c[0], c[1], l1 + c[2]);
    return locZ + l0 * normalized(radius);
  }
  // LineSurface.ipp:200-220
  void globalToLocal(const V3 &pos, const V3 &mom, double loc[2]) const {
    V3 l3 = pos - c;
    loc[0] = vperp(l3);
    loc[1] = l3[2];
    V3 dec = pos - c;
    double sign = (dot(cross(v3(0, 0, 1), mom), dec) < 0.) ? -1. : 1.;
    loc[0] *= sign;
  }
  // LineSurface.ipp:63-112
  void initJacobianToGlobal(Mat<8, 6> &J, const V3 &dir,
                            const double pars[6]) const {
    const double x = dir[0], y = dir[1], z = dir[2];
    const double cos_theta = z, sin_theta = std::sqrt(x * x + y * y);
    const double inv_sin_theta = 1. / sin_theta;
    const double cos_phi = x * inv_sin_theta, sin_phi = y * inv_sin_theta;
    double F[3][3];
    referenceFrame(dir, F);
    for (int r = 0; r < 3; ++r) {
      J.a[r][0] = F[r][0];
      J.a[r][1] = F[r][1];
    }
    J.a[3][5] = 1;
    J.a[4][2] = (-sin_theta) * sin_phi;
    J.a[4][3] = cos_theta * cos_phi;
    J.a[5][2] = sin_theta * cos_phi;
    J.a[5][3] = cos_theta * sin_phi;
    J.a[6][3] = (-sin_theta);
    J.a[7][4] = 1;
    const double ipdn = 1. / (dir[0] * F[0][2] + dir[1] * F[1][2] + dir[2] * F[2][2]);
    V3 Y = v3(F[0][1], F[1][1], F[2][1]);
    V3 X = v3(F[0][0], F[1][0], F[2][0]);
    V3 dDPhiY = cross(Y, v3(J.a[4][2], J.a[5][2], J.a[6][2]));
    V3 dDThetaY = cross(Y, v3(J.a[4][3], J.a[5][3], J.a[6][3]));
    dDPhiY = dDPhiY - dot(X, dDPhiY) * X;
    dDThetaY = dDThetaY - dot(X, dDThetaY) * X;
    for (int r = 0; r < 3; ++r) {
      J.a[r][2] = dDPhiY[r] * pars[0] * ipdn;
      J.a[r][3] = dDThetaY[r] * pars[0] * ipdn;
    }
  }
  // LineSurface.ipp:114-143
  void initJacobianToLocal(Mat<6, 8> &J, const V3 &dir, double rft[3][3]) const {
    const double x = dir[0], y = dir[1], z = dir[2];
    const double cosTheta = z, sinTheta = std::sqrt(x * x + y * y);
    const double invSinTheta = 1. / sinTheta;
    const double cosPhi = x * invSinTheta, sinPhi = y * invSinTheta;
    double F[3][3];
    referenceFrame(dir, F);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) rft[i][j] = F[j][i];
    for (int j = 0; j < 3; ++j) {
      J.a[0][j] = rft[0][j];
      J.a[1][j] = rft[1][j];
    }
    J.a[5][3] = 1;
    J.a[2][4] = -sinPhi * invSinTheta;
    J.a[2][5] = cosPhi * invSinTheta;
    J.a[3][4] = cosPhi * cosTheta;
    J.a[3][5] = sinPhi * cosTheta;
    J.a[3][6] = -sinTheta;
    J.a[4][7] = 1;
  }
  // LineSurface.ipp:145-182
  Mat<1, 6> derivativeFactors(const V3 &pos, const V3 &dir,
                              const double rft[3][3], const Mat<8, 6> &J) const {
    V3 pc = pos - c;
    V3 locz = v3(rft[1][0], rft[1][1], rft[1][2]);
    double long_c = dot(locz, dir);
    V3 nv = dir - long_c * locz;
    double s_vec[6], d_row[6];
    for (int j = 0; j < 6; ++j)
      s_vec[j] = nv[0] * J.a[0][j] + nv[1] * J.a[1][j] + nv[2] * J.a[2][j];
    double nrm = 1. / (1. - long_c * long_c);
    // diffMatrix = long_mat * diag(s_vec) - J[4:7, :]; row_vec = pc * diffMatrix
    for (int j = 0; j < 6; ++j) {
      double d0 = locz[0] * s_vec[j] - J.a[4][j];
      double d1 = locz[1] * s_vec[j] - J.a[5][j];
      double d2 = locz[2] * s_vec[j] - J.a[6][j];
      d_row[j] = pc[0] * d0 + pc[1] * d1 + pc[2] * d2;
    }
    Mat<1, 6> r;
    for (int j = 0; j < 6; ++j) r.a[0][j] = nrm * (s_vec[j] - d_row[j]);
    return r;
  }
};

// ---------------------------------------------------------------------------
// Coordinate transformations, EventData/detail/coordinate_transformations.hpp
// ---------------------------------------------------------------------------
// :65-76
static V3 parameters2globalMomentum(const double pars[6]) {
  double p = std::fabs(1. / pars[4]);
  double phi = pars[2], theta = pars[3];
  return v3(p * std::sin(theta) * std::cos(phi),
            p * std::sin(theta) * std::sin(phi), p * std::cos(theta));
}
// Utilities/UnitVectors.hpp:50-58
static V3 dirFromPhiTheta(double phi, double theta) {
  const double cosTheta = std::cos(theta), sinTheta = std::sin(theta);
  return v3(std::cos(phi) * sinTheta, std::sin(phi) * sinTheta, cosTheta);
}

// ---------------------------------------------------------------------------
// Magnetic field
// ---------------------------------------------------------------------------
struct Field {
  int kind;
  double value[3];
  double scale;
  int n[3];
  double mn[3], mx[3];
  const float *grid; // host pointer for the oracle
  // Test/Helper.hpp:17-22 (constant) or the trilinear interpolation of
  // MagneticField/InterpolatedBFieldMap.hpp:178-181 with
  // Utilities/detail/interpolation_impl.hpp (equidistant axes; positions
  // outside the grid use the boundary cell).
  V3 get(const V3 &p) const {
    if (kind == KF_FIELD_CONSTANT)
      return v3(value[0] * scale, value[1] * scale, value[2] * scale);
    if (kind == KF_FIELD_GRID_RZ) return getRZ(p);
    int idx[3];
    double f[3];
    for (int a = 0; a < 3; ++a) {
      const double w = (mx[a] - mn[a]) / (n[a] - 1);
      double g = (p[a] - mn[a]) / w;
      int i = (int)std::floor(g);
      i = std::min(std::max(i, 0), n[a] - 2);
      idx[a] = i;
      f[a] = g - i;
    }
    double out[3];
    for (int comp = 0; comp < 3; ++comp) {
      auto at = [&](int dx, int dy, int dz) {
        size_t k = ((size_t)(idx[2] + dz) * n[1] + (idx[1] + dy)) * n[0] +
                   (idx[0] + dx);
        return (double)grid[4 * k + comp];
      };
      double c00 = at(0, 0, 0) * (1 - f[0]) + at(1, 0, 0) * f[0];
      double c10 = at(0, 1, 0) * (1 - f[0]) + at(1, 1, 0) * f[0];
      double c01 = at(0, 0, 1) * (1 - f[0]) + at(1, 0, 1) * f[0];
      double c11 = at(0, 1, 1) * (1 - f[0]) + at(1, 1, 1) * f[0];
      double c0 = c00 * (1 - f[1]) + c10 * f[1];
      double c1 = c01 * (1 - f[1]) + c11 * f[1];
      out[comp] = (c0 * (1 - f[2]) + c1 * f[2]) * scale;
    }
    return v3(out[0], out[1], out[2]);
  }
  // An (r, z) map (src/MagneticField/BFieldMapUtils.cpp:17-136): the
  // position goes to (perp(pos), z) (transformPos, :97-99), the grid of
  // (br, bz) is interpolated in its cell (in r, then in z; positions outside
  // the grid use the boundary cell), and (br, bz) goes back to
  // (br cos phi, br sin phi, bz) with cos phi = x / r, sin phi = y / r, or
  // phi = 0 on the axis (transformBField, :103-116).
  V3 getRZ(const V3 &p) const {
    const double r2 = p[0] * p[0] + p[1] * p[1];
    const double q[2] = {std::sqrt(r2), p[2]};
    const int ax[2] = {0, 2};
    int idx[2];
    double f[2];
    for (int a = 0; a < 2; ++a) {
      const int k = ax[a];
      const double w = (mx[k] - mn[k]) / (n[k] - 1);
      const double g = (q[a] - mn[k]) / w;
      int i = (int)std::floor(g);
      i = std::min(std::max(i, 0), n[k] - 2);
      idx[a] = i;
      f[a] = g - i;
    }
    double v[2];
    for (int comp = 0; comp < 2; ++comp) {
      auto at = [&](int dr, int dz) {
        const size_t k = (size_t)(idx[1] + dz) * n[0] + (idx[0] + dr);
        return (double)grid[4 * k + comp];
      };
      const double c0 = at(0, 0) * (1 - f[0]) + at(1, 0) * f[0];
      const double c1 = at(0, 1) * (1 - f[0]) + at(1, 1) * f[0];
      v[comp] = (c0 * (1 - f[1]) + c1 * f[1]) * scale;
    }
    double cphi = 1., sphi = 0.;
    if (r2 > std::numeric_limits<double>::min()) {
      const double inv = 1. / std::sqrt(r2);
      cphi = p[0] * inv;
      sphi = p[1] * inv;
    }
    return v3(v[0] * cphi, v[0] * sphi, v[1]);
  }
};

// ---------------------------------------------------------------------------
// ConstrainedStep, Propagator/ConstrainedStep.hpp:22-108
// ---------------------------------------------------------------------------
enum { kAccuracy = 0, kActor = 1, kAborter = 2, kUser = 3 };
struct CStep {
  double v[4];
  int dir;
  explicit CStep(double value = DBL_MAX) {
    dir = value > 0. ? 1 : -1;
    v[0] = DBL_MAX * dir;
    v[1] = DBL_MAX * dir;
    v[2] = DBL_MAX * dir;
    v[3] = value;
  }
  double mx() const {
    double m = -DBL_MAX;
    for (int i = 0; i < 4; ++i)
      if (v[i] > m) m = v[i];
    return m;
  }
  double mn() const {
    double m = DBL_MAX;
    for (int i = 0; i < 4; ++i)
      if (v[i] < m) m = v[i];
    return m;
  }
  void release(int t) { v[t] = (dir == 1) ? mx() : mn(); }
  void update(double value, int t, bool rel = false) {
    if (rel) release(t);
    double cv = v[t];
    v[t] = std::fabs(cv) < std::fabs(value) ? cv : value;
  }
  void assign(double value) {
    v[kAccuracy] = value;
    dir = value > 0. ? 1 : -1;
  }
  double value() const { return dir == 1 ? mn() : mx(); }
};

// ---------------------------------------------------------------------------
// Stepper state, Propagator/EigenStepper.hpp:27-120
// ---------------------------------------------------------------------------
struct Stepper {
  V3 pos, dir;
  double p;
  int q;
  double t;
  int navDir;
  Mat<6, 6> jacobian;
  Mat<8, 6> jacToGlobal;
  Mat<8, 8> jacTransport;
  double derivative[8];
  Mat<6, 6> cov;
  double pathAccumulated;
  CStep stepSize;
};

struct TrackState {
  int plane;
  double pred[6], filt[6], smth[6];
  Mat<6, 6> predCov, filtCov, smthCov, jac;
  double pathLength;
};

struct Opts {
  int maxSteps, maxTrials, smoothing, faithful;
  double tol, cutoff, mass, overstep, surfTol, outlierCut;
  int materialEffects; // bit 0 multiple scattering, bit 1 energy loss
};

// ---------------------------------------------------------------------------
// Material effects at a surface (Material/detail/Interactions.ipp with
// Propagator/detail/PointwiseMaterialInteraction.hpp/.ipp), for a heavy
// (non-electron) particle.  Constants as the reference's double build sees
// them: literals written as floats there (0.038f, 0.9f) keep their float
// values.
// ---------------------------------------------------------------------------
namespace mat {
const double kMe = 0.5109989461e-3;       // electron mass (GeV), Interactions.ipp:21
const double kK = 0.307075e-3 * 10. * 10.; // Bethe prefactor K (GeV mm^2/mol), :23
const double kPlasma = 28.816e-9;          // plasma energy scale (GeV), :25

// RelativisticQuantities, Interactions.ipp:28-49
struct Rel {
  double q2OverBeta2, beta2, betaGamma, gamma;
  Rel(double m, double qop, double q) {
    q2OverBeta2 = q * q + (m * qop) * (m * qop);
    const double mOverP = m * std::fabs(qop / q);
    const double pOverM = 1.0 / mOverP;
    beta2 = 1.0 / (1.0 + mOverP * mOverP);
    betaGamma = pOverM;
    gamma = std::sqrt(1.0 + pOverM * pOverM);
  }
};
// Material::meanExcitationEnergy, Material.ipp (16 eV Z^0.9, exponent a float)
inline double meanExcitation(double Z) { return 16e-9 * std::pow(Z, (double)0.9f); }
// computeEpsilon, Interactions.ipp:101-106
inline double epsilon(double Ne, double thickness, const Rel &r) {
  return 0.5 * kK * Ne * thickness * r.q2OverBeta2;
}
// computeEnergyLossBethe, Interactions.ipp:150-176 (with computeMassTerm,
// computeWMax, computeDeltaHalf, :58-131)
inline double betheLoss(double thickness, double Z, double molarRho, double m, double qop,
                        double q) {
  const double I = meanExcitation(Z);
  const double Ne = Z * molarRho;
  const Rel r(m, qop, q);
  const double eps = epsilon(Ne, thickness, r);
  double dhalf = 0.;
  if (!(r.betaGamma < 10.0))
    dhalf = std::log(r.betaGamma) + std::log(kPlasma * std::sqrt(Ne) / I) - 0.5;
  const double u = 2 * kMe * r.betaGamma * r.betaGamma;
  const double mfrac = kMe / m;
  const double wmax = (2 * kMe * r.betaGamma * r.betaGamma) /
                      (1.0 + 2 * r.gamma * mfrac + mfrac * mfrac);
  const double running = 0.5 * std::log(u / I) + 0.5 * std::log(wmax / I) - r.beta2 - dhalf;
  return eps * running;
}
// computeEnergyLossLandauSigmaQOverP, Interactions.ipp:316-345
inline double landauSigmaQop(double thickness, double Z, double molarRho, double m, double qop,
                             double q) {
  const Rel r(m, qop, q);
  const double fwhm = 4 * epsilon(Z * molarRho, thickness, r);
  const double sigmaE = fwhm / (2 * std::sqrt(2 * std::log(2.0)));
  const double pInv = qop / q;
  return std::sqrt(r.q2OverBeta2) * pInv * pInv * sigmaE;
}
// computeMultipleScatteringTheta0 with theta0Highland, Interactions.ipp:495-546
inline double highlandTheta0(double xOverX0, double m, double qop, double q) {
  const double momentumInv = std::fabs(qop / q);
  const double q2OverBeta2 = Rel(m, qop, q).q2OverBeta2;
  const double t = std::sqrt(xOverX0 * q2OverBeta2);
  return 13.6e-3 * momentumInv * t * (1.0 + (double)0.038f * 2 * std::log(t));
}
} // namespace mat

// KalmanFitter::Actor::materialInteractor (KalmanFitter.hpp:405-449) after a
// measurement state, forward direction, full update stage: the slab scaled by
// the path correction 1/|n.d| (PlaneSurface.ipp:229-235, MaterialSlab.ipp),
// mean Bethe energy loss, Highland scattering into the phi and theta
// variances, Landau width into the q/p variance (PointwiseMaterialInteraction
// .ipp:14-51, .hpp updateState)
static void materialInteraction(Stepper &s, const Plane &pl, const Opts &o) {
  const double t0 = pl.mat[0], X0 = pl.mat[1], Ar = pl.mat[3], Z = pl.mat[4], rho = pl.mat[5];
  if (!(o.materialEffects & 3) || !(0.0 < Ar) || !(0.0 < t0)) return;
  const double eps = 2 * DBL_EPSILON;
  const double pc = 1. / std::fabs(dot(pl.normal(), s.dir));
  const double thickness = t0 * pc;
  const double xOverX0 = ((eps < X0) ? (t0 / X0) : 0.) * pc;
  const double q = s.q, qop = q / s.p, m = o.mass;
  double eloss = 0., varPhi = 0., varTheta = 0., varQop = 0.;
  if (o.materialEffects & 2) eloss = mat::betheLoss(thickness, Z, rho, m, qop, q);
  if (o.materialEffects & 1) {
    const double th0 = mat::highlandTheta0(xOverX0, m, qop, q);
    const double perp = std::sqrt(s.dir[0] * s.dir[0] + s.dir[1] * s.dir[1]);
    const double sigmaPhi = th0 * (norm(s.dir) / perp);
    varPhi = sigmaPhi * sigmaPhi;
    varTheta = th0 * th0;
  }
  if (o.materialEffects & 2) {
    const double sq = mat::landauSigmaQop(thickness, Z, rho, m, qop, q);
    varQop = sq * sq;
  }
  const double nextE = std::sqrt(m * m + s.p * s.p) - std::copysign(eloss, 1.);
  s.p = (m < nextE) ? std::sqrt(nextE * nextE - m * m) : 0;
  s.cov.a[2][2] = std::max(0., s.cov.a[2][2] + varPhi);
  s.cov.a[3][3] = std::max(0., s.cov.a[3][3] + varTheta);
  s.cov.a[4][4] = std::max(0., s.cov.a[4][4] + varQop);
}

struct Counters {
  long steps = 0;  // accepted RK steps
  long trials = 0; // RK4 stage evaluations (tryRungeKuttaStep calls)
};

// ---------------------------------------------------------------------------
// EigenStepper::step, Propagator/EigenStepper.ipp:226-332 with evaluatek
// (:18-33), propagationTime (:36-47) and transportMatrix (:50-124).
// ---------------------------------------------------------------------------
static bool step(Stepper &s, const Field &B, const Opts &o, Counters &cnt) {
  V3 Bf, Bm, Bl, k1, k2, k3, k4;
  double err = 0.;
  const double qop = s.q / s.p;
  Bf = B.get(s.pos);
  k1 = qop * cross(s.dir, Bf);
  auto tryStep = [&](double h) -> bool {
    cnt.trials++;
    const double h2 = h * h, half_h = h * 0.5;
    V3 pos1 = s.pos + half_h * s.dir + (h2 * 0.125) * k1;
    Bm = B.get(pos1);
    k2 = qop * cross(s.dir + half_h * k1, Bm);
    k3 = qop * cross(s.dir + half_h * k2, Bm);
    V3 pos2 = s.pos + h * s.dir + (h2 * 0.5) * k3;
    Bl = B.get(pos2);
    k4 = qop * cross(s.dir + h * k3, Bl);
    V3 d = k1 - k2 - k3 + k4;
    err = std::max(h2 * (std::fabs(d[0]) + std::fabs(d[1]) + std::fabs(d[2])),
                   1e-20);
    return err <= o.tol;
  };
  long nTrials = 0;
  while (!tryStep(s.stepSize.value())) {
    double scale = std::min(
        std::max(0.25, std::pow(o.tol / std::fabs(2. * err), 0.25)), 4.);
    s.stepSize.assign(s.stepSize.value() * scale);
    double hh = s.stepSize.value();
    if (hh * hh < o.cutoff * o.cutoff) return false;
    if (nTrials > o.maxTrials) return false;
    nTrials++;
  }
  const double h = s.stepSize.value();
  // propagationTime
  const double dtds = std::hypot(1., o.mass / s.p);
  s.t += h * dtds;
  s.derivative[3] = dtds;
  // transportMatrix
  {
    Mat<8, 8> D = Mat<8, 8>::identity();
    const V3 dir = s.dir;
    const double half_h = h * 0.5;
    V3 dk1dL = cross(dir, Bf);
    V3 dk2dL = cross(dir + half_h * k1, Bm) + (qop * half_h) * cross(dk1dL, Bm);
    V3 dk3dL = cross(dir + half_h * k2, Bm) + (qop * half_h) * cross(dk2dL, Bm);
    V3 dk4dL = cross(dir + h * k3, Bl) + (qop * h) * cross(dk3dL, Bl);
    Mat<3, 3> dk1dT = Mat<3, 3>::zero();
    dk1dT.a[0][1] = Bf[2];
    dk1dT.a[0][2] = -Bf[1];
    dk1dT.a[1][0] = -Bf[2];
    dk1dT.a[1][2] = Bf[0];
    dk1dT.a[2][0] = Bf[1];
    dk1dT.a[2][1] = -Bf[0];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) dk1dT.a[i][j] *= qop;
    auto next = [&](const Mat<3, 3> &prev, double hh, const V3 &Bx) {
      Mat<3, 3> m = Mat<3, 3>::identity();
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) m.a[i][j] += hh * prev.a[i][j];
      m = colcross(m, Bx);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) m.a[i][j] = qop * m.a[i][j];
      return m;
    };
    Mat<3, 3> dk2dT = next(dk1dT, half_h, Bm);
    Mat<3, 3> dk3dT = next(dk2dT, half_h, Bm);
    Mat<3, 3> dk4dT = next(dk3dT, h, Bl);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double v = (i == j) ? 1. : 0.;
        v += h / 6. * (dk1dT.a[i][j] + dk2dT.a[i][j] + dk3dT.a[i][j]);
        D.a[i][4 + j] = v * h;
        D.a[4 + i][4 + j] +=
            h / 6. *
            (dk1dT.a[i][j] + 2. * (dk2dT.a[i][j] + dk3dT.a[i][j]) + dk4dT.a[i][j]);
      }
    for (int i = 0; i < 3; ++i) {
      D.a[i][7] = (h * h) / 6. * (dk1dL[i] + dk2dL[i] + dk3dL[i]);
      D.a[4 + i][7] = h / 6. * (dk1dL[i] + 2. * (dk2dL[i] + dk3dL[i]) + dk4dL[i]);
    }
    D.a[3][7] = h * o.mass * o.mass * s.q / (s.p * std::hypot(1., o.mass / s.p));
    s.jacTransport = mul(D, s.jacTransport);
  }
  s.pos = s.pos + (h * s.dir + (h * h / 6.) * (k1 + k2 + k3));
  s.dir = s.dir + (h / 6.) * (k1 + 2. * (k2 + k3) + k4);
  {
    double n = norm(s.dir);
    s.dir = v3(s.dir[0] / n, s.dir[1] / n, s.dir[2] / n);
  }
  s.derivative[0] = s.dir[0];
  s.derivative[1] = s.dir[1];
  s.derivative[2] = s.dir[2];
  s.derivative[4] = k4[0];
  s.derivative[5] = k4[1];
  s.derivative[6] = k4[2];
  s.pathAccumulated += h;
  cnt.steps++;
  return true;
}

// ---------------------------------------------------------------------------
// Covariance transport to a surface and re-initialisation of the Jacobians,
// Propagator/detail/CovarianceEngine.hpp:106-125, :169-201, :269-290,
// followed by the BoundParameters construction of :345-371 through
// global2parameters (coordinate_transformations.hpp:115-128).
// ---------------------------------------------------------------------------
static void reinitPlane(Stepper &s, const Plane &pl) {
  // CovarianceEngine.hpp:169-201.  initJacobianToGlobal of a plane uses only
  // the direction, so the local position and angles computed there are not
  // needed for the result.
  s.jacTransport = Mat<8, 8>::identity();
  for (int i = 0; i < 8; ++i) s.derivative[i] = 0.;
  s.jacToGlobal = Mat<8, 6>::zero();
  pl.initJacobianToGlobal(s.jacToGlobal, s.dir);
}

static void boundStatePlane(Stepper &s, const Plane &pl, double out[6],
                            Mat<6, 6> &outCov) {
  const double qopF = s.q / s.p;
  s.jacToGlobal = mul(s.jacTransport, s.jacToGlobal);
  Mat<6, 8> jacToLocal = Mat<6, 8>::zero();
  double rft[3][3];
  pl.initJacobianToLocal(jacToLocal, s.dir, rft);
  Mat<1, 6> sVec = pl.derivativeFactors(s.dir, rft, s.jacToGlobal);
  for (int i = 0; i < 8; ++i)
    for (int j = 0; j < 6; ++j)
      s.jacToGlobal.a[i][j] -= s.derivative[i] * sVec.a[0][j];
  s.jacobian = mul(jacToLocal, s.jacToGlobal);
  s.cov = mul(mul(s.jacobian, s.cov), tr(s.jacobian));
  reinitPlane(s, pl);
  outCov = s.cov;
  // BoundParameters(gctx, cov, position, momentum, charge, time, surface)
  const double pabs = std::fabs(1. / qopF);
  V3 mom = pabs * s.dir;
  double charge = std::copysign(1., qopF);
  double loc[2];
  pl.globalToLocal(s.pos, loc);
  out[0] = loc[0];
  out[1] = loc[1];
  out[2] = vphi(mom);
  out[3] = vtheta(mom);
  out[4] = ((std::fabs(charge) < 1e-4) ? 1. : charge) / norm(mom);
  out[5] = s.t;
}

static void boundStateLine(Stepper &s, const Line &ln, double out[6],
                           Mat<6, 6> &outCov) {
  const double qopF = s.q / s.p;
  s.jacToGlobal = mul(s.jacTransport, s.jacToGlobal);
  Mat<6, 8> jacToLocal = Mat<6, 8>::zero();
  double rft[3][3];
  ln.initJacobianToLocal(jacToLocal, s.dir, rft);
  Mat<1, 6> sVec = ln.derivativeFactors(s.pos, s.dir, rft, s.jacToGlobal);
  for (int i = 0; i < 8; ++i)
    for (int j = 0; j < 6; ++j)
      s.jacToGlobal.a[i][j] -= s.derivative[i] * sVec.a[0][j];
  s.jacobian = mul(jacToLocal, s.jacToGlobal);
  s.cov = mul(mul(s.jacobian, s.cov), tr(s.jacobian));
  // The re-initialisation that follows in the reference has no effect on
  // the returned parameters; it is skipped.
  outCov = s.cov;
  const double pabs = std::fabs(1. / qopF);
  V3 mom = pabs * s.dir;
  double charge = std::copysign(1., qopF);
  double loc[2];
  ln.globalToLocal(s.pos, mom, loc);
  out[0] = loc[0];
  out[1] = loc[1];
  out[2] = vphi(mom);
  out[3] = vtheta(mom);
  out[4] = ((std::fabs(charge) < 1e-4) ? 1. : charge) / norm(mom);
  out[5] = s.t;
}

// EigenStepper::update, EigenStepper.ipp:554-564, fed by
// boundParameters2freeParameters (coordinate_transformations.hpp:145-158)
static void stepperUpdate(Stepper &s, const Plane &pl, const double par[6],
                          const Mat<6, 6> &cov) {
  s.pos = pl.localToGlobal(par[0], par[1]);
  s.dir = normalized(dirFromPhiTheta(par[2], par[3]));
  s.p = std::fabs(1. / par[4]);
  s.t = par[5];
  s.cov = cov;
}

// ---------------------------------------------------------------------------
// 6x6 inverse: Eigen 3's fixed-size inverse (a third-party dependency of the
// reference, version not pinned) factors the matrix with partial-pivot LU
// and solves for the identity; restated here.  Used by calculateInverse,
// Utilities/Math.hpp:103-112 (host branch).
// ---------------------------------------------------------------------------
static Mat<6, 6> inverse6(const Mat<6, 6> &M) {
  double A[6][6];
  int perm[6];
  for (int i = 0; i < 6; ++i) {
    perm[i] = i;
    for (int j = 0; j < 6; ++j) A[i][j] = M.a[i][j];
  }
  for (int k = 0; k < 6; ++k) {
    int piv = k;
    double best = std::fabs(A[k][k]);
    for (int i = k + 1; i < 6; ++i)
      if (std::fabs(A[i][k]) > best) {
        best = std::fabs(A[i][k]);
        piv = i;
      }
    if (piv != k) {
      for (int j = 0; j < 6; ++j) std::swap(A[k][j], A[piv][j]);
      std::swap(perm[k], perm[piv]);
    }
    for (int i = k + 1; i < 6; ++i) {
      A[i][k] /= A[k][k];
      for (int j = k + 1; j < 6; ++j) A[i][j] -= A[i][k] * A[k][j];
    }
  }
  Mat<6, 6> inv;
  for (int col = 0; col < 6; ++col) {
    double y[6];
    for (int i = 0; i < 6; ++i) {
      double v = (perm[i] == col) ? 1. : 0.;
      for (int j = 0; j < i; ++j) v -= A[i][j] * y[j];
      y[i] = v;
    }
    for (int i = 5; i >= 0; --i) {
      double v = y[i];
      for (int j = i + 1; j < 6; ++j) v -= A[i][j] * inv.a[j][col];
      inv.a[i][col] = v / A[i][i];
    }
  }
  return inv;
}

static bool hasNaN(const Mat<6, 6> &m) {
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j)
      if (m.a[i][j] != m.a[i][j]) return true;
  return false;
}

// ---------------------------------------------------------------------------
// Smoother arithmetic type.  The default build evaluates the reference
// smoother in FP64, as the reference's double build does.  The "precise"
// build (-DKFO_SMOOTHER_DD) evaluates the same formulas in double-double
// arithmetic (about 106 significant bits): the update
// C_s = C_f - G (C_p' - C_s') G^T cancels heavily for the q/p variance, so
// FP64 evaluations of it scatter by 1e-9 to 5e-8 relative; the double-double
// evaluation is close to the formula's exact value and is the comparison
// point for the GPU.  It is built from IEEE double operations alone
// (error-free sums, Dekker's split product; the oracle is compiled without
// FMA contraction), so it gives the same bits on every host, and it runs at
// a few times the FP64 cost where a software quad would cost ten times more.
// ---------------------------------------------------------------------------
#if defined(KFO_SMOOTHER_DD)
struct DD {
  double hi = 0., lo = 0.;
  DD() = default;
  DD(double x) : hi(x), lo(0.) {}
  DD(int x) : hi((double)x), lo(0.) {}
  static DD norm(double s, double e) { // |e| <= ulp(s) / 2 afterwards
    const double h = s + e;
    DD r;
    r.hi = h;
    r.lo = e - (h - s);
    return r;
  }
  static void twoSum(double a, double b, double &s, double &e) {
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
  }
  static void split(double a, double &h, double &l) {
    const double t = 134217729.0 * a; // 2^27 + 1
    h = t - (t - a);
    l = a - h;
  }
  static void twoProd(double a, double b, double &p, double &e) {
    p = a * b;
    double ah, al, bh, bl;
    split(a, ah, al);
    split(b, bh, bl);
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl;
  }
  explicit operator double() const { return hi; }
  friend DD operator+(const DD &a, const DD &b) {
    double s, e, t, f;
    twoSum(a.hi, b.hi, s, e);
    twoSum(a.lo, b.lo, t, f);
    e += t;
    DD r = norm(s, e);
    return norm(r.hi, r.lo + f);
  }
  friend DD operator-(const DD &a) {
    DD r;
    r.hi = -a.hi;
    r.lo = -a.lo;
    return r;
  }
  friend DD operator-(const DD &a, const DD &b) { return a + (-b); }
  friend DD operator*(const DD &a, const DD &b) {
    double p, e;
    twoProd(a.hi, b.hi, p, e);
    e += a.hi * b.lo + a.lo * b.hi;
    return norm(p, e);
  }
  friend DD operator/(const DD &a, const DD &b) {
    const double q1 = a.hi / b.hi;
    DD r = a - b * DD(q1);
    const double q2 = r.hi / b.hi;
    r = r - b * DD(q2);
    const double q3 = r.hi / b.hi;
    const DD q = norm(q1, q2);
    return q + DD(q3);
  }
  DD &operator+=(const DD &b) { return *this = *this + b; }
  DD &operator-=(const DD &b) { return *this = *this - b; }
  DD &operator*=(const DD &b) { return *this = *this * b; }
  DD &operator/=(const DD &b) { return *this = *this / b; }
  friend bool operator<(const DD &a, const DD &b) {
    return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
  }
  friend bool operator>(const DD &a, const DD &b) { return b < a; }
};
typedef DD SReal;
#else
#ifndef KFO_SMOOTHER_REAL
#define KFO_SMOOTHER_REAL double
#endif
typedef KFO_SMOOTHER_REAL SReal;
#endif
struct M6 {
  SReal a[6][6];
};
static M6 toM6(const Mat<6, 6> &m) {
  M6 r;
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) r.a[i][j] = m.a[i][j];
  return r;
}
static Mat<6, 6> fromM6(const M6 &m) {
  Mat<6, 6> r;
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) r.a[i][j] = (double)m.a[i][j];
  return r;
}
static M6 mul6(const M6 &A, const M6 &B) {
  M6 r;
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      SReal v = 0;
      for (int k = 0; k < 6; ++k) v += A.a[i][k] * B.a[k][j];
      r.a[i][j] = v;
    }
  return r;
}
static M6 tr6(const M6 &A) {
  M6 r;
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) r.a[j][i] = A.a[i][j];
  return r;
}
static M6 sub6(const M6 &A, const M6 &B) {
  M6 r;
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) r.a[i][j] = A.a[i][j] - B.a[i][j];
  return r;
}
// partial-pivot LU inverse (as inverse6) in the smoother type
static M6 inverse6s(const M6 &M) {
  SReal A[6][6];
  int perm[6];
  for (int i = 0; i < 6; ++i) {
    perm[i] = i;
    for (int j = 0; j < 6; ++j) A[i][j] = M.a[i][j];
  }
  for (int k = 0; k < 6; ++k) {
    int piv = k;
    SReal best = A[k][k] < 0 ? -A[k][k] : A[k][k];
    for (int i = k + 1; i < 6; ++i) {
      SReal v = A[i][k] < 0 ? -A[i][k] : A[i][k];
      if (v > best) {
        best = v;
        piv = i;
      }
    }
    if (piv != k) {
      for (int j = 0; j < 6; ++j) std::swap(A[k][j], A[piv][j]);
      std::swap(perm[k], perm[piv]);
    }
    for (int i = k + 1; i < 6; ++i) {
      A[i][k] /= A[k][k];
      for (int j = k + 1; j < 6; ++j) A[i][j] -= A[i][k] * A[k][j];
    }
  }
  M6 inv;
  for (int col = 0; col < 6; ++col) {
    SReal y[6];
    for (int i = 0; i < 6; ++i) {
      SReal v = (perm[i] == col) ? 1 : 0;
      for (int j = 0; j < i; ++j) v -= A[i][j] * y[j];
      y[i] = v;
    }
    for (int i = 5; i >= 0; --i) {
      SReal v = y[i];
      for (int j = i + 1; j < 6; ++j) v -= A[i][j] * inv.a[j][col];
      inv.a[i][col] = v / A[i][i];
    }
  }
  return inv;
}

// ---------------------------------------------------------------------------
// The fit of one track: KalmanFitter::fit (Fitter/KalmanFitter.hpp:716-768)
// driving Propagator::propagate (Propagator/Propagator.ipp:6-96) with the
// Kalman actor (KalmanFitter.hpp:216-393), the Kalman aborter (:682-694),
// the DirectNavigator (Propagator/DirectNavigator.hpp:158-225) and the
// PathLimitReached / SurfaceReached aborters (StandardAborters.hpp:24-132).
// ---------------------------------------------------------------------------
struct TrackIn {
  int nSeq;
  uint64_t mask;
  const double *meas; // meas[k*5 + c]
  double start[6];
  Mat<6, 6> startCov;
  V3 perigee;
};
struct TrackOut {
  double params[6];
  Mat<6, 6> cov;
  double chi2;
  int status, nMeas;
  Counters cnt;
  std::vector<TrackState> states;
};

static void fitTrack(const TrackIn &in, const std::vector<Plane> &planes,
                     const Field &B, const Opts &o, TrackOut &res) {
  res.status = KF_TRACK_NOT_FITTED;
  res.chi2 = 0.;
  res.nMeas = 0;
  for (int i = 0; i < 6; ++i) res.params[i] = 0.;
  res.cov = Mat<6, 6>::zero();
  res.states.clear();

  const Line target{in.perigee};
  int nHits = 0;
  for (int k = 0; k < in.nSeq; ++k)
    if ((in.mask >> k) & 1ull) nHits++;
  bool finite = std::isfinite(in.start[4]) && in.start[4] != 0.;
  for (int i = 0; i < 6; ++i) finite = finite && std::isfinite(in.start[i]);
  if (!finite) {
    res.status = KF_TRACK_BAD_INPUT;
    return;
  }
  if (nHits == 0) {
    res.status = KF_TRACK_NO_HITS;
    return;
  }

  // ---- EigenStepper::State from BoundParameters<LineSurface>
  //      (EigenStepper.hpp:40-61, SingleBoundTrackParameters.hpp:57-71)
  Stepper s;
  {
    V3 mom = parameters2globalMomentum(in.start);
    V3 pos = target.localToGlobal(in.start[0], in.start[1], mom);
    s.pos = pos;
    s.dir = normalized(mom);
    s.p = norm(mom);
    s.q = (in.start[4] > 0) ? 1 : -1;
    s.t = in.start[5];
    s.navDir = 1;
    s.stepSize = CStep(DBL_MAX);
    s.jacobian = Mat<6, 6>::identity();
    s.jacToGlobal = Mat<8, 6>::zero();
    s.jacTransport = Mat<8, 8>::identity();
    for (int i = 0; i < 8; ++i) s.derivative[i] = 0.;
    s.cov = in.startCov;
    s.pathAccumulated = 0.;
    target.initJacobianToGlobal(s.jacToGlobal, s.dir, in.start);
  }

  // ---- navigation + actor/aborter state
  int next = 0;
  int current = -1; // -1 none, 0..nSeq-1 plane, -2 target line
  bool targetReached = false, navigationBreak = false;
  int measStates = 0;
  bool smoothed = false, finished = false, result = true;
  std::vector<TrackState> &states = res.states;
  states.reserve(nHits);

  auto updateSurfaceStatus = [&](const Plane &pl) -> int {
    // detail::updateSingleSurfaceStatus, SteppingHelper.hpp:31-65
    V3 d = (double)s.navDir * s.dir;
    Intersection I = pl.intersect(s.pos, d, o.surfTol);
    if (I.status == kOnSurface) {
      s.stepSize.release(kActor);
      return kOnSurface;
    } else if (I.status != kMissed) {
      double pLimit = s.stepSize.v[kAborter];
      double oLimit = -o.overstep;
      double cl = I.path;
      bool accept = (cl > oLimit && cl * cl < pLimit * pLimit);
      if (accept) {
        s.stepSize.update(s.navDir * cl, kActor, true);
        return kReachable;
      }
    }
    return kMissed;
  };
  auto navStatus = [&]() {
    current = -1;
    if (next != in.nSeq) {
      if (updateSurfaceStatus(planes[next]) == kOnSurface) {
        current = next;
        ++next;
        if (next != in.nSeq) s.stepSize.release(kActor);
      }
    }
  };
  auto navTarget = [&]() {
    current = -1;
    if (next != in.nSeq) {
      if (updateSurfaceStatus(planes[next]) == kMissed) ++next;
    } else {
      navigationBreak = true;
    }
  };
  auto surfaceReached = [&]() -> bool {
    // SurfaceReached::operator(), StandardAborters.hpp:88-132
    if (targetReached) return true;
    if (current == -2) {
      targetReached = true;
      return true;
    }
    V3 d = (double)s.navDir * s.dir;
    Intersection I = target.intersect(s.pos, d, o.surfTol);
    bool reached = (I.status == kOnSurface);
    double distance = I.path;
    if (reached) {
      current = -2;
      targetReached = true;
    } else {
      s.stepSize.update(s.navDir * distance, kAborter);
    }
    return reached;
  };
  auto filter = [&](int k) -> bool {
    // Actor::filter, KalmanFitter.hpp:284-350
    if (!((in.mask >> k) & 1ull)) return true;
    const Plane &pl = planes[k];
    TrackState ts;
    ts.plane = k;
    boundStatePlane(s, pl, ts.pred, ts.predCov);
    ts.jac = s.jacobian;
    ts.pathLength = s.pathAccumulated;
    // GainMatrixUpdater::operator(), GainMatrixUpdater.hpp:34-106
    const double *m = in.meas + 5 * k;
    double S00 = ts.predCov.a[0][0] + m[2], S01 = ts.predCov.a[0][1] + m[3];
    double S10 = ts.predCov.a[1][0] + m[3], S11 = ts.predCov.a[1][1] + m[4];
    double det = S00 * S11 - S01 * S10; // get2DMatrixInverse, Helpers.hpp:387-399
    double i00 = S11 / det, i01 = -S01 / det, i10 = -S10 / det, i11 = S00 / det;
    double r0 = m[0] - ts.pred[0], r1 = m[1] - ts.pred[1];
    double chi2 = r0 * (i00 * r0 + i01 * r1) + r1 * (i10 * r0 + i11 * r1);
    bool outlier = (o.outlierCut > 0. && chi2 > o.outlierCut);
    if (outlier) {
      for (int i = 0; i < 6; ++i) ts.filt[i] = ts.pred[i];
      ts.filtCov = ts.predCov;
    } else {
      double K[6][2];
      for (int i = 0; i < 6; ++i) {
        K[i][0] = ts.predCov.a[i][0] * i00 + ts.predCov.a[i][1] * i10;
        K[i][1] = ts.predCov.a[i][0] * i01 + ts.predCov.a[i][1] * i11;
      }
      for (int i = 0; i < 6; ++i) ts.filt[i] = ts.pred[i] + (K[i][0] * r0 + K[i][1] * r1);
      Mat<6, 6> C = Mat<6, 6>::identity();
      for (int i = 0; i < 6; ++i) {
        C.a[i][0] -= K[i][0];
        C.a[i][1] -= K[i][1];
      }
      ts.filtCov = mul(C, ts.predCov);
      res.chi2 += chi2;
      // filtered state into the stepper, KalmanFitter.hpp:337-342
      stepperUpdate(s, pl, ts.filt, ts.filtCov);
      if (!o.faithful) reinitPlane(s, pl);
    }
    // the material effects after the filtering, KalmanFitter.hpp:344-345
    materialInteraction(s, pl, o);
    states.push_back(ts);
    ++measStates;
    return true;
  };
  auto finalize = [&]() -> bool {
    // Actor::finalize, KalmanFitter.hpp:360-393, with
    // GainMatrixSmoother::operator(), GainMatrixSmoother.hpp:21-94
    smoothed = true;
    const int n = (int)states.size();
    TrackState *prev = &states[n - 1];
    for (int i = 0; i < 6; ++i) prev->smth[i] = prev->filt[i];
    prev->smthCov = prev->filtCov;
    SReal xsPrev[6];
    M6 csPrev = toM6(prev->smthCov);
    for (int i = 0; i < 6; ++i) xsPrev[i] = prev->smth[i];
    for (int i = n - 2; i >= 0; --i) {
      TrackState &ts = states[i];
      const M6 cf = toM6(ts.filtCov), cp = toM6(prev->predCov);
      M6 G = mul6(mul6(cf, tr6(toM6(prev->jac))), inverse6s(cp));
      if (hasNaN(fromM6(G))) return false;
      SReal dp[6], xs[6];
      for (int j = 0; j < 6; ++j) dp[j] = xsPrev[j] - (SReal)prev->pred[j];
      for (int r = 0; r < 6; ++r) {
        SReal g = 0;
        for (int j = 0; j < 6; ++j) g += G.a[r][j] * dp[j];
        xs[r] = (SReal)ts.filt[r] + g;
        ts.smth[r] = (double)xs[r];
      }
      const M6 cs = sub6(cf, mul6(mul6(G, sub6(cp, csPrev)), tr6(G)));
      ts.smthCov = fromM6(cs);
      for (int r = 0; r < 6; ++r) xsPrev[r] = xs[r];
      csPrev = cs;
      prev = &ts;
    }
    const TrackState &first = states[0];
    stepperUpdate(s, planes[first.plane], first.smth, first.smthCov);
    if (!o.faithful) reinitPlane(s, planes[first.plane]);
    s.navDir = -1;
    s.stepSize = CStep(-1 * std::fabs(DBL_MAX));
    s.pathAccumulated = 0.;
    return true;
  };
  auto actor = [&]() {
    if (current >= 0 && !smoothed && !finished) {
      if (!filter(current)) result = false;
    }
    if ((measStates == nHits || (measStates > 0 && navigationBreak)) &&
        !smoothed && !finished) {
      if (!o.smoothing) {
        finished = true;
      } else if (!finalize()) {
        result = false;
      }
    }
    if (smoothed && !finished && surfaceReached()) {
      boundStateLine(s, target, res.params, res.cov);
      finished = true;
    }
  };
  auto kalmanAborter = [&]() { return !result || finished; };
  auto pathAborter = [&]() -> bool {
    // PathLimitReached, StandardAborters.hpp:37-56
    if (targetReached) return true;
    double distance = s.navDir * std::fabs(DBL_MAX) - s.pathAccumulated;
    s.stepSize.update(distance, kAborter);
    bool limit = distance * distance < o.surfTol * o.surfTol;
    if (limit) targetReached = true;
    return limit;
  };

  // ---- Propagator::propagate, Propagator.ipp:6-96
  navStatus();
  actor();
  bool terminatedNormally = false;
  if (!kalmanAborter() && !pathAborter()) {
    navTarget();
    for (int st = 0; st < o.maxSteps; ++st) {
      KFO_TRACE("it %d ss=(%g %g %g %g) dir=%d pos=(%g %g %g) next=%d\n", st, s.stepSize.v[0],
                s.stepSize.v[1], s.stepSize.v[2], s.stepSize.v[3], s.stepSize.dir, s.pos[0],
                s.pos[1], s.pos[2], next);
      step(s, B, o, res.cnt);
      navStatus();
      actor();
      if (kalmanAborter() || pathAborter()) {
        terminatedNormally = true;
        break;
      }
      navTarget();
    }
  }
  if (!terminatedNormally) navigationBreak = true;
  actor();

  // ---- KalmanFitter::fit result, KalmanFitter.hpp:760-767
  res.nMeas = measStates;
  if (!result)
    res.status = smoothed ? KF_TRACK_SMOOTHER_NAN : KF_TRACK_MEAS_MISMATCH;
  else if (measStates != nHits)
    res.status = KF_TRACK_MEAS_MISMATCH;
  else if (!terminatedNormally)
    res.status = KF_TRACK_MAX_STEPS;
  else if (o.smoothing && !finished)
    res.status = KF_TRACK_NOT_FITTED;
  else
    res.status = KF_TRACK_OK;
}

} // namespace kfo

// ===========================================================================
// C entry points (loaded with ctypes by the tests and the CPU baseline).
// Same structure-of-arrays layout as kf_fit_batch, in host memory; the field
// grid pointer is a host pointer here.
// ===========================================================================
extern "C" {

static const int kUpper[21][2] = {{0, 0}, {0, 1}, {0, 2}, {0, 3}, {0, 4}, {0, 5},
                                  {1, 1}, {1, 2}, {1, 3}, {1, 4}, {1, 5}, {2, 2},
                                  {2, 3}, {2, 4}, {2, 5}, {3, 3}, {3, 4}, {3, 5},
                                  {4, 4}, {4, 5}, {5, 5}};

// counters: optional [2][stride] int64 (accepted steps, RK trials)
// states:   optional [n_surfaces][63][stride] per measurement state: predicted
//           parameters (6), predicted covariance upper triangle (21) and the
//           bound-to-bound Jacobian from the previous state (36, row-major)
int32_t oracle_fit(const kf_inputs_t *in, kf_outputs_t *out,
                   const kf_config_t *cfg, const kf_geometry_t *geo,
                   const kf_field_t *field, int32_t n_threads,
                   int64_t *counters, double *states) {
  using namespace kfo;
  if (!in || !out || !cfg || !geo || !field) return KF_ERR_INVALID_ARGUMENT;
  if (geo->n_planes < in->n_surfaces || in->n_surfaces > KF_MAX_PLANES)
    return KF_ERR_INVALID_ARGUMENT;
  std::vector<Plane> planes(geo->n_planes);
  for (int k = 0; k < geo->n_planes; ++k) {
    for (int r = 0; r < 3; ++r) {
      planes[k].c[r] = geo->center[3 * k + r];
      for (int c = 0; c < 3; ++c) planes[k].R[r][c] = geo->rotation[9 * k + 3 * r + c];
    }
    if (geo->material)
      for (int e = 0; e < 6; ++e) planes[k].mat[e] = geo->material[6 * k + e];
  }
  Field B;
  B.kind = field->kind;
  B.scale = field->scale;
  for (int a = 0; a < 3; ++a) {
    B.value[a] = field->value[a];
    B.mn[a] = field->min[a];
    B.mx[a] = field->max[a];
  }
  B.n[0] = field->nx;
  B.n[1] = field->ny;
  B.n[2] = field->nz;
  B.grid = field->grid;
  Opts o;
  o.maxSteps = cfg->max_steps;
  o.maxTrials = cfg->max_rk_trials;
  o.smoothing = cfg->smoothing;
  o.faithful = cfg->faithful_jacobian;
  o.tol = cfg->tolerance;
  o.cutoff = cfg->step_size_cutoff;
  o.mass = cfg->mass;
  o.overstep = cfg->overstep_limit;
  o.surfTol = cfg->on_surface_tol;
  o.outlierCut = cfg->outlier_chi2_cut;
  o.materialEffects = geo->material ? cfg->material_effects : 0;

  const int64_t n = in->n_tracks, S = in->stride;
  const int nSurf = in->n_surfaces;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel
#endif
  {
    std::vector<double> meas(5 * nSurf);
    TrackOut res;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
    for (int64_t i = 0; i < n; ++i) {
      TrackIn t;
      t.nSeq = in->n_planes ? in->n_planes[i] : nSurf;
      if (t.nSeq > nSurf) t.nSeq = nSurf;
      t.mask = in->hit_mask ? in->hit_mask[i] : ~0ull;
      for (int k = 0; k < nSurf; ++k)
        for (int c = 0; c < 5; ++c) meas[5 * k + c] = in->meas[((int64_t)k * 5 + c) * S + i];
      t.meas = meas.data();
      for (int r = 0; r < 6; ++r) t.start[r] = in->start_params[r * S + i];
      for (int e = 0; e < 21; ++e) {
        double v = in->start_cov[e * S + i];
        t.startCov.a[kUpper[e][0]][kUpper[e][1]] = v;
        t.startCov.a[kUpper[e][1]][kUpper[e][0]] = v;
      }
      for (int r = 0; r < 3; ++r) t.perigee[r] = in->perigee[r * S + i];
      res.cnt = Counters();
      fitTrack(t, planes, B, o, res);
      for (int r = 0; r < 6; ++r) out->params[r * S + i] = res.params[r];
      for (int e = 0; e < 21; ++e)
        out->cov[e * S + i] = res.cov.a[kUpper[e][0]][kUpper[e][1]];
      out->chi2[i] = res.chi2;
      out->status[i] = res.status;
      out->n_meas[i] = res.nMeas;
      if (out->n_steps) out->n_steps[i] = (int32_t)res.cnt.steps;
      if (out->n_trials) out->n_trials[i] = (int32_t)res.cnt.trials;
      if (counters) {
        counters[i] = res.cnt.steps;
        counters[S + i] = res.cnt.trials;
      }
      if (states) {
        for (int k = 0; k < nSurf; ++k)
          for (int e = 0; e < 63; ++e) states[((int64_t)k * 63 + e) * S + i] = 0.;
        for (size_t k = 0; k < res.states.size(); ++k) {
          const TrackState &ts = res.states[k];
          double *b = states + (int64_t)k * 63 * S + i;
          for (int r = 0; r < 6; ++r) b[r * S] = ts.pred[r];
          for (int e = 0; e < 21; ++e)
            b[(6 + e) * S] = ts.predCov.a[kUpper[e][0]][kUpper[e][1]];
          for (int r = 0; r < 6; ++r)
            for (int c = 0; c < 6; ++c) b[(27 + 6 * r + c) * S] = ts.jac.a[r][c];
        }
      }
      if (out->smoothed) {
        for (int k = 0; k < nSurf; ++k)
          for (int e = 0; e < 27; ++e)
            out->smoothed[((int64_t)k * 27 + e) * S + i] = 0.;
        for (size_t k = 0; k < res.states.size(); ++k) {
          const TrackState &ts = res.states[k];
          for (int r = 0; r < 6; ++r)
            out->smoothed[((int64_t)k * 27 + r) * S + i] = ts.smth[r];
          for (int e = 0; e < 21; ++e)
            out->smoothed[((int64_t)k * 27 + 6 + e) * S + i] =
                ts.smthCov.a[kUpper[e][0]][kUpper[e][1]];
        }
      }
    }
  }
  return KF_SUCCESS;
}

// one material interaction as the fit applies it (materialInteraction)
int32_t oracle_material_interaction(const double matRow[6], int32_t flags, const double normal[3],
                                    const double dir[3], double p, double q, double mass,
                                    double out[5]) {
  using namespace kfo;
  Plane pl;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) pl.R[r][c] = (c == 2) ? normal[r] : 0.;
  for (int e = 0; e < 6; ++e) pl.mat[e] = matRow[e];
  Stepper s;
  s.dir = v3(dir[0], dir[1], dir[2]);
  s.p = p;
  s.q = (int)q;
  s.cov = Mat<6, 6>::zero();
  Opts o;
  o.materialEffects = flags;
  o.mass = mass;
  if (!(flags & 3) || !(0.0 < matRow[3]) || !(0.0 < matRow[0])) return 1;
  materialInteraction(s, pl, o);
  out[0] = s.p;
  out[1] = s.cov.a[2][2];
  out[2] = s.cov.a[3][3];
  out[3] = s.cov.a[4][4];
  out[4] = std::sqrt(mass * mass + p * p) - std::sqrt(mass * mass + s.p * s.p);
  return 0;
}

// The reference's fit defaults: maxSteps 1000 and maxRungeKuttaStepTrials
// 10000 (Propagator/Propagator.hpp:76,79), the stepper tolerance 1e-4 and no
// step-size cut-off (:92,95), the muon mass it never overrides (:73), the
// 0.01 mm overstep limit (Propagator/EigenStepper.hpp:370), the 1e-4 mm
// on-surface tolerance (Utilities/Definitions.hpp:41), smoothing on
// (Fitter/KalmanFitter.hpp:89), no outlier rejection (the void outlier
// finder, Fitter/detail/VoidKalmanComponents.hpp:67-80) and the stale
// jacToGlobal after an update (Propagator/EigenStepper.ipp:554-564).
void oracle_config_default(kf_config_t *c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->precision = KF_PRECISION_FP64;
  c->max_steps = 1000;
  c->max_rk_trials = 10000;
  c->smoothing = 1;
  c->tolerance = 1e-4;
  c->step_size_cutoff = 0.;
  c->mass = 105.6583755e-3;
  c->overstep_limit = 0.01;
  c->on_surface_tol = 1e-4;
  c->outlier_chi2_cut = 0.;
  c->faithful_jacobian = 1;
  c->kernel = KF_KERNEL_AUTO;
  c->block_size = 0;
}

// one field lookup as the fit makes it (Field::get); the grid is host memory
int32_t oracle_field_value(const kf_field_t *field, const double pos[3], double out[3]) {
  using namespace kfo;
  if (!field || !pos || !out) return KF_ERR_INVALID_ARGUMENT;
  Field B;
  B.kind = field->kind;
  B.scale = field->scale;
  for (int a = 0; a < 3; ++a) {
    B.value[a] = field->value[a];
    B.mn[a] = field->min[a];
    B.mx[a] = field->max[a];
  }
  B.n[0] = field->nx;
  B.n[1] = field->ny;
  B.n[2] = field->nz;
  B.grid = field->grid;
  const V3 b = B.get(v3(pos[0], pos[1], pos[2]));
  for (int a = 0; a < 3; ++a) out[a] = b[a];
  return KF_SUCCESS;
}

int32_t oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

} // extern "C"
