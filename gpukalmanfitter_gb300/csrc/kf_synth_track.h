// kf_synth_track.h — one synthetic track of the telescope workloads, host
// and device (the host generator's OpenMP loop in synth.cpp and the
// simulation kernel in kf_sim.cu run the same code).
//
// Stands in for the reference driver's input production
// (Run/Common/Processor.hpp:40-253; Run/GPU/KalmanFitterGPUTest.cu:245-354):
// a particle from a Gaussian vertex, truth hits where it crosses the planes
// of the (possibly misaligned) telescope, Gaussian hit smearing, outliers,
// holes, and the truth smeared into a seed on the perigee line through the
// true vertex (Processor.hpp:121-129, :177-253).  The uniform field uses the
// exact helix, restarted at each plane with material (Highland scattering,
// Bethe loss plus a Gaussian of the Landau width: the fitter's noise model,
// ActsFatras' MinimalSimulator role, include/ActsFatras/Kernel/
// MinimalSimulator.hpp:57-136); a grid field uses a fine fixed-step RK4.
//
// Every track draws from its own counter-based stream (splitmix64 keyed by
// seed and track index), so the result does not depend on threads, launch
// shape or device; host and device differ only by the last-bit rounding of
// the math library (sin, cos, log), never in a draw.
#pragma once

#include <cmath>
#include <cstdint>

#include "../../include/gb300kf_synth.h"
#include "kf_material.h"

#ifdef __CUDACC__
#define KFS_HD __host__ __device__
#define KFS_HDI __host__ __device__ __forceinline__
#else
#define KFS_HD
#define KFS_HDI inline
#endif

namespace kfs {

constexpr double kTesla = 0.000299792458; // GeV/(e*mm) per tesla
constexpr double kPi = 3.14159265358979323846;

KFS_HDI void sinCos(double x, double *sn, double *cs) {
#ifdef __CUDA_ARCH__
  sincos(x, sn, cs);
#else
  *sn = sin(x);
  *cs = cos(x);
#endif
}

// splitmix64 stream keyed by (seed, track): a counter-based generator.
struct Rng {
  uint64_t s;
  bool has;
  double cached;
  KFS_HDI static uint64_t mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  KFS_HDI Rng(uint64_t seed, uint64_t stream) : has(false), cached(0.) {
    s = mix(seed + 0x9E3779B97F4A7C15ull) ^ mix(stream * 0xD1B54A32D192ED03ull + 1);
  }
  KFS_HDI uint64_t next() {
    s += 0x9E3779B97F4A7C15ull;
    return mix(s);
  }
  KFS_HDI double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
  KFS_HDI double uniform(double a, double b) { return a + (b - a) * uniform(); }
  // Box-Muller, both values used
  KFS_HDI double normal() {
    if (has) {
      has = false;
      return cached;
    }
    double u1 = 1.0 - uniform(), u2 = uniform();
    double r = sqrt(-2.0 * log(u1));
    double sn, cs;
    sinCos(2 * kPi * u2, &sn, &cs);
    cached = r * sn;
    has = true;
    return r * cs;
  }
};

// kf_field_t grid (x fastest, float4 points), trilinear, FP64 arithmetic
struct GridView {
  int n[3];
  double mn[3], mx[3], scale;
  bool rz;           // an (r, z) grid of (br, bz) (kf_field_t kind KF_FIELD_GRID_RZ)
  const float *grid; // host or device memory, matching where the code runs;
                     // 16-byte aligned (points of 4 floats)
  KFS_HDI float at(size_t point, int comp) const {
#ifdef __CUDA_ARCH__
    const float4 q = __ldg(reinterpret_cast<const float4 *>(grid) + point);
    return comp == 0 ? q.x : comp == 1 ? q.y : q.z;
#else
    return grid[4 * point + comp];
#endif
  }
  // bilinear in (r, z), br turned by the azimuth (fieldMapperRZ)
  KFS_HDI void getRZ(const double p[3], double B[3]) const {
    const double r2 = p[0] * p[0] + p[1] * p[1], r = sqrt(r2);
    const double q[2] = {r, p[2]};
    int idx[2];
    double fr[2];
    for (int a = 0; a < 2; ++a) {
      const int ax = a == 0 ? 0 : 2;
      const double w = (mx[ax] - mn[ax]) / (n[ax] - 1);
      const double g = (q[a] - mn[ax]) / w;
      int i = (int)floor(g);
      if (i < 0) i = 0;
      if (i > n[ax] - 2) i = n[ax] - 2;
      idx[a] = i;
      fr[a] = g - i;
    }
    const size_t nr = n[0], base = (size_t)idx[1] * nr + idx[0];
    double v[2];
    for (int comp = 0; comp < 2; ++comp) {
      const double c0 = (double)at(base, comp) * (1 - fr[0]) + (double)at(base + 1, comp) * fr[0];
      const double c1 =
          (double)at(base + nr, comp) * (1 - fr[0]) + (double)at(base + nr + 1, comp) * fr[0];
      v[comp] = (c0 * (1 - fr[1]) + c1 * fr[1]) * scale;
    }
    double cphi = 1.0, sphi = 0.0;
    if (r2 > 2.2250738585072014e-308) {
      cphi = p[0] / r;
      sphi = p[1] / r;
    }
    B[0] = v[0] * cphi;
    B[1] = v[0] * sphi;
    B[2] = v[1];
  }
  KFS_HDI void get(const double p[3], double B[3]) const {
    if (rz) {
      getRZ(p, B);
      return;
    }
    int idx[3];
    double fr[3];
    for (int a = 0; a < 3; ++a) {
      const double w = (mx[a] - mn[a]) / (n[a] - 1);
      double g = (p[a] - mn[a]) / w;
      int i = (int)floor(g);
      if (i < 0) i = 0;
      if (i > n[a] - 2) i = n[a] - 2;
      idx[a] = i;
      fr[a] = g - i;
    }
    // the 8 corners, each one 16-byte (bx, by, bz, 0) point
    const size_t nx = n[0], nxy = (size_t)n[0] * n[1];
    const size_t base = (size_t)idx[2] * nxy + (size_t)idx[1] * nx + idx[0];
    const size_t off[8] = {0, 1, nx, nx + 1, nxy, nxy + 1, nxy + nx, nxy + nx + 1};
    float v[8][4];
    for (int c = 0; c < 8; ++c) {
#ifdef __CUDA_ARCH__
      const float4 q = __ldg(reinterpret_cast<const float4 *>(grid) + base + off[c]);
      v[c][0] = q.x;
      v[c][1] = q.y;
      v[c][2] = q.z;
#else
      for (int comp = 0; comp < 3; ++comp) v[c][comp] = grid[4 * (base + off[c]) + comp];
#endif
    }
    for (int comp = 0; comp < 3; ++comp) {
      double c00 = (double)v[0][comp] * (1 - fr[0]) + (double)v[1][comp] * fr[0];
      double c10 = (double)v[2][comp] * (1 - fr[0]) + (double)v[3][comp] * fr[0];
      double c01 = (double)v[4][comp] * (1 - fr[0]) + (double)v[5][comp] * fr[0];
      double c11 = (double)v[6][comp] * (1 - fr[0]) + (double)v[7][comp] * fr[0];
      double c0 = c00 * (1 - fr[1]) + c10 * fr[1];
      double c1 = c01 * (1 - fr[1]) + c11 * fr[1];
      B[comp] = (c0 * (1 - fr[2]) + c1 * fr[2]) * scale;
    }
  }
};

KFS_HDI GridView gridView(const kf_field_t &f) {
  GridView g;
  g.n[0] = f.nx;
  g.n[1] = f.ny;
  g.n[2] = f.nz;
  for (int a = 0; a < 3; ++a) {
    g.mn[a] = f.min[a];
    g.mx[a] = f.max[a];
  }
  g.scale = f.scale;
  g.rz = f.kind == KF_FIELD_GRID_RZ;
  g.grid = f.grid;
  return g;
}

// Exact helix in B = (0, 0, bz) (GeV/(e*mm)): dT/ds = qop T x B.  The
// azimuth at path s is phi0 - w s; with h = w s / 2 the chord direction is
// phi0 - h and its length 2 sin(h) / w.  One sincos(h) per point: the
// angles phi0 - h and phi0 - 2h follow from (cos, sin) of phi0 and h by the
// addition and double-angle formulas.
struct Helix {
  double x0[3], st, ct, cphi0, sphi0, w; // w = qop * bz
  KFS_HDI void at(double s, double r[3], double T[3]) const {
    const double half = 0.5 * w * s;
    double sh, ch;
    sinCos(half, &sh, &ch);
    // 2 sin(ws/2)/w, stable for small w
    const double fac = (fabs(half) < 1e-8) ? s : 2.0 * sh / w;
    const double cm = cphi0 * ch + sphi0 * sh, sm = sphi0 * ch - cphi0 * sh; // phi0 - h
    const double c2 = 1.0 - 2.0 * sh * sh, s2 = 2.0 * sh * ch;                // 2h
    r[0] = x0[0] + st * cm * fac;
    r[1] = x0[1] + st * sm * fac;
    r[2] = x0[2] + ct * s;
    T[0] = st * (cphi0 * c2 + sphi0 * s2);
    T[1] = st * (sphi0 * c2 - cphi0 * s2);
    T[2] = ct;
  }
};

KFS_HDI double dot3(const double a[3], const double b[3]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// classic RK4 step of (r, T) with dT/ds = qop T x B(r)
KFS_HDI void rk4(const GridView &F, double qop, const double r[3], const double T[3], double h,
                 double ro[3], double To[3]) {
  auto deriv = [&](const double rr[3], const double TT[3], double dr[3], double dT[3]) {
    double B[3];
    F.get(rr, B);
    dr[0] = TT[0];
    dr[1] = TT[1];
    dr[2] = TT[2];
    dT[0] = qop * (TT[1] * B[2] - TT[2] * B[1]);
    dT[1] = qop * (TT[2] * B[0] - TT[0] * B[2]);
    dT[2] = qop * (TT[0] * B[1] - TT[1] * B[0]);
  };
  double k1r[3], k1T[3], k2r[3], k2T[3], k3r[3], k3T[3], k4r[3], k4T[3], rr[3], TT[3];
  deriv(r, T, k1r, k1T);
  for (int i = 0; i < 3; ++i) {
    rr[i] = r[i] + 0.5 * h * k1r[i];
    TT[i] = T[i] + 0.5 * h * k1T[i];
  }
  deriv(rr, TT, k2r, k2T);
  for (int i = 0; i < 3; ++i) {
    rr[i] = r[i] + 0.5 * h * k2r[i];
    TT[i] = T[i] + 0.5 * h * k2T[i];
  }
  deriv(rr, TT, k3r, k3T);
  for (int i = 0; i < 3; ++i) {
    rr[i] = r[i] + h * k3r[i];
    TT[i] = T[i] + h * k3T[i];
  }
  deriv(rr, TT, k4r, k4T);
  for (int i = 0; i < 3; ++i) {
    ro[i] = r[i] + h / 6. * (k1r[i] + 2 * k2r[i] + 2 * k3r[i] + k4r[i]);
    To[i] = T[i] + h / 6. * (k1T[i] + 2 * k2T[i] + 2 * k3T[i] + k4T[i]);
  }
  double nn = sqrt(dot3(To, To));
  for (int i = 0; i < 3; ++i) To[i] /= nn;
}

// Output arrays of kf_synth_tracks (stride n); truth may be NULL.
struct TrackOut {
  double *meas;
  uint64_t *hit_mask;
  int32_t *n_planes;
  double *start, *scov, *perigee, *truth;
};

// Track i of the workload `cfg` through the truth planes (tcenter [S][3],
// trot [S][9]); bz the uniform field (GeV/(e*mm)) when F is NULL.
KFS_HD inline void simulateTrack(const kf_synth_config_t &cfg, const double *tcenter,
                                 const double *trot, const GridView *F, double bz, int64_t i,
                                 int64_t n, const TrackOut &o) {
  const int S = cfg.n_planes;
  const bool useMap = F != nullptr;
  const bool withMaterial = cfg.material[0] > 0. && cfg.material[3] > 0.;
  Rng rng(cfg.seed, (uint64_t)i);
  const double q = (rng.uniform() < 0.5) ? -1. : 1.;
  const double p = rng.uniform(cfg.p_min, cfg.p_max);
  const double phi = rng.uniform(-cfg.phi_half, cfg.phi_half);
  const double theta = rng.uniform(0.5 * kPi - cfg.theta_half, 0.5 * kPi + cfg.theta_half);
  const double vtx[3] = {0., cfg.vertex_sigma * rng.normal(), cfg.vertex_sigma * rng.normal()};
  const double qop = q / p;
  int len = cfg.min_len;
  if (cfg.max_len > cfg.min_len)
    len = cfg.min_len + (int)(rng.uniform() * (cfg.max_len - cfg.min_len + 1));
  if (len > cfg.max_len) len = cfg.max_len;
  if (o.n_planes) o.n_planes[i] = len;

  // truth hits
  uint64_t mask = 0;
  Helix hx;
  for (int a = 0; a < 3; ++a) hx.x0[a] = vtx[a];
  sinCos(theta, &hx.st, &hx.ct);
  sinCos(phi, &hx.sphi0, &hx.cphi0);
  hx.w = qop * bz;
  double r[3] = {vtx[0], vtx[1], vtx[2]};
  double T[3] = {hx.st * hx.cphi0, hx.st * hx.sphi0, hx.ct};
  double sAcc = 0.;
  double pCur = p; // momentum along the path (changes at material)
  for (int k = 0; k < S; ++k) {
    const double *c = tcenter + 3 * k;
    const double *R = trot + 9 * k;
    const double nrm[3] = {R[2], R[5], R[8]};
    // Newton stops when the correction is within rounding of the plane's
    // distance from the origin (an absolute 1e-13 mm is below one ulp there
    // and would run every iteration on rounding noise)
    const double tolS = 1e-12 * (1.0 + fabs(dot3(nrm, c)));
    double hit[3];
    if (!useMap) {
      double s = sAcc, rr[3], TT[3];
      hx.at(s, rr, TT);
      for (int it = 0; it < 50; ++it) {
        const double d[3] = {rr[0] - c[0], rr[1] - c[1], rr[2] - c[2]};
        const double ds = -dot3(nrm, d) / dot3(nrm, TT);
        s += ds;
        hx.at(s, rr, TT);
        if (fabs(ds) < tolS) break;
      }
      sAcc = s;
      for (int a = 0; a < 3; ++a) hit[a] = rr[a];
      if (withMaterial && k < len) {
        // the plane's material: Highland scattering of the direction by two
        // Gaussian angles, Bethe mean loss plus a Gaussian of the Landau width
        kfm::Effects fx{};
        const double pNow = pCur;
        kfm::interact(cfg.material, 3, nrm, TT, pNow, q, cfg.mass, fx);
        const double th0 = sqrt(fx.varTheta);
        // orthonormal u, v perpendicular to TT
        double u[3] = {-TT[1], TT[0], 0.};
        double un = sqrt(dot3(u, u));
        if (un < 1e-12) {
          u[0] = 1.;
          u[1] = u[2] = 0.;
          un = 1.;
        }
        for (int a = 0; a < 3; ++a) u[a] /= un;
        const double v[3] = {TT[1] * u[2] - TT[2] * u[1], TT[2] * u[0] - TT[0] * u[2],
                             TT[0] * u[1] - TT[1] * u[0]};
        const double a1 = th0 * rng.normal(), a2 = th0 * rng.normal();
        double Tn[3];
        for (int a = 0; a < 3; ++a) Tn[a] = TT[a] + a1 * u[a] + a2 * v[a];
        const double tn = sqrt(dot3(Tn, Tn));
        for (int a = 0; a < 3; ++a) Tn[a] /= tn;
        const double qop0 = q / pNow;
        const double sigE = sqrt(fx.varQop) * pNow * pNow /
                            sqrt(kfm::relativistic(cfg.mass, qop0, q).q2OverBeta2);
        const double E =
            sqrt(cfg.mass * cfg.mass + pNow * pNow) - fx.eloss - sigE * rng.normal();
        const double pNew = (E > cfg.mass) ? sqrt(E * E - cfg.mass * cfg.mass) : 1e-3;
        // restart the helix at the hit with the new direction and momentum
        for (int a = 0; a < 3; ++a) hx.x0[a] = rr[a];
        hx.st = sqrt(Tn[0] * Tn[0] + Tn[1] * Tn[1]);
        hx.ct = Tn[2];
        hx.cphi0 = Tn[0] / hx.st;
        hx.sphi0 = Tn[1] / hx.st;
        hx.w = (q / pNew) * bz;
        pCur = pNew;
        sAcc = 0.;
      }
    } else {
      // march with fixed steps until the plane is within one step, then
      // solve for the partial step that lands on it
      for (int guard = 0; guard < 100000; ++guard) {
        const double d[3] = {r[0] - c[0], r[1] - c[1], r[2] - c[2]};
        const double dist = -dot3(nrm, d) / dot3(nrm, T);
        if (dist <= cfg.rk_step) break;
        double ro[3], To[3];
        rk4(*F, qop, r, T, cfg.rk_step, ro, To);
        for (int a = 0; a < 3; ++a) {
          r[a] = ro[a];
          T[a] = To[a];
        }
      }
      double h;
      {
        const double d[3] = {r[0] - c[0], r[1] - c[1], r[2] - c[2]};
        h = -dot3(nrm, d) / dot3(nrm, T);
      }
      double ro[3], To[3];
      for (int it = 0; it < 30; ++it) {
        rk4(*F, qop, r, T, h, ro, To);
        const double d[3] = {ro[0] - c[0], ro[1] - c[1], ro[2] - c[2]};
        const double dh = -dot3(nrm, d) / dot3(nrm, To);
        h += dh;
        if (fabs(dh) < tolS) break;
      }
      rk4(*F, qop, r, T, h, ro, To);
      for (int a = 0; a < 3; ++a) {
        r[a] = ro[a];
        T[a] = To[a];
        hit[a] = ro[a];
      }
    }
    // truth local position, R^T (hit - c)
    const double d[3] = {hit[0] - c[0], hit[1] - c[1], hit[2] - c[2]};
    double l0 = R[0] * d[0] + R[3] * d[1] + R[6] * d[2];
    double l1 = R[1] * d[0] + R[4] * d[1] + R[7] * d[2];
    const bool onPath = k < len;
    const bool hasHit = onPath && (cfg.hit_prob >= 1. || rng.uniform() < cfg.hit_prob);
    double m0 = l0 + cfg.hit_sigma * rng.normal();
    double m1 = l1 + cfg.hit_sigma * rng.normal();
    if (hasHit && cfg.outlier_prob > 0. && rng.uniform() < cfg.outlier_prob) {
      m0 += rng.uniform(-cfg.outlier_shift, cfg.outlier_shift);
      m1 += rng.uniform(-cfg.outlier_shift, cfg.outlier_shift);
    }
    if (hasHit) mask |= (1ull << k);
    const double var = cfg.hit_sigma * cfg.hit_sigma;
    double *mk = o.meas + (int64_t)k * 5 * n;
    mk[0 * n + i] = hasHit ? m0 : 0.;
    mk[1 * n + i] = hasHit ? m1 : 0.;
    mk[2 * n + i] = var;
    mk[3 * n + i] = 0.;
    mk[4 * n + i] = var;
  }
  if (o.hit_mask) o.hit_mask[i] = mask;

  // perigee line through the true vertex; true perigee parameters are
  // (0, 0, phi, theta, q/p, 0)
  for (int a = 0; a < 3; ++a) o.perigee[a * n + i] = vtx[a];
  const double tp[6] = {0., 0., phi, theta, qop, 0.};
  if (o.truth)
    for (int a = 0; a < 6; ++a) o.truth[a * n + i] = tp[a];
  const double sl = cfg.seed_loc_sigma, sa = cfg.seed_angle_sigma,
               sq = cfg.seed_qop_rel * fabs(qop), stt = cfg.seed_time_sigma;
  double sp[6];
  sp[0] = tp[0] + sl * rng.normal();
  sp[1] = tp[1] + sl * rng.normal();
  sp[2] = tp[2] + sa * rng.normal();
  sp[3] = tp[3] + sa * rng.normal();
  sp[4] = tp[4] * (1. + cfg.seed_qop_rel * rng.normal());
  sp[5] = tp[5] + stt * rng.normal();
  for (int a = 0; a < 6; ++a) o.start[a * n + i] = sp[a];
  const double diag[6] = {sl * sl, sl * sl, sa * sa, sa * sa, sq * sq, stt * stt};
  int e = 0;
  for (int a = 0; a < 6; ++a)
    for (int b = a; b < 6; ++b) o.scov[(e++) * n + i] = (a == b) ? diag[a] : 0.;
}

} // namespace kfs
