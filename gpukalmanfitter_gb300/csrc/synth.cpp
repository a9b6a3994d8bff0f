// synth.cpp — seeded synthetic telescope workloads (host code).
//
// Stands in for the reference driver's input production
// (Run/Common/Processor.hpp:40-253; Run/GPU/KalmanFitterGPUTest.cu:245-354):
// particles from a Gaussian vertex, truth hits on every plane of the
// telescope, Gaussian hit smearing, and truth seeds smeared onto a perigee
// line surface through the true vertex (Processor.hpp:121-129, :177-253).
// Distributions follow the workload definitions (pi+-, |p| in [1,10] GeV,
// phi in +-0.1, theta in pi/2 +- 0.1, 50 um hits, 50 um / 1 mrad / 5 % seeds).

#include "../../include/gb300kf_synth.h"
#include "kf_material.h"

#include <cmath>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kTesla = 0.000299792458; // GeV/(e*mm) per tesla
constexpr double kPi = 3.14159265358979323846;

// splitmix64 stream keyed by (seed, track): a counter-based generator.
struct Rng {
  uint64_t s;
  bool has = false;
  double cached = 0.;
  static uint64_t mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  Rng(uint64_t seed, uint64_t stream) {
    s = mix(seed + 0x9E3779B97F4A7C15ull) ^ mix(stream * 0xD1B54A32D192ED03ull + 1);
  }
  uint64_t next() {
    s += 0x9E3779B97F4A7C15ull;
    return mix(s);
  }
  double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
  double uniform(double a, double b) { return a + (b - a) * uniform(); }
  double normal() {
    if (has) {
      has = false;
      return cached;
    }
    double u1 = 1.0 - uniform(), u2 = uniform();
    double r = std::sqrt(-2.0 * std::log(u1));
    cached = r * std::sin(2 * kPi * u2);
    has = true;
    return r * std::cos(2 * kPi * u2);
  }
};

struct Frame {
  double c[3];
  double R[3][3]; // columns U, V, T
};

void nominalFrame(double x, Frame &f) {
  // PlaneSurface(center, normal) with normal +x (PlaneSurface.ipp:24-46):
  // T = x, U = z cross T = y, V = T cross U = z.
  f.c[0] = x;
  f.c[1] = 0;
  f.c[2] = 0;
  const double U[3] = {0, 1, 0}, V[3] = {0, 0, 1}, T[3] = {1, 0, 0};
  for (int r = 0; r < 3; ++r) {
    f.R[r][0] = U[r];
    f.R[r][1] = V[r];
    f.R[r][2] = T[r];
  }
}

void rotXYZ(double a, double b, double g, double M[3][3]) {
  // M = Rx(a) * Ry(b) * Rz(g)
  const double ca = std::cos(a), sa = std::sin(a), cb = std::cos(b),
               sb = std::sin(b), cg = std::cos(g), sg = std::sin(g);
  const double Rx[3][3] = {{1, 0, 0}, {0, ca, -sa}, {0, sa, ca}};
  const double Ry[3][3] = {{cb, 0, sb}, {0, 1, 0}, {-sb, 0, cb}};
  const double Rz[3][3] = {{cg, -sg, 0}, {sg, cg, 0}, {0, 0, 1}};
  double T[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      T[i][j] = 0;
      for (int k = 0; k < 3; ++k) T[i][j] += Ry[i][k] * Rz[k][j];
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      M[i][j] = 0;
      for (int k = 0; k < 3; ++k) M[i][j] += Rx[i][k] * T[k][j];
    }
}

struct GridField {
  const kf_field_t *f;
  void get(const double p[3], double B[3]) const {
    if (!f || f->kind == KF_FIELD_CONSTANT) return;
    const int n[3] = {f->nx, f->ny, f->nz};
    int idx[3];
    double fr[3];
    for (int a = 0; a < 3; ++a) {
      const double w = (f->max[a] - f->min[a]) / (n[a] - 1);
      double g = (p[a] - f->min[a]) / w;
      int i = (int)std::floor(g);
      if (i < 0) i = 0;
      if (i > n[a] - 2) i = n[a] - 2;
      idx[a] = i;
      fr[a] = g - i;
    }
    for (int comp = 0; comp < 3; ++comp) {
      auto at = [&](int dx, int dy, int dz) {
        size_t k = ((size_t)(idx[2] + dz) * n[1] + (idx[1] + dy)) * n[0] + (idx[0] + dx);
        return (double)f->grid[4 * k + comp];
      };
      double c00 = at(0, 0, 0) * (1 - fr[0]) + at(1, 0, 0) * fr[0];
      double c10 = at(0, 1, 0) * (1 - fr[0]) + at(1, 1, 0) * fr[0];
      double c01 = at(0, 0, 1) * (1 - fr[0]) + at(1, 0, 1) * fr[0];
      double c11 = at(0, 1, 1) * (1 - fr[0]) + at(1, 1, 1) * fr[0];
      double c0 = c00 * (1 - fr[1]) + c10 * fr[1];
      double c1 = c01 * (1 - fr[1]) + c11 * fr[1];
      B[comp] = (c0 * (1 - fr[2]) + c1 * fr[2]) * f->scale;
    }
  }
};

// Exact helix in B = (0, 0, bz) (GeV/(e*mm)): dT/ds = qop T x B.
struct Helix {
  double x0[3], st, ct, phi0, w; // w = qop * bz
  void at(double s, double r[3], double T[3]) const {
    const double half = 0.5 * w * s;
    // 2 sin(ws/2)/w, stable for small w
    const double fac = (std::fabs(half) < 1e-8) ? s : 2.0 * std::sin(half) / w;
    const double pm = phi0 - half;
    r[0] = x0[0] + st * std::cos(pm) * fac;
    r[1] = x0[1] + st * std::sin(pm) * fac;
    r[2] = x0[2] + ct * s;
    T[0] = st * std::cos(phi0 - w * s);
    T[1] = st * std::sin(phi0 - w * s);
    T[2] = ct;
  }
};

inline double dot3(const double a[3], const double b[3]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// classic RK4 step of (r, T) with dT/ds = qop T x B(r)
void rk4(const GridField &F, double qop, const double r[3], const double T[3],
         double h, double ro[3], double To[3]) {
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
  double n = std::sqrt(dot3(To, To));
  for (int i = 0; i < 3; ++i) To[i] /= n;
}

} // namespace

extern "C" {

void kf_synth_config_default(kf_synth_config_t *c) {
  std::memset(c, 0, sizeof(*c));
  c->n_tracks = 1000;
  c->seed = 1234567890ull;
  c->n_planes = 10;
  c->min_len = 10;
  c->max_len = 10;
  c->x_first = 100.;
  c->x_step = 100.;
  c->bz_tesla = 2.;
  c->mass = 0.13957;
  c->p_min = 1.;
  c->p_max = 10.;
  c->phi_half = 0.1;
  c->theta_half = 0.1;
  c->vertex_sigma = 0.020;
  c->hit_sigma = 0.050;
  c->hit_prob = 1.;
  c->outlier_prob = 0.;
  c->outlier_shift = 5.;
  c->seed_loc_sigma = 0.050;
  c->seed_angle_sigma = 0.001;
  c->seed_qop_rel = 0.05;
  c->seed_time_sigma = 5. * 299.792458; // 5 ns (Run/Common/Processor.hpp:31)
  c->mis_shift_sigma = 0.;
  c->mis_rot_sigma = 0.;
  c->rk_step = 5.;
}

int32_t kf_synth_geometry(const kf_synth_config_t *cfg, double *center,
                          double *rotation, double *tcenter, double *trotation,
                          double *align_out) {
  if (!cfg || cfg->n_planes <= 0 || cfg->n_planes > KF_MAX_PLANES) return KF_ERR_INVALID_ARGUMENT;
  Rng rng(cfg->seed ^ 0xA5A5A5A5A5A5A5A5ull, 0xFFFFFFFFull);
  for (int k = 0; k < cfg->n_planes; ++k) {
    Frame f;
    nominalFrame(cfg->x_first + k * cfg->x_step, f);
    double a[6] = {0, 0, 0, 0, 0, 0};
    if (cfg->mis_shift_sigma > 0 || cfg->mis_rot_sigma > 0) {
      for (int i = 0; i < 3; ++i) a[i] = cfg->mis_shift_sigma * rng.normal();
      for (int i = 3; i < 6; ++i) a[i] = cfg->mis_rot_sigma * rng.normal();
    }
    double M[3][3];
    rotXYZ(a[3], a[4], a[5], M);
    for (int r = 0; r < 3; ++r) {
      if (center) center[3 * k + r] = f.c[r];
      if (tcenter) tcenter[3 * k + r] = f.c[r] + a[r];
      for (int c = 0; c < 3; ++c) {
        if (rotation) rotation[9 * k + 3 * r + c] = f.R[r][c];
        double v = 0;
        for (int m = 0; m < 3; ++m) v += M[r][m] * f.R[m][c];
        if (trotation) trotation[9 * k + 3 * r + c] = v;
      }
    }
    if (align_out)
      for (int i = 0; i < 6; ++i) align_out[6 * k + i] = a[i];
  }
  return KF_SUCCESS;
}

int32_t kf_synth_field_map(double b0_tesla, int32_t n, double half, float *grid) {
  if (n < 2 || !grid) return KF_ERR_INVALID_ARGUMENT;
  const double B0 = b0_tesla * kTesla, R = 1500., Z = 3000.;
  const double w = 2 * half / (n - 1);
  for (int iz = 0; iz < n; ++iz)
    for (int iy = 0; iy < n; ++iy)
      for (int ix = 0; ix < n; ++ix) {
        const double x = -half + ix * w, y = -half + iy * w, z = -half + iz * w;
        const double r2 = x * x + y * y;
        const double bz = B0 * (1. - 0.2 * r2 / (R * R)) * std::exp(-(z / Z) * (z / Z));
        // Br = -(r/2) dBz/dz = (r z / Z^2) Bz; Bx = Br x/r, By = Br y/r
        const size_t k = ((size_t)iz * n + iy) * n + ix;
        grid[4 * k + 0] = (float)(x * z / (Z * Z) * bz);
        grid[4 * k + 1] = (float)(y * z / (Z * Z) * bz);
        grid[4 * k + 2] = (float)bz;
        grid[4 * k + 3] = 0.f;
      }
  return KF_SUCCESS;
}

int32_t kf_synth_tracks(const kf_synth_config_t *cfg, const double *tcenter,
                        const double *trot, const kf_field_t *field, double *meas,
                        uint64_t *hit_mask, int32_t *n_planes, double *start,
                        double *scov, double *perigee, double *truth,
                        int32_t n_threads) {
  if (!cfg || !tcenter || !trot || !meas || !start || !scov || !perigee)
    return KF_ERR_INVALID_ARGUMENT;
  const int64_t n = cfg->n_tracks;
  const int S = cfg->n_planes;
  if (S <= 0 || S > KF_MAX_PLANES || cfg->min_len < 1 || cfg->max_len > S ||
      cfg->min_len > cfg->max_len)
    return KF_ERR_INVALID_ARGUMENT;
  const bool useMap = field && field->kind == KF_FIELD_GRID3D;
  const bool withMaterial = cfg->material[0] > 0. && cfg->material[3] > 0.;
  if (withMaterial && useMap) return KF_ERR_UNSUPPORTED; // material truth: uniform field only
  const double bz = cfg->bz_tesla * kTesla * ((field && !useMap) ? field->scale : 1.0);
  GridField GF{field};
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 256)
#endif
  for (int64_t i = 0; i < n; ++i) {
    Rng rng(cfg->seed, (uint64_t)i);
    const double q = (rng.uniform() < 0.5) ? -1. : 1.;
    const double p = rng.uniform(cfg->p_min, cfg->p_max);
    const double phi = rng.uniform(-cfg->phi_half, cfg->phi_half);
    const double theta = rng.uniform(0.5 * kPi - cfg->theta_half, 0.5 * kPi + cfg->theta_half);
    const double vtx[3] = {0., cfg->vertex_sigma * rng.normal(), cfg->vertex_sigma * rng.normal()};
    const double qop = q / p;
    int len = cfg->min_len;
    if (cfg->max_len > cfg->min_len)
      len = cfg->min_len + (int)(rng.uniform() * (cfg->max_len - cfg->min_len + 1));
    if (len > cfg->max_len) len = cfg->max_len;
    if (n_planes) n_planes[i] = len;

    // truth hits
    uint64_t mask = 0;
    Helix hx;
    for (int a = 0; a < 3; ++a) hx.x0[a] = vtx[a];
    hx.st = std::sin(theta);
    hx.ct = std::cos(theta);
    hx.phi0 = phi;
    hx.w = qop * bz;
    double r[3] = {vtx[0], vtx[1], vtx[2]};
    double T[3] = {hx.st * std::cos(phi), hx.st * std::sin(phi), hx.ct};
    double sAcc = 0.;
    double pCur = p; // momentum along the path (changes at material)
    for (int k = 0; k < S; ++k) {
      const double *c = tcenter + 3 * k;
      const double *R = trot + 9 * k;
      const double nrm[3] = {R[2], R[5], R[8]};
      double hit[3];
      if (!useMap) {
        double s = sAcc, rr[3], TT[3];
        hx.at(s, rr, TT);
        for (int it = 0; it < 50; ++it) {
          const double d[3] = {rr[0] - c[0], rr[1] - c[1], rr[2] - c[2]};
          const double ds = -dot3(nrm, d) / dot3(nrm, TT);
          s += ds;
          hx.at(s, rr, TT);
          if (std::fabs(ds) < 1e-13) break;
        }
        sAcc = s;
        for (int a = 0; a < 3; ++a) hit[a] = rr[a];
        if (withMaterial && k < len) {
          // the plane's material: Highland scattering of the direction by two
          // Gaussian angles, Bethe mean loss plus a Gaussian of the Landau width
          kfm::Effects fx;
          const double pNow = pCur;
          kfm::interact(cfg->material, 3, nrm, TT, pNow, q, cfg->mass, fx);
          const double th0 = std::sqrt(fx.varTheta);
          // orthonormal u, v perpendicular to TT
          double u[3] = {-TT[1], TT[0], 0.};
          double un = std::sqrt(dot3(u, u));
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
          const double tn = std::sqrt(dot3(Tn, Tn));
          for (int a = 0; a < 3; ++a) Tn[a] /= tn;
          const double qop0 = q / pNow;
          const double sigE = std::sqrt(fx.varQop) * pNow * pNow /
                              std::sqrt(kfm::relativistic(cfg->mass, qop0, q).q2OverBeta2);
          const double E = std::sqrt(cfg->mass * cfg->mass + pNow * pNow) - fx.eloss -
                           sigE * rng.normal();
          const double pNew = (E > cfg->mass) ? std::sqrt(E * E - cfg->mass * cfg->mass) : 1e-3;
          // restart the helix at the hit with the new direction and momentum
          for (int a = 0; a < 3; ++a) hx.x0[a] = rr[a];
          hx.st = std::sqrt(Tn[0] * Tn[0] + Tn[1] * Tn[1]);
          hx.ct = Tn[2];
          hx.phi0 = std::atan2(Tn[1], Tn[0]);
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
          if (dist <= cfg->rk_step) break;
          double ro[3], To[3];
          rk4(GF, qop, r, T, cfg->rk_step, ro, To);
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
          rk4(GF, qop, r, T, h, ro, To);
          const double d[3] = {ro[0] - c[0], ro[1] - c[1], ro[2] - c[2]};
          const double dh = -dot3(nrm, d) / dot3(nrm, To);
          h += dh;
          if (std::fabs(dh) < 1e-13) break;
        }
        rk4(GF, qop, r, T, h, ro, To);
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
      const bool hasHit = onPath && (cfg->hit_prob >= 1. || rng.uniform() < cfg->hit_prob);
      double m0 = l0 + cfg->hit_sigma * rng.normal();
      double m1 = l1 + cfg->hit_sigma * rng.normal();
      if (hasHit && cfg->outlier_prob > 0. && rng.uniform() < cfg->outlier_prob) {
        m0 += rng.uniform(-cfg->outlier_shift, cfg->outlier_shift);
        m1 += rng.uniform(-cfg->outlier_shift, cfg->outlier_shift);
      }
      if (hasHit) mask |= (1ull << k);
      const double var = cfg->hit_sigma * cfg->hit_sigma;
      double *mk = meas + (int64_t)k * 5 * n;
      mk[0 * n + i] = hasHit ? m0 : 0.;
      mk[1 * n + i] = hasHit ? m1 : 0.;
      mk[2 * n + i] = var;
      mk[3 * n + i] = 0.;
      mk[4 * n + i] = var;
    }
    if (hit_mask) hit_mask[i] = mask;

    // perigee line through the true vertex; true perigee parameters are
    // (0, 0, phi, theta, q/p, 0)
    for (int a = 0; a < 3; ++a) perigee[a * n + i] = vtx[a];
    const double tp[6] = {0., 0., phi, theta, qop, 0.};
    if (truth)
      for (int a = 0; a < 6; ++a) truth[a * n + i] = tp[a];
    const double sl = cfg->seed_loc_sigma, sa = cfg->seed_angle_sigma,
                 sq = cfg->seed_qop_rel * std::fabs(qop), stt = cfg->seed_time_sigma;
    double sp[6];
    sp[0] = tp[0] + sl * rng.normal();
    sp[1] = tp[1] + sl * rng.normal();
    sp[2] = tp[2] + sa * rng.normal();
    sp[3] = tp[3] + sa * rng.normal();
    sp[4] = tp[4] * (1. + cfg->seed_qop_rel * rng.normal());
    sp[5] = tp[5] + stt * rng.normal();
    for (int a = 0; a < 6; ++a) start[a * n + i] = sp[a];
    const double diag[6] = {sl * sl, sl * sl, sa * sa, sa * sa, sq * sq, stt * stt};
    int e = 0;
    for (int a = 0; a < 6; ++a)
      for (int b = a; b < 6; ++b) scov[(e++) * n + i] = (a == b) ? diag[a] : 0.;
  }
  return KF_SUCCESS;
}

} // extern "C"
