// synth.cpp — seeded synthetic telescope workloads (host code): the plane
// frames, the analytic field map, and the OpenMP loop over tracks of the
// per-track generator in kf_synth_track.h (which kf_sim.cu runs on the GPU).

#include "../../include/gb300kf_synth.h"
#include "kf_synth_track.h"

#include <cmath>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using kfs::kPi;
using kfs::kTesla;
using kfs::Rng;

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
  const bool useMap = field && (field->kind == KF_FIELD_GRID3D || field->kind == KF_FIELD_GRID_RZ);
  const bool withMaterial = cfg->material[0] > 0. && cfg->material[3] > 0.;
  if (withMaterial && useMap) return KF_ERR_UNSUPPORTED; // material truth: uniform field only
  if (useMap && !field->grid) return KF_ERR_INVALID_ARGUMENT;
  const double bz = cfg->bz_tesla * kTesla * ((field && !useMap) ? field->scale : 1.0);
  kfs::GridView gv;
  if (useMap) gv = kfs::gridView(*field);
  const kfs::TrackOut o{meas, hit_mask, n_planes, start, scov, perigee, truth};
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 256)
#endif
  for (int64_t i = 0; i < n; ++i)
    kfs::simulateTrack(*cfg, tcenter, trot, useMap ? &gv : nullptr, bz, i, n, o);
  return KF_SUCCESS;
}

} // extern "C"
