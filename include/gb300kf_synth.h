/*
 * gb300kf_synth.h — seeded synthetic inputs for the fitter (host code).
 *
 * Replaces the reference driver's input production for the telescope
 * workloads: particle generation, hit simulation and smearing, and seed
 * smearing (Run/Common/Processor.hpp:40-253, Run/GPU/KalmanFitterGPUTest.cu:
 * 245-354).  Truth hits come from the exact helix in a uniform field, or from
 * a fine fixed-step RK4 in a field map; they do not use the fitter's
 * propagator.  Each track draws from its own counter-based random stream, so
 * the output does not depend on the number of host threads.
 */
#ifndef GB300KF_SYNTH_H
#define GB300KF_SYNTH_H

#include "gb300kf.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct kf_synth_config {
  int64_t n_tracks;
  uint64_t seed;
  int32_t n_planes;        /* planes in the telescope */
  int32_t min_len, max_len;/* per-track sequence length drawn from {min..max} */
  double x_first, x_step;  /* plane k sits at x = x_first + k*x_step, normal +x */
  double bz_tesla;         /* uniform field along z (when no map is given) */
  double mass;             /* particle mass (GeV); pions 0.13957 */
  double p_min, p_max;     /* |p| uniform in [p_min, p_max] GeV */
  double phi_half;         /* phi uniform in [-phi_half, phi_half] */
  double theta_half;       /* theta uniform in pi/2 +- theta_half */
  double vertex_sigma;     /* vertex y and z Gaussian sigma (mm); x = 0 */
  double hit_sigma;        /* measurement smearing sigma per coordinate (mm) */
  double hit_prob;         /* probability that a plane on the path has a hit */
  double outlier_prob;     /* probability that a hit is an outlier */
  double outlier_shift;    /* outliers move by U(-shift, shift) per coordinate */
  double seed_loc_sigma;   /* seed smearing: loc0/loc1 (mm) */
  double seed_angle_sigma; /* seed smearing: phi/theta (rad) */
  double seed_qop_rel;     /* seed smearing: relative q/p */
  double seed_time_sigma;  /* seed smearing: time (mm of c*t) */
  double mis_shift_sigma;  /* truth-geometry misalignment: shifts (mm) */
  double mis_rot_sigma;    /* truth-geometry misalignment: rotations (rad) */
  double rk_step;          /* fixed RK4 step for field-map truth (mm) */
  double material[6];      /* every plane's material as kf_geometry_t.material
                              (thickness 0 = none); uniform-field truth only:
                              at each plane on the path the particle scatters
                              by Gaussian angles of the Highland width and
                              loses the Bethe mean energy plus a Gaussian of
                              the Landau width (the fitter's noise model) */
} kf_synth_config_t;

/* Defaults of the 10-plane uniform-field telescope workload. */
void kf_synth_config_default(kf_synth_config_t *cfg);

/* Nominal plane frames (what the fit uses) and truth frames (nominal plus
 * misalignment, what the hits come from).  Arrays: [n_planes][3] centres and
 * [n_planes][9] row-major rotations; `align_out` (may be NULL) receives the
 * applied misalignment [n_planes][6] = (dx, dy, dz, rx, ry, rz). */
int32_t kf_synth_geometry(const kf_synth_config_t *cfg, double *center,
                          double *rotation, double *truth_center,
                          double *truth_rotation, double *align_out);

/* Analytic field map sampled on a grid of n^3 points over [-half, half]^3 mm:
 * Bz = B0 (1 - 0.2 (r/1.5 m)^2) exp(-(z/3 m)^2), Br = -(r/2) dBz/dz, values in
 * GeV/(e*mm), layout [nz][ny][nx][4] (bx, by, bz, 0). */
int32_t kf_synth_field_map(double b0_tesla, int32_t n, double half,
                           float *grid_out);

/* Tracks through the truth geometry.  Output arrays follow kf_inputs_t with
 * stride n_tracks; `field` may be NULL (uniform bz_tesla) or a grid field
 * whose `grid` pointer is HOST memory.  `truth` (may be NULL) receives
 * [6][n] true perigee parameters.  Returns 0 on success. */
int32_t kf_synth_tracks(const kf_synth_config_t *cfg, const double *truth_center,
                        const double *truth_rotation, const kf_field_t *field,
                        double *meas, uint64_t *hit_mask, int32_t *n_planes,
                        double *start_params, double *start_cov,
                        double *perigee, double *truth, int32_t n_threads);

/* The same tracks generated on the GPU: one thread per track runs the
 * per-track code of kf_synth_tracks, so every random draw, hit, hole,
 * outlier and length is the host generator's, and the values agree with it
 * to the last-bit rounding of the math library.  Output arrays and
 * `field->grid` are DEVICE memory; truth_center / truth_rotation are host
 * arrays (copied into the launch).  Asynchronous on `stream` (a
 * cudaStream_t, NULL = legacy default stream); nothing is allocated. */
int32_t kf_simulate_tracks(const kf_synth_config_t *cfg, const double *truth_center,
                           const double *truth_rotation, const kf_field_t *field,
                           double *meas, uint64_t *hit_mask, int32_t *n_planes,
                           double *start_params, double *start_cov, double *perigee,
                           double *truth, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GB300KF_SYNTH_H */
