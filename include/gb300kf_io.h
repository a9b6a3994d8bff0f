/*
 * gb300kf_io.h — output files of the fit, ROOT-free (host code, no GPU).
 *
 * The reference driver's writers (Run/Common/Writer.hpp): simulated hits and
 * fitted states as Wavefront obj polylines (writeSimHitsObj :16-40,
 * writeStatesObj :42-78), the fitted perigee parameters as CSV
 * (writeParamsCsv :80-110), and the per-track truth / fit / error / residual
 * / pull record that writeParamsRoot (:112-229) fills into a ROOT tree,
 * written here as CSV with the tree's branch names as columns.
 *
 * Arrays follow kf_inputs_t / kf_outputs_t (structure of arrays, element
 * [row][i] at ptr[row * stride + i]) in host memory.  Tracks whose status is
 * not KF_TRACK_OK are skipped, as the reference skips unsuccessful fits.
 * Numbers are printed as a default-formatted C++ stream prints them (%g, six
 * significant digits), so the files match the reference's byte for byte.
 * Returns 0, KF_ERR_INVALID_ARGUMENT, or KF_ERR_IO when the file cannot be
 * opened or written (kf_last_error_string() names the file and the reason).
 */
#ifndef GB300KF_IO_H
#define GB300KF_IO_H

#include "gb300kf.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Header "trackIdx, fit_BoundLoc0, fit_BoundLoc1, fit_BoundPhi,
 * fit_BoundTheta, fit_BoundQOverP, fit_BoundTime", then "i,p0,...,p5" for
 * every fitted track i.  params = kf_outputs_t.params [6][stride]. */
int32_t kf_write_params_csv(const char *path, const double *params, const int32_t *status,
                            int64_t n_tracks, int64_t stride);

/* One polyline per fitted track through its smoothed states: "v x y z" at
 * the global position of each state on its plane (centre + loc0 U + loc1 V
 * of the fit geometry), then "l a b" joining consecutive vertices (1-based
 * obj indices, counted as the reference counts them).  smoothed =
 * kf_outputs_t.smoothed [n_surfaces][27][stride] with n_meas states per
 * track; state k lies on the plane of the k-th set bit of hit_mask (NULL:
 * on plane k). */
int32_t kf_write_states_obj(const char *path, const double *smoothed, const int32_t *n_meas,
                            const uint64_t *hit_mask, const int32_t *status, int64_t n_tracks,
                            int64_t stride, const kf_geometry_t *geo);

/* One polyline per track through its hits (every track, as writeSimHitsObj
 * writes every particle): positions [n_surfaces][3][stride] global (mm),
 * hit k of track i at the k-th set bit of hit_mask[i] (NULL: planes
 * 0..n_hits-1); n_hits [stride] (NULL: every plane of the mask, or
 * n_surfaces). */
int32_t kf_write_hits_obj(const char *path, const double *positions, const uint64_t *hit_mask,
                          const int32_t *n_hits, int32_t n_surfaces, int64_t n_tracks,
                          int64_t stride);

/* The writeParamsRoot record of every fitted track, comma separated, with
 * the header row
 *   t_charge,t_time,t_vx,t_vy,t_vz,t_px,t_py,t_pz,t_theta,t_phi,t_eta,t_pT,
 *   eLOC0_fit,eLOC1_fit,ePHI_fit,eTHETA_fit,eQOP_fit,eT_fit,
 *   err_eLOC0_fit,...,err_eT_fit, res_eLOC0,...,res_eT, pull_eLOC0,...,pull_eT
 * (no spaces).  truth [6][stride] = the true perigee parameters (loc0, loc1,
 * phi, theta, q/p, t) on the perigee line through the true vertex, vertex
 * [3][stride] = that vertex (kf_inputs_t.perigee); the particle's charge is
 * the sign of the true q/p (unit charge) and its momentum |1/(q/p)| along
 * the direction (phi, theta).  err = sqrt of the covariance diagonal, res =
 * fit - truth, pull = res / err. */
int32_t kf_write_params_table(const char *path, const double *params, const double *cov,
                              const int32_t *status, const double *truth, const double *vertex,
                              int64_t n_tracks, int64_t stride);

#ifdef __cplusplus
}
#endif

#endif /* GB300KF_IO_H */
