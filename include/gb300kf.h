/*
 * gb300kf.h — C ABI of the GB300-native Kalman track fitter.
 *
 * One call fits a batch of tracks: RK4 (Nystroem) propagation with transport
 * Jacobian through the magnetic field, direct navigation over a sequence of
 * plane surfaces, gain-matrix Kalman update on every hit, gain-matrix (RTS)
 * smoothing, and back-propagation of the first smoothed state to the per-track
 * perigee line surface.  It replaces the per-track call
 *
 *   Acts::KalmanFitter<P,U,S,O>::fit(sourcelinks, startParameters, kfOptions,
 *                                    kfResult, surfaceSequence, nSurfaces)
 *     reference: include/Fitter/KalmanFitter.hpp:716-768
 *
 * and its device twin fitOnDevice (include/Fitter/KalmanFitter.hpp:790-850),
 * launched per track by fitKernelThreadPerTrack / fitKernelBlockPerTrack
 * (Run/GPU/Kernels.cu:6-94).
 *
 * Conventions
 *  - Units are the reference's native units: mm, GeV, e; time in mm (c = 1);
 *    magnetic field in GeV/(e*mm) (1 T = 0.000299792458).
 *  - Bound parameter order (reference eBoundLoc0..eBoundTime):
 *      0 loc0, 1 loc1, 2 phi, 3 theta, 4 q/p, 5 t.
 *  - Covariances are passed as the 21 upper-triangle elements of the 6x6
 *    matrix, row-major: (0,0) (0,1) .. (0,5) (1,1) .. (1,5) .. (5,5).
 *  - Per-track arrays are structure-of-arrays: element `row` of track `i`
 *    lives at ptr[row * stride + i].  `stride` >= n_tracks.
 *  - All data pointers in kf_inputs_t / kf_outputs_t / workspace are DEVICE
 *    pointers (kf_fit_batch) or HOST pointers (kf_fit_batch_host).
 *    kf_geometry_t and kf_config_t are always read from host memory at call
 *    time; the grid of a kf_field_t must be a device pointer.
 *  - Calls are stream-ordered and asynchronous; nothing is allocated inside a
 *    call.  Concurrent calls on different streams need distinct workspaces.
 *  - Return codes: 0 on success, a negative kf_error on an API or CUDA error
 *    (text via kf_last_error_string()).  The library never exits the process.
 */
#ifndef GB300KF_H
#define GB300KF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KF_ABI_VERSION 1
#define KF_MAX_PLANES 64 /* surfaces in one sequence */

/* ---- call-level error codes (negative) ---------------------------------- */
enum kf_error {
  KF_SUCCESS = 0,
  KF_ERR_INVALID_ARGUMENT = -1,
  KF_ERR_WORKSPACE_TOO_SMALL = -2,
  KF_ERR_CUDA = -3,
  KF_ERR_UNSUPPORTED = -4,
  KF_ERR_NO_DEVICE = -5,
  KF_ERR_IO = -6 /* an output file could not be written (gb300kf_io.h) */
};

/* ---- per-track status (kf_outputs_t.status) ------------------------------ *
 * KF_TRACK_OK corresponds to the reference fit() returning true; every other
 * value to it returning false (KalmanFitter.hpp:760-767), with the cause.   */
enum kf_track_status {
  KF_TRACK_OK = 0,
  KF_TRACK_MEAS_MISMATCH = 1, /* measurement states != hits on the track */
  KF_TRACK_SMOOTHER_NAN = 2,  /* smoothing gain had a NaN (GainMatrixSmoother.hpp:63-66) */
  KF_TRACK_MAX_STEPS = 3,     /* propagation hit maxSteps without the aborter */
  KF_TRACK_NO_HITS = 4,       /* no measurement on the track */
  KF_TRACK_BAD_INPUT = 5,     /* q/p == 0 or non-finite start parameters */
  KF_TRACK_NOT_FITTED = 6,    /* target surface never reached */
  KF_TRACK_ADJOINT_FAILED = 7 /* kf_adjoint_batch: a step failed or the
                                 segment tape was full; no gradient */
};

enum kf_precision {
  KF_PRECISION_FP64 = 0, /* plain form: FP64 throughout */
  KF_PRECISION_MIXED = 1 /* FP32 RK4/field/transport, FP64 gain/update/smoother */
};

enum kf_field_kind {
  KF_FIELD_CONSTANT = 0, /* Test::ConstantBField (Test/Helper.hpp:17-22) */
  KF_FIELD_GRID3D = 1,   /* trilinear on an (x, y, z) grid (fieldMapperXYZ) */
  KF_FIELD_GRID_RZ = 2   /* bilinear on an (r, z) grid of (br, bz), rotated by the
                            position's azimuth (fieldMapperRZ,
                            src/MagneticField/BFieldMapUtils.cpp:17-136) */
};

enum kf_kernel_kind {
  KF_KERNEL_AUTO = 0,
  KF_KERNEL_THREAD_PER_TRACK = 1, /* one thread per track, grid over tracks */
  KF_KERNEL_PERSISTENT = 2        /* persistent CTAs pulling a sorted queue */
};

/* Steering of the fit: PropagatorOptions (Propagator.hpp:52-111) plus
 * KalmanFitterOptions (KalmanFitter.hpp:48-96) plus launch shape. */
typedef struct kf_config {
  int32_t precision;         /* kf_precision */
  int32_t max_steps;         /* PropagatorOptions::maxSteps (1000) */
  int32_t max_rk_trials;     /* PropagatorOptions::maxRungeKuttaStepTrials (10000) */
  int32_t smoothing;         /* KalmanFitterOptions::smoothing (1) */
  double tolerance;          /* RK error tolerance, PropagatorOptions::tolerance (1e-4) */
  double step_size_cutoff;   /* PropagatorOptions::stepSizeCutOff (0) */
  double mass;               /* particle mass used in dt/ds; the reference fit
                                never sets it, so the muon default applies
                                (Propagator.hpp:73): 0.1056583755 GeV */
  double overstep_limit;     /* EigenStepper::m_overstepLimit (0.01 mm) */
  double on_surface_tol;     /* s_onSurfaceTolerance (1e-4 mm) */
  double outlier_chi2_cut;   /* > 0: hits whose predicted chi2 exceeds it are
                                outliers (no update); 0 = off, as in the
                                reference's VoidOutlierFinder */
  int32_t faithful_jacobian; /* 1: keep the reference's jacToGlobal (not rebuilt
                                after the update, EigenStepper.ipp:554-564);
                                0: rebuild it at the updated state */
  int32_t kernel;            /* kf_kernel_kind: kf_fit_batch_host runs the batched
                                form for KF_KERNEL_PERSISTENT and the
                                thread-per-track grid otherwise; the device-buffer
                                entry points each run their own form */
  int32_t block_size;        /* batched form: threads per CTA (64, 128, 256),
                                0 = 128 */
  int32_t min_blocks_per_sm; /* batched form: CTAs per SM the persistent kernel
                                is compiled for (its register budget), 0 = 4;
                                compiled shapes (threads x CTAs): 128 x 2..5,
                                64 x 4, 64 x 8, 256 x 1, 256 x 2; kf_autotune
                                picks one */
  int32_t material_effects;  /* bit 0: multiple scattering, bit 1: energy loss
                                at the surfaces' material (kf_geometry_t.material)
                                after each filter update (KalmanFitter.hpp:405-449,
                                KalmanFitterOptions::multipleScattering /
                                energyLoss); 0 (default) = none.  With material
                                the smoother takes the reference's general gain
                                C_f J^T C_p^-1 and the workspace grows (sizes
                                depend on this field); the batched form runs its
                                material instantiation (128 threads x 4 CTAs per
                                SM) whatever the shape fields say */
  int32_t adjoint_tape;      /* kf_adjoint_batch only: 0 (default) = the forward
                                records the tape of the whole track (256 doubles
                                per track and surface, at least 3072); 1 = it
                                saves checkpoints every 5 measurement states
                                and the reverse sweep recomputes one 5-state
                                segment at a time (3072 doubles per track).
                                The results are bitwise the same; 0 is faster
                                and is also what a track falls back to 1 from
                                when its tape runs over */
} kf_config_t;

/* The surface sequence: boundless plane surfaces (PlaneSurface<InfiniteBounds>,
 * Surfaces/detail/PlaneSurface.ipp:24-69), in navigation order. */
typedef struct kf_geometry {
  int32_t n_planes;   /* <= KF_MAX_PLANES */
  int32_t reserved0;
  const double *center;   /* [n_planes][3] host memory */
  const double *rotation; /* [n_planes][9] host memory, row-major 3x3 whose
                             columns are the local axes U, V and the normal T */
  const double *material; /* [n_planes][6] host memory or NULL: homogeneous
                             surface material (Material/MaterialSlab.hpp,
                             Material.hpp) as thickness (mm), radiation length
                             X0 (mm), interaction length L0 (mm), relative
                             atomic mass Ar, nuclear charge Z and molar density
                             (mol/mm^3); thickness 0 = no material on the plane */
} kf_geometry_t;

/* Magnetic field: Test::ConstantBField (include/Test/Helper.hpp:17-22) or an
 * equidistant 3D grid with trilinear interpolation
 * (MagneticField/InterpolatedBFieldMap.hpp:87-208). */
typedef struct kf_field {
  int32_t kind;             /* kf_field_kind */
  int32_t nx, ny, nz;       /* grid points per axis (grid only); (r, z) grid:
                               nx points in r, ny = 1, nz points in z */
  double value[3];          /* constant field (constant only) */
  double scale;             /* global multiplier applied to every lookup */
  double min[3], max[3];    /* grid extent in mm: point i at min + i*(max-min)/(n-1);
                               (r, z) grid: r over min[0]..max[0], z over
                               min[2]..max[2] */
  const float *grid;        /* DEVICE [nz][ny][nx][4] = (bx, by, bz, 0) in
                               GeV/(e*mm); index ((iz*ny)+iy)*nx+ix.  (r, z)
                               grid: [nz][nx][4] = (br, bz, 0, 0), index
                               iz*nx+ir */
} kf_field_t;

/* Per-track inputs (structure of arrays). */
typedef struct kf_inputs {
  int64_t n_tracks;
  int64_t stride;             /* elements between SoA rows, >= n_tracks */
  int32_t n_surfaces;         /* planes in the sequence (== geometry n_planes) */
  int32_t reserved0;
  const double *meas;         /* [n_surfaces][5][stride]: loc0, loc1, var0,
                                 cov01, var1 of the 2D pixel measurement
                                 (EventData/PixelSourceLink.hpp:22-75) */
  const uint64_t *hit_mask;   /* [stride] bit k set: plane k has a hit;
                                 NULL: every plane has a hit */
  const int32_t *n_planes;    /* [stride] length of the track's surface sequence
                                 (first n planes); NULL: n_surfaces */
  const double *start_params; /* [6][stride] bound parameters on the perigee line */
  const double *start_cov;    /* [21][stride] upper triangle */
  const double *perigee;      /* [3][stride] centre of the perigee line surface
                                 (LineSurface with axis z, Run/Common/Processor.hpp:121-129) */
} kf_inputs_t;

/* Per-track outputs (structure of arrays). */
typedef struct kf_outputs {
  double *params;     /* [6][stride] fitted parameters at the perigee line */
  double *cov;        /* [21][stride] their covariance */
  double *chi2;       /* [stride] sum of predicted-residual chi2 over updates */
  int32_t *status;    /* [stride] kf_track_status */
  int32_t *n_meas;    /* [stride] measurement states (hits incl. outliers) */
  int32_t *n_steps;   /* [stride] accepted RK steps (may be NULL) */
  int32_t *n_trials;  /* [stride] RK4 stage evaluations incl. rejected trials
                         (may be NULL) */
  double *smoothed;   /* [n_surfaces][27][stride] smoothed parameters (6) and
                         covariance (21) per measurement state; may be NULL */
} kf_outputs_t;

/* Version and diagnostics. */
int32_t kf_version(void);
const char *kf_last_error_string(void);

/* Material interaction at one plane crossing (host; no GPU involved): the
 * same computation the fit applies after a measurement with material
 * (Propagator/detail/PointwiseMaterialInteraction.hpp/.ipp, formulas of
 * Material/detail/Interactions.ipp).  mat as one row of
 * kf_geometry_t.material, flags as kf_config_t.material_effects, unit
 * plane normal and unit direction, |p| (GeV), charge, mass (GeV).
 * out = (|p| after the mean energy loss, phi variance, theta variance, q/p
 * variance, mean energy loss).  Returns 0, or 1 when nothing applies (no
 * material or no effect selected; out untouched). */
int32_t kf_material_interaction(const double mat[6], int32_t flags, const double normal[3],
                                const double dir[3], double p, double q, double mass,
                                double out[5]);

/* Default configuration (reference defaults, FP64). */
void kf_config_default(kf_config_t *cfg);

/* Device workspace bytes kf_fit_batch needs for this batch shape. */
size_t kf_workspace_size(const kf_config_t *cfg, int64_t n_tracks,
                         int32_t n_surfaces);

/* Fit a batch; all kf_inputs_t/kf_outputs_t pointers are device pointers.
 * `stream` is a cudaStream_t (NULL = legacy default stream). */
int32_t kf_fit_batch(const kf_inputs_t *in, kf_outputs_t *out,
                     const kf_config_t *cfg, const kf_geometry_t *geo,
                     const kf_field_t *field, void *workspace,
                     size_t workspace_bytes, void *stream);

/* Device bytes kf_fit_batch_host needs: workspace plus staging of inputs and
 * outputs. */
size_t kf_host_staging_size(const kf_config_t *cfg, int64_t n_tracks,
                            int32_t n_surfaces, int32_t with_smoothed);

/* Fit a batch held in HOST memory (pinned memory gives async copies): copies
 * inputs into `device_staging`, fits, copies the outputs back, and blocks
 * until the results are on the host.  Batches of 262144 tracks or more run as
 * 2 or 4 chunks alternating between `stream` and a second stream the library
 * keeps per device, so that the copies of one chunk overlap the fit of
 * another (with pinned host memory); results are the same as one chunk's. */
int32_t kf_fit_batch_host(const kf_inputs_t *host_in, kf_outputs_t *host_out,
                          const kf_config_t *cfg, const kf_geometry_t *geo,
                          const kf_field_t *field, void *device_staging,
                          size_t staging_bytes, void *stream);

/* ---- batched form ---------------------------------------------------------
 * Replaces the reference's one-thread-per-track launch
 * (Run/GPU/Kernels.cu:6-45 from Run/GPU/KalmanFitterGPUTest.cu:461-472) for
 * large batches with uneven track lengths, holes and outliers: tracks are
 * ordered by expected work (sequence length, then |q/p|; longest first) by a
 * counting sort on the device, and a persistent kernel (one resident grid,
 * warps claiming 32 queue positions at a time) fits them.  Results are the
 * same as kf_fit_batch's; the workspace is kf_batch_workspace_size bytes. */
size_t kf_batch_workspace_size(const kf_config_t *cfg, int64_t n_tracks,
                               int32_t n_surfaces);
int32_t kf_fit_batch_sorted(const kf_inputs_t *in, kf_outputs_t *out,
                            const kf_config_t *cfg, const kf_geometry_t *geo,
                            const kf_field_t *field, void *workspace,
                            size_t workspace_bytes, void *stream);

/* A plan captures the whole batched pipeline (queue reset, sort, persistent
 * fit) for fixed buffers into a CUDA graph; each launch replays it with one
 * call.  `stream` must be a created stream (capture is not possible on the
 * legacy default stream).  The buffers must outlive the plan. */
typedef struct kf_batch_plan kf_batch_plan_t;
int32_t kf_batch_plan_create(kf_batch_plan_t **plan, const kf_inputs_t *in,
                             kf_outputs_t *out, const kf_config_t *cfg,
                             const kf_geometry_t *geo, const kf_field_t *field,
                             void *workspace, size_t workspace_bytes,
                             void *stream);
int32_t kf_batch_plan_launch(kf_batch_plan_t *plan, void *stream);
void kf_batch_plan_destroy(kf_batch_plan_t *plan);

/* Times every compiled persistent-kernel shape (threads per CTA and CTAs per
 * SM, see kf_config_t.min_blocks_per_sm) of cfg->precision on the first min(n, 524288) tracks of the batch
 * (best of three runs after a warm-up) and returns the fastest configuration
 * in *tuned (and its time per fit of the sample in *best_ms).  Overwrites
 * the outputs of those tracks.  Shapes differ in register allocation only;
 * results agree to rounding (not bitwise) across shapes. */
int32_t kf_autotune(const kf_inputs_t *in, kf_outputs_t *out,
                    const kf_config_t *cfg, const kf_geometry_t *geo,
                    const kf_field_t *field, void *workspace,
                    size_t workspace_bytes, void *stream, kf_config_t *tuned,
                    double *best_ms);

/* ---- fitting without allocation ------------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (a host framework owns all device memory through its own pool, a plugin
 * host forbids foreign allocations, or cudaMalloc's implicit synchronisation
 * or mid-run failure is unacceptable): same inputs and outputs as
 * kf_fit_batch, with the workspace taken from a static device array of
 * KF_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until the
 * process exits.  A batch needing more scratch than that (kf_workspace_size)
 * is rejected with KF_ERR_WORKSPACE_TOO_SMALL and a message from
 * kf_noalloc_last_error_string() (this thread's last call; empty after a
 * success); split it or use kf_fit_batch.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress), and so does the first call after that device's
 * context was replaced (cudaDeviceReset); make such a call before any stream
 * capture.
 * All calls share the one array: calls that overlap on the GPU (different
 * streams, or host threads without ordering) race on it.  Nothing is
 * allocated, and nothing needs clearing between calls. */
#define KF_NOALLOC_SCRATCH_BYTES (64ull << 20)

int32_t kf_fit_batch_noalloc(const kf_inputs_t *in, kf_outputs_t *out,
                             const kf_config_t *cfg, const kf_geometry_t *geo,
                             const kf_field_t *field, void *stream);
size_t kf_noalloc_scratch_bytes(void);
const char *kf_noalloc_last_error_string(void);

/* ---- chi2 adjoint ---------------------------------------------------------
 * No counterpart in the reference (it has no derivatives).  Objective: the
 * total smoothed chi2, sum over tracks with status KF_TRACK_OK and their
 * non-outlier measurement states of (m - H x_s)^T V^-1 (m - H x_s), x_s the
 * smoothed parameters of the same fit as kf_fit_batch.  Gradients by a
 * hand-written reverse sweep (FP64) with respect to
 *   - the alignment of each plane: centre shift (dx, dy, dz) in mm and small
 *     rotations (wx, wy, wz) in rad about the global axes applied to the
 *     plane frame, at the geometry given (zero alignment);
 *   - each track's start parameters (perigee d0, z0, phi, theta, q/p, t);
 *   - the field scale (kf_field_t.scale).
 * Supported: cfg->precision FP64, uniform field, faithful_jacobian = 1.
 * The forward states are checkpointed every 5 measurement states and each
 * segment is recomputed during the reverse sweep. */
typedef struct kf_adjoint_outputs {
  double *chi2;             /* [n] smoothed chi2 per track (0 unless OK) */
  int32_t *status;          /* [n] kf_track_status */
  double *grad_start;       /* [6][stride] d chi2_track / d start parameter, or NULL */
  double *grad_align;       /* [n_surfaces][6] d chi2_total / d alignment, or NULL */
  double *grad_field_scale; /* [1] d chi2_total / d field scale, or NULL */
  double *chi2_total;       /* [1] total chi2, or NULL */
  double *grad_field_scale_track; /* [n] d chi2_track / d field scale, or NULL */
} kf_adjoint_outputs_t;

/* Device workspace bytes kf_adjoint_batch needs: the fit's state store,
 * the smoother adjoints, checkpoints and the tape, whose size follows
 * cfg->adjoint_tape (262144 tracks of 20 surfaces: 15.2 GB with 0, 10.9 GB
 * with 1).  cfg may be NULL (adjoint_tape = 0). */
size_t kf_adjoint_workspace_size(const kf_config_t *cfg, int64_t n_tracks, int32_t n_surfaces);

/* compute_gradient = 0 runs the forward part only (chi2, status), the
 * function the gradient differentiates, for finite-difference checks. */
int32_t kf_adjoint_batch(const kf_inputs_t *in, kf_adjoint_outputs_t *out,
                         const kf_config_t *cfg, const kf_geometry_t *geo,
                         const kf_field_t *field, int32_t compute_gradient, void *workspace,
                         size_t workspace_bytes, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GB300KF_H */
