// KalmanFitter.hpp — header-only C++ drop-in over the gb300kf C ABI.
//
// Keeps the shape of the reference's fitter API so that a caller written
// against it ports by changing includes:
//   Acts::KalmanFitter<P,U,S>::fit(sourcelinks, startParameters, kfOptions,
//                                  kfResult, surfaceSequence, nSurfaces)
//       reference: include/Fitter/KalmanFitter.hpp:716-768
//   KalmanFitterOptions       include/Fitter/KalmanFitter.hpp:48-96
//   KalmanFitterResult        include/Fitter/KalmanFitter.hpp:98-120
//   PropagatorOptions fields  include/Propagator/Propagator.hpp:66-95
//   PixelSourceLink           include/EventData/PixelSourceLink.hpp:22-75
//   BoundParameters           include/EventData/SingleBoundTrackParameters.hpp:27-105
//   PlaneSurface(center, normal)  include/Surfaces/detail/PlaneSurface.ipp:24-46
//   LineSurface(point)        include/Surfaces/detail/LineSurface.ipp:19-21
//   InterpolatedBFieldMap from a text map, as Options::readBField reads it
//                             src/Plugins/BFieldOptions.cpp:33-61
//
// The reference fits one track per call.  fit() here does the same (a batch
// of one, convenient but slow); fitBatch() fits many tracks in one GPU launch
// and is the intended use.  Tracks' measurements are matched to surfaces by
// geometry id, as the reference's SurfaceFinder does (KalmanFitter.hpp:31-38).
//
// Names live in namespace gb300kf; define GB300KF_ACTS_NAMESPACE before the
// include to also expose them as namespace Acts.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include <ios>

#include "../gb300kf.h"
#include "../gb300kf_fieldmap.h"
#include "../gb300kf_io.h"

namespace gb300kf {

using ActsScalar = double;
using Vector2D = std::array<double, 2>;
using Vector3D = std::array<double, 3>;
using BoundVector = std::array<double, 6>;
using BoundSymMatrix = std::array<std::array<double, 6>, 6>;
using SymMatrix2D = std::array<std::array<double, 2>, 2>;

constexpr double kTesla = 0.000299792458; // GeV/(e*mm)

/// Geometry identifier (the reference packs volume/layer/sensitive bits,
/// Geometry/GeometryID.hpp:30-33); any unique integer per surface works here.
struct GeometryID {
  uint64_t value = 0;
  bool operator==(const GeometryID &o) const { return value == o.value; }
};

struct GeometryContext {};
struct MagneticFieldContext {};

/// Boundless plane surface with the reference's curvilinear frame:
/// T = normal, U = z x T (x x T near z), V = T x U.
/// Homogeneous surface material (Material/MaterialSlab.hpp, Material.hpp):
/// thickness (mm), X0, L0 (mm), Ar, Z, molar density (mol/mm^3).
struct MaterialSlab {
  double thickness = 0., X0 = 0., L0 = 0., Ar = 0., Z = 0., molarDensity = 0.;
  /// silicon as Test/Helper.hpp:25-29 builds it
  static MaterialSlab silicon(double thicknessMm) {
    return {thicknessMm, 93.70, 465.2, 28.0855, 14., (2.329 / 28.0855) / 1000.};
  }
};

class PlaneSurface {
public:
  PlaneSurface(const Vector3D &center, const Vector3D &normal, MaterialSlab material = {})
      : m_center(center), m_material(material) {
    double n = std::sqrt(normal[0] * normal[0] + normal[1] * normal[1] + normal[2] * normal[2]);
    Vector3D T{normal[0] / n, normal[1] / n, normal[2] / n};
    Vector3D a = (std::fabs(T[2]) < 0.999995) ? Vector3D{0, 0, 1} : Vector3D{1, 0, 0};
    Vector3D U = cross(a, T);
    double un = std::sqrt(U[0] * U[0] + U[1] * U[1] + U[2] * U[2]);
    for (auto &u : U) u /= un;
    Vector3D V = cross(T, U);
    for (int r = 0; r < 3; ++r) {
      m_rot[3 * r + 0] = U[r];
      m_rot[3 * r + 1] = V[r];
      m_rot[3 * r + 2] = T[r];
    }
  }
  void assignGeoID(GeometryID id) { m_id = id; }
  GeometryID geoID() const { return m_id; }
  const Vector3D &center() const { return m_center; }
  const std::array<double, 9> &rotation() const { return m_rot; }
  const MaterialSlab &material() const { return m_material; }

private:
  static Vector3D cross(const Vector3D &a, const Vector3D &b) {
    return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
  }
  Vector3D m_center;
  MaterialSlab m_material;
  std::array<double, 9> m_rot{};
  GeometryID m_id{};
};

/// Line surface through a point with axis z (the perigee target).
class LineSurface {
public:
  LineSurface() = default;
  explicit LineSurface(const Vector3D &point) : m_center(point) {}
  const Vector3D &center() const { return m_center; }

private:
  Vector3D m_center{0, 0, 0};
};

/// 2D pixel measurement.
class PixelSourceLink {
public:
  PixelSourceLink() = default;
  PixelSourceLink(const Vector2D &values, const SymMatrix2D &cov, GeometryID gid)
      : m_values(values), m_cov(cov), m_geometryId(gid) {}
  const Vector2D &localPosition() const { return m_values; }
  const SymMatrix2D &covariance() const { return m_cov; }
  GeometryID geometryId() const { return m_geometryId; }

private:
  Vector2D m_values{};
  SymMatrix2D m_cov{};
  GeometryID m_geometryId{};
};

/// Bound parameters (loc0, loc1, phi, theta, q/p, t) with covariance on a surface.
template <typename surface_t> class BoundParameters {
public:
  using ReferenceSurfaceType = surface_t;
  BoundParameters() = default;
  BoundParameters(const GeometryContext &, const BoundSymMatrix &cov, const BoundVector &pars,
                  const surface_t *surface)
      : m_pars(pars), m_cov(cov), m_surface(surface) {}
  const BoundVector &parameters() const { return m_pars; }
  const BoundSymMatrix *covariance() const { return &m_cov; }
  const surface_t &referenceSurface() const { return *m_surface; }
  double charge() const { return m_pars[4] > 0 ? 1. : -1.; }

private:
  BoundVector m_pars{};
  BoundSymMatrix m_cov{};
  const surface_t *m_surface = nullptr;
};

/// Smoothed state on a measurement surface (subset of the reference TrackState).
struct TrackState {
  BoundVector smoothed{};
  BoundSymMatrix smoothedCovariance{};
  unsigned int surfaceIndex = 0; // position of the state's plane in the surface sequence
};

struct KalmanFitterOptions {
  KalmanFitterOptions() = default;
  KalmanFitterOptions(const GeometryContext &g, const MagneticFieldContext &m,
                      bool rsmoothing = true, const LineSurface *rSurface = nullptr)
      : geoContext(g), magFieldContext(m), smoothing(rsmoothing), referenceSurface(rSurface) {}
  GeometryContext geoContext;
  MagneticFieldContext magFieldContext;
  bool smoothing = true;
  const LineSurface *referenceSurface = nullptr;
  double outlierChi2Cut = 0.; // 0: no outlier rejection (reference VoidOutlierFinder)
  bool batched = false;       // fitBatch: length-sorted persistent kernel (batched form)
  bool mixedPrecision = false; // FP32 propagation and Jacobian transport, FP64 Kalman algebra
  bool multipleScattering = true; // at surfaces with material (KalmanFitter.hpp:92)
  bool energyLoss = true;         // at surfaces with material (KalmanFitter.hpp:95)
};

struct KalmanFitterResult {
  std::vector<TrackState> fittedStates;
  BoundParameters<LineSurface> fittedParameters;
  size_t measurementStates = 0;
  bool smoothed = false;
  bool finished = false;
  bool result = false;
  double chi2 = 0.;
  int status = KF_TRACK_NOT_FITTED;
};

/// Propagator options that steer the fit (reference defaults).
struct PropagatorOptions {
  unsigned int maxSteps = 1000;
  unsigned int maxRungeKuttaStepTrials = 10000;
  double tolerance = 1e-4;
  double stepSizeCutOff = 0.;
  double mass = 105.6583755e-3;
  double overstepLimit = 0.01; // EigenStepper::m_overstepLimit
  double targetTolerance = 1e-4;
};

/// Uniform field (Test::ConstantBField), value in GeV/(e*mm).
struct ConstantBField {
  Vector3D value{0., 0., 2. * kTesla};
};

/// Field map (MagneticField/InterpolatedBFieldMap.hpp, trilinear on an
/// equidistant 3D grid) read from a text file of "x y z bx by bz" lines as
/// Options::readBField reads the driver's map (src/Plugins/BFieldOptions.cpp:
/// 33-61: lengths in mm, field in tesla); the grid is copied to the current
/// device and shared by the copies of this object.  `scale` multiplies
/// every lookup (InterpolatedBFieldMap::Config::scale).
class InterpolatedBFieldMap {
public:
  explicit InterpolatedBFieldMap(const std::string &xyzFile, double lengthUnit = 1.,
                                 double bFieldUnit = kTesla, bool firstOctant = false,
                                 double scale = 1.) {
    float *host = nullptr;
    if (kf_field_map_read_xyz(xyzFile.c_str(), lengthUnit, bFieldUnit, firstOctant ? 1 : 0,
                              &m_field, &host) != 0)
      throw std::runtime_error(std::string("field map: ") + kf_last_error_string());
    const size_t bytes = (size_t)m_field.nx * m_field.ny * m_field.nz * 4 * sizeof(float);
    void *dev = nullptr;
    const bool ok = cudaMalloc(&dev, bytes) == cudaSuccess &&
                    cudaMemcpy(dev, host, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
    kf_field_map_free(host);
    if (!ok) {
      if (dev) cudaFree(dev);
      throw std::runtime_error("field map: device copy failed");
    }
    m_grid = std::shared_ptr<void>(dev, [](void *q) { cudaFree(q); });
    m_field.grid = static_cast<const float *>(dev);
    m_field.scale = scale;
  }
  /// the grid as the C ABI takes it (device memory)
  const kf_field_t &field() const { return m_field; }

private:
  kf_field_t m_field{};
  std::shared_ptr<void> m_grid;
};

/// One track's inputs for fitBatch.
struct TrackInput {
  std::vector<PixelSourceLink> sourcelinks;
  BoundParameters<LineSurface> start;
};

class KalmanFitter {
public:
  explicit KalmanFitter(ConstantBField field = ConstantBField(),
                        PropagatorOptions options = PropagatorOptions())
      : m_options(options) {
    m_field.kind = KF_FIELD_CONSTANT;
    m_field.scale = 1.;
    for (int a = 0; a < 3; ++a) m_field.value[a] = field.value[a];
  }
  explicit KalmanFitter(const InterpolatedBFieldMap &map,
                        PropagatorOptions options = PropagatorOptions())
      : m_field(map.field()), m_map{map}, m_options(options) {}
  KalmanFitter(const KalmanFitter &) = delete;
  KalmanFitter &operator=(const KalmanFitter &) = delete;
  ~KalmanFitter() {
    if (m_staging) cudaFree(m_staging);
  }

  /// Reference-shaped single-track fit (a batch of one).
  bool fit(const std::vector<PixelSourceLink> &sourcelinks,
           const BoundParameters<LineSurface> &sParameters, const KalmanFitterOptions &kfOptions,
           KalmanFitterResult &kfResult, const PlaneSurface *surfaceSequence,
           size_t surfaceSequenceSize) {
    std::vector<TrackInput> one(1);
    one[0].sourcelinks = sourcelinks;
    one[0].start = sParameters;
    std::vector<KalmanFitterResult> res;
    fitBatch(one, kfOptions, res, surfaceSequence, surfaceSequenceSize);
    kfResult = res[0];
    return kfResult.result;
  }

  /// Fit every track of `tracks` through the same surface sequence in one
  /// launch.  The perigee line of each track is its start parameters'
  /// reference surface (the reference sets kfOptions.referenceSurface to it,
  /// Run/GPU/Kernels.cu:35).
  void fitBatch(const std::vector<TrackInput> &tracks, const KalmanFitterOptions &kfOptions,
                std::vector<KalmanFitterResult> &results, const PlaneSurface *surfaces,
                size_t nSurfaces, cudaStream_t stream = nullptr) {
    if (nSurfaces == 0 || nSurfaces > KF_MAX_PLANES)
      throw std::invalid_argument("surface sequence must hold 1..64 planes");
    const int64_t n = static_cast<int64_t>(tracks.size());
    const int S = static_cast<int>(nSurfaces);
    results.assign(tracks.size(), KalmanFitterResult());
    if (n == 0) return;
    std::vector<double> center(3 * S), rot(9 * S), mat(6 * S);
    bool anyMaterial = false;
    for (int k = 0; k < S; ++k) {
      const MaterialSlab &m = surfaces[k].material();
      const double row[6] = {m.thickness, m.X0, m.L0, m.Ar, m.Z, m.molarDensity};
      for (int e = 0; e < 6; ++e) mat[6 * k + e] = row[e];
      anyMaterial = anyMaterial || (m.thickness > 0. && m.Ar > 0.);
    }
    for (int k = 0; k < S; ++k) {
      for (int r = 0; r < 3; ++r) center[3 * k + r] = surfaces[k].center()[r];
      for (int e = 0; e < 9; ++e) rot[9 * k + e] = surfaces[k].rotation()[e];
    }
    std::vector<double> meas((size_t)S * 5 * n, 0.), start(6 * n), scov(21 * n), per(3 * n);
    std::vector<uint64_t> mask(n, 0);
    for (int64_t i = 0; i < n; ++i) {
      for (int k = 0; k < S; ++k) {
        meas[((size_t)k * 5 + 2) * n + i] = 1.;
        meas[((size_t)k * 5 + 4) * n + i] = 1.;
      }
      for (const auto &sl : tracks[i].sourcelinks) {
        int k = 0;
        while (k < S && !(surfaces[k].geoID() == sl.geometryId())) ++k;
        if (k == S) continue; // no such surface: the measurement is never visited
        mask[i] |= (1ull << k);
        const auto &v = sl.localPosition();
        const auto &c = sl.covariance();
        const double m[5] = {v[0], v[1], c[0][0], c[0][1], c[1][1]};
        for (int e = 0; e < 5; ++e) meas[((size_t)k * 5 + e) * n + i] = m[e];
      }
      const auto &p = tracks[i].start.parameters();
      const auto &C = *tracks[i].start.covariance();
      for (int e = 0; e < 6; ++e) start[e * n + i] = p[e];
      int e = 0;
      for (int a = 0; a < 6; ++a)
        for (int b = a; b < 6; ++b) scov[(e++) * n + i] = C[a][b];
      const auto &pc = tracks[i].start.referenceSurface().center();
      for (int r = 0; r < 3; ++r) per[r * n + i] = pc[r];
    }
    kf_inputs_t in{};
    in.n_tracks = n;
    in.stride = n;
    in.n_surfaces = S;
    in.meas = meas.data();
    in.hit_mask = mask.data();
    in.n_planes = nullptr;
    in.start_params = start.data();
    in.start_cov = scov.data();
    in.perigee = per.data();
    std::vector<double> oPar(6 * n), oCov(21 * n), oChi(n), oSm((size_t)S * 27 * n);
    std::vector<int32_t> oSt(n), oNm(n);
    kf_outputs_t out{};
    out.params = oPar.data();
    out.cov = oCov.data();
    out.chi2 = oChi.data();
    out.status = oSt.data();
    out.n_meas = oNm.data();
    out.smoothed = oSm.data();
    kf_config_t cfg;
    kf_config_default(&cfg);
    cfg.max_steps = (int32_t)m_options.maxSteps;
    cfg.max_rk_trials = (int32_t)m_options.maxRungeKuttaStepTrials;
    cfg.tolerance = m_options.tolerance;
    cfg.step_size_cutoff = m_options.stepSizeCutOff;
    cfg.mass = m_options.mass;
    cfg.overstep_limit = m_options.overstepLimit;
    cfg.on_surface_tol = m_options.targetTolerance;
    cfg.smoothing = kfOptions.smoothing ? 1 : 0;
    cfg.outlier_chi2_cut = kfOptions.outlierChi2Cut;
    cfg.kernel = kfOptions.batched ? KF_KERNEL_PERSISTENT : KF_KERNEL_THREAD_PER_TRACK;
    cfg.precision = kfOptions.mixedPrecision ? KF_PRECISION_MIXED : KF_PRECISION_FP64;
    if (anyMaterial)
      cfg.material_effects = (kfOptions.multipleScattering ? 1 : 0) | (kfOptions.energyLoss ? 2 : 0);
    kf_geometry_t geo{S, 0, center.data(), rot.data(), anyMaterial ? mat.data() : nullptr};
    const kf_field_t field = m_field;
    const size_t need = kf_host_staging_size(&cfg, n, S, 1);
    if (need > m_stagingBytes) {
      if (m_staging) cudaFree(m_staging);
      m_staging = nullptr;
      m_stagingBytes = 0;
      if (cudaMalloc(&m_staging, need) != cudaSuccess)
        throw std::runtime_error("cudaMalloc of the fit staging buffer failed");
      m_stagingBytes = need;
    }
    const int32_t rc = kf_fit_batch_host(&in, &out, &cfg, &geo, &field, m_staging,
                                         m_stagingBytes, stream);
    if (rc != 0) throw std::runtime_error(std::string("kf_fit_batch_host: ") + kf_last_error_string());
    for (int64_t i = 0; i < n; ++i) {
      KalmanFitterResult &r = results[i];
      r.status = oSt[i];
      r.result = (oSt[i] == KF_TRACK_OK);
      r.measurementStates = (size_t)oNm[i];
      r.smoothed = kfOptions.smoothing && r.measurementStates > 0;
      r.finished = r.result;
      r.chi2 = oChi[i];
      BoundVector p{};
      BoundSymMatrix C{};
      for (int e = 0; e < 6; ++e) p[e] = oPar[e * n + i];
      int e = 0;
      for (int a = 0; a < 6; ++a)
        for (int b = a; b < 6; ++b) {
          C[a][b] = C[b][a] = oCov[(e++) * n + i];
        }
      const LineSurface *target =
          kfOptions.referenceSurface ? kfOptions.referenceSurface : &tracks[i].start.referenceSurface();
      r.fittedParameters = BoundParameters<LineSurface>(GeometryContext{}, C, p, target);
      r.fittedStates.resize(r.measurementStates);
      uint64_t bits = mask[i];
      for (size_t k = 0; k < r.measurementStates; ++k) {
        TrackState &ts = r.fittedStates[k];
        ts.surfaceIndex = bits ? (unsigned)__builtin_ctzll(bits) : (unsigned)k;
        bits &= bits ? bits - 1 : 0;
        for (int q = 0; q < 6; ++q) ts.smoothed[q] = oSm[((size_t)k * 27 + q) * n + i];
        int f = 0;
        for (int a = 0; a < 6; ++a)
          for (int b = a; b < 6; ++b) {
            ts.smoothedCovariance[a][b] = ts.smoothedCovariance[b][a] =
                oSm[((size_t)k * 27 + 6 + (f++)) * n + i];
          }
      }
    }
  }

private:
  kf_field_t m_field{};
  std::vector<InterpolatedBFieldMap> m_map; // keeps a map's device grid alive
  PropagatorOptions m_options;
  void *m_staging = nullptr;
  size_t m_stagingBytes = 0;
};

/// writeParamsCsv (Run/Common/Writer.hpp:80-110): the fitted parameters of
/// the tracks whose status is true, one CSV row each (kf_write_params_csv).
template <typename parameters_t>
void writeParamsCsv(const parameters_t *params, const bool *status, unsigned int nTracks,
                    std::string fileName) {
  if (fileName.empty()) fileName = "params-fitted.obj"; // the reference's default name
  std::vector<double> p((size_t)6 * nTracks);
  std::vector<int32_t> st(nTracks);
  for (unsigned int i = 0; i < nTracks; ++i) {
    for (int e = 0; e < 6; ++e) p[(size_t)e * nTracks + i] = params[i].parameters()[e];
    st[i] = status[i] ? KF_TRACK_OK : KF_TRACK_NOT_FITTED;
  }
  if (kf_write_params_csv(fileName.c_str(), p.data(), st.data(), nTracks, nTracks) != 0)
    throw std::ios_base::failure(kf_last_error_string());
}

/// writeStatesObj (Run/Common/Writer.hpp:42-78) with parameters = "smoothed":
/// one obj polyline per successful fit through its smoothed states, placed on
/// the planes of `surfaces` (kf_write_states_obj).  Takes the fit results and
/// the surface sequence where the reference takes its track-state array.
inline void writeStatesObj(const KalmanFitterResult *results, unsigned int nTracks,
                           const PlaneSurface *surfaces, unsigned int nSurfaces,
                           std::string fileName) {
  if (fileName.empty()) fileName = "tracks-fitted.obj";
  if (nSurfaces == 0 || nSurfaces > KF_MAX_PLANES)
    throw std::invalid_argument("surface sequence must hold 1..64 planes");
  const size_t n = nTracks, S = nSurfaces;
  std::vector<double> sm(S * 27 * n, 0.), center(3 * S), rot(9 * S);
  std::vector<int32_t> nm(n), st(n);
  std::vector<uint64_t> mask(n, 0);
  for (size_t k = 0; k < S; ++k) {
    for (int r = 0; r < 3; ++r) center[3 * k + r] = surfaces[k].center()[r];
    for (int e = 0; e < 9; ++e) rot[9 * k + e] = surfaces[k].rotation()[e];
  }
  for (size_t i = 0; i < n; ++i) {
    const KalmanFitterResult &r = results[i];
    st[i] = r.result ? KF_TRACK_OK : KF_TRACK_NOT_FITTED;
    nm[i] = (int32_t)std::min(r.fittedStates.size(), S);
    for (int k = 0; k < nm[i]; ++k) {
      const TrackState &ts = r.fittedStates[k];
      mask[i] |= 1ull << ts.surfaceIndex;
      for (int q = 0; q < 6; ++q) sm[((size_t)k * 27 + q) * n + i] = ts.smoothed[q];
    }
  }
  const kf_geometry_t geo{(int32_t)S, 0, center.data(), rot.data(), nullptr};
  if (kf_write_states_obj(fileName.c_str(), sm.data(), nm.data(), mask.data(), st.data(),
                          (int64_t)n, (int64_t)n, &geo) != 0)
    throw std::ios_base::failure(kf_last_error_string());
}

} // namespace gb300kf

#ifdef GB300KF_ACTS_NAMESPACE
namespace Acts = gb300kf;
#endif
