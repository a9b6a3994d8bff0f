// A caller written in the reference driver's shape, compiled against the
// drop-in header instead of the reference's own: the driver's typedefs
// (Run/Common/FitData.hpp:26-43), its surfaces, source links, perigee
// targets and start parameters built as Run/GPU/KalmanFitterGPUTest.cu:
// 245-354 and Run/Common/Processor.hpp:120-253 build them, and its CPU fit
// loop (KalmanFitterGPUTest.cu:539-560: an OpenMP loop, one fit() per track)
// and GPU launch (Run/GPU/Kernels.cu:6-45, here fitBatch over the same
// arrays).  Inputs are the seeded telescope workload of kf_synth_tracks; the
// results are checked against a direct kf_fit_batch_host call on the same
// arrays.  Prints "mismatches=0" when every per-track fit, the batched call
// and the C ABI agree bitwise.
#define GB300KF_ACTS_NAMESPACE
#include "../../include/gb300kf/KalmanFitter.hpp"
#include "../../include/gb300kf_synth.h"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include <unistd.h>

#ifdef _OPENMP
#include <omp.h>
#endif

// ---- the reference driver's typedefs (the simulator's aside)
using PlaneSurfaceType = Acts::PlaneSurface<Acts::InfiniteBounds>;
using Stepper = Acts::EigenStepper<Test::ConstantBField>;
using PropagatorType = Acts::Propagator<Stepper>;
using PropResultType = Acts::PropagatorResult;
using Smoother = Acts::GainMatrixSmoother<Acts::BoundParameters<PlaneSurfaceType>>;
using KalmanFitterType = Acts::KalmanFitter<PropagatorType, Acts::GainMatrixUpdater, Smoother>;
using KalmanFitterResultType =
    Acts::KalmanFitterResult<Acts::PixelSourceLink, Acts::BoundParameters<PlaneSurfaceType>,
                             Acts::LineSurface>;
using TSType = typename KalmanFitterResultType::TrackStateType;
using FitOptionsType = Acts::KalmanFitterOptions<Acts::VoidOutlierFinder>;
using Size = unsigned int;

// the field map case: the same typedefs with the map's stepper
template <typename bfield_t> struct Types {
  using StepperT = Acts::EigenStepper<bfield_t>;
  using PropagatorT = Acts::Propagator<StepperT>;
  using FitterT = Acts::KalmanFitter<PropagatorT, Acts::GainMatrixUpdater, Smoother>;
};

template <typename bfield_t>
static int run(const char *name, const bfield_t &bField, const kf_field_t &abiField,
               const float *hostGrid, double siliconMm, long &mismatches) {
  const Size nTracks = 3000, nSurfaces = 10;
  const bool smoothing = true;
  Acts::GeometryContext gctx(0);
  Acts::MagneticFieldContext mctx(0);

  // synthetic inputs: the 10-plane telescope at x = 100..1000 mm
  kf_synth_config_t sc;
  kf_synth_config_default(&sc);
  sc.n_tracks = nTracks;
  sc.seed = 4242;
  if (siliconMm > 0) {
    const Acts::Material si = Test::makeSilicon();
    const double row[6] = {siliconMm, si.X0(), si.L0(), si.Ar(), si.Z(), si.molarDensity()};
    for (int e = 0; e < 6; ++e) sc.material[e] = row[e];
  }
  const int S = (int)nSurfaces;
  const int64_t n = nTracks;
  std::vector<double> center(3 * S), rot(9 * S), tc(3 * S), tr(9 * S);
  kf_synth_geometry(&sc, center.data(), rot.data(), tc.data(), tr.data(), nullptr);
  std::vector<double> meas((size_t)S * 5 * n), start(6 * n), scov(21 * n), per(3 * n);
  std::vector<uint64_t> mask(n);
  std::vector<int32_t> np(n);
  kf_field_t truthField = abiField;
  truthField.grid = hostGrid;
  if (kf_synth_tracks(&sc, tc.data(), tr.data(), hostGrid ? &truthField : nullptr, meas.data(),
                      mask.data(), np.data(), start.data(), scov.data(), per.data(), nullptr,
                      0) != 0)
    return 1;

  // ---- the geometry, as the driver builds it
  Acts::MaterialSlab matProp(Test::makeSilicon(), siliconMm * Acts::units::_mm);
  Acts::HomogeneousSurfaceMaterial surfaceMaterial(matProp);
  PlaneSurfaceType *surfaces = new PlaneSurfaceType[nSurfaces];
  for (Size isur = 0; isur < nSurfaces; isur++) {
    Acts::Vector3D translation(center[3 * isur], center[3 * isur + 1], center[3 * isur + 2]);
    surfaces[isur] = siliconMm > 0
                         ? PlaneSurfaceType(translation, Acts::Vector3D(1, 0, 0), surfaceMaterial)
                         : PlaneSurfaceType(translation, Acts::Vector3D(1, 0, 0));
    auto geoID = Acts::GeometryID().setVolume(0u).setLayer(isur).setSensitive(isur);
    surfaces[isur].assignGeoID(geoID);
  }
  const Acts::Surface *surfacePtrs = surfaces;

  // ---- source links, perigee targets and start parameters
  std::vector<Acts::PixelSourceLink> sourcelinks(nTracks * nSurfaces);
  std::vector<Acts::LineSurface> targetSurfaces(nTracks);
  std::vector<Acts::BoundParameters<Acts::LineSurface>> startParsCollection;
  startParsCollection.reserve(nTracks);
  for (Size ip = 0; ip < nTracks; ip++) {
    for (Size ih = 0; ih < nSurfaces; ih++) {
      const double *m = &meas[(size_t)ih * 5 * n];
      Acts::Vector2D values;
      values << m[ip], m[n + ip];
      Acts::SymMatrix2D cov;
      cov << m[2 * n + ip], m[3 * n + ip], m[3 * n + ip], m[4 * n + ip];
      sourcelinks[ip * nSurfaces + ih] = Acts::PixelSourceLink(values, cov, surfaces[ih].geoID());
    }
    targetSurfaces[ip] = Acts::LineSurface(Acts::Vector3D(per[ip], per[n + ip], per[2 * n + ip]));
    Acts::BoundVector params = Acts::BoundVector::Zero();
    for (int e = 0; e < 6; ++e) params[e] = start[e * n + ip];
    Acts::BoundSymMatrix cov = Acts::BoundSymMatrix::Zero();
    int e = 0;
    for (int a = 0; a < 6; ++a)
      for (int b = a; b < 6; ++b) cov(a, b) = cov(b, a) = scov[(e++) * n + ip];
    startParsCollection.emplace_back(gctx, cov, params, &targetSurfaces[ip]);
  }

  // ---- the fitter: the reference's objects; the overstep limit is the
  // stepper's second argument (0.1 mm: at the reference's 0.01 mm a quarter
  // of this workload's tracks skip planes)
  typename Types<bfield_t>::StepperT stepper(bField, 0.1 * Acts::units::_mm);
  typename Types<bfield_t>::PropagatorT propagator(stepper);
  typename Types<bfield_t>::FitterT kFitter(propagator);
  std::vector<FitOptionsType> fitOptions(nTracks);
  std::vector<TSType> fitStates(nTracks * nSurfaces);
  std::vector<Acts::BoundParameters<Acts::LineSurface>> fitPars(nTracks);
  std::unique_ptr<bool[]> fitStatus(new bool[nTracks]);
  for (Size it = 0; it < nTracks; it++) {
    fitOptions[it] = FitOptionsType(gctx, mctx, smoothing);
    fitStatus[it] = false;
  }

  // ---- the CPU driver's loop: one fit per track from an OpenMP loop
  int threads = 1;
#pragma omp parallel for
  for (Size it = 0; it < nTracks; it++) {
    KalmanFitterResultType kfResult;
    kfResult.fittedStates =
        Acts::CudaKernelContainer<TSType>(&fitStates[it * nSurfaces], nSurfaces);
    auto sourcelinkTrack = Acts::CudaKernelContainer<Acts::PixelSourceLink>(
        sourcelinks.data() + it * nSurfaces, nSurfaces);
    fitOptions[it].referenceSurface = &targetSurfaces[it];
    auto status = kFitter.fit(sourcelinkTrack, startParsCollection[it], fitOptions[it], kfResult,
                              surfacePtrs, nSurfaces);
    fitStatus[it] = status;
    fitPars[it] = kfResult.fittedParameters;
#ifdef _OPENMP
    threads = omp_get_num_threads();
#endif
  }

  // ---- the GPU driver's launch over the same arrays, in one call
  std::vector<TSType> batchStates(nTracks * nSurfaces);
  std::vector<Acts::BoundParameters<Acts::LineSurface>> batchPars(nTracks);
  std::unique_ptr<bool[]> batchStatus(new bool[nTracks]);
  kFitter.fitBatch(sourcelinks.data(), startParsCollection.data(), fitOptions.data(),
                   batchStates.data(), batchPars.data(), batchStatus.get(), nTracks, surfacePtrs,
                   nSurfaces);

  // ---- the C ABI on the same arrays
  kf_config_t cfg;
  kf_config_default(&cfg);
  cfg.overstep_limit = 0.1;
  std::vector<double> mat(6 * S, 0.);
  if (siliconMm > 0) {
    cfg.material_effects = 3;
    for (int k = 0; k < S; ++k)
      for (int e = 0; e < 6; ++e) mat[6 * k + e] = sc.material[e];
  }
  kf_inputs_t in{};
  in.n_tracks = n;
  in.stride = n;
  in.n_surfaces = S;
  in.meas = meas.data();
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
  kf_geometry_t geo{S, 0, center.data(), rot.data(), siliconMm > 0 ? mat.data() : nullptr};
  const kf_field_t field = abiField;
  void *staging = nullptr;
  const size_t bytes = kf_host_staging_size(&cfg, n, S, 1);
  if (cudaMalloc(&staging, bytes) != cudaSuccess) return 2;
  const int32_t rc = kf_fit_batch_host(&in, &out, &cfg, &geo, &field, staging, bytes, nullptr);
  cudaFree(staging);
  if (rc != 0) {
    std::printf("kf_fit_batch_host: %s\n", kf_last_error_string());
    return 3;
  }

  long bad = 0, ok = 0;
  for (int64_t i = 0; i < n; ++i) {
    const bool abiOk = oSt[i] == KF_TRACK_OK && oNm[i] == S;
    if (fitStatus[i] != abiOk || batchStatus[i] != abiOk) ++bad;
    ok += abiOk;
    for (int e = 0; e < 6; ++e) {
      if (fitPars[i].parameters()[e] != oPar[e * n + i]) ++bad;
      if (batchPars[i].parameters()[e] != oPar[e * n + i]) ++bad;
    }
    int e = 0;
    for (int a = 0; a < 6; ++a)
      for (int b = a; b < 6; ++b, ++e) {
        if ((*fitPars[i].covariance())(a, b) != oCov[e * n + i]) ++bad;
        if ((*batchPars[i].covariance())(a, b) != oCov[e * n + i]) ++bad;
      }
    if (&fitPars[i].referenceSurface() != &targetSurfaces[i]) ++bad;
    for (int k = 0; k < oNm[i]; ++k) {
      const TSType &a = fitStates[i * nSurfaces + k], &b = batchStates[i * nSurfaces + k];
      if (!a.isType(Acts::MeasurementFlag) || !(a.geometryId() == surfaces[k].geoID())) ++bad;
      for (int q = 0; q < 6; ++q) {
        const double want = oSm[((size_t)k * 27 + q) * n + i];
        if (a.parameter.smoothed.parameters()[q] != want) ++bad;
        if (b.parameter.smoothed.parameters()[q] != want) ++bad;
      }
      if (a.measurement.uncalibrated.localPosition()[0] != meas[(size_t)k * 5 * n + i]) ++bad;
    }
  }
  // the driver's writers on the results
  const std::string csv = "/tmp/gb300kf_driver_params_" + std::to_string(getpid()) + ".csv";
  Acts::writeParamsCsv(fitPars.data(), fitStatus.get(), nTracks, csv);
  std::ifstream f(csv);
  std::string header;
  std::getline(f, header);
  if (header.rfind("trackIdx, fit_BoundLoc0", 0) != 0) ++bad;
  std::remove(csv.c_str());
  std::printf("%s: %u tracks, %ld fitted, %d host threads, mismatches %ld\n", name, nTracks, ok,
              threads, bad);
  mismatches += bad;
  delete[] surfaces;
  return ok > (long)nTracks * 9 / 10 ? 0 : 4;
}

int main() {
  long mismatches = 0;
  kf_field_t uniform{};
  uniform.kind = KF_FIELD_CONSTANT;
  uniform.scale = 1.;
  uniform.value[2] = 2. * Acts::kTesla;
  int rc = run("uniform 2 T", Test::ConstantBField(), uniform, nullptr, 0.0, mismatches);
  if (!rc) rc = run("uniform 2 T, 0.5 mm silicon", Test::ConstantBField(), uniform, nullptr, 0.5,
                    mismatches);
  if (!rc) {
    // a field map as a text file of "x y z bx by bz" lines (mm, tesla): the
    // analytic map on 31^3 points over +-1.5 m, read back as the reference
    // driver reads its map
    const int nm = 31;
    const double half = 1500.;
    std::vector<float> grid((size_t)nm * nm * nm * 4);
    kf_synth_field_map(2.0, nm, half, grid.data());
    const std::string path = "/tmp/gb300kf_driver_map_" + std::to_string(getpid()) + ".txt";
    {
      std::ofstream f(path);
      const double w = 2 * half / (nm - 1);
      for (int ix = 0; ix < nm; ++ix)
        for (int iy = 0; iy < nm; ++iy)
          for (int iz = 0; iz < nm; ++iz) {
            const float *v = &grid[4 * (((size_t)iz * nm + iy) * nm + ix)];
            f << (-half + ix * w) << " " << (-half + iy * w) << " " << (-half + iz * w) << " "
              << v[0] / Acts::kTesla << " " << v[1] / Acts::kTesla << " " << v[2] / Acts::kTesla
              << "\n";
          }
    }
    Acts::InterpolatedBFieldMap map(path);
    kf_field_t hostMap{};
    float *host = nullptr;
    if (kf_field_map_read_xyz(path.c_str(), 1., Acts::kTesla, 0, &hostMap, &host) != 0) rc = 6;
    std::remove(path.c_str());
    if (!rc) rc = run("field map from a text file", map, map.field(), host, 0.0, mismatches);
    kf_field_map_free(host);
  }
  if (rc) {
    std::printf("run failed: %d\n", rc);
    return rc;
  }
  std::printf("mismatches=%ld\n", mismatches);
  return mismatches == 0 ? 0 : 5;
}
