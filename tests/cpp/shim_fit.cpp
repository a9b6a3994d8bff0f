// Fits a synthetic telescope workload through the C++ drop-in shim
// (include/gb300kf/KalmanFitter.hpp) written in the reference fitter's call
// shape, and checks it against a direct kf_fit_batch_host call.
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>
#include <vector>

#include "../../include/gb300kf/KalmanFitter.hpp"
#include "../../include/gb300kf_synth.h"

int main() {
  using namespace gb300kf;
  const int64_t n = 500;
  const int S = 10;
  kf_synth_config_t sc;
  kf_synth_config_default(&sc);
  sc.n_tracks = n;
  std::vector<double> center(3 * S), rot(9 * S), tc(3 * S), tr(9 * S);
  kf_synth_geometry(&sc, center.data(), rot.data(), tc.data(), tr.data(), nullptr);
  std::vector<double> meas((size_t)S * 5 * n), start(6 * n), scov(21 * n), per(3 * n);
  std::vector<uint64_t> mask(n);
  std::vector<int32_t> np(n);
  kf_synth_tracks(&sc, tc.data(), tr.data(), nullptr, meas.data(), mask.data(), np.data(),
                  start.data(), scov.data(), per.data(), nullptr, 0);

  // reference-style objects: planes at x = 100..1000 mm with normal +x
  std::vector<PlaneSurface> planes;
  for (int k = 0; k < S; ++k) {
    planes.emplace_back(Vector3D{100. * (k + 1), 0., 0.}, Vector3D{1., 0., 0.});
    planes.back().assignGeoID(GeometryID{(uint64_t)(1000 + k)});
  }
  std::vector<LineSurface> targets(n);
  std::vector<TrackInput> tracks(n);
  for (int64_t i = 0; i < n; ++i) {
    targets[i] = LineSurface(Vector3D{per[i], per[n + i], per[2 * n + i]});
    for (int k = S - 1; k >= 0; --k) { // any order: matched by geometry id
      const double *m = &meas[(size_t)k * 5 * n];
      tracks[i].sourcelinks.emplace_back(Vector2D{m[i], m[n + i]},
                                         SymMatrix2D{{{m[2 * n + i], m[3 * n + i]},
                                                      {m[3 * n + i], m[4 * n + i]}}},
                                         GeometryID{(uint64_t)(1000 + k)});
    }
    BoundVector p;
    BoundSymMatrix C{};
    for (int e = 0; e < 6; ++e) p[e] = start[e * n + i];
    int e = 0;
    for (int a = 0; a < 6; ++a)
      for (int b = a; b < 6; ++b) C[a][b] = C[b][a] = scov[(e++) * n + i];
    tracks[i].start = BoundParameters<LineSurface>(GeometryContext{}, C, p, &targets[i]);
  }
  PropagatorOptions popt;
  popt.overstepLimit = 0.1;
  KalmanFitter fitter(ConstantBField{}, popt);
  KalmanFitterOptions opt(GeometryContext{}, MagneticFieldContext{}, true);
  std::vector<KalmanFitterResult> res;
  fitter.fitBatch(tracks, opt, res, planes.data(), planes.size());

  // direct C ABI call on the same arrays
  kf_config_t cfg;
  kf_config_default(&cfg);
  cfg.overstep_limit = 0.1;
  kf_inputs_t in{};
  in.n_tracks = n;
  in.stride = n;
  in.n_surfaces = S;
  in.meas = meas.data();
  in.start_params = start.data();
  in.start_cov = scov.data();
  in.perigee = per.data();
  std::vector<double> oPar(6 * n), oCov(21 * n), oChi(n);
  std::vector<int32_t> oSt(n), oNm(n);
  kf_outputs_t out{};
  out.params = oPar.data();
  out.cov = oCov.data();
  out.chi2 = oChi.data();
  out.status = oSt.data();
  out.n_meas = oNm.data();
  kf_geometry_t geo{S, 0, center.data(), rot.data(), nullptr};
  kf_field_t field{};
  field.kind = KF_FIELD_CONSTANT;
  field.scale = 1.;
  field.value[2] = 2. * kTesla;
  void *dev = nullptr;
  const size_t bytes = kf_host_staging_size(&cfg, n, S, 0);
  if (cudaMalloc(&dev, bytes) != cudaSuccess) return 2;
  if (kf_fit_batch_host(&in, &out, &cfg, &geo, &field, dev, bytes, nullptr) != 0) return 3;
  cudaFree(dev);

  int bad = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (!res[i].result || oSt[i] != 0 || res[i].measurementStates != 10) ++bad;
    for (int e = 0; e < 6; ++e)
      if (res[i].fittedParameters.parameters()[e] != oPar[e * n + i]) ++bad;
    if (res[i].chi2 != oChi[i]) ++bad;
    if (res[i].fittedStates.size() != 10) ++bad;
  }
  // the single-track call gives the same answer as the batch
  KalmanFitterResult one;
  const bool ok = fitter.fit(tracks[7].sourcelinks, tracks[7].start, opt, one, planes.data(),
                             planes.size());
  if (!ok) ++bad;
  for (int e = 0; e < 6; ++e)
    if (one.fittedParameters.parameters()[e] != res[7].fittedParameters.parameters()[e]) ++bad;
  // the batched form (sorted queue, persistent kernel) gives the same fits
  KalmanFitterOptions bopt = opt;
  bopt.batched = true;
  std::vector<KalmanFitterResult> bres;
  fitter.fitBatch(tracks, bopt, bres, planes.data(), planes.size());
  for (int64_t i = 0; i < n; ++i) {
    if (bres[i].status != res[i].status || bres[i].chi2 != res[i].chi2) ++bad;
    for (int e = 0; e < 6; ++e)
      if (bres[i].fittedParameters.parameters()[e] != res[i].fittedParameters.parameters()[e]) ++bad;
  }
  // planes carrying 0.5 mm of silicon: the shim passes the slabs with the
  // reference's default scattering and energy-loss options
  std::vector<PlaneSurface> mplanes;
  std::vector<double> mat(6 * S);
  for (int k = 0; k < S; ++k) {
    mplanes.emplace_back(Vector3D{100. * (k + 1), 0., 0.}, Vector3D{1., 0., 0.},
                         MaterialSlab::silicon(0.5));
    mplanes.back().assignGeoID(GeometryID{(uint64_t)(1000 + k)});
    const MaterialSlab &m = mplanes.back().material();
    const double row[6] = {m.thickness, m.X0, m.L0, m.Ar, m.Z, m.molarDensity};
    for (int e = 0; e < 6; ++e) mat[6 * k + e] = row[e];
  }
  std::vector<KalmanFitterResult> mres;
  fitter.fitBatch(tracks, opt, mres, mplanes.data(), mplanes.size());
  kf_config_t mcfg = cfg;
  mcfg.material_effects = 3;
  kf_geometry_t mgeo{S, 0, center.data(), rot.data(), mat.data()};
  const size_t mbytes = kf_host_staging_size(&mcfg, n, S, 0);
  if (cudaMalloc(&dev, mbytes) != cudaSuccess) return 2;
  if (kf_fit_batch_host(&in, &out, &mcfg, &mgeo, &field, dev, mbytes, nullptr) != 0) return 4;
  cudaFree(dev);
  int changed = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (mres[i].status != oSt[i] || mres[i].chi2 != oChi[i]) ++bad;
    for (int e = 0; e < 6; ++e) {
      if (mres[i].fittedParameters.parameters()[e] != oPar[e * n + i]) ++bad;
      if (mres[i].fittedParameters.parameters()[e] != res[i].fittedParameters.parameters()[e]) ++changed;
    }
  }
  if (changed < n) ++bad; // the material must change the fits

  // a field map file ("x y z bx by bz" in mm and tesla, the driver's format):
  // the shim's InterpolatedBFieldMap against the C ABI reader and a direct call
  const char *tmp = std::getenv("TMPDIR");
  const std::string path = std::string(tmp ? tmp : "/tmp") + "/gb300kf_shim_map.txt";
  {
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) return 5;
    std::fprintf(f, "%% x y z bx by bz\n");
    for (int ix = 0; ix < 27; ++ix)
      for (int iy = 0; iy < 13; ++iy)
        for (int iz = 0; iz < 13; ++iz) {
          const double x = -100. + 50. * ix, y = -300. + 50. * iy, z = -300. + 50. * iz;
          std::fprintf(f, "%.17g %.17g %.17g %.17g %.17g %.17g\n", x, y, z, 1e-5 * z,
                       -1e-5 * y, 2.0 * (1. - 2e-5 * x));
        }
    std::fclose(f);
  }
  InterpolatedBFieldMap map(path);
  KalmanFitter mfitter(map, popt);
  std::vector<KalmanFitterResult> fres;
  mfitter.fitBatch(tracks, opt, fres, planes.data(), planes.size());
  kf_field_t mf;
  float *hgrid = nullptr;
  if (kf_field_map_read_xyz(path.c_str(), 1., kTesla, 0, &mf, &hgrid) != 0) return 6;
  const size_t gbytes = (size_t)mf.nx * mf.ny * mf.nz * 4 * sizeof(float);
  void *dgrid = nullptr;
  if (cudaMalloc(&dgrid, gbytes) != cudaSuccess) return 2;
  cudaMemcpy(dgrid, hgrid, gbytes, cudaMemcpyHostToDevice);
  kf_field_map_free(hgrid);
  mf.grid = static_cast<const float *>(dgrid);
  const size_t fbytes = kf_host_staging_size(&cfg, n, S, 0);
  if (cudaMalloc(&dev, fbytes) != cudaSuccess) return 2;
  if (kf_fit_batch_host(&in, &out, &cfg, &geo, &mf, dev, fbytes, nullptr) != 0) return 7;
  cudaFree(dev);
  cudaFree(dgrid);
  std::remove(path.c_str());
  int fitted = 0, moved = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (fres[i].status != oSt[i] || fres[i].chi2 != oChi[i]) ++bad;
    fitted += fres[i].result ? 1 : 0;
    for (int e = 0; e < 6; ++e) {
      if (fres[i].fittedParameters.parameters()[e] != oPar[e * n + i]) ++bad;
      if (fres[i].fittedParameters.parameters()[e] != res[i].fittedParameters.parameters()[e]) ++moved;
    }
  }
  if (fitted < n * 9 / 10 || moved < n) ++bad; // the map fits, and differently from 2 T

  // the reference writers' signatures: the same CSV as the C ABI writer on the
  // same numbers, and one obj vertex per smoothed state of a fitted track
  {
    const std::string csvA = std::string(tmp ? tmp : "/tmp") + "/gb300kf_shim_a.csv";
    const std::string csvB = std::string(tmp ? tmp : "/tmp") + "/gb300kf_shim_b.csv";
    const std::string obj = std::string(tmp ? tmp : "/tmp") + "/gb300kf_shim.obj";
    std::vector<BoundParameters<LineSurface>> fp(n);
    std::unique_ptr<bool[]> okv(new bool[n]);
    size_t states = 0, lines = 0;
    for (int64_t i = 0; i < n; ++i) {
      fp[i] = fres[i].fittedParameters;
      okv[i] = fres[i].result;
      if (fres[i].result) {
        states += fres[i].fittedStates.size();
        lines += fres[i].fittedStates.size() - 1;
      }
    }
    writeParamsCsv(fp.data(), okv.get(), (unsigned)n, csvA);
    if (kf_write_params_csv(csvB.c_str(), oPar.data(), oSt.data(), n, n) != 0) return 8;
    auto slurp = [](const std::string &f) {
      std::string t;
      FILE *h = std::fopen(f.c_str(), "rb");
      if (!h) return t;
      char buf[4096];
      size_t k;
      while ((k = std::fread(buf, 1, sizeof(buf), h)) > 0) t.append(buf, k);
      std::fclose(h);
      return t;
    };
    if (slurp(csvA).empty() || slurp(csvA) != slurp(csvB)) ++bad;
    writeStatesObj(fres.data(), (unsigned)n, planes.data(), (unsigned)planes.size(), obj);
    const std::string o = slurp(obj);
    size_t nv = 0, nl = 0;
    for (size_t k = 0; k + 1 < o.size(); ++k)
      if (k == 0 || o[k - 1] == '\n') {
        nv += o[k] == 'v';
        nl += o[k] == 'l';
      }
    if (nv != states || nl != lines) ++bad;
    std::remove(csvA.c_str());
    std::remove(csvB.c_str());
    std::remove(obj.c_str());
  }
  std::printf("shim tracks=%lld mismatches=%d\n", (long long)n, bad);
  return bad == 0 ? 0 : 1;
}
