// kf_io.cpp — output files of the fit (gb300kf_io.h): the reference driver's
// writers (Run/Common/Writer.hpp) without ROOT.
//
// Tracks are formatted in parallel chunks (OpenMP) into memory and written in
// track order, so a million-track file costs a fraction of a second instead of
// one stream insertion per number.  Every number goes through "%g", which is
// what a default-formatted std::ostream prints for a double (precision 6).
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <string>
#include <vector>

#include "gb300kf_io.h"

namespace kfh {
char *errorBuffer(); // kf_capi.cu: the text behind kf_last_error_string()
}

namespace {

constexpr int64_t kChunk = 8192; // tracks formatted per task
constexpr int kDiag[6] = {0, 6, 11, 15, 18, 20}; // diagonal of the upper triangle

int32_t invalid(const char *what) {
  std::snprintf(kfh::errorBuffer(), 512, "invalid argument: %s", what);
  return KF_ERR_INVALID_ARGUMENT;
}

int32_t ioError(const char *path, const char *what) {
  std::snprintf(kfh::errorBuffer(), 512, "%s %s: %s", what, path, std::strerror(errno));
  return KF_ERR_IO;
}

void put(std::string &s, const char *fmt, double v) {
  char b[40];
  const int k = std::snprintf(b, sizeof(b), fmt, v);
  s.append(b, (size_t)k);
}
void putG(std::string &s, double v) { put(s, "%g", v); }
void putI(std::string &s, long long v) {
  char b[24];
  const int k = std::snprintf(b, sizeof(b), "%lld", v);
  s.append(b, (size_t)k);
}

// file body = header + chunks formatted by body(chunk, out) in parallel,
// written in chunk order
template <class Body>
int32_t writeChunked(const char *path, const std::string &header, int64_t n, Body body) {
  FILE *f = std::fopen(path, "wb");
  if (!f) return ioError(path, "cannot open");
  bool ok = std::fwrite(header.data(), 1, header.size(), f) == header.size();
  const int64_t nChunks = (n + kChunk - 1) / kChunk;
  const int64_t wave = 64; // chunks formatted between writes (bounds the memory)
  std::vector<std::string> text((size_t)std::min<int64_t>(nChunks, wave));
  for (int64_t c0 = 0; ok && c0 < nChunks; c0 += wave) {
    const int64_t c1 = std::min(nChunks, c0 + wave);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t c = c0; c < c1; ++c) {
      std::string &s = text[(size_t)(c - c0)];
      s.clear();
      body(c * kChunk, std::min(n, (c + 1) * kChunk), s);
    }
    for (int64_t c = c0; ok && c < c1; ++c) {
      const std::string &s = text[(size_t)(c - c0)];
      ok = std::fwrite(s.data(), 1, s.size(), f) == s.size();
    }
  }
  if (std::fclose(f) != 0) ok = false;
  return ok ? 0 : ioError(path, "cannot write");
}

// plane of the k-th state of a track with this hit mask (k-th set bit)
int planeOfState(uint64_t mask, int k) {
  for (int j = 0; j < k; ++j) mask &= mask - 1;
  return mask ? __builtin_ctzll(mask) : -1;
}

bool strided(int64_t n, int64_t stride) { return n >= 0 && stride >= n; }

// bits of the planes 0..S-1 of a sequence
uint64_t planeBits(int S) { return S >= 64 ? ~0ull : ((1ull << S) - 1); }

// obj vertex numbering of the reference writers: the counter advances by one
// before a track's vertices and then along its line segments, so a track of
// c >= 1 vertices starts at (previous end + 1) and ends c - 1 further, and a
// track of no vertices still advances it by one.  start[i] = first index of
// the i-th track (0 = not written), from the per-track vertex counts.
std::vector<int64_t> objStarts(const std::vector<int32_t> &count, const std::vector<char> &written) {
  std::vector<int64_t> start(count.size(), 0);
  int64_t v = 0;
  for (size_t i = 0; i < count.size(); ++i) {
    if (!written[i]) continue;
    start[i] = ++v;
    if (count[i] > 1) v += count[i] - 1;
  }
  return start;
}

void putVertex(std::string &s, double x, double y, double z) {
  s += "v ";
  putG(s, x);
  s += ' ';
  putG(s, y);
  s += ' ';
  putG(s, z);
  s += '\n';
}

void putLines(std::string &s, int64_t first, int32_t count) {
  for (int64_t a = first; a < first + count - 1; ++a) {
    s += "l ";
    putI(s, a);
    s += ' ';
    putI(s, a + 1);
    s += '\n';
  }
}

} // namespace

extern "C" {

int32_t kf_write_params_csv(const char *path, const double *params, const int32_t *status,
                            int64_t n, int64_t stride) {
  if (!path || !params || !status || !strided(n, stride)) return invalid("kf_write_params_csv");
  const std::string header = "trackIdx, fit_BoundLoc0, fit_BoundLoc1, fit_BoundPhi, "
                             "fit_BoundTheta, fit_BoundQOverP, fit_BoundTime\n";
  return writeChunked(path, header, n, [&](int64_t i0, int64_t i1, std::string &s) {
    for (int64_t i = i0; i < i1; ++i) {
      if (status[i] != KF_TRACK_OK) continue;
      putI(s, i);
      for (int r = 0; r < 6; ++r) {
        s += ',';
        putG(s, params[r * stride + i]);
      }
      s += '\n';
    }
  });
}

int32_t kf_write_states_obj(const char *path, const double *smoothed, const int32_t *n_meas,
                            const uint64_t *hit_mask, const int32_t *status, int64_t n,
                            int64_t stride, const kf_geometry_t *geo) {
  if (!path || !smoothed || !n_meas || !status || !geo || !geo->center || !geo->rotation ||
      geo->n_planes < 1 || geo->n_planes > KF_MAX_PLANES || !strided(n, stride))
    return invalid("kf_write_states_obj");
  const int S = geo->n_planes;
  std::vector<int32_t> count((size_t)n);
  std::vector<char> written((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    written[i] = status[i] == KF_TRACK_OK;
    int c = std::min(n_meas[i], S);
    if (hit_mask) c = std::min(c, __builtin_popcountll(hit_mask[i] & planeBits(S)));
    count[i] = std::max(0, c);
  }
  const std::vector<int64_t> start = objStarts(count, written);
  return writeChunked(path, std::string(), n, [&](int64_t i0, int64_t i1, std::string &s) {
    for (int64_t i = i0; i < i1; ++i) {
      if (!written[i]) continue;
      for (int k = 0; k < count[i]; ++k) {
        const int pl = hit_mask ? planeOfState(hit_mask[i] & planeBits(S), k) : k;
        const double l0 = smoothed[((int64_t)k * 27 + 0) * stride + i];
        const double l1 = smoothed[((int64_t)k * 27 + 1) * stride + i];
        const double *c = geo->center + 3 * pl;
        const double *R = geo->rotation + 9 * pl;
        // PlaneSurface::localToGlobal: R (l0, l1, 0) + centre
        putVertex(s, (R[0] * l0 + R[1] * l1 + R[2] * 0.0) + c[0],
                  (R[3] * l0 + R[4] * l1 + R[5] * 0.0) + c[1],
                  (R[6] * l0 + R[7] * l1 + R[8] * 0.0) + c[2]);
      }
      putLines(s, start[i], count[i]);
    }
  });
}

int32_t kf_write_hits_obj(const char *path, const double *positions, const uint64_t *hit_mask,
                          const int32_t *n_hits, int32_t S, int64_t n, int64_t stride) {
  if (!path || !positions || S < 1 || S > KF_MAX_PLANES || !strided(n, stride))
    return invalid("kf_write_hits_obj");
  std::vector<int32_t> count((size_t)n);
  std::vector<char> written((size_t)n, 1);
  for (int64_t i = 0; i < n; ++i) {
    int c = n_hits ? n_hits[i] : S;
    if (hit_mask) c = std::min(c, __builtin_popcountll(hit_mask[i] & planeBits(S)));
    count[i] = std::max(0, std::min(c, S));
  }
  const std::vector<int64_t> start = objStarts(count, written);
  return writeChunked(path, std::string(), n, [&](int64_t i0, int64_t i1, std::string &s) {
    for (int64_t i = i0; i < i1; ++i) {
      for (int k = 0; k < count[i]; ++k) {
        const int64_t pl = hit_mask ? planeOfState(hit_mask[i] & planeBits(S), k) : k;
        putVertex(s, positions[(pl * 3 + 0) * stride + i], positions[(pl * 3 + 1) * stride + i],
                  positions[(pl * 3 + 2) * stride + i]);
      }
      putLines(s, start[i], count[i]);
    }
  });
}

int32_t kf_write_params_table(const char *path, const double *params, const double *cov,
                              const int32_t *status, const double *truth, const double *vertex,
                              int64_t n, int64_t stride) {
  if (!path || !params || !cov || !status || !truth || !vertex || !strided(n, stride))
    return invalid("kf_write_params_table");
  static const char *kPar[6] = {"eLOC0", "eLOC1", "ePHI", "eTHETA", "eQOP", "eT"};
  std::string header = "t_charge,t_time,t_vx,t_vy,t_vz,t_px,t_py,t_pz,t_theta,t_phi,t_eta,t_pT";
  for (const char *pre : {"", "err_"})
    for (int r = 0; r < 6; ++r) header += std::string(",") + pre + kPar[r] + "_fit";
  for (const char *pre : {"res_", "pull_"})
    for (int r = 0; r < 6; ++r) header += std::string(",") + pre + kPar[r];
  header += '\n';
  return writeChunked(path, header, n, [&](int64_t i0, int64_t i1, std::string &s) {
    for (int64_t i = i0; i < i1; ++i) {
      if (status[i] != KF_TRACK_OK) continue;
      // the truth particle (writeParamsRoot, Writer.hpp:199-213)
      const double qop = truth[4 * stride + i], phi0 = truth[2 * stride + i],
                   th0 = truth[3 * stride + i];
      const int charge = qop > 0 ? 1 : -1;
      const double p = std::fabs(1.0 / qop);
      const double d[3] = {std::cos(phi0) * std::sin(th0), std::sin(phi0) * std::sin(th0),
                           std::cos(th0)};
      const double perp = std::sqrt(d[0] * d[0] + d[1] * d[1]);
      const double theta = std::atan2(perp, d[2]);
      const double phi = std::atan2(d[1], d[0]);
      const double eta = std::atanh(d[2] / std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]));
      const double time = truth[5 * stride + i];
      putI(s, charge);
      for (double v : {time, vertex[i], vertex[stride + i], vertex[2 * stride + i], p * d[0],
                       p * d[1], p * d[2], theta, phi, eta, p * perp}) {
        s += ',';
        putG(s, v);
      }
      // truth parameters (Writer.hpp:215-216) and the fit's fit / err / res /
      // pull (:217-222)
      const double tp[6] = {truth[i], truth[stride + i], phi, theta, charge / p, time};
      double fit[6], err[6], res[6], pull[6];
      for (int r = 0; r < 6; ++r) {
        fit[r] = params[r * stride + i];
        err[r] = std::sqrt(cov[kDiag[r] * stride + i]);
        res[r] = fit[r] - tp[r];
        pull[r] = res[r] / err[r];
      }
      for (const double *row : {fit, err, res, pull})
        for (int r = 0; r < 6; ++r) {
          s += ',';
          putG(s, row[r]);
        }
      s += '\n';
    }
  });
}

} // extern "C"
