// kf_fieldmap.cpp — text field maps into the fitter's grid
// (gb300kf_fieldmap.h).  Host code.
//
// The reference builds an Acts::detail::Grid from the file's points
// (src/MagneticField/BFieldMapUtils.cpp:17-240): per axis the sorted unique
// coordinates give the bin count n and the range [min, max + step), where
// step = (max - min) / (n - 1); each point is the lower edge of its bin; the
// bins outside the range hold zero.  Its lookup interpolates between a
// bin's lower corner and the next bin's (the overflow bin's zero above the
// last point).  The fitter's kf_field_t grid interpolates between n points
// spanning [min, max]; so the grid built here has the file's points plus one
// zero plane at max + step per axis, spanning [min, max + step] with the
// reference's bin width.
#include <algorithm>
#include <cerrno>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gb300kf_fieldmap.h"

namespace kfh {
char *errorBuffer(); // kf_capi.cu: the text behind kf_last_error_string()
}

namespace {

int32_t fail(int32_t code, const char *path, long line, const char *what) {
  if (line > 0)
    std::snprintf(kfh::errorBuffer(), 512, "%s:%ld: %s", path, line, what);
  else
    std::snprintf(kfh::errorBuffer(), 512, "%s: %s", path, what);
  return code;
}

// rows of `cols` numbers from a map file (BFieldUtils.cpp:35-49, :75-93):
// skips empty and blank lines and lines starting with '%' or '#'
int32_t readRows(const char *path, int cols, std::vector<double> &v) {
  FILE *f = std::fopen(path, "rb");
  if (!f) {
    std::snprintf(kfh::errorBuffer(), 512, "cannot open %s: %s", path, std::strerror(errno));
    return KF_ERR_IO;
  }
  std::fseek(f, 0, SEEK_END);
  const long size = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  std::string text(size > 0 ? (size_t)size : 0, '\0');
  const bool ok = size <= 0 || std::fread(&text[0], 1, (size_t)size, f) == (size_t)size;
  std::fclose(f);
  if (!ok) return fail(KF_ERR_IO, path, 0, "read error");
  v.clear();
  v.reserve((size_t)(size / 12) + 16);
  const char *p = text.c_str(), *end = p + text.size();
  long line = 0;
  while (p < end) {
    ++line;
    const char *eol = static_cast<const char *>(std::memchr(p, '\n', (size_t)(end - p)));
    if (!eol) eol = end;
    const char *q = p;
    while (q < eol && (*q == ' ' || *q == '\t' || *q == '\r')) ++q;
    if (q < eol && p[0] != '%' && p[0] != '#') {
      for (int c = 0; c < cols; ++c) {
        char *next = nullptr;
        const double x = std::strtod(q, &next);
        if (next == q || next > eol)
          return fail(KF_ERR_INVALID_ARGUMENT, path, line, "expected a number");
        v.push_back(x);
        q = next;
      }
    }
    p = eol + 1;
  }
  return 0;
}

// sorted unique coordinates of column c
std::vector<double> axisPoints(const std::vector<double> &v, int cols, int c) {
  std::vector<double> a;
  a.reserve(v.size() / cols);
  for (size_t i = c; i < v.size(); i += cols) a.push_back(v[i]);
  std::sort(a.begin(), a.end());
  a.erase(std::unique(a.begin(), a.end()), a.end());
  return a;
}

// The reference's equidistant axis of one coordinate (BFieldMapUtils.cpp:
// 47-66, 158-188): file points `pts`, mirrored to -max when `mirror`.
struct Axis {
  int nFile;     // distinct coordinates in the file
  int nBins;     // bins of the reference's axis (2 nFile - 1 mirrored)
  double lo, hi; // its range (length units applied), hi = max + step
  double width() const { return (hi - lo) / nBins; }
};

int32_t makeAxis(const char *path, const std::vector<double> &pts, bool mirror, double unit,
                 const char *name, Axis &ax) {
  if (pts.size() < 2) {
    char m[96];
    std::snprintf(m, sizeof(m), "axis %s has fewer than two distinct points", name);
    return fail(KF_ERR_INVALID_ARGUMENT, path, 0, m);
  }
  const double mn = pts.front(), mx = pts.back();
  const double step = std::fabs(mx - mn) / (double)(pts.size() - 1);
  ax.nFile = (int)pts.size();
  ax.nBins = ax.nFile;
  double lo = mn, hi = mx + step;
  if (mirror) {
    if (mn != 0.0) {
      char m[96];
      std::snprintf(m, sizeof(m), "mirrored axis %s must start at 0", name);
      return fail(KF_ERR_INVALID_ARGUMENT, path, 0, m);
    }
    lo = -mx;
    ax.nBins = 2 * ax.nFile - 1;
  }
  ax.lo = lo * unit;
  ax.hi = hi * unit;
  return 0;
}

// file row of local bin b (0-based) of a possibly mirrored axis
// (BFieldMapUtils.cpp:84-96, 206-224)
inline int fileIndex(const Axis &ax, int b, bool mirror) {
  return mirror ? std::abs(b + 1 - ax.nFile) : b;
}

// kf_field_t over the reference's bins plus the zero plane above the last
// bin: point i at lo + i * width, i = 0..nBins
void describe(kf_field_t *field, const Axis ax[3]) {
  std::memset(field, 0, sizeof(*field));
  field->kind = KF_FIELD_GRID3D;
  int *n[3] = {&field->nx, &field->ny, &field->nz};
  for (int a = 0; a < 3; ++a) {
    *n[a] = ax[a].nBins + 1;
    field->min[a] = ax[a].lo;
    field->max[a] = ax[a].hi;
  }
  field->scale = 1.0;
  field->grid = nullptr;
}

float *allocGrid(const kf_field_t *field) {
  const size_t n = (size_t)field->nx * field->ny * field->nz * 4;
  float *g = static_cast<float *>(std::calloc(n, sizeof(float)));
  return g;
}

} // namespace

extern "C" {

int32_t kf_field_map_read_xyz(const char *path, double length_unit, double field_unit,
                              int32_t first_octant, kf_field_t *field, float **grid_host) {
  if (!path || !field || !grid_host || !(length_unit > 0) || !std::isfinite(field_unit))
    return fail(KF_ERR_INVALID_ARGUMENT, path ? path : "(null)", 0, "invalid argument");
  *grid_host = nullptr;
  std::vector<double> v;
  if (int32_t rc = readRows(path, 6, v)) return rc;
  const bool mirror = first_octant != 0;
  Axis ax[3];
  std::vector<double> pts[3];
  static const char *names[3] = {"x", "y", "z"};
  for (int a = 0; a < 3; ++a) {
    pts[a] = axisPoints(v, 6, a);
    if (int32_t rc = makeAxis(path, pts[a], mirror, length_unit, names[a], ax[a])) return rc;
  }
  const size_t rows = v.size() / 6;
  const size_t nx = ax[0].nFile, ny = ax[1].nFile, nz = ax[2].nFile;
  if (rows != nx * ny * nz) {
    char m[160];
    std::snprintf(m, sizeof(m), "%zu points, but the axes have %zu x %zu x %zu", rows, nx, ny,
                  nz);
    return fail(KF_ERR_INVALID_ARGUMENT, path, 0, m);
  }
  // row (ix * ny + iy) * nz + iz must sit at (x_ix, y_iy, z_iz): the order
  // the reference's localToGlobalBin assumes (BFieldOptions.cpp:44-47)
  for (size_t ix = 0; ix < nx; ++ix)
    for (size_t iy = 0; iy < ny; ++iy)
      for (size_t iz = 0; iz < nz; ++iz) {
        const double *r = &v[((ix * ny + iy) * nz + iz) * 6];
        if (r[0] != pts[0][ix] || r[1] != pts[1][iy] || r[2] != pts[2][iz]) {
          char m[160];
          std::snprintf(m, sizeof(m),
                        "point %zu is out of order (x slowest, z fastest expected)",
                        (ix * ny + iy) * nz + iz);
          return fail(KF_ERR_INVALID_ARGUMENT, path, 0, m);
        }
      }
  describe(field, ax);
  float *g = allocGrid(field);
  if (!g) return fail(KF_ERR_INVALID_ARGUMENT, path, 0, "out of host memory");
  const size_t gx = field->nx, gxy = (size_t)field->nx * field->ny;
  for (int k = 0; k < ax[2].nBins; ++k)
    for (int j = 0; j < ax[1].nBins; ++j)
      for (int i = 0; i < ax[0].nBins; ++i) {
        const size_t row = ((size_t)fileIndex(ax[0], i, mirror) * ny +
                            fileIndex(ax[1], j, mirror)) * nz + fileIndex(ax[2], k, mirror);
        float *o = g + 4 * ((size_t)k * gxy + (size_t)j * gx + i);
        for (int c = 0; c < 3; ++c) o[c] = (float)(v[row * 6 + 3 + c] * field_unit);
      }
  *grid_host = g;
  return 0;
}

} // extern "C"

namespace {
// An (r, z) map file: its rows, and the reference's r and z axes (r never
// mirrored, BFieldMapUtils.cpp:61-64 mirrors z only), checked for the
// reference's point order (r slowest, z fastest).
int32_t readRZ(const char *path, double length_unit, bool mirror, std::vector<double> &v,
               std::vector<double> &pr, std::vector<double> &pz, Axis &ar, Axis &az) {
  if (int32_t rc = readRows(path, 4, v)) return rc;
  pr = axisPoints(v, 4, 0);
  pz = axisPoints(v, 4, 1);
  if (int32_t rc = makeAxis(path, pr, false, length_unit, "r", ar)) return rc;
  if (int32_t rc = makeAxis(path, pz, mirror, length_unit, "z", az)) return rc;
  const size_t rows = v.size() / 4, nr = ar.nFile, nz = az.nFile;
  if (rows != nr * nz) {
    char m[160];
    std::snprintf(m, sizeof(m), "%zu points, but the axes have %zu x %zu", rows, nr, nz);
    return fail(KF_ERR_INVALID_ARGUMENT, path, 0, m);
  }
  for (size_t ir = 0; ir < nr; ++ir)
    for (size_t iz = 0; iz < nz; ++iz) {
      const double *r = &v[(ir * nz + iz) * 4];
      if (r[0] != pr[ir] || r[1] != pz[iz]) {
        char m[160];
        std::snprintf(m, sizeof(m), "point %zu is out of order (r slowest, z fastest expected)",
                      ir * nz + iz);
        return fail(KF_ERR_INVALID_ARGUMENT, path, 0, m);
      }
    }
  return 0;
}
} // namespace

extern "C" {

int32_t kf_field_map_read_rz_native(const char *path, double length_unit, double field_unit,
                                    int32_t first_quadrant, kf_field_t *field,
                                    float **grid_host) {
  if (!path || !field || !grid_host || !(length_unit > 0) || !std::isfinite(field_unit))
    return fail(KF_ERR_INVALID_ARGUMENT, path ? path : "(null)", 0, "invalid argument");
  *grid_host = nullptr;
  const bool mirror = first_quadrant != 0;
  std::vector<double> v, pr, pz;
  Axis ar, az;
  if (int32_t rc = readRZ(path, length_unit, mirror, v, pr, pz, ar, az)) return rc;
  const size_t nzFile = az.nFile;
  // the reference's bins plus the zero row above the last bin on each axis:
  // point i at lo + i * width, i = 0..nBins
  std::memset(field, 0, sizeof(*field));
  field->kind = KF_FIELD_GRID_RZ;
  field->nx = ar.nBins + 1;
  field->ny = 1;
  field->nz = az.nBins + 1;
  field->min[0] = ar.lo;
  field->max[0] = ar.hi;
  field->min[2] = az.lo;
  field->max[2] = az.hi;
  field->scale = 1.0;
  const size_t nPts = (size_t)field->nx * field->nz;
  float *g = static_cast<float *>(std::calloc(nPts * 4, sizeof(float)));
  if (!g) return fail(KF_ERR_INVALID_ARGUMENT, path, 0, "out of host memory");
  for (int iz = 0; iz < az.nBins; ++iz)
    for (int ir = 0; ir < ar.nBins; ++ir) {
      const size_t row = (size_t)ir * nzFile + fileIndex(az, iz, mirror);
      float *o = g + 4 * ((size_t)iz * field->nx + ir);
      o[0] = (float)(v[row * 4 + 2] * field_unit);
      o[1] = (float)(v[row * 4 + 3] * field_unit);
    }
  *grid_host = g;
  return 0;
}

int32_t kf_field_map_read_rz(const char *path, double length_unit, double field_unit,
                             int32_t first_quadrant, const int32_t *n_xyz, const double *min_xyz,
                             const double *max_xyz, kf_field_t *field, float **grid_host) {
  if (!path || !field || !grid_host || !(length_unit > 0) || !std::isfinite(field_unit))
    return fail(KF_ERR_INVALID_ARGUMENT, path ? path : "(null)", 0, "invalid argument");
  *grid_host = nullptr;
  std::vector<double> v, pr, pz;
  const bool mirror = first_quadrant != 0;
  Axis ar, az;
  if (int32_t rc = readRZ(path, length_unit, mirror, v, pr, pz, ar, az)) return rc;
  const size_t nr = ar.nFile, nz = az.nFile;
  (void)nr;
  // the reference's 2D grid: bins 0..nBins-1 per axis, zero outside
  auto value = [&](int br, int bz, int c) -> double {
    if (br < 0 || br >= ar.nBins || bz < 0 || bz >= az.nBins) return 0.0;
    const size_t row = (size_t)br * nz + fileIndex(az, bz, mirror);
    return v[row * 4 + 2 + c] * field_unit;
  };
  const double wr = ar.width(), wz = az.width();
  // (r, z) -> (br, bz): the bin of the position, its edges, and the
  // interpolation over z and then r (Utilities/detail/interpolation_impl.hpp)
  auto lookup = [&](double r, double z, double out[2]) {
    const int br = (int)std::floor((r - ar.lo) / wr), bz = (int)std::floor((z - az.lo) / wz);
    const double r0 = ar.lo + br * wr, r1 = ar.lo + (br + 1) * wr;
    const double z0 = az.lo + bz * wz, z1 = az.lo + (bz + 1) * wz;
    const double fz = (z - z0) / (z1 - z0), fr = (r - r0) / (r1 - r0);
    for (int c = 0; c < 2; ++c) {
      const double a0 = (1 - fz) * value(br, bz, c) + fz * value(br, bz + 1, c);
      const double a1 = (1 - fz) * value(br + 1, bz, c) + fz * value(br + 1, bz + 1, c);
      out[c] = (1 - fr) * a0 + fr * a1;
    }
  };
  int32_t n[3];
  double mn[3], mx[3];
  if (n_xyz) {
    if (!min_xyz || !max_xyz)
      return fail(KF_ERR_INVALID_ARGUMENT, path, 0, "n_xyz given without min_xyz / max_xyz");
    for (int a = 0; a < 3; ++a) {
      n[a] = n_xyz[a];
      mn[a] = min_xyz[a];
      mx[a] = max_xyz[a];
      if (n[a] < 2 || !(mx[a] > mn[a]))
        return fail(KF_ERR_INVALID_ARGUMENT, path, 0, "invalid Cartesian grid");
    }
  } else {
    // x, y over [-r_max, r_max] at the r step, z over the map's z range
    const double rmax = pr.back() * length_unit;
    const int nrr = (int)nr - 1;
    n[0] = n[1] = 2 * nrr + 1;
    mn[0] = mn[1] = -rmax;
    mx[0] = mx[1] = rmax;
    n[2] = az.nBins;
    mn[2] = az.lo;
    mx[2] = az.lo + (az.nBins - 1) * wz;
  }
  std::memset(field, 0, sizeof(*field));
  field->kind = KF_FIELD_GRID3D;
  field->nx = n[0];
  field->ny = n[1];
  field->nz = n[2];
  for (int a = 0; a < 3; ++a) {
    field->min[a] = mn[a];
    field->max[a] = mx[a];
  }
  field->scale = 1.0;
  float *g = allocGrid(field);
  if (!g) return fail(KF_ERR_INVALID_ARGUMENT, path, 0, "out of host memory");
  for (int k = 0; k < n[2]; ++k) {
    const double z = mn[2] + k * (mx[2] - mn[2]) / (n[2] - 1);
    for (int j = 0; j < n[1]; ++j) {
      const double y = mn[1] + j * (mx[1] - mn[1]) / (n[1] - 1);
      for (int i = 0; i < n[0]; ++i) {
        const double x = mn[0] + i * (mx[0] - mn[0]) / (n[0] - 1);
        // transformPos (x, y, z) -> (perp, z) and transformBField
        // (BFieldMapUtils.cpp:101-127)
        const double r2 = x * x + y * y;
        double cphi = 1.0, sphi = 0.0;
        if (r2 > DBL_MIN) {
          const double inv = 1.0 / std::sqrt(r2);
          cphi = x * inv;
          sphi = y * inv;
        }
        double b[2];
        lookup(std::sqrt(r2), z, b);
        float *o = g + 4 * (((size_t)k * n[1] + j) * n[0] + i);
        o[0] = (float)(b[0] * cphi);
        o[1] = (float)(b[0] * sphi);
        o[2] = (float)b[1];
      }
    }
  }
  *grid_host = g;
  return 0;
}

void kf_field_map_free(float *grid_host) { std::free(grid_host); }

} // extern "C"
