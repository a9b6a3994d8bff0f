"""The oracle of field-map ingestion (test infrastructure): the reference's
map construction and lookup restated in numpy, independent of the library's
reader.  Only tests/ use it.

- parse: BField::txt::fieldMapperXYZ / fieldMapperRZ (src/Plugins/
  BFieldUtils.cpp:35-49, :75-93): skip empty lines, lines starting with '%'
  or '#', and lines of spaces; read the numbers of each remaining line.
- grid: Acts::fieldMapperXYZ / fieldMapperRZ (src/MagneticField/
  BFieldMapUtils.cpp:17-240): per axis the sorted unique coordinates, n bins
  over [min, max + step) (mirrored: 2n - 1 bins over [-max, max + step)),
  bin b holding the file row localToGlobalBin(b) = (ix * ny + iy) * nz + iz
  (src/Plugins/BFieldOptions.cpp:44-47) of the possibly mirrored index
  |b + 1 - n|, values times the field unit; bins outside the range zero.
- lookup: InterpolatedBFieldMapper::getField (include/MagneticField/
  InterpolatedBFieldMap.hpp:178-210) with detail::interpolate_impl
  (include/Utilities/detail/interpolation_impl.hpp): the bin of the
  position, its lower and upper edges, linear interpolation over the last
  axis first; for RZ then (br cos phi, br sin phi, bz).
"""
from __future__ import annotations

import numpy as np


def parse(path, cols: int) -> np.ndarray:
    rows = []
    with open(path) as f:
        for line in f:
            line = line.rstrip("\n")
            if not line or line[0] in "%#" or line.strip(" \t\r") == "":
                continue
            rows.append([float(t) for t in line.split()[:cols]])
    return np.array(rows, dtype=np.float64).reshape(-1, cols)


class _Axis:
    def __init__(self, pts: np.ndarray, mirror: bool, unit: float):
        u = np.unique(pts)
        self.n_file = len(u)
        mn, mx = u[0], u[-1]
        step = abs(mx - mn) / (len(u) - 1)
        lo, hi = mn, mx + step
        self.n = len(u)
        if mirror:
            lo = -mx
            self.n = 2 * len(u) - 1
        self.lo, self.hi = lo * unit, hi * unit
        self.mirror = mirror

    @property
    def width(self) -> float:
        return (self.hi - self.lo) / self.n

    def file_index(self, b: int) -> int:
        return abs(b + 1 - self.n_file) if self.mirror else b

    def bin(self, x: float) -> int:
        return int(np.floor((x - self.lo) / self.width))

    def edges(self, b: int):
        return self.lo + b * self.width, self.lo + (b + 1) * self.width


class MapXYZ:
    """The reference's 3D map from an XYZ file."""

    def __init__(self, path, length_unit=1.0, field_unit=1.0, first_octant=False):
        rows = parse(path, 6)
        self.ax = [_Axis(rows[:, a], first_octant, length_unit) for a in range(3)]
        nf = [a.n_file for a in self.ax]
        self.values = rows[:, 3:6] * field_unit
        self.nf = nf

    def bin_value(self, b) -> np.ndarray:
        if any(b[a] < 0 or b[a] >= self.ax[a].n for a in range(3)):
            return np.zeros(3)
        i, j, k = (self.ax[a].file_index(b[a]) for a in range(3))
        return self.values[(i * self.nf[1] + j) * self.nf[2] + k]

    def field(self, pos) -> np.ndarray:
        b = [self.ax[a].bin(pos[a]) for a in range(3)]
        lo = [self.ax[a].edges(b[a])[0] for a in range(3)]
        hi = [self.ax[a].edges(b[a])[1] for a in range(3)]
        # corners in the order (x, y, z) with z fastest; reduce z, then y, then x
        c = np.array([[[self.bin_value((b[0] + i, b[1] + j, b[2] + k)) for k in (0, 1)]
                       for j in (0, 1)] for i in (0, 1)])
        for d in (2, 1, 0):
            f = (pos[d] - lo[d]) / (hi[d] - lo[d])
            c = (1 - f) * np.take(c, 0, axis=d) + f * np.take(c, 1, axis=d)
        return c


class MapRZ:
    """The reference's 2D (r, z) map from an RZ file."""

    def __init__(self, path, length_unit=1.0, field_unit=1.0, first_quadrant=False):
        rows = parse(path, 4)
        self.ar = _Axis(rows[:, 0], False, length_unit)
        self.az = _Axis(rows[:, 1], first_quadrant, length_unit)
        self.values = rows[:, 2:4] * field_unit

    def bin_value(self, br: int, bz: int) -> np.ndarray:
        if br < 0 or br >= self.ar.n or bz < 0 or bz >= self.az.n:
            return np.zeros(2)
        return self.values[br * self.az.n_file + self.az.file_index(bz)]

    def field(self, pos) -> np.ndarray:
        x, y, z = pos
        r2 = x * x + y * y
        r = np.sqrt(r2)
        br, bz = self.ar.bin(r), self.az.bin(z)
        r0, r1 = self.ar.edges(br)
        z0, z1 = self.az.edges(bz)
        fz = (z - z0) / (z1 - z0)
        fr = (r - r0) / (r1 - r0)
        a0 = (1 - fz) * self.bin_value(br, bz) + fz * self.bin_value(br, bz + 1)
        a1 = (1 - fz) * self.bin_value(br + 1, bz) + fz * self.bin_value(br + 1, bz + 1)
        b = (1 - fr) * a0 + fr * a1
        if r2 > np.finfo(np.float64).tiny:
            cphi, sphi = x / r, y / r
        else:
            cphi, sphi = 1.0, 0.0
        return np.array([b[0] * cphi, b[0] * sphi, b[1]])


def trilinear(grid: np.ndarray, dims, mn, mx, pos) -> np.ndarray:
    """The fitter's lookup of a kf_field_t grid ([nz][ny][nx][4], points
    spanning [min, max]) at one position, in double."""
    idx, f = [], []
    for a in range(3):
        g = (pos[a] - mn[a]) * (dims[a] - 1) / (mx[a] - mn[a])
        i = min(max(int(np.floor(g)), 0), dims[a] - 2)
        idx.append(i)
        f.append(g - i)
    g3 = grid.reshape(dims[2], dims[1], dims[0], 4).astype(np.float64)
    c = g3[idx[2]:idx[2] + 2, idx[1]:idx[1] + 2, idx[0]:idx[0] + 2, :3]  # [z][y][x]
    for d, w in ((2, f[0]), (1, f[1]), (0, f[2])):
        c = (1 - w) * np.take(c, 0, axis=d) + w * np.take(c, 1, axis=d)
    return c
