"""Magnetic field maps from text files (gb300kf_fieldmap.h): the reference's
BField::txt::fieldMapperXYZ / fieldMapperRZ (src/Plugins/BFieldUtils.cpp)
and Acts::fieldMapperXYZ / fieldMapperRZ (src/MagneticField/BFieldMapUtils.cpp)
through the library's C ABI.

    fm = read_field_map_xyz("bfield.txt")          # "x y z bx by bz" in mm, T
    tel = make_telescope(n, field_map=fm)          # truth and fit in that map
    fm.device()                                    # torch tensor for kf_field_t.grid
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import TESLA, KfField, _check, load


@dataclass
class FieldMap:
    """A grid ready for kf_field_t: `grid` float32 [nz, ny, nx, 4] (host),
    `dims` (nx, ny, nz), `min` / `max` per axis in mm, `kind` the
    kf_field_kind (1: (x, y, z) grid; 2: (r, z) grid of (br, bz), ny = 1)."""
    grid: np.ndarray
    dims: tuple
    min: tuple
    max: tuple
    kind: int = 1

    def field(self, grid_ptr: int | None = None, scale: float = 1.0) -> KfField:
        f = KfField()
        f.kind = self.kind
        f.nx, f.ny, f.nz = self.dims
        for a in range(3):
            f.min[a], f.max[a] = self.min[a], self.max[a]
        f.scale = scale
        f.grid = grid_ptr if grid_ptr is not None else self.grid.ctypes.data
        return f

    def device(self, device: str = "cuda"):
        import torch
        return torch.from_numpy(self.grid.reshape(-1)).to(device)


def _lib() -> C.CDLL:
    lib = load()
    if not getattr(lib, "_fieldmap_bound", False):
        lib.kf_field_map_read_xyz.argtypes = [C.c_char_p, C.c_double, C.c_double, C.c_int32,
                                              C.POINTER(KfField), C.POINTER(C.c_void_p)]
        lib.kf_field_map_read_rz.argtypes = [C.c_char_p, C.c_double, C.c_double, C.c_int32,
                                             C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.POINTER(KfField), C.POINTER(C.c_void_p)]
        lib.kf_field_map_read_rz_native.argtypes = [C.c_char_p, C.c_double, C.c_double,
                                                    C.c_int32, C.POINTER(KfField),
                                                    C.POINTER(C.c_void_p)]
        lib.kf_field_map_read_xyz.restype = C.c_int32
        lib.kf_field_map_read_rz.restype = C.c_int32
        lib.kf_field_map_read_rz_native.restype = C.c_int32
        lib.kf_field_map_free.argtypes = [C.c_void_p]
        lib.kf_field_map_free.restype = None
        lib._fieldmap_bound = True
    return lib


def _take(lib, f: KfField, ptr: C.c_void_p) -> FieldMap:
    dims = (f.nx, f.ny, f.nz)
    n = dims[0] * dims[1] * dims[2] * 4
    try:
        grid = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_float)), shape=(n,)).copy()
    finally:
        lib.kf_field_map_free(ptr)
    return FieldMap(grid.reshape(dims[2], dims[1], dims[0], 4), dims, tuple(f.min), tuple(f.max),
                    int(f.kind))


def read_field_map_xyz(path, length_unit: float = 1.0, field_unit: float = TESLA,
                       first_octant: bool = False) -> FieldMap:
    """An XYZ map: lines "x y z bx by bz", x slowest and z fastest; positions
    times length_unit (mm), values times field_unit (GeV/(e*mm), tesla by
    default), as Options::readBField reads the driver's map
    (src/Plugins/BFieldOptions.cpp:33-61)."""
    lib = _lib()
    f = KfField()
    ptr = C.c_void_p()
    _check(lib.kf_field_map_read_xyz(os.fsencode(os.fspath(path)), length_unit, field_unit,
                                     int(first_octant), C.byref(f), C.byref(ptr)))
    return _take(lib, f, ptr)


def read_field_map_rz(path, length_unit: float = 1.0, field_unit: float = TESLA,
                      first_quadrant: bool = False, n_xyz=None, min_xyz=None,
                      max_xyz=None, native: bool = True) -> FieldMap:
    """An RZ map ("r z br bz", r slowest).  native (default): the (r, z) grid
    the fit interpolates in (r, z) as the reference does
    (kf_field_map_read_rz_native); native=False: resampled onto a Cartesian
    grid (default: x, y over +-r_max at the r step, z over the map's range)."""
    lib = _lib()
    f = KfField()
    ptr = C.c_void_p()
    if native and n_xyz is None:
        _check(lib.kf_field_map_read_rz_native(os.fsencode(os.fspath(path)), length_unit,
                                               field_unit, int(first_quadrant), C.byref(f),
                                               C.byref(ptr)))
        return _take(lib, f, ptr)
    args = [None, None, None]
    keep = []
    if n_xyz is not None:
        n = np.ascontiguousarray(n_xyz, dtype=np.int32)
        lo = np.ascontiguousarray(min_xyz, dtype=np.float64)
        hi = np.ascontiguousarray(max_xyz, dtype=np.float64)
        keep = [n, lo, hi]
        args = [a.ctypes.data for a in keep]
    _check(lib.kf_field_map_read_rz(os.fsencode(os.fspath(path)), length_unit, field_unit,
                                    int(first_quadrant), *args, C.byref(f), C.byref(ptr)))
    return _take(lib, f, ptr)


def write_field_map_xyz(path, x, y, z, b, fmt: str = "%.9g") -> None:
    """Write an XYZ map file from axis points x, y, z and field values
    b [nx, ny, nz, 3] (file units), x slowest and z fastest."""
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    rows = np.column_stack([X.ravel(), Y.ravel(), Z.ravel(), np.asarray(b).reshape(-1, 3)])
    np.savetxt(path, rows, fmt=fmt, header="x y z bx by bz", comments="# ")


def write_field_map_rz(path, r, z, b, fmt: str = "%.9g") -> None:
    """Write an RZ map file from axis points r, z and values b [nr, nz, 2]."""
    R, Z = np.meshgrid(r, z, indexing="ij")
    rows = np.column_stack([R.ravel(), Z.ravel(), np.asarray(b).reshape(-1, 2)])
    np.savetxt(path, rows, fmt=fmt, header="r z br bz", comments="% ")
