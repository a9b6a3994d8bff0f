"""The oracle: a CPU FP64 restatement of the reference fitter (test infrastructure).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package.  It is the checker the CUDA fitter is compared with and the CPU
baseline timed beside it; the product library never links or calls it.

``build()`` compiles ``kf_oracle.cpp`` with g++ (OpenMP, no FMA contraction so
results do not depend on the host ISA) into ``oracle/_build/libkforacle.so``.
The same library also carries the seeded workload generator (the package's
host source ``csrc/synth.cpp``, compiled with the package's host flags), so
the CPU baseline can build its inputs and fit them without mapping the
product library: ``make_telescope(..., lib=oracle.load())`` and
``oracle.default_config()``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "kf_oracle.cpp"
# the workload generator: host code of the package, compiled in as well
SYNTH_SRC = HERE.parent / "gpukalmanfitter_gb300" / "csrc" / "synth.cpp"
SYNTH_DEPS = [SYNTH_SRC, HERE.parent / "gpukalmanfitter_gb300" / "csrc" / "kf_synth_track.h",
              HERE.parent / "gpukalmanfitter_gb300" / "csrc" / "kf_material.h",
              HERE.parent / "include" / "gb300kf_synth.h"]
LIB = HERE / "_build" / "libkforacle.so"
# Same source with the smoother evaluated in double-double arithmetic (about
# 106 bits, the same on every host): the comparison point for the GPU (see
# the note on the smoother in kf_oracle.cpp).
LIB_PRECISE = HERE / "_build" / "libkforacle_precise.so"
HEADER = HERE.parent / "include" / "gb300kf.h"

_LIBS: dict = {}


def _compile(target: Path, flags: list[str], force: bool) -> Path:
    deps = [SRC, HEADER, *SYNTH_DEPS]
    if not force and target.exists() and target.stat().st_mtime >= max(d.stat().st_mtime
                                                                       for d in deps):
        return target
    target.parent.mkdir(parents=True, exist_ok=True)
    tmp = target.with_suffix(".so.tmp")
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", *flags, "-fPIC", "-shared", "-o", str(tmp),
           str(SRC), "-ffp-contract=off", "-I", str(HEADER.parent), str(SYNTH_SRC)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    os.replace(tmp, target)
    return target


def build(force: bool = False, variant: str = "default") -> Path:
    """Compile the oracle.  ``variant="precise"`` evaluates the smoother in
    double-double arithmetic; the default build is FP64 throughout (the CPU
    baseline)."""
    if variant == "precise":
        return _compile(LIB_PRECISE, ["-ffp-contract=off", "-DKFO_SMOOTHER_DD"], force)
    return _compile(LIB, ["-ffp-contract=off"], force)


def load(variant: str = "default"):
    if variant not in _LIBS:
        lib = C.CDLL(str(build(variant=variant)))
        lib.oracle_fit.restype = C.c_int32
        lib.oracle_num_threads.restype = C.c_int32
        lib.oracle_config_default.restype = None
        lib.kf_synth_geometry.restype = C.c_int32
        lib.kf_synth_field_map.restype = C.c_int32
        lib.kf_synth_field_map.argtypes = [C.c_double, C.c_int32, C.c_double, C.c_void_p]
        lib.kf_synth_tracks.restype = C.c_int32
        lib.oracle_field_value.restype = C.c_int32
        _LIBS[variant] = lib
    return _LIBS[variant]


def default_config(variant: str = "default", **overrides):
    """The reference's fit defaults (oracle_config_default) as a KfConfig,
    filled by the oracle library alone."""
    import gpukalmanfitter_gb300 as kf
    cfg = kf.KfConfig()
    load(variant).oracle_config_default(C.byref(cfg))
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return cfg


class Fitter:
    """One workload bound to ``oracle_fit``: the structures and the output
    arrays are made once, so that ``run()`` is the OpenMP track loop alone
    (the CPU baseline times it per step)."""

    def __init__(self, tel, cfg=None, *, smoothed: bool = False, masks: bool = True,
                 field_scale: float = 1.0, center=None, rotation=None, states: bool = False,
                 variant: str = "default"):
        import gpukalmanfitter_gb300 as kf
        self.lib = load(variant)
        self.cfg = cfg or default_config(variant)
        n, S = tel.n, tel.n_surfaces
        self.out = kf.host_outputs(n, S, smoothed)
        for v in self.out.values():
            v.fill(0)  # touch the pages outside any timed region
        self.arrays = kf.tel_arrays(tel, masks)
        self.ins = kf.inputs_struct(self.arrays, n, S, lambda x: x.ctypes.data)
        self.outs = kf._outputs_struct(self.out)
        if center is None:
            self.geo, self._keep = tel.geometry()
        else:
            c = np.ascontiguousarray(center, dtype=np.float64)
            r = np.ascontiguousarray(rotation, dtype=np.float64)
            m = None if tel.material is None else np.ascontiguousarray(tel.material, dtype=np.float64)
            self.geo = kf.KfGeometry(S, 0, c.ctypes.data_as(C.POINTER(C.c_double)),
                                     r.ctypes.data_as(C.POINTER(C.c_double)),
                                     m.ctypes.data_as(C.POINTER(C.c_double)) if m is not None else None)
            self._keep = (c, r, m)
        self.fld = tel.field(None, field_scale)
        self.st = np.zeros((S, 63, n)) if states else None

    def run(self, threads: int = 0) -> dict:
        rc = self.lib.oracle_fit(C.byref(self.ins), C.byref(self.outs), C.byref(self.cfg),
                                 C.byref(self.geo), C.byref(self.fld), C.c_int32(threads), None,
                                 self.st.ctypes.data_as(C.POINTER(C.c_double))
                                 if self.st is not None else None)
        if rc != 0:
            raise RuntimeError(f"oracle_fit returned {rc}")
        if self.st is not None:
            self.out["states"] = self.st
        return self.out


def field_value(field, pos) -> np.ndarray:
    """One lookup of a kf_field_t (grid in host memory) as the oracle's fit
    makes it."""
    lib = load()
    out = np.zeros(3)
    p = np.ascontiguousarray(pos, dtype=np.float64)
    rc = lib.oracle_field_value(C.byref(field), p.ctypes.data_as(C.POINTER(C.c_double)),
                                out.ctypes.data_as(C.POINTER(C.c_double)))
    if rc != 0:
        raise RuntimeError(f"oracle_field_value returned {rc}")
    return out


def fit(tel, cfg=None, *, threads: int = 0, smoothed: bool = False, masks: bool = True,
        field_scale: float = 1.0, center=None, rotation=None, states: bool = False,
        variant: str = "default") -> dict:
    """Fit a Telescope workload on the host; returns the same arrays as the GPU.

    With ``states=True`` the result also holds ``states`` [S,63,n]: predicted
    parameters, predicted covariance (upper triangle) and the bound-to-bound
    Jacobian of every measurement state.
    """
    return Fitter(tel, cfg, smoothed=smoothed, masks=masks, field_scale=field_scale,
                  center=center, rotation=rotation, states=states, variant=variant).run(threads)
