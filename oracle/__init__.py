"""The oracle: a CPU FP64 restatement of the reference fitter (test infrastructure).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package.  It is the checker the CUDA fitter is compared with and the CPU
baseline timed beside it; the product library never links or calls it.

``build()`` compiles ``kf_oracle.cpp`` with g++ (OpenMP, no FMA contraction so
results do not depend on the host ISA) into ``oracle/_build/libkforacle.so``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "kf_oracle.cpp"
LIB = HERE / "_build" / "libkforacle.so"
# Same source with the smoother evaluated in extended precision (long double):
# the comparison point for the GPU (see the note on the smoother in
# kf_oracle.cpp).
LIB_PRECISE = HERE / "_build" / "libkforacle_precise.so"
HEADER = HERE.parent / "include" / "gb300kf.h"

_LIBS: dict = {}


def _compile(target: Path, flags: list[str], force: bool) -> Path:
    if not force and target.exists() and target.stat().st_mtime >= max(SRC.stat().st_mtime,
                                                                       HEADER.stat().st_mtime):
        return target
    target.parent.mkdir(parents=True, exist_ok=True)
    tmp = target.with_suffix(".so.tmp")
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", *flags, "-fPIC", "-shared", "-o", str(tmp),
           str(SRC)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    os.replace(tmp, target)
    return target


def build(force: bool = False, variant: str = "default") -> Path:
    """Compile the oracle.  ``variant="precise"`` evaluates the smoother in
    long double; the default build is FP64 throughout (the CPU baseline)."""
    if variant == "precise":
        return _compile(LIB_PRECISE, ["-ffp-contract=off", "-DKFO_SMOOTHER_REAL=long double"], force)
    return _compile(LIB, ["-ffp-contract=off"], force)


def load(variant: str = "default"):
    if variant not in _LIBS:
        lib = C.CDLL(str(build(variant=variant)))
        lib.oracle_fit.restype = C.c_int32
        lib.oracle_num_threads.restype = C.c_int32
        _LIBS[variant] = lib
    return _LIBS[variant]


def fit(tel, cfg=None, *, threads: int = 0, smoothed: bool = False, masks: bool = True,
        field_scale: float = 1.0, center=None, rotation=None, states: bool = False,
        variant: str = "default") -> dict:
    """Fit a Telescope workload on the host; returns the same arrays as the GPU.

    With ``states=True`` the result also holds ``states`` [S,63,n]: predicted
    parameters, predicted covariance (upper triangle) and the bound-to-bound
    Jacobian of every measurement state.
    """
    import gpukalmanfitter_gb300 as kf
    lib = load(variant)
    cfg = cfg or kf.default_config()
    n, S = tel.n, tel.n_surfaces
    out = kf.host_outputs(n, S, smoothed)
    arrays = kf.tel_arrays(tel, masks)
    ins = kf.inputs_struct(arrays, n, S, lambda x: x.ctypes.data)
    outs = kf._outputs_struct(out)
    if center is None:
        geo, keep = tel.geometry()
    else:
        c = np.ascontiguousarray(center, dtype=np.float64)
        r = np.ascontiguousarray(rotation, dtype=np.float64)
        m = None if tel.material is None else np.ascontiguousarray(tel.material, dtype=np.float64)
        geo = kf.KfGeometry(S, 0, c.ctypes.data_as(C.POINTER(C.c_double)),
                            r.ctypes.data_as(C.POINTER(C.c_double)),
                            m.ctypes.data_as(C.POINTER(C.c_double)) if m is not None else None)
        keep = (c, r, m)
    fld = tel.field(None, field_scale)
    st = np.zeros((S, 63, n)) if states else None
    rc = lib.oracle_fit(C.byref(ins), C.byref(outs), C.byref(cfg), C.byref(geo), C.byref(fld),
                        C.c_int32(threads), None,
                        st.ctypes.data_as(C.POINTER(C.c_double)) if states else None)
    if states:
        out["states"] = st
    if rc != 0:
        raise RuntimeError(f"oracle_fit returned {rc}")
    del keep
    return out
