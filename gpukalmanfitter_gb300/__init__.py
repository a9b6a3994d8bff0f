"""GB300-native Kalman track fitter: Python bindings of the C ABI.

The product is ``libgb300kf.so`` (CUDA kernels for sm_103a plus the C ABI of
``include/gb300kf.h``).  This module loads it with ctypes and mirrors the
reference fitter's call shape: one ``fit`` over a batch of tracks with the
reference's options (maxSteps, tolerance, mass, smoothing), its bound-parameter
convention (loc0, loc1, phi, theta, q/p, t) and its per-track success flag
(reference: Fitter/KalmanFitter.hpp:716-768).

Device memory and streams come from PyTorch; the library itself takes plain
pointers.  There is no CPU fallback: if the library or a GPU is missing the
calls raise.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import build as _build

__all__ = [
    "load", "KfConfig", "KfGeometry", "KfField", "KfInputs", "KfOutputs", "SynthConfig",
    "default_config", "Telescope", "make_telescope", "fit_device", "fit_host",
    "TRACK_STATUS", "KfError", "AdjointBatch", "align_geometry",
]

KF_MAX_PLANES = 64
TRACK_STATUS = {0: "ok", 1: "meas_mismatch", 2: "smoother_nan", 3: "max_steps",
                4: "no_hits", 5: "bad_input", 6: "not_fitted", 7: "adjoint_failed"}
TESLA = 0.000299792458  # GeV/(e*mm)


class KfError(RuntimeError):
    pass


class KfConfig(C.Structure):
    _fields_ = [("precision", C.c_int32), ("max_steps", C.c_int32),
                ("max_rk_trials", C.c_int32), ("smoothing", C.c_int32),
                ("tolerance", C.c_double), ("step_size_cutoff", C.c_double),
                ("mass", C.c_double), ("overstep_limit", C.c_double),
                ("on_surface_tol", C.c_double), ("outlier_chi2_cut", C.c_double),
                ("faithful_jacobian", C.c_int32), ("kernel", C.c_int32),
                ("block_size", C.c_int32), ("min_blocks_per_sm", C.c_int32),
                ("material_effects", C.c_int32), ("adjoint_tape", C.c_int32)]


class KfGeometry(C.Structure):
    _fields_ = [("n_planes", C.c_int32), ("reserved0", C.c_int32),
                ("center", C.POINTER(C.c_double)), ("rotation", C.POINTER(C.c_double)),
                ("material", C.POINTER(C.c_double))]


class KfField(C.Structure):
    _fields_ = [("kind", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("value", C.c_double * 3), ("scale", C.c_double),
                ("min", C.c_double * 3), ("max", C.c_double * 3), ("grid", C.c_void_p)]


class KfInputs(C.Structure):
    _fields_ = [("n_tracks", C.c_int64), ("stride", C.c_int64), ("n_surfaces", C.c_int32),
                ("reserved0", C.c_int32), ("meas", C.c_void_p), ("hit_mask", C.c_void_p),
                ("n_planes", C.c_void_p), ("start_params", C.c_void_p),
                ("start_cov", C.c_void_p), ("perigee", C.c_void_p)]


class KfOutputs(C.Structure):
    _fields_ = [("params", C.c_void_p), ("cov", C.c_void_p), ("chi2", C.c_void_p),
                ("status", C.c_void_p), ("n_meas", C.c_void_p), ("n_steps", C.c_void_p),
                ("n_trials", C.c_void_p), ("smoothed", C.c_void_p)]


class SynthConfig(C.Structure):
    _fields_ = [("n_tracks", C.c_int64), ("seed", C.c_uint64), ("n_planes", C.c_int32),
                ("min_len", C.c_int32), ("max_len", C.c_int32),
                ("x_first", C.c_double), ("x_step", C.c_double), ("bz_tesla", C.c_double),
                ("mass", C.c_double), ("p_min", C.c_double), ("p_max", C.c_double),
                ("phi_half", C.c_double), ("theta_half", C.c_double),
                ("vertex_sigma", C.c_double), ("hit_sigma", C.c_double),
                ("hit_prob", C.c_double), ("outlier_prob", C.c_double),
                ("outlier_shift", C.c_double), ("seed_loc_sigma", C.c_double),
                ("seed_angle_sigma", C.c_double), ("seed_qop_rel", C.c_double),
                ("seed_time_sigma", C.c_double), ("mis_shift_sigma", C.c_double),
                ("mis_rot_sigma", C.c_double), ("rk_step", C.c_double),
                ("material", C.c_double * 6)]


_LIB = None
EXPORTS = ["kf_version", "kf_last_error_string", "kf_config_default", "kf_workspace_size",
           "kf_fit_batch", "kf_host_staging_size", "kf_fit_batch_host", "kf_batch_workspace_size",
           "kf_fit_batch_sorted", "kf_batch_plan_create", "kf_batch_plan_launch",
           "kf_batch_plan_destroy", "kf_autotune",
           "kf_synth_config_default", "kf_synth_geometry", "kf_synth_field_map",
           "kf_synth_tracks", "kf_simulate_tracks"]


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libgb300kf.so (building it in-tree if absent)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    lib_path = _build.LIB
    if not lib_path.exists():
        if not build_if_missing:
            raise KfError(f"{lib_path} is missing; run gpukalmanfitter_gb300.build.build()")
        _build.build()
    lib = C.CDLL(str(lib_path))
    lib.kf_version.restype = C.c_int32
    lib.kf_last_error_string.restype = C.c_char_p
    lib.kf_config_default.argtypes = [C.POINTER(KfConfig)]
    lib.kf_workspace_size.restype = C.c_size_t
    lib.kf_workspace_size.argtypes = [C.POINTER(KfConfig), C.c_int64, C.c_int32]
    lib.kf_fit_batch.restype = C.c_int32
    lib.kf_fit_batch.argtypes = [C.POINTER(KfInputs), C.POINTER(KfOutputs), C.POINTER(KfConfig),
                                 C.POINTER(KfGeometry), C.POINTER(KfField), C.c_void_p,
                                 C.c_size_t, C.c_void_p]
    lib.kf_host_staging_size.restype = C.c_size_t
    lib.kf_host_staging_size.argtypes = [C.POINTER(KfConfig), C.c_int64, C.c_int32, C.c_int32]
    lib.kf_fit_batch_host.restype = C.c_int32
    lib.kf_fit_batch_host.argtypes = lib.kf_fit_batch.argtypes
    lib.kf_batch_workspace_size.restype = C.c_size_t
    lib.kf_batch_workspace_size.argtypes = [C.POINTER(KfConfig), C.c_int64, C.c_int32]
    lib.kf_fit_batch_sorted.restype = C.c_int32
    lib.kf_fit_batch_sorted.argtypes = lib.kf_fit_batch.argtypes
    lib.kf_batch_plan_create.restype = C.c_int32
    lib.kf_batch_plan_create.argtypes = [C.POINTER(C.c_void_p)] + lib.kf_fit_batch.argtypes
    lib.kf_batch_plan_launch.restype = C.c_int32
    lib.kf_batch_plan_launch.argtypes = [C.c_void_p, C.c_void_p]
    lib.kf_batch_plan_destroy.argtypes = [C.c_void_p]
    lib.kf_autotune.restype = C.c_int32
    lib.kf_autotune.argtypes = lib.kf_fit_batch.argtypes + [C.POINTER(KfConfig),
                                                            C.POINTER(C.c_double)]
    lib.kf_fit_batch_noalloc.restype = C.c_int32
    lib.kf_noalloc_scratch_bytes.restype = C.c_size_t
    lib.kf_noalloc_last_error_string.restype = C.c_char_p
    lib.kf_diag_fp64_fma_rate.restype = C.c_int32
    lib.kf_adjoint_workspace_size.restype = C.c_size_t
    lib.kf_adjoint_workspace_size.argtypes = [C.POINTER(KfConfig), C.c_int64, C.c_int32]
    lib.kf_adjoint_batch.restype = C.c_int32
    lib.kf_adjoint_batch.argtypes = [C.POINTER(KfInputs), C.c_void_p, C.POINTER(KfConfig),
                                     C.POINTER(KfGeometry), C.POINTER(KfField), C.c_int32,
                                     C.c_void_p, C.c_size_t, C.c_void_p]
    lib.kf_synth_config_default.argtypes = [C.POINTER(SynthConfig)]
    lib.kf_synth_geometry.restype = C.c_int32
    lib.kf_synth_field_map.restype = C.c_int32
    lib.kf_synth_field_map.argtypes = [C.c_double, C.c_int32, C.c_double, C.c_void_p]
    lib.kf_synth_tracks.restype = C.c_int32
    lib.kf_simulate_tracks.restype = C.c_int32
    lib.kf_field_map_read_rz_native.restype = C.c_int32
    _LIB = lib
    return lib


def _check(rc: int) -> None:
    if rc != 0:
        raise KfError(f"libgb300kf error {rc}: {load().kf_last_error_string().decode()}")


def default_config(**overrides) -> KfConfig:
    cfg = KfConfig()
    load().kf_config_default(C.byref(cfg))
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return cfg


def _ptr(a: np.ndarray, ctype=C.c_double):
    return a.ctypes.data_as(C.POINTER(ctype))


# ---------------------------------------------------------------------------
# Workloads
# ---------------------------------------------------------------------------
@dataclass
class Telescope:
    """A synthetic telescope workload in host memory (structure of arrays)."""
    n: int
    n_surfaces: int
    center: np.ndarray        # [S,3] nominal plane centres (what the fit uses)
    rotation: np.ndarray      # [S,9]
    meas: np.ndarray          # [S,5,n]
    hit_mask: np.ndarray      # [n] uint64
    n_planes: np.ndarray      # [n] int32
    start: np.ndarray         # [6,n]
    start_cov: np.ndarray     # [21,n]
    perigee: np.ndarray       # [3,n]
    truth: np.ndarray         # [6,n]
    bz_tesla: float
    field_grid: np.ndarray | None = None   # [n^3*4] float32 (host copy)
    field_n: int = 0
    field_half: float = 0.0
    truth_center: np.ndarray | None = None
    truth_rotation: np.ndarray | None = None
    misalignment: np.ndarray | None = None  # [S,6]
    material: np.ndarray | None = None      # [S,6] surface material (None: vacuum)
    # a grid that is not the cube of field_n points over +-field_half (an
    # ingested map, gpukalmanfitter_gb300.fieldmap): points and extent per axis
    field_dims: tuple | None = None
    field_min: tuple | None = None
    field_max: tuple | None = None
    field_kind: int = 1                     # kf_field_kind of a grid field
    synth_cfg: object = None                # SynthConfig of a GPU-simulated telescope

    def geometry(self) -> tuple[KfGeometry, tuple]:
        c = np.ascontiguousarray(self.center, dtype=np.float64)
        r = np.ascontiguousarray(self.rotation, dtype=np.float64)
        m = None if self.material is None else np.ascontiguousarray(self.material, dtype=np.float64)
        g = KfGeometry(self.n_surfaces, 0, _ptr(c), _ptr(r), _ptr(m) if m is not None else None)
        return g, (c, r, m)

    def field(self, grid_ptr: int | None = None, scale: float = 1.0) -> KfField:
        f = KfField()
        f.scale = scale
        if self.field_grid is None:
            f.kind = 0
            f.value[0], f.value[1], f.value[2] = 0.0, 0.0, self.bz_tesla * TESLA
        else:
            f.kind = self.field_kind
            if self.field_dims is not None:
                f.nx, f.ny, f.nz = self.field_dims
                for a in range(3):
                    f.min[a] = self.field_min[a]
                    f.max[a] = self.field_max[a]
            else:
                f.nx = f.ny = f.nz = self.field_n
                for a in range(3):
                    f.min[a] = -self.field_half
                    f.max[a] = self.field_half
            f.grid = grid_ptr if grid_ptr is not None else self.field_grid.ctypes.data
        return f

    def simulate(self, stream=None) -> None:
        """(Re)generate the tracks of a GPU-simulated telescope into its own
        device arrays with kf_simulate_tracks on `stream` (asynchronous)."""
        import torch
        field = None
        if self.field_grid is not None:
            field = self.field(self.field_grid.data_ptr())
        s = stream if stream is not None else torch.cuda.current_stream()
        tc = np.ascontiguousarray(self.truth_center, dtype=np.float64)
        tr = np.ascontiguousarray(self.truth_rotation, dtype=np.float64)
        _check(load().kf_simulate_tracks(C.byref(self.synth_cfg), _ptr(tc), _ptr(tr),
                                         C.byref(field) if field is not None else None,
                                         *[C.c_void_p(a.data_ptr()) for a in
                                           (self.meas, self.hit_mask, self.n_planes, self.start,
                                            self.start_cov, self.perigee, self.truth)],
                                         C.c_void_p(s.cuda_stream)))

    def to_host(self) -> "Telescope":
        """A copy whose per-track arrays (torch tensors of a GPU-simulated
        telescope) are numpy arrays."""
        import copy
        t = copy.copy(self)
        for k in ("meas", "hit_mask", "n_planes", "start", "start_cov", "perigee", "truth",
                  "field_grid"):
            v = getattr(self, k)
            if v is not None and hasattr(v, "detach"):
                a = v.detach().cpu().numpy()
                setattr(t, k, a.view(np.uint64) if k == "hit_mask" else a)
        return t


def silicon(thickness_mm: float) -> np.ndarray:
    """Surface material row (thickness, X0, L0, Ar, Z, molar density) of
    silicon, as the reference's test helper builds it (Test/Helper.hpp:25-29:
    X0 9.370 cm, L0 46.52 cm, Ar 28.0855, Z 14, 2.329 g/cm^3)."""
    return np.array([thickness_mm, 93.70, 465.2, 28.0855, 14.0, (2.329 / 28.0855) / 1000.0])


def synth_config(lib=None, **kw) -> SynthConfig:
    c = SynthConfig()
    (lib or load()).kf_synth_config_default(C.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def make_telescope(n: int, *, seed: int = 1234567890, n_planes: int = 10,
                   x_first: float = 100.0, x_step: float = 100.0, min_len: int | None = None,
                   max_len: int | None = None, hit_prob: float = 1.0,
                   outlier_prob: float = 0.0, field_map=False, field_n: int = 101,
                   field_half: float = 1500.0, mis_shift: float = 0.0, mis_rot: float = 0.0,
                   material: float = 0.0, threads: int = 0, device: str | None = None,
                   lib=None, **extra) -> Telescope:
    """Seeded synthetic telescope workload (host arrays).  material > 0: every
    plane carries that many mm of silicon (the reference driver's 0.5 mm,
    Run/GPU/KalmanFitterGPUTest.cu:253) in the geometry and in the truth.
    field_map: True for the analytic map of field_n^3 points over
    +-field_half, or a FieldMap (gpukalmanfitter_gb300.fieldmap) read from a
    file; the truth and the fit then use that grid.  device ("cuda", ...):
    the tracks are simulated on that GPU (kf_simulate_tracks, the same
    tracks as the host generator's) and the per-track arrays are torch
    tensors there (Telescope.to_host() gives the numpy form).  lib: another
    library exporting the host generator's kf_synth_* entry points (the
    oracle's, which carries the same host code), in place of this one's; host
    generation only."""
    if lib is not None and device is not None:
        raise KfError("make_telescope: lib= generates on the host; device= needs libgb300kf")
    lib = lib or load()
    cfg = synth_config(lib, n_tracks=n, seed=seed, n_planes=n_planes, x_first=x_first, x_step=x_step,
                       min_len=min_len or n_planes, max_len=max_len or n_planes,
                       hit_prob=hit_prob, outlier_prob=outlier_prob,
                       mis_shift_sigma=mis_shift, mis_rot_sigma=mis_rot, **extra)
    mat = None
    if material > 0:
        mat = np.tile(silicon(material), (n_planes, 1))
        for e in range(6):
            cfg.material[e] = mat[0, e]
    S = n_planes
    center = np.zeros((S, 3)); rot = np.zeros((S, 9))
    tcenter = np.zeros((S, 3)); trot = np.zeros((S, 9)); align = np.zeros((S, 6))
    _check(lib.kf_synth_geometry(C.byref(cfg), _ptr(center), _ptr(rot), _ptr(tcenter),
                                 _ptr(trot), _ptr(align)))
    grid = None
    field = None
    ingested = field_map is not None and not isinstance(field_map, bool)
    if ingested:
        grid = np.ascontiguousarray(field_map.grid, dtype=np.float32).reshape(-1)
    elif field_map:
        grid = np.zeros(field_n ** 3 * 4, dtype=np.float32)
        _check(lib.kf_synth_field_map(C.c_double(cfg.bz_tesla), field_n, C.c_double(field_half),
                                      grid.ctypes.data))
    if device is not None:
        import torch
        z = lambda *shape, dt=torch.float64: torch.zeros(shape, dtype=dt, device=device)
        meas, mask, nplanes = z(S, 5, n), z(n, dt=torch.int64), z(n, dt=torch.int32)
        start, scov, per, truth = z(6, n), z(21, n), z(3, n), z(6, n)
        if grid is not None:
            grid = torch.from_numpy(grid).to(device)
    else:
        meas = np.zeros((S, 5, n)); mask = np.zeros(n, dtype=np.uint64)
        nplanes = np.zeros(n, dtype=np.int32); start = np.zeros((6, n)); scov = np.zeros((21, n))
        per = np.zeros((3, n)); truth = np.zeros((6, n))
    tel = Telescope(n, S, center, rot, meas, mask, nplanes, start, scov, per, truth,
                    cfg.bz_tesla, grid, field_n if field_map else 0, field_half,
                    tcenter, trot, align, mat)
    if ingested:
        tel.field_dims = tuple(field_map.dims)
        tel.field_min = tuple(field_map.min)
        tel.field_max = tuple(field_map.max)
        tel.field_kind = int(getattr(field_map, "kind", 1))
    if field_map is not None and field_map is not False:
        field = tel.field(grid.data_ptr() if device is not None else None)
    if device is not None:
        import torch
        tel.synth_cfg = cfg
        tel.simulate(torch.cuda.current_stream(device))
        return tel
    _check(lib.kf_synth_tracks(C.byref(cfg), _ptr(tcenter), _ptr(trot),
                               C.byref(field) if field is not None else None,
                               _ptr(meas), _ptr(mask, C.c_uint64), _ptr(nplanes, C.c_int32),
                               _ptr(start), _ptr(scov), _ptr(per), _ptr(truth),
                               C.c_int32(threads)))
    return tel


# ---------------------------------------------------------------------------
# Fitting
# ---------------------------------------------------------------------------
OUT_FIELDS = ("params", "cov", "chi2", "status", "n_meas", "n_steps", "n_trials")


def host_outputs(n: int, n_surfaces: int, smoothed: bool = False) -> dict:
    out = {"params": np.zeros((6, n)), "cov": np.zeros((21, n)), "chi2": np.zeros(n),
           "status": np.zeros(n, dtype=np.int32), "n_meas": np.zeros(n, dtype=np.int32),
           "n_steps": np.zeros(n, dtype=np.int32), "n_trials": np.zeros(n, dtype=np.int32)}
    if smoothed:
        out["smoothed"] = np.zeros((n_surfaces, 27, n))
    return out


def _outputs_struct(d: dict) -> KfOutputs:
    o = KfOutputs()
    for k in OUT_FIELDS + ("smoothed",):
        v = d.get(k)
        if v is None:
            setattr(o, k, None)
        elif isinstance(v, np.ndarray):
            setattr(o, k, v.ctypes.data)
        else:  # torch tensor
            setattr(o, k, v.data_ptr())
    return o


def inputs_struct(tel_or_arrays, n: int, n_surfaces: int, ptr) -> KfInputs:
    a = tel_or_arrays
    i = KfInputs()
    i.n_tracks = n
    i.stride = n
    i.n_surfaces = n_surfaces
    i.meas = ptr(a["meas"])
    i.hit_mask = ptr(a["hit_mask"]) if a.get("hit_mask") is not None else None
    i.n_planes = ptr(a["n_planes"]) if a.get("n_planes") is not None else None
    i.start_params = ptr(a["start"])
    i.start_cov = ptr(a["start_cov"])
    i.perigee = ptr(a["perigee"])
    return i


def tel_arrays(tel: Telescope, masks: bool = True) -> dict:
    return {"meas": tel.meas, "hit_mask": tel.hit_mask if masks else None,
            "n_planes": tel.n_planes if masks else None, "start": tel.start,
            "start_cov": tel.start_cov, "perigee": tel.perigee}


def fit_host(tel: Telescope, cfg: KfConfig | None = None, *, smoothed: bool = False,
             staging=None, stream=None, field_grid_dev=None, field_scale: float = 1.0,
             masks: bool = True) -> dict:
    """Fit host-resident tracks through kf_fit_batch_host (copies in and out).

    ``staging`` is a device buffer (torch uint8 tensor) of at least
    kf_host_staging_size bytes; it is allocated with torch if not given.
    """
    import torch
    lib = load()
    cfg = cfg or default_config()
    n, S = tel.n, tel.n_surfaces
    size = lib.kf_host_staging_size(C.byref(cfg), n, S, int(smoothed))
    if staging is None:
        staging = torch.empty(size, dtype=torch.uint8, device="cuda")
    out = host_outputs(n, S, smoothed)
    arrays = tel_arrays(tel, masks)
    ins = inputs_struct(arrays, n, S, lambda x: x.ctypes.data)
    outs = _outputs_struct(out)
    geo, keep = tel.geometry()
    grid_ptr = field_grid_dev.data_ptr() if field_grid_dev is not None else None
    fld = tel.field(grid_ptr, field_scale)
    s = stream if stream is not None else torch.cuda.current_stream()
    _check(lib.kf_fit_batch_host(C.byref(ins), C.byref(outs), C.byref(cfg), C.byref(geo),
                                 C.byref(fld), C.c_void_p(staging.data_ptr()),
                                 C.c_size_t(staging.numel()), C.c_void_p(s.cuda_stream)))
    return out


class DeviceBatch:
    """A workload resident in HBM (torch tensors) plus outputs and workspace."""

    def __init__(self, tel: Telescope, cfg: KfConfig | None = None, *, smoothed: bool = False,
                 masks: bool = True, device: str = "cuda"):
        import torch
        self.tel = tel
        self.cfg = cfg or default_config()
        n, S = tel.n, tel.n_surfaces
        t = lambda a: a if hasattr(a, "data_ptr") else torch.from_numpy(np.ascontiguousarray(a)).to(device)
        self.arrays = {k: (t(v) if v is not None else None) for k, v in tel_arrays(tel, masks).items()}
        self.out = {"params": torch.zeros((6, n), dtype=torch.float64, device=device),
                    "cov": torch.zeros((21, n), dtype=torch.float64, device=device),
                    "chi2": torch.zeros(n, dtype=torch.float64, device=device),
                    "status": torch.zeros(n, dtype=torch.int32, device=device),
                    "n_meas": torch.zeros(n, dtype=torch.int32, device=device),
                    "n_steps": torch.zeros(n, dtype=torch.int32, device=device),
                    "n_trials": torch.zeros(n, dtype=torch.int32, device=device)}
        if smoothed:
            self.out["smoothed"] = torch.zeros((S, 27, n), dtype=torch.float64, device=device)
        lib = load()
        self.ws_bytes = max(lib.kf_workspace_size(C.byref(self.cfg), n, S),
                            lib.kf_batch_workspace_size(C.byref(self.cfg), n, S))
        self.ws = torch.empty(max(self.ws_bytes, 1), dtype=torch.uint8, device=device)
        self.plan = None
        self.grid = t(tel.field_grid) if tel.field_grid is not None else None
        self.ins = inputs_struct(self.arrays, n, S, lambda x: x.data_ptr())
        self.outs = _outputs_struct(self.out)
        self.geo, self._keep = tel.geometry()
        self.field = tel.field(self.grid.data_ptr() if self.grid is not None else None)

    def fit(self, stream=None) -> None:
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        _check(load().kf_fit_batch(C.byref(self.ins), C.byref(self.outs), C.byref(self.cfg),
                                   C.byref(self.geo), C.byref(self.field),
                                   C.c_void_p(self.ws.data_ptr()), C.c_size_t(self.ws_bytes),
                                   C.c_void_p(s.cuda_stream)))

    def fit_sorted(self, stream=None) -> None:
        """The batched form: length-sorted queue and persistent kernel."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        _check(load().kf_fit_batch_sorted(C.byref(self.ins), C.byref(self.outs),
                                          C.byref(self.cfg), C.byref(self.geo),
                                          C.byref(self.field), C.c_void_p(self.ws.data_ptr()),
                                          C.c_size_t(self.ws_bytes), C.c_void_p(s.cuda_stream)))

    def make_plan(self, stream) -> None:
        """Capture the batched pipeline into a CUDA graph (see kf_batch_plan_create)."""
        self.destroy_plan()
        p = C.c_void_p()
        _check(load().kf_batch_plan_create(C.byref(p), C.byref(self.ins), C.byref(self.outs),
                                           C.byref(self.cfg), C.byref(self.geo),
                                           C.byref(self.field), C.c_void_p(self.ws.data_ptr()),
                                           C.c_size_t(self.ws_bytes),
                                           C.c_void_p(stream.cuda_stream)))
        self.plan = p

    def launch_plan(self, stream) -> None:
        _check(load().kf_batch_plan_launch(self.plan, C.c_void_p(stream.cuda_stream)))

    def destroy_plan(self) -> None:
        if getattr(self, "plan", None):
            load().kf_batch_plan_destroy(self.plan)
            self.plan = None

    def autotune(self, stream=None) -> tuple:
        """Pick the persistent kernel shape; sets self.cfg and returns (cfg, ms)."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        tuned = KfConfig()
        ms = C.c_double(0)
        _check(load().kf_autotune(C.byref(self.ins), C.byref(self.outs), C.byref(self.cfg),
                                  C.byref(self.geo), C.byref(self.field),
                                  C.c_void_p(self.ws.data_ptr()), C.c_size_t(self.ws_bytes),
                                  C.c_void_p(s.cuda_stream), C.byref(tuned), C.byref(ms)))
        self.cfg = tuned
        return tuned, ms.value

    def __del__(self):
        try:
            self.destroy_plan()
        except Exception:
            pass

    def results(self) -> dict:
        return {k: v.cpu().numpy() for k, v in self.out.items()}


def fit_device(tel: Telescope, cfg: KfConfig | None = None, **kw) -> dict:
    b = DeviceBatch(tel, cfg, **kw)
    b.fit()
    return b.results()


# ---------------------------------------------------------------------------
# chi2 adjoint (kf_adjoint_batch)
# ---------------------------------------------------------------------------
class KfAdjointOutputs(C.Structure):
    _fields_ = [("chi2", C.c_void_p), ("status", C.c_void_p), ("grad_start", C.c_void_p),
                ("grad_align", C.c_void_p), ("grad_field_scale", C.c_void_p),
                ("chi2_total", C.c_void_p), ("grad_field_scale_track", C.c_void_p)]


def _rot(a: np.ndarray) -> np.ndarray:
    """R = Rx(wx) Ry(wy) Rz(wz) for a = (wx, wy, wz) (the same composition as
    the alignment frame rotation of the adjoint's tests)."""
    cx, sx, cy, sy, cz, sz = np.cos(a[0]), np.sin(a[0]), np.cos(a[1]), np.sin(a[1]), np.cos(a[2]), np.sin(a[2])
    rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    return rx @ ry @ rz


def align_geometry(center: np.ndarray, rotation: np.ndarray, alignment: np.ndarray):
    """Plane centres shifted by alignment[:, 0:3] and frames (U, V, T columns of
    rotation[k].reshape(3, 3)) rotated by alignment[:, 3:6] about the global axes."""
    c = np.array(center, dtype=np.float64).reshape(-1, 3) + alignment[:, :3]
    r = np.array(rotation, dtype=np.float64).reshape(-1, 3, 3).copy()
    for k in range(r.shape[0]):
        r[k] = _rot(alignment[k, 3:]) @ r[k]
    return c, r.reshape(-1, 9)


def rotation_increment_jacobian(a: np.ndarray) -> np.ndarray:
    """E with (incremental global rotation vector) = E d(wx, wy, wz) for
    R = Rx(wx) Ry(wy) Rz(wz): columns e_x, Rx e_y, Rx Ry e_z."""
    cx, sx, cy, sy = np.cos(a[0]), np.sin(a[0]), np.cos(a[1]), np.sin(a[1])
    rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    return np.stack([np.array([1., 0., 0.]), rx @ np.array([0., 1., 0.]),
                     rx @ ry @ np.array([0., 0., 1.])], axis=1)


class AdjointBatch:
    """d(total smoothed chi2) / d(plane alignment, start parameters, field
    scale) of a batch on the device (kf_adjoint_batch)."""

    def __init__(self, tel: Telescope, cfg: KfConfig | None = None, device: str = "cuda"):
        import torch
        self.tel = tel
        self.cfg = cfg or default_config()
        n, S = tel.n, tel.n_surfaces
        t = lambda a: a if hasattr(a, "data_ptr") else torch.from_numpy(np.ascontiguousarray(a)).to(device)
        self.arrays = {k: (t(v) if v is not None else None) for k, v in tel_arrays(tel, True).items()}
        self.out = {"chi2": torch.zeros(n, dtype=torch.float64, device=device),
                    "status": torch.zeros(n, dtype=torch.int32, device=device),
                    "grad_start": torch.zeros((6, n), dtype=torch.float64, device=device),
                    "grad_align": torch.zeros((S, 6), dtype=torch.float64, device=device),
                    "grad_field_scale": torch.zeros(1, dtype=torch.float64, device=device),
                    "chi2_total": torch.zeros(1, dtype=torch.float64, device=device),
                    "grad_field_scale_track": torch.zeros(n, dtype=torch.float64, device=device)}
        self.aout = KfAdjointOutputs(*[self.out[k].data_ptr() for k in
                                       ("chi2", "status", "grad_start", "grad_align",
                                        "grad_field_scale", "chi2_total",
                                        "grad_field_scale_track")])
        lib = load()
        self.ws_bytes = int(lib.kf_adjoint_workspace_size(C.byref(self.cfg), n, S))
        if n > 0 and self.ws_bytes < n * S * 37 * 8:
            raise KfError(f"implausible adjoint workspace size {self.ws_bytes}")
        self.ws = torch.empty(max(self.ws_bytes, 1), dtype=torch.uint8, device=device)
        self.ins = inputs_struct(self.arrays, n, S, lambda x: x.data_ptr())
        self.center = np.array(tel.center, dtype=np.float64)
        self.rotation = np.array(tel.rotation, dtype=np.float64)

    def run(self, grad: bool = True, alignment: np.ndarray | None = None,
            field_scale: float = 1.0, stream=None) -> dict:
        """One call; alignment (S, 6) perturbs the geometry first (the gradient
        is then taken at that geometry, with respect to incremental alignment)."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        if alignment is None:
            c, r = self.center, self.rotation
        else:
            c, r = align_geometry(self.center, self.rotation, np.asarray(alignment, np.float64))
        c = np.ascontiguousarray(c, dtype=np.float64)
        r = np.ascontiguousarray(r, dtype=np.float64)
        m = None if self.tel.material is None else np.ascontiguousarray(self.tel.material, np.float64)
        geo = KfGeometry(self.tel.n_surfaces, 0, _ptr(c), _ptr(r), _ptr(m) if m is not None else None)
        field = self.tel.field(scale=field_scale)
        _check(load().kf_adjoint_batch(C.byref(self.ins), C.byref(self.aout), C.byref(self.cfg),
                                       C.byref(geo), C.byref(field), C.c_int32(1 if grad else 0),
                                       C.c_void_p(self.ws.data_ptr()), C.c_size_t(self.ws_bytes),
                                       C.c_void_p(s.cuda_stream)))
        s.synchronize()
        return {k: v.cpu().numpy() for k, v in self.out.items()}

    def set_start(self, start: np.ndarray) -> None:
        import torch
        self.arrays["start"].copy_(torch.from_numpy(np.ascontiguousarray(start, np.float64)))
