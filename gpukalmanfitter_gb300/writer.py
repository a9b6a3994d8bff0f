"""Output files of the fit — the reference driver's writers
(Run/Common/Writer.hpp) through the library's C ABI (gb300kf_io.h), without
ROOT.  Results are the host dictionaries of fit_host / DeviceBatch.results /
the oracle; inputs come from a Telescope.

    write_params_csv(path, res)            writeParamsCsv      (Writer.hpp:80-110)
    write_states_obj(path, res, tel)       writeStatesObj      (Writer.hpp:42-78)
    write_sim_hits_obj(path, tel)          writeSimHitsObj     (Writer.hpp:16-40)
    write_params_table(path, res, tel)     writeParamsRoot     (Writer.hpp:112-229),
                                           as CSV with the tree's branch names
    resolution_report(table)               the pull fits of Performance/Scripts/
                                           perigeeParamResolution.C
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import KfError, Telescope, _check, load

_I64, _I32, _P = C.c_int64, C.c_int32, C.c_void_p


def _lib() -> C.CDLL:
    lib = load()
    if not getattr(lib, "_io_bound", False):
        lib.kf_write_params_csv.argtypes = [C.c_char_p, _P, _P, _I64, _I64]
        lib.kf_write_states_obj.argtypes = [C.c_char_p, _P, _P, _P, _P, _I64, _I64, _P]
        lib.kf_write_hits_obj.argtypes = [C.c_char_p, _P, _P, _P, _I32, _I64, _I64]
        lib.kf_write_params_table.argtypes = [C.c_char_p, _P, _P, _P, _P, _P, _I64, _I64]
        for f in ("kf_write_params_csv", "kf_write_states_obj", "kf_write_hits_obj",
                  "kf_write_params_table"):
            getattr(lib, f).restype = C.c_int32
        lib._io_bound = True
    return lib


def _arr(a, dtype) -> np.ndarray:
    a = np.asarray(a)
    if a.dtype != dtype or not a.flags.c_contiguous:
        raise KfError(f"expected a C-contiguous {np.dtype(dtype).name} array, got {a.dtype}")
    return a


def _host(a):
    """numpy view of a host array or a (device) torch tensor"""
    if hasattr(a, "detach"):
        return a.detach().cpu().numpy()
    return a


def _path(p) -> bytes:
    return os.fsencode(os.fspath(p))


def write_params_csv(path, res: dict) -> None:
    params = _arr(_host(res["params"]), np.float64)
    status = _arr(_host(res["status"]), np.int32)
    n = status.shape[0]
    _check(_lib().kf_write_params_csv(_path(path), params.ctypes.data, status.ctypes.data, n,
                                      params.shape[1]))


def write_states_obj(path, res: dict, tel: Telescope) -> None:
    """Smoothed states (fit with smoothed=True) on the fit geometry."""
    sm = _arr(_host(res["smoothed"]), np.float64)
    n_meas = _arr(_host(res["n_meas"]), np.int32)
    status = _arr(_host(res["status"]), np.int32)
    mask = _arr(tel.hit_mask, np.uint64)
    geo, keep = tel.geometry()
    _check(_lib().kf_write_states_obj(_path(path), sm.ctypes.data, n_meas.ctypes.data,
                                      mask.ctypes.data, status.ctypes.data, status.shape[0],
                                      sm.shape[2], C.byref(geo)))


def measurement_positions(tel: Telescope) -> np.ndarray:
    """Global positions [S,3,n] of the measurements on the planes that
    produced them (truth geometry when the telescope is misaligned)."""
    c = tel.truth_center if tel.truth_center is not None else tel.center
    r = tel.truth_rotation if tel.truth_rotation is not None else tel.rotation
    r = np.asarray(r).reshape(-1, 3, 3)
    loc = np.stack([tel.meas[:, 0], tel.meas[:, 1], np.zeros_like(tel.meas[:, 0])], axis=1)
    return np.ascontiguousarray(np.einsum("sab,sbn->san", r, loc) + np.asarray(c)[:, :, None])


def write_sim_hits_obj(path, tel: Telescope, positions: np.ndarray | None = None) -> None:
    """One polyline per track through its hits (the measurements' global
    positions unless `positions` [S,3,n] is given)."""
    pos = _arr(measurement_positions(tel) if positions is None else positions, np.float64)
    mask = _arr(tel.hit_mask, np.uint64)
    _check(_lib().kf_write_hits_obj(_path(path), pos.ctypes.data, mask.ctypes.data, None,
                                    tel.n_surfaces, tel.n, pos.shape[2]))


def write_params_table(path, res: dict, tel: Telescope) -> None:
    params = _arr(_host(res["params"]), np.float64)
    cov = _arr(_host(res["cov"]), np.float64)
    status = _arr(_host(res["status"]), np.int32)
    truth = _arr(tel.truth, np.float64)
    vertex = _arr(tel.perigee, np.float64)
    _check(_lib().kf_write_params_table(_path(path), params.ctypes.data, cov.ctypes.data,
                                        status.ctypes.data, truth.ctypes.data, vertex.ctypes.data,
                                        status.shape[0], params.shape[1]))


PARAMS = ("eLOC0", "eLOC1", "ePHI", "eTHETA", "eQOP", "eT")
# residual histogram half-ranges of Performance/Scripts/perigeeParamResolution.C:45-50
RESIDUAL_RANGE = (0.25, 0.25, 0.08, 0.08, 0.002, 5000.0)


def _gauss_fit(values: np.ndarray, lo: float, hi: float, bins: int = 100) -> dict:
    """Binned Gaussian fit of a histogram of `values` over [lo, hi): chi2 with
    sqrt(N) bin errors over the non-empty bins (ROOT's default TH1::Fit with
    "gaus"); mean, sigma and their errors."""
    from scipy.optimize import curve_fit
    h, edges = np.histogram(values, bins=bins, range=(lo, hi))
    x = 0.5 * (edges[1:] + edges[:-1])
    use = h > 0
    if use.sum() < 3:
        return {"entries": int(h.sum()), "mean": float("nan"), "sigma": float("nan")}
    inside = values[(values >= lo) & (values < hi)]
    p0 = (float(h.max()), float(inside.mean()), float(max(inside.std(), (hi - lo) / bins)))
    f = lambda t, a, m, s: a * np.exp(-0.5 * ((t - m) / s) ** 2)
    popt, pcov = curve_fit(f, x[use], h[use], p0=p0, sigma=np.sqrt(h[use]), absolute_sigma=True)
    err = np.sqrt(np.diag(pcov))
    return {"entries": int(h.sum()), "mean": float(popt[1]), "mean_err": float(err[1]),
            "sigma": float(abs(popt[2])), "sigma_err": float(err[2])}


def resolution_report(table) -> dict:
    """The pull and residual summary of perigeeParamResolution.C on a params
    table (read_params_table, or any mapping of the writeParamsRoot column
    names to arrays): per parameter, a Gaussian fit to the pull histogram in
    [-5, 5) with 100 bins, and the residual RMS within the script's range."""
    out = {}
    for k, name in enumerate(PARAMS):
        pull = np.asarray(table["pull_" + name], dtype=np.float64)
        res = np.asarray(table["res_" + name], dtype=np.float64)
        r = RESIDUAL_RANGE[k]
        inr = res[(res >= -r) & (res < r)]
        out[name] = {"pull": _gauss_fit(pull, -5.0, 5.0),
                     "residual_rms": float(np.sqrt(np.mean(inr ** 2))) if inr.size else float("nan")}
    return out


def read_params_table(path) -> np.ndarray:
    """A file of write_params_table as a structured array (columns by name)."""
    return np.genfromtxt(path, delimiter=",", names=True)
