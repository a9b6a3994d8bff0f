"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session")
def kf():
    import gpukalmanfitter_gb300 as kf
    kf.load()
    return kf


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.load()
    return oracle


def rel_close(gpu: dict, ref: dict, tol: float = 1e-9, mask=None):
    """Compare fit outputs with a relative tolerance.

    Parameters use max(|ref|, sigma) as scale (sigma from the reference
    covariance), covariance elements use sqrt(C_ii C_jj), chi2 uses
    max(|chi2|, 1).  Returns the worst ratio |diff| / (tol * scale).
    """
    diag = [0, 6, 11, 15, 18, 20]
    sel = slice(None) if mask is None else mask
    rc = ref["cov"][:, sel]
    sig = np.sqrt(np.abs(rc[diag]))
    worst = 0.0
    scale_p = np.maximum(np.abs(ref["params"][:, sel]), sig)
    scale_p = np.where(scale_p > 0, scale_p, 1.0)
    worst = max(worst, float(np.max(np.abs(gpu["params"][:, sel] - ref["params"][:, sel]) / (tol * scale_p), initial=0)))
    e = 0
    for i in range(6):
        for j in range(i, 6):
            s = np.sqrt(np.abs(rc[diag[i]] * rc[diag[j]]))
            s = np.where(s > 0, s, 1.0)
            worst = max(worst, float(np.max(np.abs(gpu["cov"][e, sel] - rc[e]) / (tol * s), initial=0)))
            e += 1
    sc = np.maximum(np.abs(ref["chi2"][sel]), 1.0)
    worst = max(worst, float(np.max(np.abs(gpu["chi2"][sel] - ref["chi2"][sel]) / (tol * sc), initial=0)))
    return worst


def parity_report(gpu: dict, ref: dict, tol: float = 1e-9, mask=None):
    """Worst deviations in units of ``tol`` and the number of covariance
    elements above ``tol``.

    Parameters use the scale max(|x|, sigma_x), chi2 max(chi2, 1) and
    covariance elements sqrt(C_ii C_jj).
    """
    diag = [0, 6, 11, 15, 18, 20]
    sel = np.ones(ref["chi2"].shape, bool) if mask is None else mask
    rc = ref["cov"][:, sel]
    sig = np.sqrt(np.abs(rc[diag]))
    sp = np.maximum(np.abs(ref["params"][:, sel]), sig)
    sp = np.where(sp > 0, sp, 1.0)
    rep = {"params": float(np.max(np.abs(gpu["params"][:, sel] - ref["params"][:, sel]) / (tol * sp), initial=0))}
    sc = np.maximum(np.abs(ref["chi2"][sel]), 1.0)
    rep["chi2"] = float(np.max(np.abs(gpu["chi2"][sel] - ref["chi2"][sel]) / (tol * sc), initial=0))
    worst, over, e = 0.0, 0, 0
    for i in range(6):
        for j in range(i, 6):
            s = np.sqrt(np.abs(rc[diag[i]] * rc[diag[j]]))
            s = np.where(s > 0, s, 1.0)
            r = np.abs(gpu["cov"][e, sel] - rc[e]) / (tol * s)
            worst = max(worst, float(np.max(r, initial=0)))
            over += int(np.sum(r > 1.0))
            e += 1
    rep["cov"] = worst
    rep["cov_elements_over_tol"] = over
    return rep
