"""Algorithmic FP64 operation counts of the fit, per counted event.

Counted by hand from the structure-exploiting kernel in csrc/kf_device.cuh
(one add, multiply, divide, square root or transcendental call = 1 FLOP; a
fused multiply-add = 2).  The kernel reports, per track, the RK trials, the
accepted RK steps and the measurement states, so the FLOPs of a batch are

    F = trials*RK_TRIAL + steps*RK_STEP + states*FILTER
        + (states - tracks_fitted)*SMOOTH + tracks*FIXED

with POLY_TRIAL/POLY_STEP in place of RK_TRIAL/RK_STEP in a uniform field.

The dense formulation of the reference (8x8 D*J per step, 8x8*8x6 and 6x8*8x6
per surface, dense 6x6 products in updater and smoother) would count about
2.7x more for the same events; DENSE_* give those figures for context.
"""
from __future__ import annotations

import numpy as np

# structure-exploiting kernel (what runs on the GPU)
RK_TRIAL = 94      # field map: one tryRungeKuttaStep: 2 field points, k1..k4, error estimate
RK_STEP = 591      # field map: accepted step: time, transport matrix blocks, D*J on 25 entries, motion
# uniform field: the step through c = d x B, e = c x B (kfa::polyPrep/polyCoef/polyAcceptFwd)
POLY_TRIAL = 24    # trial coefficients and error estimate
POLY_STEP = 354    # c, e (23) + motion, k4, D blocks (173) + D*J (139) + path (1) + navigation (18)
FILTER = 936       # boundState to a plane (J C J^T on the non-zeros) + gain update + reload
SMOOTH = 367       # one RTS smoother state: structured J^-1 (gain), state, Pg <- G Pg
FIXED = 1270       # start state on the perigee line, C_s(0) = Pg C Pg^T, final transport

# dense reference formulation, same events
DENSE_RK_TRIAL = 94
DENSE_RK_STEP = 1024 + 400 + 60
DENSE_FILTER = 768 + 96 + 576 + 864 + 432 + 300
DENSE_SMOOTH = 6 * 6 * 6 * 2 * 4 + 500
DENSE_FIXED = 2400


def batch_flops(n_trials, n_steps, n_meas, status, dense: bool = False,
                uniform: bool = False) -> float:
    """FP64 FLOPs of one fit of a batch from the kernel's per-track counters
    (uniform: the uniform-field step formulation)."""
    t = np.asarray(n_trials, dtype=np.float64).sum()
    s = np.asarray(n_steps, dtype=np.float64).sum()
    m = np.asarray(n_meas, dtype=np.float64)
    fitted = np.asarray(status) == 0
    smooth = np.clip(m - 1, 0, None)[fitted].sum()
    if dense:
        return (t * DENSE_RK_TRIAL + s * DENSE_RK_STEP + m.sum() * DENSE_FILTER
                + smooth * DENSE_SMOOTH + len(m) * DENSE_FIXED)
    trial, step = (POLY_TRIAL, POLY_STEP) if uniform else (RK_TRIAL, RK_STEP)
    return t * trial + s * step + m.sum() * FILTER + smooth * SMOOTH + len(m) * FIXED


def batch_bytes(n_tracks: int, n_surfaces: int) -> dict:
    """Algorithmic HBM bytes of one fit: inputs read once, outputs written
    once, smoother states written and read back once."""
    inputs = n_tracks * (n_surfaces * 5 * 8 + 8 + 4 + 6 * 8 + 21 * 8 + 3 * 8)
    outputs = n_tracks * (6 * 8 + 21 * 8 + 8 + 4 * 4)
    workspace = 2 * n_tracks * n_surfaces * 37 * 8  # stored states (kStateStride doubles)
    return {"inputs": inputs, "outputs": outputs, "workspace": workspace,
            "total": inputs + outputs + workspace}
