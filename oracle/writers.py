"""The oracle of the output writers (test infrastructure): the reference
driver's writers restated in pure Python, as plain loops that follow
Run/Common/Writer.hpp statement by statement.  A default-formatted C++
stream prints a double as "%g" and an integer in decimal; both are written
with Python's printf-style formatting here, which follows C's.

Only tests/ use this module, as the checker of gpukalmanfitter_gb300.writer.
"""
from __future__ import annotations

import math

import numpy as np

DIAG = (0, 6, 11, 15, 18, 20)


def _g(x: float) -> str:
    return "%g" % x


def _obj_polylines(points_per_track) -> str:
    """writeSimHitsObj / writeStatesObj body (Writer.hpp:25-39, :55-76): the
    vertex counter advances once before a track's vertices and then along
    its segments; `points_per_track` yields a list of (x, y, z) per written
    track."""
    out = []
    v = 0
    for pts in points_per_track:
        v += 1
        for x, y, z in pts:
            out.append("v %s %s %s\n" % (_g(x), _g(y), _g(z)))
        brk = v + len(pts) - 1
        while v < brk:
            out.append("l %d %d\n" % (v, v + 1))
            v += 1
    return "".join(out)


def _plane_of_state(mask: int, k: int, S: int) -> int:
    bits = [j for j in range(S) if (mask >> j) & 1]
    return bits[k]


def states_obj(smoothed, n_meas, hit_mask, status, center, rotation) -> str:
    """writeStatesObj (Writer.hpp:42-78) on the smoothed states; state k of a
    track lies on the plane of the k-th hit; position = R (loc0, loc1, 0) + c
    (PlaneSurface::localToGlobal)."""
    S = len(center)

    def tracks():
        for i in range(len(status)):
            if status[i] != 0:  # Writer.hpp:57-59
                continue
            pts = []
            cnt = min(int(n_meas[i]), S, bin(int(hit_mask[i]) & ((1 << S) - 1)).count("1"))
            for k in range(max(cnt, 0)):
                pl = _plane_of_state(int(hit_mask[i]), k, S)
                l0, l1 = float(smoothed[k, 0, i]), float(smoothed[k, 1, i])
                R, c = rotation[pl], center[pl]
                pts.append(tuple((R[3 * a] * l0 + R[3 * a + 1] * l1 + R[3 * a + 2] * 0.0) + c[a]
                                 for a in range(3)))
            yield pts
    return _obj_polylines(tracks())


def sim_hits_obj(positions, hit_mask) -> str:
    """writeSimHitsObj (Writer.hpp:16-40): every track, its hits in plane
    order."""
    S = positions.shape[0]

    def tracks():
        for i in range(positions.shape[2]):
            m = int(hit_mask[i]) & ((1 << S) - 1)
            yield [tuple(float(positions[j, a, i]) for a in range(3)) for j in range(S)
                   if (m >> j) & 1]
    return _obj_polylines(tracks())


def params_csv(params, status) -> str:
    """writeParamsCsv (Writer.hpp:80-110)."""
    out = ["trackIdx, fit_BoundLoc0, fit_BoundLoc1, fit_BoundPhi, fit_BoundTheta, "
           "fit_BoundQOverP, fit_BoundTime\n"]
    for i in range(len(status)):
        if status[i] != 0:
            continue
        out.append("%d,%s\n" % (i, ",".join(_g(float(params[r, i])) for r in range(6))))
    return "".join(out)


PAR = ("eLOC0", "eLOC1", "ePHI", "eTHETA", "eQOP", "eT")
TABLE_COLUMNS = (["t_charge", "t_time", "t_vx", "t_vy", "t_vz", "t_px", "t_py", "t_pz",
                  "t_theta", "t_phi", "t_eta", "t_pT"] + [p + "_fit" for p in PAR]
                 + ["err_" + p + "_fit" for p in PAR] + ["res_" + p for p in PAR]
                 + ["pull_" + p for p in PAR])


def params_table(params, cov, status, truth, vertex) -> str:
    """writeParamsRoot's record per fitted track (Writer.hpp:188-225): the
    truth particle from the true perigee parameters (unit charge of the sign
    of q/p, momentum 1/|q/p| along (phi, theta)), truth parameters (loc0,
    loc1, phi, theta, q/p, t), fit, sqrt of the covariance diagonal, fit -
    truth and their ratio."""
    out = [",".join(TABLE_COLUMNS) + "\n"]
    for i in range(len(status)):
        if status[i] != 0:
            continue
        qop, phi0, th0 = float(truth[4, i]), float(truth[2, i]), float(truth[3, i])
        charge = 1 if qop > 0 else -1
        p = abs(1.0 / qop)
        d = (math.cos(phi0) * math.sin(th0), math.sin(phi0) * math.sin(th0), math.cos(th0))
        perp = math.sqrt(d[0] * d[0] + d[1] * d[1])
        theta = math.atan2(perp, d[2])
        phi = math.atan2(d[1], d[0])
        eta = math.atanh(d[2] / math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]))
        t = float(truth[5, i])
        row = ["%d" % charge] + [_g(x) for x in (t, float(vertex[0, i]), float(vertex[1, i]),
                                                 float(vertex[2, i]), p * d[0], p * d[1],
                                                 p * d[2], theta, phi, eta, p * perp)]
        tp = (float(truth[0, i]), float(truth[1, i]), phi, theta, charge / p, t)
        fit = [float(params[r, i]) for r in range(6)]
        err = [math.sqrt(float(cov[DIAG[r], i])) for r in range(6)]
        res = [fit[r] - tp[r] for r in range(6)]
        pull = [res[r] / err[r] for r in range(6)]
        row += [_g(x) for x in fit + err + res + pull]
        out.append(",".join(row) + "\n")
    return "".join(out)


def read_table(path) -> np.ndarray:
    """The params table as a structured array (column names as fields)."""
    return np.genfromtxt(path, delimiter=",", names=True)
