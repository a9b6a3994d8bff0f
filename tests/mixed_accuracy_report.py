"""Accuracy of the mixed-precision form against the FP64 oracle (a report,
not a test; needs a GPU).  For each workload it fits the same seeded tracks
with the batched mixed-precision form on the GPU and with the oracle's
precise build on the host, and prints one JSON line per workload:

- per fitted parameter (d0, z0, phi, theta, q/p, t): median / p99 / max of
  |mixed - FP64| / max(|FP64|, sigma), and of |mixed - FP64| / sigma;
- chi2: median / p99 of |mixed - FP64| / FP64;
- pull widths (std of (fit - truth) / sigma) of both, and their ratio;
- fractions of tracks with equal status and equal RK step counts.

    python tests/mixed_accuracy_report.py [n_tracks]
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

DIAG = [0, 6, 11, 15, 18, 20]
NAMES = ["d0", "z0", "phi", "theta", "qop", "t"]
WORKLOADS = {
    "uniform10": {},
    "map30": dict(n_planes=30, x_first=50., x_step=50., field_map=True),
}


def report(n: int) -> None:
    import gpukalmanfitter_gb300 as kf
    import oracle
    for name, kw in WORKLOADS.items():
        tel = kf.make_telescope(n, seed=2024, **kw)
        cfg = kf.default_config(overstep_limit=0.1, precision=1)
        b = kf.DeviceBatch(tel, cfg)
        b.fit_sorted()
        g = b.results()
        o = oracle.fit(tel, kf.default_config(overstep_limit=0.1), threads=0, variant="precise")
        ok = (g["status"] == 0) & (o["status"] == 0)
        sig = np.sqrt(np.abs(o["cov"][DIAG]))[:, ok]
        d = np.abs(g["params"][:, ok] - o["params"][:, ok])
        rel = d / np.maximum(np.abs(o["params"][:, ok]), sig)
        ins = d / np.where(sig > 0, sig, 1.0)
        out = {"workload": name, "tracks": n,
               "status_equal": float(np.mean(g["status"] == o["status"])),
               "steps_equal": float(np.mean(g["n_steps"] == o["n_steps"]))}
        for k, nm in enumerate(NAMES):
            out[nm] = {"rel_median": float(np.median(rel[k])), "rel_p99": float(np.percentile(rel[k], 99)),
                       "rel_max": float(rel[k].max()), "sigma_median": float(np.median(ins[k])),
                       "sigma_max": float(ins[k].max())}
        c = np.abs(g["chi2"][ok] - o["chi2"][ok]) / np.maximum(o["chi2"][ok], 1e-300)
        out["chi2_rel"] = {"median": float(np.median(c)), "p99": float(np.percentile(c, 99))}
        pw = {}
        for lab, r in (("mixed", g), ("fp64", o)):
            pulls = (r["params"] - tel.truth)[:5, ok] / np.sqrt(np.abs(r["cov"][DIAG]))[:5, ok]
            pw[lab] = pulls.std(axis=1)
        out["pull_width_mixed"] = [round(float(x), 5) for x in pw["mixed"]]
        out["pull_width_fp64"] = [round(float(x), 5) for x in pw["fp64"]]
        out["pull_width_ratio_minus_1"] = [float(x) for x in pw["mixed"] / pw["fp64"] - 1]
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    report(int(sys.argv[1]) if len(sys.argv) > 1 else 50_000)
