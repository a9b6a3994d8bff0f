"""Writes the golden fixtures of this directory: small seeded workloads
(inputs) with the oracle's fits of them (outputs) and the output writers'
files of one of them.

    python tests/golden/make_golden.py

Each case_<name>.npz holds the fit's inputs (measurements, hit masks,
lengths, seeds, perigee lines, plane frames, material, field grid), the
configuration fields that differ from the defaults, and the precise
oracle's outputs (parameters, covariance, chi2, status, steps; smoothed
states for two cases).  The inputs are stored, not regenerated, so the fixtures pin the
fit alone.  Regenerate only when the oracle's algorithm changes on purpose.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

# name -> (tracks, make_telescope keywords, config overrides)
CASES = {
    "uniform10": (48, dict(seed=101), dict(overstep_limit=0.1)),
    "reference_overstep": (48, dict(seed=102), dict()),  # the reference's 0.01 mm overstep
    "holes30": (48, dict(seed=103, n_planes=30, x_first=50., x_step=50., min_len=5, max_len=30,
                         hit_prob=0.9, outlier_prob=0.05),
                dict(overstep_limit=0.1, outlier_chi2_cut=25.0)),
    "map10": (32, dict(seed=104, field_map=True, field_n=11), dict(overstep_limit=0.1)),
    "material10": (48, dict(seed=105, material=0.5), dict(overstep_limit=0.1, material_effects=3)),
    "misaligned20": (32, dict(seed=106, n_planes=20, x_first=50., x_step=50., mis_shift=0.1,
                              mis_rot=1e-3), dict(overstep_limit=0.1)),
}

SMOOTHED = ("holes30", "material10")  # cases that keep the smoothed states
INPUTS = ("meas", "hit_mask", "n_planes", "start", "start_cov", "perigee", "truth", "center",
          "rotation")
OUTPUTS = ("params", "cov", "chi2", "status", "n_meas", "n_steps", "smoothed")


def main() -> None:
    import gpukalmanfitter_gb300 as kf
    import oracle
    from oracle import writers as ow
    for name, (n, tkw, ckw) in CASES.items():
        tel = kf.make_telescope(n, **tkw)
        cfg = kf.default_config(**ckw)
        out = oracle.fit(tel, cfg, threads=1, smoothed=True, variant="precise")
        arrays = {f"in_{k}": np.asarray(getattr(tel, k)) for k in INPUTS}
        if tel.material is not None:
            arrays["in_material"] = tel.material
        if tel.field_grid is not None:
            arrays["in_field_grid"] = tel.field_grid
            arrays["in_field_n"] = np.array(tel.field_n)
            arrays["in_field_half"] = np.array(tel.field_half)
        arrays["in_bz_tesla"] = np.array(tel.bz_tesla)
        for k in OUTPUTS:
            if k != "smoothed" or name in SMOOTHED:
                arrays[f"out_{k}"] = out[k]
        arrays["config_keys"] = np.array(list(ckw.keys()), dtype="U32")
        arrays["config_values"] = np.array(list(ckw.values()), dtype=np.float64)
        np.savez_compressed(HERE / f"case_{name}.npz", **arrays)
        if name == "holes30":
            (HERE / "holes30_params.csv").write_text(ow.params_csv(out["params"], out["status"]))
            (HERE / "holes30_states.obj").write_text(
                ow.states_obj(out["smoothed"], out["n_meas"], tel.hit_mask, out["status"],
                              tel.center, tel.rotation))
            (HERE / "holes30_table.csv").write_text(
                ow.params_table(out["params"], out["cov"], out["status"], tel.truth,
                                tel.perigee))
        print(name, n, "tracks", int((out["status"] == 0).sum()), "fitted")


if __name__ == "__main__":
    main()
