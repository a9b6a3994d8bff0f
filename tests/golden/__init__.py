"""Golden fixtures (see make_golden.py) and their loader."""
from __future__ import annotations

from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
NAMES = ("uniform10", "reference_overstep", "holes30", "map10", "material10", "misaligned20")


def load(name: str):
    """(Telescope, config, expected outputs) of one golden case."""
    import gpukalmanfitter_gb300 as kf
    z = np.load(HERE / f"case_{name}.npz")
    g = lambda k: z[f"in_{k}"]
    n = g("meas").shape[2]
    S = g("meas").shape[0]
    grid = z["in_field_grid"] if "in_field_grid" in z else None
    tel = kf.Telescope(n, S, g("center"), g("rotation"), g("meas"), g("hit_mask"),
                       g("n_planes"), g("start"), g("start_cov"), g("perigee"), g("truth"),
                       float(z["in_bz_tesla"]), grid,
                       int(z["in_field_n"]) if grid is not None else 0,
                       float(z["in_field_half"]) if grid is not None else 0.0,
                       material=z["in_material"] if "in_material" in z else None)
    cfg = kf.default_config(**{str(k): (int(v) if str(k) == "material_effects" else float(v))
                               for k, v in zip(z["config_keys"], z["config_values"])})
    out = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return tel, cfg, out
