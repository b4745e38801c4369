"""Writes column_12800_30k.json: the shape of the 12,800-point column collapse
after 30,000 FP64 oracle steps (0.3 s), for the long-horizon test of the GPU
paths. Run from the repository root (takes a few minutes on one core):

    python tests/golden/make_long_horizon.py

The oracle runs single-threaded so that its summation order, and so the
result, is reproducible.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from libhybridgrains_gb300 import scenes  # noqa: E402

STEPS = 30000
STRIP = 0.01  # m


def shape(q, xmax=1.0):
    bins = np.floor(q[:, 0] / STRIP).astype(int)
    prof = np.zeros(int(round(xmax / STRIP)))
    np.maximum.at(prof, np.clip(bins, 0, len(prof) - 1), q[:, 1])
    return float(q[:, 0].max()), prof


def main():
    cfg = scenes.mpm_column("column_12800")
    p = scenes.seed_column_points(cfg)
    m = oracle.MPM(cfg["grid_min"], cfg["grid_max"], cfg["h"], basis=0,
                   shear_modulus=cfg["shear_modulus"], bulk_modulus=cfg["bulk_modulus"],
                   dp_alpha=cfg["dp_alpha"], flip_alpha=cfg["flip_alpha"],
                   gravity=scenes.GRAVITY)
    for (x, n, st, lb) in cfg["planes"]:
        m.add_plane(x, n, st, lb)
    m.set_particles(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    m.set_threads(0)
    m.step(cfg["dt"], STEPS)
    front, prof = shape(m.particles()["q"])
    out = {"scene": "column_12800", "steps": STEPS, "dt": cfg["dt"], "strip_width_m": STRIP,
           "front_x_m": front, "profile_top_y_m": [round(float(v), 12) for v in prof]}
    with open(os.path.join(HERE, "column_12800_30k.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
