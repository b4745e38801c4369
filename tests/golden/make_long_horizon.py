"""Writes column_12800_50k.json: the shape of the 12,800-point column collapse
after 30,000 and 50,000 FP64 oracle steps (0.3 s and 0.5 s; by 0.5 s the
front has reached the far wall of the 1 m domain), for the long-horizon test
of the GPU paths. Run from the repository root (takes a few minutes on one core):

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

CHECKPOINTS = (30000, 50000)
STRIP = 0.01  # m


def shape(q, xmax=1.0, pct=95.0, nmin=10):
    """Front position and the free-surface height per strip: the 95th
    percentile of the heights of the strip's points (strips with fewer than
    10 points: 0), which single points thrown up at the walls do not move."""
    bins = np.floor(q[:, 0] / STRIP).astype(int)
    prof = np.zeros(int(round(xmax / STRIP)))
    for k in range(len(prof)):
        y = q[bins == k, 1]
        if len(y) >= nmin:
            prof[k] = np.percentile(y, pct)
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
    out = {"scene": "column_12800", "dt": cfg["dt"], "strip_width_m": STRIP, "checkpoints": []}
    done = 0
    for steps in CHECKPOINTS:
        m.step(cfg["dt"], steps - done)
        done = steps
        front, prof = shape(m.particles()["q"])
        out["checkpoints"].append({"steps": steps, "front_x_m": front,
                                   "profile_p95_y_m": [round(float(v), 12) for v in prof]})
    with open(os.path.join(HERE, "column_12800_50k.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
