"""Small cases run through whichever libhg_gpu variant HG_GPU_VARIANT selects
(a helper of tests/test_gpu_bounds.py, run as a subprocess: a process loads
one variant). Writes the final states and status words to an .npz file."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import libhybridgrains_gb300 as hg  # noqa: E402
from libhybridgrains_gb300 import scenes, serving  # noqa: E402
from libhybridgrains_gb300.hybrid import HybridSim  # noqa: E402


def main(out):
    ctx = hg.Context(0)
    res = {}
    # MIXED column: crosses periodic re-sorts, graph chunks and per-step calls
    cfg = scenes.serving_column(30000, 1.5, 30.0)
    p = scenes.seed_column_points(cfg)
    m = hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
               cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
               cfg["planes"], capacity=len(p["m"]))
    m.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    m.flow(cfg["dt"], 150)
    for _ in range(5):
        m.flow(cfg["dt"], 3)
    res["mixed_q"] = m.download()["q"]
    res["mixed_status"] = m.status()
    # batch of three scenes
    b = hg.Batch(ctx, 4)
    ms = []
    for n in (5000, 12000, 20000):
        c = scenes.serving_column(n, 2.0, 25.0)
        pp = scenes.seed_column_points(c)
        x = hg.MPM(ctx, c["grid_min"], c["grid_max"], c["h"], c["shear_modulus"],
                   c["bulk_modulus"], c["dp_alpha"], c["flip_alpha"], scenes.GRAVITY,
                   c["planes"], capacity=len(pp["m"]))
        x.upload(pp["q"], pp["v"], pp["m"], pp["vol"], pp["hl"])
        b.add(x, c["dt"])
        ms.append(x)
    b.step(120)
    res["batch_status"] = np.array([x.status() for x in ms])
    res["batch_q0"] = ms[0].download()["q"]
    # DEM piles with an edit
    piles = [serving.dem_pile(serving.Request(k, 0.0, None, 0, ndisks=600, aspect=1.0), k)
             for k in range(3)]
    d = serving.dem_for_piles(ctx, 2000)
    d.upload(*[np.concatenate([q[f] for q in piles[:2]]) for f in ("q", "v", "r", "m", "I")])
    d.flow(1e-5, 300)
    keep = np.concatenate([np.full(600, -1), np.arange(600)]).astype(np.int32)
    d.edit_async(keep, **{f: piles[2][f] for f in ("q", "v", "r", "m", "I")})
    d.flow(1e-5, 301)
    res["dem_q"], res["dem_v"] = d.download()
    res["dem_contacts"] = d.contacts()
    res["dem_status"] = d.status()
    # hybrid column, small
    sim = HybridSim(ctx, scenes.hybrid_column(scale=0.05))
    sim.step(60)
    res["hybrid_status"] = np.array([sim.mpm.status(), sim.dem.status()])
    res["hybrid_q"] = sim.mpm.download()["q"]
    np.savez(out, **res)


if __name__ == "__main__":
    main(sys.argv[1])
