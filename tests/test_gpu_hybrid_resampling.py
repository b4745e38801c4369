"""The hybrid column with the resampling interval (HybridGrains2DSim): device
node-node steps, host zone labels and resampling every freq + 1 steps, state
copied back with the DEM contact history renumbered.

Checked on a reduced hybrid column (about 5,000 points under 1,000 disks,
resampling every 200 steps): the device status words stay clean, the
resampling inserts and deletes bodies, the DEM contact history survives the
renumbering, and the zone labels computed by the library at the last
interval equal the oracle's on the same FP64 positions (bit-exact, the
config-2 check of the zone labels).
"""
import numpy as np
import pytest

import oracle
import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import hybrid, scenes

pytestmark = pytest.mark.gpu


def test_hybrid_column_with_resampling(ctx):
    scene = scenes.hybrid_column(scale=0.05)
    sim = hybrid.HybridSim(ctx, scene)
    n0 = sim.counts()
    sim.step(450)
    assert sim.resamplings == 3  # the initial one and two intervals
    assert sim.mpm.status() == 0 and sim.dem.status() == 0
    st = sim.stats
    assert sum(s["points_inserted"] for s in st) > 0
    assert sum(s["points_deleted"] for s in st) + sum(s["grains_deleted"] for s in st) > 0
    assert sim.counts() != n0
    P = sim.mpm.download()
    q3, v3 = sim.dem.download()
    assert np.isfinite(P["q"]).all() and np.isfinite(q3).all() and np.isfinite(v3).all()
    assert sim.dem.num_contacts() > 0
    # zone labels on the current positions: library vs oracle, bit-exact
    z = scene["zones"]
    g = sim.mpm
    ours = hg.Zones(g.grid_min, scene["mpm"]["h"], (g.nx, g.ny), z["level_set_cell_width"],
                    z["phi_window_size"], z["phi_samples_per_cell_side"], z["phi_threshold"],
                    z["rzone_level_set"], z["rzone_half_thickness"])
    ref = oracle.Zones(g.grid_min, scene["mpm"]["h"], (g.nx, g.ny), z["level_set_cell_width"])
    ours.update(q3, sim.G["r"], sim.G["fixed"], P["q"])
    ref.update(q3, sim.G["r"], sim.G["fixed"], P["q"], z["phi_window_size"],
               z["phi_samples_per_cell_side"], z["phi_threshold"], z["rzone_level_set"],
               z["rzone_half_thickness"])
    a, b = ours.fields(), ref.fields()
    for k in ("phi", "dist", "ls", "mpm"):
        assert np.array_equal(a[k], b[k]), k
    assert (a["mpm"] == hg.HYBRID).any()
