"""The host loops of the zone update and the resampling step give the same
results whatever the number of host threads (hg_set_host_threads): the
hybrid column's first zone update and resampling (100,000 material points
under 20,000 disks; about 27,000 points and 4,000 grains inserted), run with
one thread and with eight, bit for bit. The bit-exactness of the step
itself against the oracle is tested on a small scene in test_resampling.py;
this scene is large enough for every threaded loop to split.
"""
import math

import numpy as np
import pytest

import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import CONTINUUM, DISCRETE, scenes


def resample(threads):
    hg.set_host_threads(threads)
    try:
        scene = scenes.hybrid_column()
        cfg, sc, zs, rs = scene["mpm"], scene["dem"], scene["zones"], scene["resampling"]
        p = scenes.seed_column_points(cfg)
        h = cfg["h"]
        nx = math.ceil((cfg["grid_max"][0] - cfg["grid_min"][0]) / h)
        ny = math.ceil((cfg["grid_max"][1] - cfg["grid_min"][1]) / h)
        cx = 0.5 * (cfg["grid_min"][0] + cfg["grid_max"][0])
        cy = 0.5 * (cfg["grid_min"][1] + cfg["grid_max"][1])
        gmin = (cx - 0.5 * nx * h, cy - 0.5 * ny * h)
        gmax = (cx + 0.5 * nx * h, cy + 0.5 * ny * h)
        zargs = (gmin, h, (nx, ny), zs["level_set_cell_width"], zs["phi_window_size"],
                 zs["phi_samples_per_cell_side"], zs["phi_threshold"], zs["rzone_level_set"],
                 zs["rzone_half_thickness"], zs["allow_direct_transitions"])
        zones = hg.Zones(*zargs[:-1], allow_direct_transitions=zargs[-1])
        res = hg.Resampler(zargs, gmax, 1, h / 2, cfg["rho"], rs["dem_r_mean"],
                           rs["dem_r_std"], rs["rho_dem"], cfg["bulk_modulus"],
                           cfg["shear_modulus"], rs["newly_inserted_continuum_stress_free"],
                           rs["homogenize_stress"], rs["homogenize_velocity"])
        q = p["q"]
        i = np.floor((q[:, 0] - gmin[0]) / h).astype(int)
        j = np.floor((q[:, 1] - gmin[1]) / h).astype(int)
        labels = np.full(nx * ny, DISCRETE, dtype=np.int32)
        labels[j * nx + i] = CONTINUUM
        zones.set_labels(labels)
        zones.update(sc["q"], sc["r"], sc["fixed"], q)
        n = len(p["m"])
        rng = np.random.default_rng(1)
        be = np.tile([1.0, 0.0, 0.0, 1.0], (n, 1)) + rng.normal(scale=1e-4, size=(n, 4))
        v = rng.normal(scale=0.1, size=(n, 2))
        res.set_points(q, q, v, p["m"], p["vol"], p["m"], p["vol"], p["hl"], be,
                       np.ones(n), np.zeros(n, dtype=np.int32))
        M0 = np.stack([sc["m"], sc["m"], sc["I"]], axis=1)
        res.set_grains(sc["q"], sc["q"], sc["v"], sc["r"], M0, sc["fixed"])
        nn = (nx + 1) * (ny + 1)
        res.set_homogenized(rng.normal(size=(nn, 4)), rng.normal(size=(nn, 2)))
        res.run(zones)
        return zones.fields(), res.points(), res.grains(), res.stats()
    finally:
        hg.set_host_threads(0)


def test_results_do_not_depend_on_host_threads():
    Z1, P1, G1, S1 = resample(1)
    Z8, P8, G8, S8 = resample(8)
    for k in Z1:
        assert np.array_equal(Z1[k], Z8[k]), k
    assert S1[:2] == S8[:2]
    counts = ("points_inserted", "grains_inserted", "points_deleted", "grains_deleted")
    assert all(S1[2][k] == S8[2][k] for k in counts)
    assert S1[2]["points_inserted"] > 10000 and S1[2]["grains_inserted"] > 1000
    for k in P1:
        assert np.array_equal(P1[k], P8[k], equal_nan=True), k
    for k in G1:
        assert np.array_equal(G1[k], G8[k], equal_nan=True), k


def test_host_threads_are_checked():
    with pytest.raises(hg.HGError):
        hg.set_host_threads(-1)
