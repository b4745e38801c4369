"""Node-node hybrid step through the C ABI against the CPU oracle
(hybridgrains2dnew/HybridGrains2DSim.cpp:116-220, Coupling.cpp).

FP64 on both sides; the grain-to-grid scatters use FP64 atomics, so the
comparison tolerance is 1e-10 relative (summation order only)."""
import numpy as np
import pytest

import oracle
import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import scenes

pytestmark = pytest.mark.gpu


def rel(a, b):
    den = np.abs(b).max()
    return np.abs(a - b).max() / (den if den > 0 else 1.0)


def hybrid_scene(basis):
    cfg = scenes.mpm_column("column_12800", grid_min=(-0.01, -0.01))
    cfg["rect_min"], cfg["rect_max"] = (0.1, 0.0), (0.3, 0.1)
    p = scenes.seed_column_points(cfg)
    # grains in the upper part of the column and above it (hybrid band)
    sc = scenes.dem_column(n=800, per_row=40, pitch=4.4e-3, rmin=1.8e-3, rmax=2.2e-3,
                           jitter=0.1e-3, x0=0.11, y0=0.07, rho=1550.0)
    sc["v"][:, 1] = -0.05
    w = np.where(sc["q"][:, 1] < 0.1, 0.5, 1.0)
    return cfg, p, sc, w


@pytest.mark.parametrize("basis", [0, 1])
def test_hybrid_step_matches_oracle(ctx, basis):
    cfg, p, sc, w = hybrid_scene(basis)
    dp = scenes.dem_params(kn=1e4)
    planes_dem = [((0.0, 0.0), (0.0, 1.0)), ((0.0, 0.0), (1.0, 0.0))]
    gm = hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
                cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
                cfg["planes"], basis=basis, precision=hg.FP64, capacity=len(p["m"]))
    gm.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    gd = hg.DEM(ctx, scenes.GRAVITY, dp["kn"], dp["kt"], dp["gamman"], dp["gammat"], dp["mu"],
                planes_dem, capacity=len(sc["r"]))
    gd.upload(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"])
    gd.set_weights(w)
    gh = hg.Hybrid(ctx, gm, gd)

    cm = oracle.MPM(cfg["grid_min"], cfg["grid_max"], cfg["h"], basis=basis,
                    shear_modulus=cfg["shear_modulus"], bulk_modulus=cfg["bulk_modulus"],
                    dp_alpha=cfg["dp_alpha"], flip_alpha=cfg["flip_alpha"],
                    gravity=scenes.GRAVITY)
    for (x, n, st, lb) in cfg["planes"]:
        cm.add_plane(x, n, st, lb)
    cm.set_particles(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    cd = oracle.DEM(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"], scenes.GRAVITY,
                    dp["kn"], dp["kt"], dp["gamman"], dp["gammat"], dp["mu"], 1.0)
    for (x, n) in planes_dem:
        cd.add_plane(x, n)
    cd.set_weights(w)
    ch = oracle.Hybrid(cm, cd)

    dt = 1e-5
    for _ in range(2):
        gh.step(dt, 3, homogenize_stress=True, homogenize_velocity=True)
        ch.step(dt, 3, homogenize_stress=True, homogenize_velocity=True)
        A, B = gh.coupling(), ch.coupling()
        assert len(B["packed_dem"]) > 0 and len(B["packed_mpm"]) > 0
        assert np.array_equal(A["packed_dem"], B["packed_dem"])
        assert np.array_equal(A["packed_mpm"], B["packed_mpm"])
        for k in ("dem_mass_grid", "dem_mom_grid", "v_after", "at_after", "homog_stress",
                  "homog_velocity"):
            assert rel(A[k], B[k]) <= 1e-10, k
        assert np.array_equal(A["homog_factor"], B["homog_factor"])
        qg, vg = gd.download()
        qc, vc = cd.state()
        assert np.abs(qg - qc).max() <= 1e-15
        assert rel(vg, vc) <= 1e-10
        P, Q = gm.download(), cm.particles()
        assert np.abs(P["q"] - Q["q"]).max() <= 1e-15
        assert rel(P["v"], Q["v"]) <= 1e-10
