"""Parity at the benchmark sizes, against the CPU oracle.

* 2,000,000-point column (2048 x 1024 grid, h = 1 mm, dt = 2e-6 s): one step
  from a stressed state on the GPU in FP64 and in mixed precision against one
  oracle step (OpenMP over the host cores). FP64: grid fields and particle
  state within 1e-12 relative (1e-15 m on positions); mixed: grid velocity
  ||dv||_2 / ||v||_2 <= 1e-5 over the active nodes, grid mass 1e-6
  relative, positions 1e-12 m, J and be_bar 1e-6.
* 10,000 disks compacted to about 2.5 contacts per disk, FP64: 300 steps
  with positions, velocities and the whole collision cache bit-exact.
* hybrid column at full scale (100,000 uGIMP points under 20,000 disks):
  three coupled steps before the first resampling, coupling buffers and
  states within 1e-10 relative (FP64 atomics change summation order only).

Set HG_PARITY_REPORT to a file name to append each measured error to it as
JSON lines.
"""
import json
import os

import numpy as np
import pytest

import oracle
import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import scenes

pytestmark = pytest.mark.gpu


def rel(a, b):
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))


def report(case, **errors):
    path = os.environ.get("HG_PARITY_REPORT")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps(dict(case=case, **{k: float(v) for k, v in errors.items()})) + "\n")


def gpu_mpm(ctx, cfg, precision, n):
    g = hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
               cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
               cfg["planes"], precision=precision, capacity=n)
    return g


def cpu_mpm(cfg, threads):
    c = oracle.MPM(cfg["grid_min"], cfg["grid_max"], cfg["h"],
                   shear_modulus=cfg["shear_modulus"], bulk_modulus=cfg["bulk_modulus"],
                   dp_alpha=cfg["dp_alpha"], flip_alpha=cfg["flip_alpha"],
                   gravity=scenes.GRAVITY, threads=threads)
    for (x, n, st, lb) in cfg["planes"]:
        c.add_plane(x, n, st, lb)
    return c


def test_column_2M_one_step_fp64_and_mixed_against_oracle(ctx):
    cfg = scenes.mpm_column("column_2M")
    p = scenes.seed_column_points(cfg)
    n = len(p["m"])
    assert n == 2000000
    dt = cfg["dt"]
    # a stressed state: 5,000 mixed-precision steps (10 ms) from rest, so
    # that the elastic wave has crossed half the column
    warm = gpu_mpm(ctx, cfg, hg.MIXED, n)
    warm.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    warm.flow(dt, 5000)
    s = warm.download()
    assert warm.status() == 0
    warm.close()
    assert np.abs(s["be"] - [1.0, 0.0, 0.0, 1.0]).max() > 1e-4
    c = cpu_mpm(cfg, os.cpu_count() or 1)
    c.set_particles(s["q"], s["v"], p["m"], p["vol"], p["hl"], s["be"], s["J"], s["jh"])
    c.step(dt)
    C, Q = c.grid(), c.particles()
    act = C["mass"] > 0
    assert act.sum() > 400000

    f = gpu_mpm(ctx, cfg, hg.FP64, n)
    f.upload(s["q"], s["v"], p["m"], p["vol"], p["hl"], s["be"], s["J"], s["jh"])
    f.flow(dt)
    G, P = f.grid(), f.download()
    errs = {k: rel(G[k], C[k]) for k in ("mass", "mom", "mom_new", "force", "vel", "acc")}
    errs["q_abs"] = float(np.abs(P["q"] - Q["q"]).max())
    errs["v"] = rel(P["v"], Q["v"])
    errs["J_abs"] = float(np.abs(P["J"] - Q["J"]).max())
    errs["be_abs"] = float(np.abs(P["be"] - Q["be"]).max())
    report("column_2M fp64", **errs)
    for k in ("mass", "mom", "mom_new", "force", "vel", "acc", "v"):
        assert errs[k] <= 1e-12, (k, errs[k])
    assert errs["q_abs"] <= 1e-15
    assert errs["J_abs"] <= 1e-13 and errs["be_abs"] <= 1e-13
    assert np.array_equal(P["jh"], Q["jh"])
    assert f.status() == 0
    f.close()

    m = gpu_mpm(ctx, cfg, hg.MIXED, n)
    m.upload(s["q"], s["v"], p["m"], p["vol"], p["hl"], s["be"], s["J"], s["jh"])
    m.flow(dt)
    G, P = m.grid(), m.download()
    assert np.array_equal(G["mass"] > 0, act)
    errs = {"grid_velocity_l2": float(np.linalg.norm(G["vel"][act] - C["vel"][act]) /
                                      np.linalg.norm(C["vel"][act])),
            "grid_mass": rel(G["mass"], C["mass"]),
            "grid_acceleration_l2": float(np.linalg.norm(G["acc"][act] - C["acc"][act]) /
                                          np.linalg.norm(C["acc"][act])),
            "q_abs": float(np.abs(P["q"] - Q["q"]).max()),
            "v_l2": float(np.linalg.norm(P["v"] - Q["v"]) / np.linalg.norm(Q["v"])),
            "J_abs": float(np.abs(P["J"] - Q["J"]).max()),
            "be_abs": float(np.abs(P["be"] - Q["be"]).max())}
    report("column_2M mixed", **errs)
    assert errs["grid_velocity_l2"] <= 1e-5, errs
    assert errs["grid_mass"] <= 1e-6, errs
    assert errs["q_abs"] <= 1e-12, errs
    assert errs["J_abs"] <= 1e-6 and errs["be_abs"] <= 1e-6, errs
    assert m.status() == 0
    m.close()


def test_dense_dem_10k_bit_exact(ctx):
    sc = scenes.dem_packed(n=10000, per_row=100)
    dp = scenes.dem_params()
    n = len(sc["r"])
    g = hg.DEM(ctx, scenes.GRAVITY, dp["kn"], dp["kt"], dp["gamman"], dp["gammat"], dp["mu"],
               sc["planes"], capacity=n, contact_capacity=8 * n)
    g.upload(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"])
    c = oracle.DEM(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"], scenes.GRAVITY,
                   dp["kn"], dp["kt"], dp["gamman"], dp["gammat"], dp["mu"], 1.0)
    for (x, nn) in sc["planes"]:
        c.add_plane(x, nn)
    for _ in range(3):
        g.flow(1e-6, 100)
        c.step(1e-6, 100)
        Qg, Vg = g.download()
        Qc, Vc = c.state()
        assert np.array_equal(Qg, Qc)
        assert np.array_equal(Vg, Vc)
        Rg, Rc = g.contacts(), c.contacts()
        assert Rg.shape == Rc.shape
        assert np.array_equal(Rg, Rc)
        assert len(Rc) >= 2 * n  # at least two contacts per disk throughout
    report("dem_packed_10k fp64", contacts_per_disk=len(Rc) / n, q_equal=1.0, v_equal=1.0,
           cache_equal=1.0)
    assert g.status() == 0


def test_hybrid_full_scale_coupled_steps_against_oracle(ctx):
    scene = scenes.hybrid_column()
    cfg, sc, dp = scene["mpm"], scene["dem"], scene["dem_params"]
    p = scenes.seed_column_points(cfg)
    assert len(p["m"]) == 100000 and len(sc["r"]) == 20000
    # grains below the top of the bulk are in the coupling band
    w = np.where(sc["q"][:, 1] < cfg["rect_max"][1], 0.5, 1.0)
    planes_dem = [(pl[0], pl[1]) for pl in cfg["planes"]]
    gm = hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
                cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
                cfg["planes"], basis=hg.UGIMP, precision=hg.FP64, capacity=len(p["m"]))
    gm.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    gd = hg.DEM(ctx, scenes.GRAVITY, dp["kn"], dp["kt"], dp["gamman"], dp["gammat"], dp["mu"],
                planes_dem, capacity=len(sc["r"]))
    gd.upload(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"])
    gd.set_weights(w)
    gh = hg.Hybrid(ctx, gm, gd)
    cm = oracle.MPM(cfg["grid_min"], cfg["grid_max"], cfg["h"], basis=1,
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
    dt = cfg["dt"]
    worst = {}
    for _ in range(3):
        gh.step(dt, 1, homogenize_stress=True, homogenize_velocity=True)
        ch.step(dt, 1, homogenize_stress=True, homogenize_velocity=True)
        A, B = gh.coupling(), ch.coupling()
        assert len(B["packed_dem"]) > 400 and len(B["packed_mpm"]) > 400
        assert np.array_equal(A["packed_dem"], B["packed_dem"])
        assert np.array_equal(A["packed_mpm"], B["packed_mpm"])
        assert np.array_equal(A["homog_factor"], B["homog_factor"])
        errs = {k: rel(A[k], B[k]) for k in ("dem_mass_grid", "dem_mom_grid", "v_after",
                                             "at_after", "homog_stress", "homog_velocity")}
        qg, vg = gd.download()
        qc, vc = cd.state()
        errs["grain_q_abs"] = float(np.abs(qg - qc).max())
        errs["grain_v"] = rel(vg, vc)
        P, Q = gm.download(), cm.particles()
        errs["point_q_abs"] = float(np.abs(P["q"] - Q["q"]).max())
        errs["point_v"] = rel(P["v"], Q["v"])
        G, C = gm.grid(), cm.grid()
        errs["grid_vel"] = rel(G["vel"], C["vel"])
        for k, v in errs.items():
            worst[k] = max(worst.get(k, 0.0), v)
        for k in ("dem_mass_grid", "dem_mom_grid", "v_after", "at_after", "homog_stress",
                  "homog_velocity", "grain_v", "point_v", "grid_vel"):
            assert errs[k] <= 1e-10, (k, errs[k])
        assert errs["grain_q_abs"] <= 1e-15 and errs["point_q_abs"] <= 1e-15, errs
    report("hybrid_column full scale fp64", **worst)
    assert gm.status() == 0 and gd.status() == 0
