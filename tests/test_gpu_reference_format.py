"""The reference's MPM snapshot and frame datasets from device objects.

A snapshot written from a device FP64 scene, read back and loaded into a new
object steps on as the original does (1e-12 m: FP64 atomic order); frame
files carry the reference's dataset names and shapes.
"""
import numpy as np
import pytest

import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import frames, reference_format as rf, scenes, serving

pytestmark = pytest.mark.gpu


def test_snapshot_resume(ctx, tmp_path):
    cfg = scenes.mpm_column("column_12800")
    p = scenes.seed_column_points(cfg)
    a = hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
               cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
               cfg["planes"], precision=hg.FP64, capacity=len(p["m"]))
    a.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    a.flow(cfg["dt"], 20)
    state = rf.snapshot_from_device(a, cfg, p["m"], p["vol"], p["hl"], q0=p["q"])
    run = dict(iteration=20, dt=(1, 100000), end_time=0.5, steps_per_save=100)
    path = tmp_path / "serial_00001.bin"
    rf.write_mpm_snapshot(path, state, run)
    s2, r2 = rf.read_mpm_snapshot(path)
    assert r2["iteration"] == 20 and tuple(r2["dt"]) == (1, 100000)
    assert np.array_equal(s2["points"]["q"], a.download()["q"])
    assert np.array_equal(s2["grid"]["mass"], a.grid()["mass"])
    b = rf.device_from_snapshot(ctx, s2)
    a.flow(cfg["dt"], 10)
    b.flow(cfg["dt"], 10)
    A, B = a.download(), b.download()
    assert np.abs(A["q"] - B["q"]).max() <= 1e-12
    assert np.abs(A["J"] - B["J"]).max() <= 1e-12
    assert a.status() == 0 and b.status() == 0


def test_frame_datasets(ctx, tmp_path):
    cfg = scenes.serving_column(20000, 2.0, 30.0)
    p = scenes.seed_column_points(cfg)
    m = hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
               cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
               cfg["planes"], capacity=len(p["m"]))
    m.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    m.flow(cfg["dt"], 50)
    pile = serving.dem_pile(serving.Request(1, 0.0, None, 0, ndisks=500, aspect=1.0), 0)
    d = serving.dem_for_piles(ctx, 500)
    d.upload(pile["q"], pile["v"], pile["r"], pile["m"], pile["I"], pile["fixed"])
    d.flow(1e-5, 50)
    path = frames.frame_path(tmp_path, 3)
    assert path.endswith("config_00003.npz")
    frames.write(path, frames.mpm_frame(m, cfg, p["m"], p["vol"], p["hl"]),
                 frames.dem_frame(d, pile["r"], pile["m"]))
    f = frames.read(path)
    n = len(p["m"])
    assert int(f["mpm/npoints"]) == n and f["mpm/q"].shape == (2, n)
    assert np.array_equal(f["mpm/q"].T, m.download()["q"])
    nn = (m.nx + 1) * (m.ny + 1)
    assert f["mpm/grid_node_positions"].shape == (2 * nn,)
    assert np.allclose(f["mpm/grid_node_positions"][2 * (m.nx + 2):2 * (m.nx + 2) + 2],
                       np.add(m.grid_min, cfg["h"]))
    assert f["mpm/grid_node_masses"].sum() == pytest.approx(p["m"].sum(), rel=1e-5)
    assert np.all(f["mpm/p"] >= -1.0) and f["mpm/p"].max() > 0  # compressed column
    assert f["discrete/q"].shape == (3 * 500,) and f["discrete/m"].shape == (3 * 500,)
    assert np.array_equal(f["discrete/q"].reshape(-1, 3), d.download()[0])
