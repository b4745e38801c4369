"""Launch-shape autotuning of the MIXED kernels on the GPU.

* the tuner times every candidate shape per kernel with CUDA events, then
  every pair of a fused and an update shape on whole graph-replayed steps,
  and keeps the fastest pair; the choice is recorded under the scene's size
  class and a later scene of the same class starts with it;
* a shape changes only the order of FP32 atomic sums: a tuned scene follows
  an untuned twin stepped the same number of steps within 1e-9 m;
* the batched kernels are tuned the same way.
"""
import numpy as np
import pytest

import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import scenes

pytestmark = pytest.mark.gpu


def column(ctx, npoints=60000):
    cfg = scenes.serving_column(npoints, 1.5, 30.0)
    p = scenes.seed_column_points(cfg)
    m = hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
               cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
               cfg["planes"], capacity=len(p["m"]))
    m.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    return cfg, m


def test_autotune_picks_the_fastest_and_records_it(ctx):
    hg.tune_clear()
    cfg, a = column(ctx)
    _, b = column(ctx)
    assert a.launch_shape() == (0, 0)
    r = a.autotune(cfg["dt"], 10)
    assert len(r["tried"]) == 4
    for k in ("fused_ms", "update_ms"):
        assert all(np.isfinite(t) and t > 0 for t in r[k])
    # the fastest pair of shapes on whole graph-replayed steps
    sm = np.array(r["step_ms"])
    assert sm.shape == (4, 4) and np.isfinite(sm).all() and (sm > 0).all()
    i, j = np.unravel_index(int(np.argmin(sm)), sm.shape)
    assert r["chosen"] == (r["tried"][i][0], r["tried"][j][1])
    assert a.launch_shape() == r["chosen"]
    # 4 candidates x (1 untimed + 10 timed) steps per kernel, then 16 pairs x
    # 3 graph chunks of 16 steps; the twin keeps the default
    assert r["steps"] == 4 * 11 + 16 * 48
    b.flow(cfg["dt"], r["steps"])
    assert np.abs(a.download()["q"] - b.download()["q"]).max() <= 1e-9
    assert a.status() == 0 and b.status() == 0
    # a new scene of the same size class starts with the recorded shape
    _, c = column(ctx)
    c.flow(cfg["dt"], 1)
    assert c.launch_shape() == r["chosen"]
    c.set_launch_shape(3, 8)
    c.flow(cfg["dt"], 20)  # graph chunk with the explicit shape
    assert c.launch_shape() == (3, 8) and c.status() == 0
    with pytest.raises(hg.HGError):
        c.set_launch_shape(-1, 8)
    for m in (a, b, c):
        m.close()
    hg.tune_clear()


def test_batch_autotune(ctx):
    hg.tune_clear()
    batch = hg.Batch(ctx, 8)
    ms = []
    for n in (8000, 20000, 45000):
        cfg, m = column(ctx, n)
        batch.add(m, cfg["dt"])
        ms.append(m)
    r = batch.autotune(5)
    assert len(r["tried"]) == 4 and all(t > 0 for t in r["fused_ms"])
    assert r["steps"] == 4 * 6
    assert batch.launch_shape() == r["chosen"]
    batch.step(40)
    assert all(m.status() == 0 for m in ms)
    batch.close()
    for m in ms:
        m.close()
    hg.tune_clear()
