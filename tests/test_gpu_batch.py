"""Batches of MIXED MPM scenes (hg_batch_*): every member steps as it would
alone.

A batch runs all members through one grid-update launch and one fused
G2P/P2G launch per step. The kernels per (scene, tile) are the ones the
single-scene path runs, so a member differs from the same scene stepped alone
only by the order of FP32 atomic additions into shared nodes. Tolerance:
positions within 1e-9 m and velocities within 1e-5 relative (2-norm) after 80
steps, which cross one periodic re-sort; status words stay clean.
"""
import numpy as np
import pytest

import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import scenes

pytestmark = pytest.mark.gpu

STEPS = 80


def make(ctx, cfg, precision=hg.MIXED):
    p = scenes.seed_column_points(cfg)
    m = hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
               cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
               cfg["planes"], precision=precision, capacity=len(p["m"]))
    rng = np.random.default_rng(len(p["m"]))
    m.upload(p["q"], rng.normal(scale=0.05, size=p["v"].shape), p["m"], p["vol"], p["hl"])
    return m


def mix():
    return [scenes.serving_column(2000, 0.5, 20.0), scenes.serving_column(9000, 2.0, 30.0),
            scenes.serving_column(30000, 4.0, 40.0)]


def close(a, b):
    A, B = a.download(), b.download()
    assert np.abs(A["q"] - B["q"]).max() <= 1e-9
    assert np.linalg.norm(A["v"] - B["v"]) <= 1e-5 * np.linalg.norm(B["v"])
    assert np.abs(A["J"] - B["J"]).max() <= 1e-6


def test_batch_matches_scenes_stepped_alone(ctx):
    cfgs = mix()
    alone = [make(ctx, c) for c in cfgs]
    together = [make(ctx, c) for c in cfgs]
    dts = [1.0e-5, 0.8e-5, 1.2e-5]
    for m, dt in zip(alone, dts):
        m.flow(dt, STEPS)
    b = hg.Batch(ctx, 8)
    for m, dt in zip(together, dts):
        b.add(m, dt)
    assert len(b) == 3
    b.step(STEPS)
    for a, t in zip(alone, together):
        close(t, a)
        assert t.status() == 0
        assert t.rebin_count() >= 2
    b.close()


def test_members_join_and_leave_between_steps(ctx):
    cfgs = mix()
    alone = [make(ctx, c) for c in cfgs]
    together = [make(ctx, c) for c in cfgs]
    dt = 1.0e-5
    # scene 0 for all 80 steps, scene 1 leaves after 30, scene 2 joins at 30
    alone[0].flow(dt, STEPS)
    alone[1].flow(dt, 30)
    alone[2].flow(dt, STEPS - 30)
    b = hg.Batch(ctx, 4)
    b.add(together[0], dt)
    b.add(together[1], dt)
    b.step(30)
    b.remove(together[1])
    b.add(together[2], dt)
    b.step(STEPS - 30)
    for a, t in zip(alone, together):
        close(t, a)
    # a former member keeps stepping on its own
    together[1].flow(dt, 10)
    alone[1].flow(dt, 10)
    close(together[1], alone[1])
    b.close()


def test_batch_rejects_bad_members(ctx):
    cfg = scenes.serving_column(2000, 1.0, 30.0)
    a, c = make(ctx, cfg), make(ctx, cfg)
    f = make(ctx, cfg, precision=hg.FP64)
    b = hg.Batch(ctx, 1)
    with pytest.raises(hg.HGError):
        b.add(f, 1e-5)  # FP64 objects run the unfused drop-in path
    b.add(a, 1e-5)
    with pytest.raises(hg.HGError):
        b.add(a, 1e-5)  # already a member
    with pytest.raises(hg.HGError):
        b.add(c, 1e-5)  # full
    with pytest.raises(hg.HGError):
        b.remove(c)  # not a member
    with pytest.raises(hg.HGError):
        hg.Batch(ctx, hg._capi.HG_MAX_BATCH + 1)
    b.step(0)
    b.close()
