"""Empty and ragged inputs through the C ABI: objects with no points or
bodies step, download and export nothing without setting a status bit; a
batch holds an empty member beside a full one; a single material point and a
single disk step like any other; the candidate-pair search of no boxes is
empty."""
import numpy as np
import pytest

import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import scenes, serving

pytestmark = pytest.mark.gpu


def mpm(ctx, cfg, precision, basis=hg.LINEAR, capacity=64):
    return hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
                  cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
                  cfg["planes"], basis=basis, precision=precision, capacity=capacity)


@pytest.mark.parametrize("precision,basis", [(hg.FP64, hg.LINEAR), (hg.MIXED, hg.LINEAR),
                                             (hg.MIXED, hg.UGIMP)])
def test_mpm_without_points(ctx, precision, basis):
    cfg = dict(scenes.mpm_column("column_12800"), grid_min=(-0.01, -0.01))
    m = mpm(ctx, cfg, precision, basis)
    z = np.zeros((0, 2))
    m.upload(z, z, np.zeros(0), np.zeros(0), np.zeros(0))
    m.flow(cfg["dt"], 20)  # a graph chunk and per-step calls
    m.flow(cfg["dt"], 3)
    st = m.download()
    assert st["q"].shape == (0, 2) and m.status() == 0
    assert not m.grid()["mass"].any()
    blob = m.state()
    m.load_state(blob)
    assert m.n == 0


@pytest.mark.parametrize("precision,basis", [(hg.FP64, hg.LINEAR), (hg.MIXED, hg.LINEAR),
                                             (hg.MIXED, hg.UGIMP)])
def test_single_point(ctx, precision, basis):
    cfg = dict(scenes.mpm_column("column_12800"), grid_min=(-0.01, -0.01))
    m = mpm(ctx, cfg, precision, basis)
    h = cfg["h"]
    m.upload(np.array([[0.4, 0.2]]), np.array([[0.1, -0.05]]), np.array([1e-3]),
             np.array([1e-6]), np.array([h / 4]))
    m.flow(cfg["dt"], 30)
    q = m.download()["q"]
    assert m.status() == 0 and np.isfinite(q).all()
    # free fall under gravity for 30 steps of 1e-5 s: it moved down
    assert q[0, 1] < 0.2 and abs(q[0, 0] - 0.4 - 30 * cfg["dt"] * 0.1) < 1e-6


def test_batch_with_an_empty_member(ctx):
    cfg = scenes.serving_column(8000, 1.0, 30.0)
    p = scenes.seed_column_points(cfg)
    full = mpm(ctx, cfg, hg.MIXED, capacity=len(p["m"]))
    full.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    empty = mpm(ctx, cfg, hg.MIXED)
    z = np.zeros((0, 2))
    empty.upload(z, z, np.zeros(0), np.zeros(0))
    alone = mpm(ctx, cfg, hg.MIXED, capacity=len(p["m"]))
    alone.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    b = hg.Batch(ctx, 4)
    b.add(empty, cfg["dt"])
    b.add(full, cfg["dt"])
    b.step(40)
    alone.flow(cfg["dt"], 40)
    assert full.status() == 0 and empty.status() == 0 and empty.n == 0
    assert np.abs(full.download()["q"] - alone.download()["q"]).max() <= 1e-9
    b.close()


def test_dem_without_bodies_and_with_one(ctx):
    d = serving.dem_for_piles(ctx, 16)
    d.flow(1e-5, 10)  # nothing uploaded
    d.upload(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0), np.zeros(0), np.zeros(0))
    d.flow(1e-5, 10)
    assert d.n == 0 and len(d.contacts()) == 0 and d.status() == 0
    r, rho = 1e-3, 2600.0
    mass = rho * np.pi * r * r
    d.upload(np.array([[0.0, 0.5 * r, 0.0]]), np.zeros((1, 3)), np.array([r]), np.array([mass]),
             np.array([0.5 * mass * r * r]))
    d.flow(1e-5, 10)  # resting on the floor: one plane contact
    q, v = d.download()
    c = d.contacts()
    assert len(c) == 1 and int(c[0, 0]) == 0 and d.status() == 0
    assert np.isfinite(q).all() and np.isfinite(v).all()
    pairs = hg.candidate_pairs(ctx, np.zeros((0, 2)), np.zeros((0, 2)))
    assert len(pairs) == 0
