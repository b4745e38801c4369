"""Checkpoint and resume of device objects on the GPU.

An object loaded from a state blob holds the saved buffers byte for byte (its
own blob equals the loaded one) and continues as the saved object does: the
DEM bit for bit (its step is deterministic), MPM within the order of atomic
sums (1e-9 m MIXED, 1e-12 m FP64), and a hybrid simulation, whose zone labels,
random streams and host arrays are in the checkpoint too, through a
resampling step with the same point and grain counts.
"""
import numpy as np
import pytest

import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import checkpoint, scenes, serving
from libhybridgrains_gb300.hybrid import HybridSim

pytestmark = pytest.mark.gpu


def column(ctx, precision, npoints=40000):
    cfg = scenes.serving_column(npoints, 1.5, 30.0)
    p = scenes.seed_column_points(cfg)
    m = hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
               cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
               cfg["planes"], precision=precision, capacity=len(p["m"]))
    return cfg, p, m


@pytest.mark.parametrize("precision,tol", [(hg.MIXED, 1e-9), (hg.FP64, 1e-12)])
def test_mpm_resume(ctx, tmp_path, precision, tol):
    cfg, p, a = column(ctx, precision)
    a.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    a.flow(cfg["dt"], 70)  # past a periodic re-sort
    path = tmp_path / "mpm.hgckpt"
    checkpoint.save_objects(path, mpm=a)
    _, _, b = column(ctx, precision)
    checkpoint.load_objects(path, mpm=b)
    assert b.n == a.n
    assert np.array_equal(b.state(), checkpoint.read(path)[0]["mpm"])
    a.flow(cfg["dt"], 45)
    b.flow(cfg["dt"], 45)
    A, B = a.download(), b.download()
    assert np.abs(A["q"] - B["q"]).max() <= tol
    assert np.abs(A["J"] - B["J"]).max() <= 1e3 * tol
    assert a.status() == 0 and b.status() == 0
    # another grid is refused
    other = scenes.serving_column(90000, 1.5, 30.0)
    c = hg.MPM(ctx, other["grid_min"], other["grid_max"], other["h"], other["shear_modulus"],
               other["bulk_modulus"], other["dp_alpha"], other["flip_alpha"], scenes.GRAVITY,
               other["planes"], precision=precision, capacity=len(p["m"]))
    with pytest.raises(hg.HGError):
        c.load_state(a.state())
    for m in (a, b, c):
        m.close()


def test_dem_resume_is_exact(ctx, tmp_path):
    pile = serving.dem_pile(serving.Request(1, 0.0, None, 0, ndisks=3000, aspect=1.0), 0)
    a = serving.dem_for_piles(ctx, 3000)
    a.upload(pile["q"], pile["v"], pile["r"], pile["m"], pile["I"], pile["fixed"])
    a.flow(1e-5, 1000)
    path = tmp_path / "dem.hgckpt"
    checkpoint.save_objects(path, dem=a)
    b = serving.dem_for_piles(ctx, 3000)
    checkpoint.load_objects(path, dem=b)
    assert np.array_equal(b.state(), checkpoint.read(path)[0]["dem"])
    a.flow(1e-5, 501)
    b.flow(1e-5, 501)
    (qa, va), (qb, vb) = a.download(), b.download()
    assert np.array_equal(qa, qb) and np.array_equal(va, vb)
    ca, cb = a.contacts(), b.contacts()
    assert len(ca) > 100 and np.array_equal(ca, cb)
    small = serving.dem_for_piles(ctx, 1000)
    with pytest.raises(hg.HGError):
        small.load_state(a.state())
    for d in (a, b, small):
        d.close()


def test_hybrid_resume_through_a_resampling(ctx, tmp_path):
    sc = scenes.hybrid_column(scale=0.05)
    a = HybridSim(ctx, sc)
    a.step(150)
    path = tmp_path / "hybrid.hgckpt"
    a.save(path)
    b = HybridSim(ctx, sc)
    b.restore(path)
    assert b.counts() == a.counts() and b.steps == a.steps == 150
    a.step(200)
    b.step(200)
    assert a.resamplings == b.resamplings >= 2
    assert a.counts() == b.counts()
    qa, qb = a.mpm.download()["q"], b.mpm.download()["q"]
    assert np.abs(qa - qb).max() <= 1e-9
    (da, _), (db, _) = a.dem.download(), b.dem.download()
    assert np.abs(da - db).max() <= 1e-9
    assert a.mpm.status() == 0 and a.dem.status() == 0
