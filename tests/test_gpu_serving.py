"""Asynchronous pieces of the serving path and the serving loop on the GPU.

* fences and frames: a frame copied without waiting equals the synchronous
  download bit for bit (the same conversion kernel);
* admission estimate: hg_mpm_estimate_bytes bounds the device bytes an MPM
  object really holds after upload and downloads, within 10% + 1 MiB;
* continuous batching: every request's frames (the column's front and its
  DEM pile's front per 100 steps) equal those of the same scene served alone
  within 1e-9 m, with the piles' contact law in mixed precision (the
  serving default) and in FP64. For the columns FP32 atomic summation order is the only
  difference; the piles share one DEM object in the mix, shifted by their
  lane, where alone each sits at x = 0, so their FP64 positions round
  differently.
"""
import numpy as np
import pytest

import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import scenes, serving

pytestmark = pytest.mark.gpu


def build(ctx, cfg, n):
    return hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
                  cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
                  cfg["planes"], capacity=n)


def test_async_upload_and_frame_match_sync_download(ctx):
    cfg = scenes.serving_column(20000, 2.0, 30.0)
    p = scenes.seed_column_points(cfg)
    n = len(p["m"])
    host = {k: hg.pinned(p[k].shape) for k in ("q", "v", "m", "vol")}
    for k in host:
        host[k][...] = p[k]
    m = build(ctx, cfg, n)
    m.upload_async(host["q"], host["v"], host["m"], host["vol"])
    f0 = ctx.fence()
    m.flow(cfg["dt"], 50)
    q, v = hg.pinned((n, 2)), hg.pinned((n, 2))
    m.frame_async(q, v)
    f1 = ctx.fence()
    assert f1 == f0 + 1
    ctx.fence_wait(f1)
    assert ctx.fence_done(f0) and ctx.fence_done(f1)
    ref = m.download()
    assert np.array_equal(q, ref["q"]) and np.array_equal(v, ref["v"])
    assert np.abs(ref["q"] - p["q"]).max() > 0  # it moved
    with pytest.raises(hg.HGError):
        ctx.fence_done(f1 + 5)


@pytest.mark.parametrize("precision", [hg.FP64, hg.MIXED])
def test_device_seed_is_host_seed_bit_for_bit(ctx, precision):
    cfg = scenes.serving_column(30000, 1.5, 30.0)
    n_host = len(scenes.seed_column_points(cfg)["m"])
    a = hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
               cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
               cfg["planes"], precision=precision, capacity=3 * n_host)
    b = hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
               cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
               cfg["planes"], precision=precision, capacity=3 * n_host)
    lo, hi = (cfg["rect_min"][0] + 0.3 * cfg["h"], 0.0), cfg["rect_max"]  # ragged edge
    p = a.seed_rectangle(lo, hi, 1550.0, 3, vel=(0.5, -0.25), omega=2.0)
    a.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    n = b.seed_rectangle_device(lo, hi, 1550.0, 3, vel=(0.5, -0.25), omega=2.0)
    assert n == len(p["m"]) > 0
    A, B = a.download(), b.download()
    for k in ("q", "v", "be", "J", "jh"):
        assert np.array_equal(A[k], B[k]), k
    # stepping from the two states agrees up to the order of atomic sums
    # (FP64 atomics: 1e-12 m; FP32 atomics of the MIXED path: 1e-9 m)
    a.flow(cfg["dt"], 3)
    b.flow(cfg["dt"], 3)
    tol = 1e-12 if precision == hg.FP64 else 1e-9
    assert np.abs(a.download()["q"] - b.download()["q"]).max() <= tol
    with pytest.raises(hg.HGError):  # more points than the capacity
        b.seed_rectangle_device(lo, hi, 1550.0, 4)


def test_estimate_bounds_device_bytes(ctx):
    cfg = scenes.serving_column(100000, 1.0, 30.0)
    p = scenes.seed_column_points(cfg)
    n = len(p["m"])
    ctx.synchronize()
    b0 = ctx.device_bytes()
    m = build(ctx, cfg, n)
    m.upload(p["q"], p["v"], p["m"], p["vol"])
    m.flow(cfg["dt"], 2)
    m.download()
    m.grid()
    ctx.synchronize()
    used = ctx.device_bytes() - b0
    est = hg.mpm_estimate_bytes(cfg["grid_min"], cfg["grid_max"], cfg["h"], n)
    assert used > 0
    assert est >= used, (est, used)
    assert est <= 1.1 * used + 2**20, (est, used)
    m.close()


@pytest.mark.parametrize("dem_precision", [hg.MIXED, hg.FP64])
def test_serving_results_match_scenes_served_alone(ctx, dem_precision):
    reqs = serving.column_requests(n=6, rate=400.0, seed=11, steps=300, nmax=3.0e4)
    for r, t in zip(reqs, (0.0, 0.0, 0.0, 0.002, 0.004, 0.006)):
        r.arrival = t  # three at once, three while those run
    assert sum(r.ndisks > 0 for r in reqs) >= 4
    alone = [r.copy() for r in reqs]
    be = serving.DeviceBackend(ctx, max_members=8, dem_precision=dem_precision)
    srv = serving.Server(be, 2**33, max_members=8)
    srv.run(reqs)
    be.shutdown()
    serving.run_one_at_a_time(ctx, alone, dem_precision=dem_precision)
    assert srv.peak_members >= 2  # they overlapped on the device
    for a, b in zip(reqs, alone):
        assert [s for s, _ in a.frames] == [100, 200, 300]
        assert [s for s, _ in b.frames] == [100, 200, 300]
        for (_, x), (_, y) in zip(a.frames, b.frames):
            assert (x[1] is None) == (a.ndisks == 0) and (y[1] is None) == (a.ndisks == 0)
            assert serving.frame_diff(x, y) <= 1e-9, (a.rid, x, y)
        assert a.finished >= a.admitted >= a.arrival
