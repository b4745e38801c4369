"""Host transfers of the MIXED state through the C ABI: chunked uploads and
downloads, and the upload that keeps the points in the slots of the last
re-sort.

An upload of the same number of points after a re-sort puts every point in
the slot it had (no re-sort) unless one of them left its slot's tile window;
then the points are re-sorted as for a first upload. Either way a step gives
the same result as an object that only ever stepped (positions within 1e-9 m
and J within 1e-6 after the steps; velocities within 1e-4 relative: the
positions pass through the reference's world coordinates at each upload) and
as a fresh object given the same points (grid velocity within 1e-6 relative:
only the order of the FP32 atomic sums differs).
"""
import numpy as np
import pytest

import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import scenes

pytestmark = pytest.mark.gpu


def column(h=1.0e-3):
    # 320,000 points: two transfer chunks
    cfg = scenes.mpm_column("column_12800", h=h)
    return cfg, scenes.seed_column_points(cfg)


def make(ctx, cfg, n):
    return hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
                  cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
                  cfg["planes"], precision=hg.MIXED, capacity=n)


def host_array(a, pinned):
    """a copy of a in page-locked memory (read and written in place by the
    transfer kernels) or in ordinary pageable memory (copied through staging)"""
    if not pinned:
        return np.array(a)
    torch = pytest.importorskip("torch")
    t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)), pin_memory=True).numpy()
    t[...] = a
    return t


@pytest.mark.parametrize("pinned", [True, False])
def test_upload_step_download_loop_matches_a_continuous_run(ctx, pinned):
    cfg, p = column()
    n = len(p["m"])
    assert n > 2 * 131072
    dt = cfg["dt"]
    steps = 12
    a = make(ctx, cfg, n)
    a.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    a.flow(dt, steps)
    A = a.download()
    b = make(ctx, cfg, n)
    st = {k: host_array(x, pinned) for k, x in (
        ("q", p["q"]), ("v", p["v"]), ("m", p["m"]), ("vol", p["vol"]),
        ("be", np.tile([1.0, 0.0, 0.0, 1.0], (n, 1))), ("J", np.ones(n)),
        ("jh", np.zeros(n, dtype=np.int32)))}
    launches = []
    for k in range(steps):
        l0 = hg.kernel_launch_count()
        b.upload(st["q"], st["v"], st["m"], st["vol"], None, st["be"], st["J"], st["jh"])
        launches.append(hg.kernel_launch_count() - l0)
        b.flow(dt, 1)
        b.download_into(st["q"], st["v"], st["be"], st["J"], st["jh"])
    # after the first upload the points keep their slots: no re-sort launches
    assert all(x < launches[0] for x in launches[1:]), launches
    assert np.abs(st["q"] - A["q"]).max() <= 1e-9
    assert np.abs(st["J"] - A["J"]).max() <= 1e-6
    assert np.abs(st["be"] - A["be"]).max() <= 1e-6
    assert np.linalg.norm(st["v"] - A["v"]) / np.linalg.norm(A["v"]) <= 1e-4
    assert np.array_equal(st["jh"], A["jh"])
    assert a.status() == 0 and b.status() == 0


def test_points_moved_out_of_their_slots_are_resorted(ctx):
    cfg, p = column()
    n = len(p["m"])
    dt = cfg["dt"]
    b = make(ctx, cfg, n)
    b.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    b.flow(dt, 2)
    # the same points 40 cells to the right and 8 up: every point leaves
    # its slot's window
    q = p["q"] + np.array([40 * cfg["h"], 8 * cfg["h"]])
    l0 = hg.kernel_launch_count()
    b.upload(q, p["v"], p["m"], p["vol"], p["hl"])
    moved = hg.kernel_launch_count() - l0
    f = make(ctx, cfg, n)
    l0 = hg.kernel_launch_count()
    f.upload(q, p["v"], p["m"], p["vol"], p["hl"])
    fresh = hg.kernel_launch_count() - l0
    assert moved > fresh  # the slot upload, then the re-sort of a first upload
    b.flow(dt, 1)
    f.flow(dt, 1)
    G, F = b.grid(), f.grid()
    act = F["mass"] > 0
    assert np.array_equal(G["mass"] > 0, act)
    err = np.linalg.norm(G["vel"][act] - F["vel"][act]) / np.linalg.norm(F["vel"][act])
    assert err <= 1e-6, err
    Pb, Pf = b.download(), f.download()
    assert np.abs(Pb["q"] - Pf["q"]).max() <= 1e-12
    assert b.status() == 0 and f.status() == 0


def test_chunked_download_equals_the_frame_path(ctx):
    cfg, p = column()
    n = len(p["m"])
    b = make(ctx, cfg, n)
    b.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    b.flow(cfg["dt"], 20)
    D = b.download()
    fq, fv = np.empty((n, 2)), np.empty((n, 2))
    b.frame_async(fq, fv)
    ctx.synchronize()
    assert np.array_equal(D["q"], fq)
    assert np.array_equal(D["v"], fv)


def test_unaligned_and_tiny_host_arrays(ctx):
    """Page-locked arrays that start 8 bytes past a 16-byte boundary (the
    upload reads them element by element, the download takes the staging
    copies), and uploads of 1 and 0 points, give what aligned arrays give."""
    torch = pytest.importorskip("torch")
    cfg, p = column(h=2.5e-3)
    n = len(p["m"])
    dt = cfg["dt"]

    def shifted(a):
        # a page-locked copy of a whose data starts 8 bytes past the buffer
        raw = torch.empty(a.size + 2, dtype=torch.float64, pin_memory=True).numpy()
        flat = raw[1:1 + a.size]
        assert flat.ctypes.data % 16 == 8
        flat[...] = a.ravel()
        return flat.reshape(a.shape)

    ref = make(ctx, cfg, n)
    ref.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    ref.flow(dt, 3)
    R = ref.download()
    b = make(ctx, cfg, n)
    q, v, m, vol = (shifted(p[k]) for k in ("q", "v", "m", "vol"))
    b.upload(q, v, m, vol, None)
    b.flow(dt, 3)
    out = {"q": shifted(np.zeros((n, 2))), "v": shifted(np.zeros((n, 2))),
           "be": shifted(np.zeros((n, 4))), "J": shifted(np.zeros(n))}
    jh = np.zeros(n, dtype=np.int32)
    b.download_into(out["q"], out["v"], out["be"], out["J"], jh)
    assert np.abs(out["q"] - R["q"]).max() <= 1e-12
    assert np.abs(out["J"] - R["J"]).max() <= 1e-9
    assert np.linalg.norm(out["v"] - R["v"]) / np.linalg.norm(R["v"]) <= 1e-6
    for k in (1, 0):
        t = make(ctx, cfg, max(k, 1))
        t.upload(p["q"][:k].copy(), p["v"][:k].copy(), p["m"][:k].copy(), p["vol"][:k].copy(),
                 None)
        t.flow(dt, 2)
        t.upload(p["q"][:k].copy(), p["v"][:k].copy(), p["m"][:k].copy(), p["vol"][:k].copy(),
                 None)
        t.flow(dt, 1)
        D = t.download()
        assert D["q"].shape == (k, 2) and t.status() == 0
        if k:
            assert np.abs(D["q"] - p["q"][:k]).max() < cfg["h"]


def test_upload_of_a_different_point_count_resorts(ctx):
    cfg, p = column(h=2.5e-3)
    n = len(p["m"])
    dt = cfg["dt"]
    b = make(ctx, cfg, n)
    b.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    b.flow(dt, 2)
    k = n // 2  # the first half of the points: a new point count
    sub = {x: p[x][:k].copy() for x in ("q", "v", "m", "vol")}
    b.upload(sub["q"], sub["v"], sub["m"], sub["vol"], None)
    b.flow(dt, 2)
    f = make(ctx, cfg, n)
    f.upload(sub["q"], sub["v"], sub["m"], sub["vol"], None)
    f.flow(dt, 2)
    G, F = b.grid(), f.grid()
    assert np.array_equal(G["mass"] > 0, F["mass"] > 0)
    act = F["mass"] > 0
    assert np.linalg.norm(G["vel"][act] - F["vel"][act]) / np.linalg.norm(F["vel"][act]) <= 1e-6
    assert np.abs(b.download()["q"] - f.download()["q"]).max() <= 1e-12
