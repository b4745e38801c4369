"""Penalty-DEM step through the C ABI against the CPU oracle.

The FP64 DEM path evaluates every contact with the reference's operation order
and gathers body forces in the reference's summation order, so positions,
velocities and the collision cache are compared for exact equality.
"""
import numpy as np
import pytest

import oracle
import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import scenes

pytestmark = pytest.mark.gpu


def build_pair(ctx, sc, p, planes, fixed=None, gravity=scenes.GRAVITY, ccap=None):
    fixed = sc["fixed"] if fixed is None else fixed
    n = len(sc["r"])
    g = hg.DEM(ctx, gravity, p["kn"], p["kt"], p["gamman"], p["gammat"], p["mu"], planes,
               capacity=n, contact_capacity=ccap or 8 * n)
    g.upload(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], fixed)
    c = oracle.DEM(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], fixed, gravity, p["kn"],
                   p["kt"], p["gamman"], p["gammat"], p["mu"], 1.0)
    for (x, nn) in planes:
        c.add_plane(x, nn)
    return g, c


def test_candidate_pairs_bit_exact(ctx):
    rng = np.random.default_rng(21)
    n = 3000
    c = rng.uniform(0, 0.1, size=(n, 2))
    r = rng.uniform(0.9e-3, 1.1e-3, size=n)
    mn, mx = c - r[:, None], c + r[:, None]
    mn[1] = [mx[0, 0], mn[0, 1]]  # touching boxes count as overlapping
    mx[1] = mn[1] + 2e-3
    got = hg.candidate_pairs(ctx, mn, mx)
    ref, _, _, _ = oracle.candidate_pairs(mn, mx, 1.0)
    assert len(ref) > 0
    assert np.array_equal(got, ref)


def column_scene(n=600, per_row=30, fall=True):
    sc = scenes.dem_column(n=n, per_row=per_row)
    if fall:
        sc["v"][:, 1] = -2.0  # rows close their 0.2 mm gaps within the run
    return sc


@pytest.mark.parametrize("weighted", [False, True])
def test_dem_step_bit_exact(ctx, weighted):
    sc = column_scene()
    p = scenes.dem_params()
    fixed = np.zeros(len(sc["r"]), dtype=np.uint8)
    fixed[: 30] = 1  # a kinematic bottom row, at rest (fixed bodies keep their velocity)
    sc["v"][: 30] = 0.0
    # the left wall touches part of the first column of disks
    planes = [((0.15e-3, 0.0), (1.0, 0.0)), ((0.0, 0.0), (0.0, 1.0))]
    g, c = build_pair(ctx, sc, p, planes, fixed=fixed)
    if weighted:
        w = np.where(np.arange(len(sc["r"])) % 3 == 0, 0.5, 1.0)
        g.set_weights(w)
        c.set_weights(w)
    for _ in range(3):
        if weighted:
            g.flow_with_weights(1e-6, 100)
        else:
            g.flow(1e-6, 100)
        c.step(1e-6, 100, weighted=weighted)
        Qg, Vg = g.download()
        Qc, Vc = c.state()
        assert np.array_equal(Qg, Qc)
        assert np.array_equal(Vg, Vc)
        Rg, Rc = g.contacts(), c.contacts()
        assert Rg.shape == Rc.shape and len(Rc) > 0
        assert np.array_equal(Rg, Rc)
    kinds = Rc[:, 0]
    assert (kinds == 0).any() and (kinds == 1).any() and (kinds == 2).any()
    assert g.status() == 0


def test_contact_capacity_overflow_is_reported(ctx):
    sc = column_scene(n=200, per_row=20)
    sc["v"][:, 1] = -2.0
    p = scenes.dem_params()
    g, _ = build_pair(ctx, sc, p, [((0.0, 0.0), (0.0, 1.0))], ccap=4)
    g.flow(1e-6, 400)
    assert g.status() & 4  # HG_STATUS_CONTACT_OVERFLOW
    q, v = g.download()
    assert np.isfinite(q).all() and np.isfinite(v).all()


def test_upload_relabel_keeps_renumbered_history(ctx):
    """After bodies are removed (the resampling step), the contact history
    keeps the surviving contacts, renumbered, with their tangential springs
    (PenaltyImpactFrictionMap::deleteCacheEntries); bit-exact bookkeeping."""
    sc = scenes.dem_column(n=2000, per_row=50)
    dp = scenes.dem_params()
    d = hg.DEM(ctx, scenes.GRAVITY, dp["kn"], dp["kt"], dp["gamman"], dp["gammat"], dp["mu"],
               [((0.0, 0.0), (0.0, 1.0))], capacity=2100)
    d.upload(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"])
    d.flow(1e-6, 200)
    before = d.contacts()
    q, v = d.download()
    n = len(sc["r"])
    keep = np.ones(n, dtype=bool)
    keep[::7] = False
    old_to_new = np.where(keep, np.cumsum(keep) - 1, -1).astype(np.int32)
    # two bodies appended after the survivors, as the resampling step does
    extra_q = np.array([[0.5, 0.5, 0.0], [0.6, 0.5, 0.0]])
    nq = np.concatenate([q[keep], extra_q])
    nv = np.concatenate([v[keep], np.zeros((2, 3))])
    nr = np.concatenate([sc["r"][keep], [1e-3, 1e-3]])
    nm = np.concatenate([sc["m"][keep], sc["m"][:2]])
    nI = np.concatenate([sc["I"][keep], sc["I"][:2]])
    d.upload_relabel(nq, nv, nr, nm, nI, np.zeros(len(nr), dtype=np.uint8), old_to_new)
    after = d.contacts()
    kind, a, b = before[:, 0].astype(int), before[:, 1].astype(int), before[:, 2].astype(int)
    alive = keep[a] & ((kind == 0) | keep[np.where(kind == 0, 0, b)])
    exp = before[alive].copy()
    exp[:, 1] = old_to_new[a[alive]]
    nb = b[alive]
    exp[:, 2] = np.where(kind[alive] == 0, nb, old_to_new[np.where(kind[alive] == 0, 0, nb)])
    assert len(exp) > 20 and len(exp) < len(before)
    assert np.array_equal(after, exp)
    d.flow(1e-6, 10)
    assert d.status() == 0


def test_edit_async_matches_the_scene_without_the_removed_pile(ctx):
    """hg_dem_edit_async (bodies removed by a stable compaction, new ones
    appended, all on the device): three piles A, B, C step together, B leaves
    and D joins; a second object that never held B (A and C, then D appended)
    gives the same positions, velocities and collision cache bit for bit,
    so the compaction renumbered the contact history of A and C exactly."""
    from libhybridgrains_gb300 import serving

    def pile(rid, n, lane):
        return serving.dem_pile(serving.Request(rid, 0.0, None, 0, ndisks=n, aspect=1.5), lane)

    A, B, C, D = pile(1, 700, 0), pile(2, 500, 1), pile(3, 900, 2), pile(4, 400, 3)

    def cat(*ps):
        return {k: np.concatenate([p[k] for p in ps]) for k in ("q", "v", "r", "m", "I")}

    x = serving.dem_for_piles(ctx, 3000)
    y = serving.dem_for_piles(ctx, 3000)
    for d, s in ((x, cat(A, B, C)), (y, cat(A, C))):
        d.edit_async(np.zeros(0, dtype=np.int32), **s)
    x.flow(1e-5, 1000)  # 10 ms: the piles settle into contact
    y.flow(1e-5, 1000)
    nA, nB, nC = 700, 500, 900
    assert x.n == nA + nB + nC and y.n == nA + nC
    drop = np.concatenate([np.arange(nA), np.full(nB, -1), nA + np.arange(nC)]).astype(np.int32)
    x.edit_async(drop, **D)
    y.edit_async(np.arange(nA + nC, dtype=np.int32), **D)
    assert x.n == y.n == nA + nC + 400
    x.flow(1e-5, 1001)  # graph replays and one plain step
    y.flow(1e-5, 1001)
    qx, vx = x.download()
    qy, vy = y.download()
    assert np.array_equal(qx, qy) and np.array_equal(vx, vy)
    cx, cy = x.contacts(), y.contacts()
    assert len(cx) > 500 and np.array_equal(cx, cy)
    assert np.abs(cx[:, 6:8]).max() > 0  # tangential springs carried over
    assert x.status() == 0 and y.status() == 0
    # everything removed, then refilled
    x.edit_async(np.full(x.n, -1, dtype=np.int32))
    assert x.n == 0
    x.flow(1e-5, 5)
    x.edit_async(np.zeros(0, dtype=np.int32), **A)
    x.flow(1e-5, 5)
    assert x.n == nA and np.isfinite(x.download()[0]).all()
    # host-side checks: capacity, order of the kept bodies
    with pytest.raises(hg.HGError):
        x.edit_async(np.arange(nA, dtype=np.int32), **cat(B, C, D, D, D, D))
    bad = np.arange(nA, dtype=np.int32)
    bad[[0, 1]] = bad[[1, 0]]
    with pytest.raises(hg.HGError):
        x.edit_async(bad)
    x.close()
    y.close()


def test_mixed_precision_against_fp64(ctx):
    """HG_PRECISION_MIXED (FP32 contact law and integration; FP64 positions,
    pairwise differences, contact points and position update) against the
    bit-exact FP64 step from the same settled state with its contact
    history. The contact set is identical (the broadphase and the contact
    tests are shared and exact); after one step every output field is within
    FP32 rounding of the FP64 values (measured: 4e-8 relative for velocities,
    6e-8 for depths and spring lengths, 1e-7 for forces, 7e-11 m for
    positions); positions stay within 1e-7 m after 10 more steps (measured
    1.2e-9 m; contacts amplify the difference over longer runs)."""
    sc = scenes.dem_column(n=4000, per_row=40)
    dp = scenes.dem_params()
    planes = [((0.0, 0.0), (0.0, 1.0))]

    def make(precision):
        return hg.DEM(ctx, scenes.GRAVITY, dp["kn"], dp["kt"], dp["gamman"], dp["gammat"],
                      dp["mu"], planes, capacity=4000, precision=precision)

    base = make(hg.FP64)
    base.upload(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"])
    base.flow(1e-5, 2000)  # settle into contact, with friction history
    blob = base.state()
    f64, mix = make(hg.FP64), make(hg.MIXED)
    f64.load_state(blob)
    mix.load_state(blob)
    f64.flow(1e-5, 1)
    mix.flow(1e-5, 1)
    ca, cb = f64.contacts(), mix.contacts()
    assert len(ca) > 300 and np.array_equal(ca[:, :3], cb[:, :3])  # same contact set

    def rel(a, b):
        return np.linalg.norm(a - b) / np.linalg.norm(b)

    (qa, va), (qb, vb) = f64.download(), mix.download()
    assert rel(vb[:, :2], va[:, :2]) <= 2e-6
    assert rel(vb[:, 2], va[:, 2]) <= 2e-6
    assert np.abs(qb - qa).max() <= 1e-9
    # depth, spring, relative velocity, lever arms, normal and friction force
    for cols in ((3,), (6, 7), (8, 9), (10, 11), (17, 18), (19, 20)):
        assert rel(cb[:, cols], ca[:, cols]) <= 5e-6, cols
    f64.flow(1e-5, 10)
    mix.flow(1e-5, 10)
    assert np.abs(mix.download()[0] - f64.download()[0]).max() <= 1e-7
    assert mix.status() == 0
    for d in (base, f64, mix):
        d.close()


def test_concurrent_stream_gives_the_same_steps(ctx):
    """A DEM object in concurrent mode (its own stream) steps, edits and
    copies frames exactly as on the context's stream, the MPM work queued in
    between notwithstanding; join orders the context's later work after it."""
    from libhybridgrains_gb300 import serving

    def pile(rid, n, lane):
        return serving.dem_pile(serving.Request(rid, 0.0, None, 0, ndisks=n, aspect=1.5), lane)

    A, B = pile(1, 800, 0), pile(2, 500, 1)
    cfg = scenes.serving_column(20000, 1.5, 30.0)
    p = scenes.seed_column_points(cfg)
    out = []
    for concurrent in (False, True):
        d = serving.dem_for_piles(ctx, 2000)
        d.set_concurrent(concurrent)
        d.edit_async(np.zeros(0, dtype=np.int32), **{f: A[f] for f in ("q", "v", "r", "m", "I")})
        m = hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
                   cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
                   cfg["planes"], capacity=len(p["m"]))
        m.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
        frame = hg.pinned((2000, 3))
        for k in range(3):
            m.flow(cfg["dt"], 100)       # context stream
            d.flow(1e-5, 100)            # DEM stream in concurrent mode
            if k == 1:
                d.edit_async(np.arange(800, dtype=np.int32),
                             **{f: B[f] for f in ("q", "v", "r", "m", "I")})
        d.frame_async(frame[:d.n])
        d.join()
        f = ctx.fence()
        ctx.fence_wait(f)
        out.append((frame[:d.n].copy(), d.download()[0], d.contacts(), d.status()))
        m.close()
        d.close()
    (fa, qa, ca, sa), (fb, qb, cb, sb) = out
    assert sa == 0 and sb == 0
    assert np.array_equal(fa, qa) and np.array_equal(fb, qb)  # frames landed by the fence
    assert np.array_equal(qa, qb) and np.array_equal(ca, cb)


def drum_scene():
    """Disks of the DEM column's lattice inside two static drums of radius
    50 mm whose centres lie 2 mm apart (each drum is the nearer wall on one
    side), above a floor plane that cuts the drums' bottom, moving outwards
    at 2 m/s: contacts with both drums, with the floor and with each other,
    several static objects per body near the bottom."""
    c = np.array([0.05, 0.05])
    c2 = c + np.array([0.002, 0.0])
    sc = scenes.dem_column(n=2400, per_row=48, x0=0.0, y0=0.0)
    xy = sc["q"][:, :2]
    d1 = np.linalg.norm(xy - c, axis=1)
    d2 = np.linalg.norm(xy - c2, axis=1)
    # 1.05 mm below the lattice's seventh row (rows at 2.2 mm (1/2 + k sqrt(3)/2))
    floor_y = 2.2e-3 * (0.5 + 6.0 * np.sqrt(3.0) / 2.0) - 1.05e-3
    keep = (d1 <= 0.0495) & (d2 <= 0.0495) & (xy[:, 1] >= floor_y + 0.95e-3)
    for k in ("q", "v", "r", "m", "I", "fixed"):
        sc[k] = np.ascontiguousarray(sc[k][keep])
    rel = sc["q"][:, :2] - c
    sc["v"][:, :2] = 2.0 * rel / np.maximum(np.linalg.norm(rel, axis=1), 1e-12)[:, None]
    drums = [(tuple(c), 0.05), (tuple(c2), 0.05)]
    planes = [((0.0, floor_y), (0.0, 1.0))]
    return sc, drums, planes


@pytest.mark.parametrize("weighted", [False, True])
def test_static_drums_bit_exact(ctx, weighted):
    """StaticDrumCircleConstraint (StaticDrumCircleConstraint.cpp:7-159),
    the drum branch of the collision cache and force loop
    (PenaltyImpactFrictionMap.cpp:84-111, 361-401, 696-767) and the drum
    active set (RigidBody2DSim.cpp:844-884), FP64 against the oracle."""
    sc, drums, planes = drum_scene()
    n = len(sc["r"])
    assert n > 1000
    p = scenes.dem_params()
    g = hg.DEM(ctx, scenes.GRAVITY, p["kn"], p["kt"], p["gamman"], p["gammat"], p["mu"], planes,
               capacity=n, contact_capacity=8 * n, drums=drums)
    g.upload(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"])
    c = oracle.DEM(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"], scenes.GRAVITY,
                   p["kn"], p["kt"], p["gamman"], p["gammat"], p["mu"], 1.0)
    for (x, nn) in planes:
        c.add_plane(x, nn)
    for (x, r) in drums:
        c.add_drum(x, r)
    if weighted:
        w = np.where(np.arange(n) % 3 == 0, 0.5, 1.0)
        g.set_weights(w)
        c.set_weights(w)
    for _ in range(3):
        if weighted:
            g.flow_with_weights(1e-6, 100)
        else:
            g.flow(1e-6, 100)
        c.step(1e-6, 100, weighted=weighted)
        Qg, Vg = g.download()
        Qc, Vc = c.state()
        assert np.array_equal(Qg, Qc)
        assert np.array_equal(Vg, Vc)
        Rg, Rc = g.contacts(), c.contacts()
        assert Rg.shape == Rc.shape
        assert np.array_equal(Rg, Rc)
    kinds = Rc[:, 0]
    assert (kinds == 0).any() and (kinds == 1).any()
    drum_rows = Rc[kinds == 3]
    assert set(drum_rows[:, 2].astype(int)) == {0, 1}
    assert g.status() == 0


def test_static_drums_mixed_precision_tracks_fp64(ctx):
    sc, drums, planes = drum_scene()
    n = len(sc["r"])
    p = scenes.dem_params()
    objs = []
    for prec in (hg.FP64, hg.MIXED):
        d = hg.DEM(ctx, scenes.GRAVITY, p["kn"], p["kt"], p["gamman"], p["gammat"], p["mu"],
                   planes, capacity=n, contact_capacity=8 * n, drums=drums, precision=prec)
        d.upload(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"])
        d.flow(1e-6, 10)
        objs.append(d)
    (qf, vf), (qm, vm) = objs[0].download(), objs[1].download()
    Rf, Rm = objs[0].contacts(), objs[1].contacts()
    assert np.array_equal(Rf[:, :3], Rm[:, :3])  # the same contacts
    assert (Rf[:, 0] == 3).sum() > 10
    assert np.abs(qf[:, :2] - qm[:, :2]).max() <= 1e-9
    assert np.linalg.norm(vf - vm) / np.linalg.norm(vf) <= 1e-5
    # the drum contacts' normal forces, FP32 against FP64
    dr = Rf[:, 0] == 3
    assert np.abs(Rm[dr, 17:19] - Rf[dr, 17:19]).max() <= 1e-5 * np.abs(Rf[dr, 17:19]).max()
    assert objs[1].status() == 0
