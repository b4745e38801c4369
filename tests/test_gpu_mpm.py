"""MPM step through the C ABI (libhg_gpu.so) against the CPU oracle.

Tolerances:
  FP64 path   - relative max error <= 1e-12 on grid fields and particle state
                (only the summation order of the FP64 atomics differs);
  MIXED path  - one-step grid-velocity error ||dv||_2 / ||v||_2 <= 1e-5 over
                active nodes (from the same FP64 state), positions within
                1e-9 m and J within 1e-6 after 20 steps;
  cell index  - bit-exact.
"""
import numpy as np
import pytest

import oracle
import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import scenes

pytestmark = pytest.mark.gpu


def rel(a, b):
    den = np.abs(b).max()
    return np.abs(a - b).max() / (den if den > 0 else 1.0)


def gpu_mpm(ctx, cfg, precision, basis=hg.LINEAR, capacity=None):
    return hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
                  cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
                  cfg["planes"], basis=basis, precision=precision,
                  capacity=capacity or 200000)


def cpu_mpm(cfg, basis=0):
    m = oracle.MPM(cfg["grid_min"], cfg["grid_max"], cfg["h"], basis=basis,
                   shear_modulus=cfg["shear_modulus"], bulk_modulus=cfg["bulk_modulus"],
                   dp_alpha=cfg["dp_alpha"], flip_alpha=cfg["flip_alpha"],
                   gravity=scenes.GRAVITY)
    for (x, n, st, lb) in cfg["planes"]:
        m.add_plane(x, n, st, lb)
    return m


def column(cfg, seed=11, vscale=0.05):
    p = scenes.seed_column_points(cfg)
    rng = np.random.default_rng(seed)
    p["v"] = rng.normal(scale=vscale, size=p["v"].shape)
    return p


@pytest.fixture(scope="module")
def cfg0():
    return scenes.mpm_column("column_12800")


def test_seed_rectangle_matches_oracle(ctx, cfg0):
    g = gpu_mpm(ctx, cfg0, hg.FP64)
    a = g.seed_rectangle(cfg0["rect_min"], cfg0["rect_max"], cfg0["rho"], 2)
    o = cpu_mpm(cfg0).seed_rectangle(cfg0["rect_min"], cfg0["rect_max"], cfg0["rho"], 2)
    assert len(a["m"]) == 12800
    for k in ("q", "v", "m", "vol", "hl"):
        assert np.array_equal(a[k], o[k]), k
    assert (g.nx, g.ny) == (200, 100)


@pytest.mark.parametrize("basis", [0, 1])
def test_fp64_step_matches_oracle(ctx, cfg0, basis):
    cfg = dict(cfg0)
    if basis == 1:
        cfg["grid_min"] = (-0.01, -0.01)
    p = column(cfg)
    g = gpu_mpm(ctx, cfg, hg.FP64, basis=basis)
    c = cpu_mpm(cfg, basis=basis)
    g.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    c.set_particles(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    dt = cfg["dt"]
    for nsteps in (1, 9):
        g.flow(dt, nsteps)
        c.step(dt, nsteps)
        G, C = g.grid(), c.grid()
        for k in ("mass", "mom", "mom_new", "force", "vel", "acc"):
            assert rel(G[k], C[k]) <= 1e-12, k
        P, Q = g.download(), c.particles()
        assert np.abs(P["q"] - Q["q"]).max() <= 1e-15
        assert rel(P["v"], Q["v"]) <= 1e-12
        assert np.abs(P["J"] - Q["J"]).max() <= 1e-13
        assert np.abs(P["be"] - Q["be"]).max() <= 1e-13
        assert np.array_equal(P["jh"], Q["jh"])
    assert g.status() == 0


def test_fp64_phases_match_oracle(ctx, cfg0):
    p = column(cfg0)
    g = gpu_mpm(ctx, cfg0, hg.FP64)
    c = cpu_mpm(cfg0)
    g.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    c.set_particles(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    dt = cfg0["dt"]
    g.flow_zero_phase()
    c.phase0()
    G, C = g.grid(), c.grid()
    assert rel(G["mass"], C["mass"]) <= 1e-12 and rel(G["mom"], C["mom"]) <= 1e-12
    g.flow_first_phase(dt)
    c.phase1(dt)
    G, C = g.grid(), c.grid()
    assert rel(G["force"], C["force"]) <= 1e-12 and rel(G["mom_new"], C["mom_new"]) <= 1e-12
    g.flow_second_phase(dt)
    c.phase2(dt)
    G, C = g.grid(), c.grid()
    assert rel(G["vel"], C["vel"]) <= 1e-12 and rel(G["acc"], C["acc"]) <= 1e-12


def stressed_state(cfg, steps=200):
    """FP64 oracle state after `steps` steps of the column (non-trivial stress)."""
    c = cpu_mpm(cfg)
    p = scenes.seed_column_points(cfg)
    c.set_particles(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    c.step(cfg["dt"], steps)
    return c, p


def test_mixed_one_step_grid_velocity_error(ctx, cfg0):
    c, p = stressed_state(cfg0)
    s = c.particles()
    g = gpu_mpm(ctx, cfg0, hg.MIXED)
    g.upload(s["q"], s["v"], p["m"], p["vol"], p["hl"], s["be"], s["J"], s["jh"])
    dt = cfg0["dt"]
    g.flow(dt)
    c.step(dt)
    G, C = g.grid(), c.grid()
    act = C["mass"] > 0
    assert np.array_equal(G["mass"] > 0, act)
    err = np.linalg.norm(G["vel"][act] - C["vel"][act]) / np.linalg.norm(C["vel"][act])
    assert err <= 1e-5, err
    assert rel(G["mass"], C["mass"]) <= 1e-6
    P, Q = g.download(), c.particles()
    assert np.abs(P["q"] - Q["q"]).max() <= 1e-12
    assert np.abs(P["J"] - Q["J"]).max() <= 1e-6


def test_mixed_multi_step_tracks_oracle(ctx, cfg0):
    p = column(cfg0, vscale=0.02)
    g = gpu_mpm(ctx, cfg0, hg.MIXED)
    c = cpu_mpm(cfg0)
    g.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    c.set_particles(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    g.flow(cfg0["dt"], 20)
    c.step(cfg0["dt"], 20)
    P, Q = g.download(), c.particles()
    assert np.abs(P["q"] - Q["q"]).max() <= 1e-9
    assert np.abs(P["J"] - Q["J"]).max() <= 1e-6
    assert np.abs(P["be"] - Q["be"]).max() <= 1e-6
    assert np.linalg.norm(P["v"] - Q["v"]) / np.linalg.norm(Q["v"]) <= 1e-4
    assert g.status() == 0


@pytest.mark.parametrize("basis", [0, 1])
def test_mixed_fast_particles_resort(ctx, basis):
    """Isolated points crossing several tiles: exercises the out-of-window
    path and the re-sort, stepping both per step (calls of fewer steps than a
    captured chunk, re-sort decisions every step) and through the graph of
    captured chunks (decisions between chunks); results follow the FP64
    oracle either way. With the uGIMP basis every point has its own
    half-width, which the re-sorts carry along."""
    # no elastic stiffness: at 0.2 cells per step the elastic CFL limit of the
    # column material would be exceeded, so these points carry no stress
    cfg = scenes.mpm_column("column_12800", shear_modulus=0.0, bulk_modulus=0.0)
    cfg["planes"] = []
    rng = np.random.default_rng(5)
    n = 300
    q = np.stack([rng.uniform(0.3, 0.7, n), rng.uniform(0.15, 0.35, n)], axis=1)
    v = np.tile([[2.0, 1.0]], (n, 1))
    m = np.full(n, 1e-3)
    vol = np.full(n, 1e-6)
    hl = np.full(n, 1.25e-3) if basis == 0 else rng.uniform(0.15, 0.5, n) * cfg["h"]
    g = gpu_mpm(ctx, cfg, hg.MIXED, basis=basis)
    gc = gpu_mpm(ctx, cfg, hg.MIXED, basis=basis)
    c = cpu_mpm(cfg, basis=basis)
    g.upload(q, v, m, vol, hl)
    gc.upload(q, v, m, vol, hl)
    c.set_particles(q, v, m, vol, hl)
    dt = 5e-4  # 0.2 cells per step
    for _ in range(5):
        g.flow(dt, 8)
    gc.flow(dt, 40)
    c.step(dt, 40)
    Q = c.particles()
    for x in (g, gc):
        # FP32 velocities integrated over 40 steps of 0.2 cells each
        assert np.abs(x.download()["q"] - Q["q"]).max() <= 2e-8
        assert x.status() == 0
    assert g.rebin_count() >= 2


@pytest.mark.parametrize("varying", [False, True])
def test_mixed_ugimp_against_the_oracle(ctx, cfg0, varying):
    """MIXED with the uGIMP basis (FP32 weights of the particle-size
    integrated hat functions, 3 x 3 stencils near cell edges) against the
    FP64 oracle with uGIMP: one-step grid-velocity error from a stressed FP64
    state within the MIXED bound, and positions / J after 20 steps within the
    linear path's tolerances; with the seeded half-width h / 4 for every
    point, and with per-point half-widths from 0.15 h to h / 2 (the resampling
    gives inserted points their own)."""
    cfg = dict(cfg0, grid_min=(-0.01, -0.01))
    c = cpu_mpm(cfg, basis=1)
    p = scenes.seed_column_points(cfg)
    hl = p["hl"].copy()
    if varying:
        hl *= np.random.default_rng(5).uniform(0.6, 2.0, len(hl))
    c.set_particles(p["q"], p["v"], p["m"], p["vol"], hl)
    c.step(cfg["dt"], 200)
    s = c.particles()
    g = gpu_mpm(ctx, cfg, hg.MIXED, basis=hg.UGIMP)
    g.upload(s["q"], s["v"], p["m"], p["vol"], hl, s["be"], s["J"], s["jh"])
    dt = cfg["dt"]
    g.flow(dt)
    c.step(dt)
    G, C = g.grid(), c.grid()
    # the edges of uGIMP supports carry weights down to FP32's underflow:
    # compare on the nodes that hold a non-negligible mass
    act = C["mass"] > 1e-6 * C["mass"].max()
    assert (G["mass"][act] > 0).all()
    assert (C["mass"][G["mass"] > 1e-6 * C["mass"].max()] > 0).all()
    err = np.linalg.norm(G["vel"][act] - C["vel"][act]) / np.linalg.norm(C["vel"][act])
    assert err <= 1e-5, err
    assert rel(G["mass"], C["mass"]) <= 1e-6
    P, Q = g.download(), c.particles()
    assert np.abs(P["q"] - Q["q"]).max() <= 1e-12
    g.flow(dt, 20)
    c.step(dt, 20)
    P, Q = g.download(), c.particles()
    assert np.abs(P["q"] - Q["q"]).max() <= 1e-9
    assert np.abs(P["J"] - Q["J"]).max() <= 1e-6
    assert np.abs(P["be"] - Q["be"]).max() <= 1e-6
    assert g.status() == 0
    # half-widths above h / 2 are refused; batches take the linear basis
    wide = hl.copy()
    wide[3] = 0.6 * cfg["h"]
    with pytest.raises(hg.HGError):
        g.upload(p["q"], p["v"], p["m"], p["vol"], wide)
    b = hg.Batch(ctx, 2)
    with pytest.raises(hg.HGError):
        b.add(g, dt)
    b.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_cell_index_bit_exact(ctx, cfg0, precision):
    rng = np.random.default_rng(9)
    n = 4000
    h = cfg0["h"]
    # points exactly on, and one ulp either side of, cell boundaries
    k = rng.integers(1, 150, size=(n, 2)).astype(np.float64)
    q = k * h
    q[: n // 3] = np.nextafter(q[: n // 3], -np.inf)
    q[n // 3: 2 * n // 3] = np.nextafter(q[n // 3: 2 * n // 3], np.inf)
    q[:, 1] *= 0.5
    g = gpu_mpm(ctx, dict(cfg0, planes=[]), precision)
    g.upload(q, np.zeros_like(q), np.full(n, 1e-3), np.full(n, 1e-6), np.full(n, 1e-3))
    cells = g.cell_index()
    ref = np.floor((q - g.grid_min) / h).astype(np.int32)
    assert np.array_equal(cells, ref)


@pytest.mark.parametrize("precision", [0, 1])
def test_out_of_grid_point_sets_status(ctx, cfg0, precision):
    p = scenes.seed_column_points(cfg0)
    q = p["q"].copy()
    q[5] = (-0.5, 0.2)  # outside the grid: detected, skipped, reported
    g = gpu_mpm(ctx, cfg0, precision)
    g.upload(q, p["v"], p["m"], p["vol"], p["hl"])
    g.flow(cfg0["dt"], 2)
    assert g.status() & 2  # HG_STATUS_OUT_OF_GRID
    P = g.download()
    assert np.isfinite(P["q"]).all() and np.isfinite(P["v"]).all()
    g.clear_status()
    assert g.status() == 0


def test_invalid_arguments_are_rejected(ctx, cfg0):
    with pytest.raises(hg.HGError):
        hg.MPM(ctx, (0, 0), (1, 1), -1.0, 1, 1, 0.3, 0.99)
    g = gpu_mpm(ctx, cfg0, hg.MIXED, capacity=10)
    p = scenes.seed_column_points(cfg0)
    with pytest.raises(hg.HGError):
        g.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])  # over capacity
    with pytest.raises(hg.HGError):
        g.flow_zero_phase()  # phase calls need FP64


def sliding_scene(cfg0, seed=3):
    """The 12,800-point column with every plane behaviour of MPMStaticPlane
    (mpmgrains2d/StaticPlane.h:6-22): a sticking floor; a SLIDING left wall 2
    mm inside the column, so that points start behind it; a SLIDING right wall
    2 mm inside the column that acts only from y = 0.2 m up (finite
    lower_bound); a tilted SLIDING plane across the column's upper left corner
    from y = 0.3 m up; and the sticking far wall. Random velocities of 0.5 m/s
    give both signs of the normal velocity at every plane, so the separating
    (v_n > 0) and the projecting branches of PhysicsGrid.cpp:611-673 and
    MaterialPoints.cpp:371-423 both run."""
    cfg = dict(cfg0)
    p = column(cfg, seed=seed, vscale=0.5)
    s = 1.0 / np.sqrt(2.0)
    cfg["planes"] = [((0.0, 0.0), (0.0, 1.0), True, -np.inf),
                     ((0.102, 0.0), (1.0, 0.0), False, -np.inf),
                     ((0.298, 0.0), (-1.0, 0.0), False, 0.2),
                     ((0.1, 0.37), (s, -s), False, 0.3),
                     ((1.0, 0.0), (-1.0, 0.0), True, -np.inf)]
    return cfg, p


@pytest.mark.parametrize("basis", [0, 1])
def test_fp64_sliding_planes_and_lower_bound_match_oracle(ctx, cfg0, basis):
    cfg, p = sliding_scene(cfg0)
    if basis == 1:
        cfg["grid_min"] = (-0.01, -0.01)
    g = gpu_mpm(ctx, cfg, hg.FP64, basis=basis)
    c = cpu_mpm(cfg, basis=basis)
    g.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    c.set_particles(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    q0 = p["q"]
    behind_left = q0[:, 0] < 0.102
    behind_right_high = (q0[:, 0] > 0.298) & (q0[:, 1] >= 0.2)
    behind_right_low = (q0[:, 0] > 0.298) & (q0[:, 1] < 0.2)
    assert behind_left.sum() > 100 and behind_right_high.sum() > 50 and behind_right_low.sum() > 50
    dt = cfg["dt"]
    for nsteps in (1, 9):
        g.flow(dt, nsteps)
        c.step(dt, nsteps)
        G, C = g.grid(), c.grid()
        for k in ("mass", "mom", "mom_new", "force", "vel", "acc"):
            assert rel(G[k], C[k]) <= 1e-12, k
        P, Q = g.download(), c.particles()
        assert np.abs(P["q"] - Q["q"]).max() <= 1e-15
        assert rel(P["v"], Q["v"]) <= 1e-12
        assert np.abs(P["J"] - Q["J"]).max() <= 1e-13
        assert np.abs(P["be"] - Q["be"]).max() <= 1e-13
    # the planes acted: points behind the left wall and behind the bounded
    # right wall above its lower bound were projected onto them, points
    # below that bound were not
    Q = c.particles()
    assert (Q["q"][behind_left, 0] >= 0.102 - 1e-12).all()
    assert (Q["q"][behind_right_high, 0] <= 0.298 + 1e-12).all()
    assert (Q["q"][behind_right_low, 0] > 0.298).any()
    assert g.status() == 0


def test_mixed_sliding_planes_and_lower_bound_track_oracle(ctx, cfg0):
    cfg, p = sliding_scene(cfg0)
    g = gpu_mpm(ctx, cfg, hg.MIXED)
    c = cpu_mpm(cfg)
    g.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    c.set_particles(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    dt = cfg["dt"]
    g.flow(dt)
    c.step(dt)
    G, C = g.grid(), c.grid()
    act = C["mass"] > 0
    assert np.array_equal(G["mass"] > 0, act)
    err = np.linalg.norm(G["vel"][act] - C["vel"][act]) / np.linalg.norm(C["vel"][act])
    assert err <= 1e-5, err
    P, Q = g.download(), c.particles()
    # the projection onto a plane is formed in FP64 on both sides
    assert np.abs(P["q"] - Q["q"]).max() <= 1e-12
    assert np.linalg.norm(P["v"] - Q["v"]) / np.linalg.norm(Q["v"]) <= 1e-5
    g.flow(dt, 19)
    c.step(dt, 19)
    P, Q = g.download(), c.particles()
    assert np.abs(P["q"] - Q["q"]).max() <= 1e-9
    assert np.abs(P["J"] - Q["J"]).max() <= 1e-6
    assert np.abs(P["be"] - Q["be"]).max() <= 1e-6
    assert np.linalg.norm(P["v"] - Q["v"]) / np.linalg.norm(Q["v"]) <= 1e-4
    assert g.status() == 0
