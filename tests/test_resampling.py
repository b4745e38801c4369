"""The hybrid method's resampling step (ResamplingTools, CAvoidAVoid) in
libhg_gpu's host code against the pure-Python oracle (oracle/resampling.py),
and the random streams against the reference's own MT19937
(hybridgrains2dnew/random.c, via oracle/_ref where a checkout is present).

All comparisons are bit-exact: inserted positions come from the random
streams and overlap tests, and every quantity is an FP64 expression in the
reference's order. The scene is a small hybrid column in the units of the
reference's column-collapse assets: grains on the left, material points on
the right, overlapping over 0.4 units, so that all three zone kinds and
every resampling branch occur.
"""
import math

import numpy as np
import pytest

import oracle
from oracle import resampling as ores
import libhybridgrains_gb300 as hg

GMIN, GMAX, CW, CELLS = (0.0, 0.0), (6.0, 3.0), 0.2, (30, 15)
SIZE, RHO, KAPPA, MU = 0.1, 0.96, 4.15e6, 1.9e6
R_MEAN, R_STD, RHO_DEM = 0.0575, 0.00575, 2.53
# the column-collapse settings, with the reconciliation level set at 0.6
# (1.25 there) so that the small scene has continuum cells
ZONES = dict(ls_cw=0.2, window=0.25, samples=1, thr=0.3, level=0.6, half=0.1)


def scene(seed=4):
    rng = np.random.default_rng(seed)
    # grains: hexagonal rows in [0.2, 2.8] x [0, 2.5]
    xs, ys = [], []
    for row in range(24):
        y = 0.06 + row * 0.1
        off = 0.055 if row % 2 else 0.0
        for col in range(24):
            xs.append(0.2 + off + col * 0.11)
            ys.append(y)
    n = len(xs)
    r = rng.uniform(0.048, 0.054, n)
    gq = np.stack([np.array(xs) + rng.uniform(-0.004, 0.004, n),
                   np.array(ys) + rng.uniform(-0.004, 0.004, n), rng.uniform(0, 6.28, n)], axis=1)
    gq0 = gq + rng.normal(scale=0.01, size=gq.shape)
    gv = rng.normal(scale=0.3, size=gq.shape)
    m = RHO_DEM * math.pi * r * r
    M0 = np.stack([m, m, 0.5 * m * r * r], axis=1)
    fixed = np.zeros(n, dtype=np.uint8)
    fixed[:24] = 1  # the bottom row
    # points: 2 x 2 per cell in [2.4, 5.0] x [0, 2.4]
    px, py = np.meshgrid(2.4 + SIZE * (np.arange(26) + 0.5), SIZE * (np.arange(24) + 0.5))
    q = np.stack([px.ravel(), py.ravel()], axis=1) + rng.uniform(-0.01, 0.01, (px.size, 2))
    k = len(q)
    vol0 = np.full(k, SIZE * SIZE)
    pts = dict(q0=q + rng.normal(scale=0.01, size=q.shape), q=q,
               v=rng.normal(scale=0.2, size=q.shape), m=RHO * vol0 * 0.9, vol=vol0 * 0.9,
               m0=RHO * vol0, vol0=vol0, hl=np.full(k, 0.5 * SIZE),
               be=np.tile([1.0, 0.0, 0.0, 1.0], (k, 1)) + rng.normal(scale=1e-3, size=(k, 4)),
               J=1.0 + rng.normal(scale=1e-3, size=k))
    grains = dict(q0=gq0, q=gq, v=gv, r=r, M0=M0, fixed=fixed)
    nn = (CELLS[0] + 1) * (CELLS[1] + 1)
    hs = rng.normal(scale=1e3, size=(nn, 4))
    hs[:, 2] = hs[:, 1]  # symmetric stresses
    hv = rng.normal(scale=0.2, size=(nn, 2))
    return pts, grains, hs, hv


def make(basis, direct, stress_free, hom_s, hom_v, pts, grains, hs, hv):
    z = ZONES
    zargs = (GMIN, CW, CELLS, z["ls_cw"], z["window"], z["samples"], z["thr"], z["level"],
             z["half"], direct)
    ours = hg.Resampler(zargs, GMAX, basis, SIZE, RHO, R_MEAN, R_STD, RHO_DEM, KAPPA, MU,
                        stress_free, hom_s, hom_v)
    ours.set_points(pts["q0"], pts["q"], pts["v"], pts["m"], pts["vol"], pts["m0"], pts["vol0"],
                    pts["hl"], pts["be"], pts["J"])
    ours.set_grains(grains["q0"], grains["q"], grains["v"], grains["r"], grains["M0"],
                    grains["fixed"])
    ours.set_homogenized(hs, hv)
    ref = ores.Resampler(GMIN, GMAX, CW, CELLS, basis, SIZE, RHO, R_MEAN, R_STD, RHO_DEM, KAPPA,
                         MU, stress_free, hom_s, hom_v)
    ref.set_points(pts["q0"], pts["q"], pts["v"], pts["m"], pts["vol"], pts["m0"], pts["vol0"],
                   pts["hl"], pts["be"], pts["J"])
    ref.set_grains(grains["q0"], grains["q"], grains["v"], grains["r"], grains["M0"],
                   grains["fixed"])
    ref.set_homogenized(hs, hv)
    zo = hg.Zones(GMIN, CW, CELLS, z["ls_cw"], z["window"], z["samples"], z["thr"], z["level"],
                  z["half"], allow_direct_transitions=direct)
    zr = oracle.Zones(GMIN, CW, CELLS, z["ls_cw"], direct)
    return ours, ref, zo, zr


def update_zones(zo, zr, grains, pts):
    z = ZONES
    zo.update(grains["q"], grains["r"], grains["fixed"], pts["q"])
    zr.update(grains["q"], grains["r"], grains["fixed"], pts["q"], z["window"], z["samples"],
              z["thr"], z["level"], z["half"])
    assert np.array_equal(zo.fields()["mpm"], zr.fields()["mpm"])


def compare(ours, ref):
    P, G = ours.points(), ours.grains()
    RP, RG = ref.P, ref.G
    assert len(P["m"]) == len(RP["m"]) and len(G["r"]) == len(RG["r"])
    for k in ("q0", "q", "v", "be"):
        assert np.array_equal(P[k], np.array(RP[k]).reshape(P[k].shape), equal_nan=True), k
    for k in ("m", "vol", "m0", "vol0", "w", "hl", "J"):
        assert np.array_equal(P[k], np.array(RP[k]), equal_nan=True), k
    for k in ("q0", "q", "v", "M0"):
        assert np.array_equal(G[k], np.array(RG[k]).reshape(G[k].shape)), "grain " + k
    assert np.array_equal(G["r"], np.array(RG["r"]))
    assert np.array_equal(G["w"], np.array(RG["w"]))
    assert np.array_equal(G["fixed"], np.array(RG["fixed"], dtype=np.uint8))
    assert np.array_equal(G["old_to_new"], np.array(ref.dem_map, dtype=np.int32))
    _, _, st = ours.stats()
    assert {k: st[k] for k in ref.stats} == ref.stats  # the counts; st also has timings
    return st


def test_random_streams_match_the_reference_and_the_oracle():
    zargs = (GMIN, CW, CELLS, 0.2, 0.25, 1, 0.3, 1.25, 0.1, False)
    r = hg.Resampler(zargs, GMAX, hg.LINEAR, SIZE, RHO, R_MEAN, R_STD, RHO_DEM, KAPPA, MU)
    mt = ores.MT()
    a = [r.random_u32() for _ in range(1500)]  # crosses two regenerations
    assert a == [mt.u32() for _ in range(1500)]
    assert [r.random_f32() for _ in range(10)] == [mt.f32() for _ in range(10)]
    nrm = ores.Normal(R_MEAN, R_STD)
    assert [r.random_radius() for _ in range(101)] == [nrm() for _ in range(101)]
    ref = oracle.reference_lib()
    if ref is not None:  # random.c itself: its stream is process-global
        ref.seedMT(4357)
        mt2 = ores.MT()
        assert [ref.randomMT_i() for _ in range(1500)] == [mt2.u32() for _ in range(1500)]
        assert [ref.randomMT() for _ in range(10)] == [mt2.f32() for _ in range(10)]


@pytest.mark.parametrize("basis,direct,stress_free,hom_s,hom_v", [
    (hg.LINEAR, False, False, False, False),
    (hg.UGIMP, False, True, False, False),
    (hg.UGIMP, True, False, True, True),
    (hg.LINEAR, True, True, False, True),
])
def test_resampling_step_matches_the_oracle(basis, direct, stress_free, hom_s, hom_v):
    pts, grains, hs, hv = scene()
    ours, ref, zo, zr = make(basis, direct, stress_free, hom_s, hom_v, pts, grains, hs, hv)
    update_zones(zo, zr, grains, pts)
    ours.run(zo)
    ref.run(zr, direct)
    st = compare(ours, ref)
    assert st["points_inserted"] > 0 and st["grains_inserted"] > 0
    assert st["points_deleted"] > 0
    # without direct transitions no cell turns continuum on the first update
    # (the previous labels are discrete), so grains go only with them
    assert (st["grains_deleted"] > 0) == direct


def test_second_interval_continues_the_streams():
    """Two resampling steps in a row: the random streams and the zone
    hysteresis carry over."""
    pts, grains, hs, hv = scene(seed=9)
    ours, ref, zo, zr = make(hg.UGIMP, False, False, False, False, pts, grains, hs, hv)
    for k in range(2):
        update_zones(zo, zr, grains, pts)
        ours.run(zo)
        ref.run(zr, False)
        st = compare(ours, ref)
        if k == 1:  # continuum cells exist now: grains inside them go
            assert st["grains_deleted"] > 0
        P, G = ours.points(), ours.grains()
        # the next interval starts from the resampled state, moved a little
        pts = dict(q0=P["q0"], q=P["q"] + 0.02, v=P["v"], m=P["m"], vol=P["vol"], m0=P["m0"],
                   vol0=P["vol0"], hl=P["hl"], be=P["be"], J=P["J"])
        grains = dict(q0=G["q0"], q=G["q"] + np.array([0.02, 0.0, 0.0]), v=G["v"], r=G["r"],
                      M0=G["M0"], fixed=G["fixed"])
        for obj in (ours,):
            obj.set_points(pts["q0"], pts["q"], pts["v"], pts["m"], pts["vol"], pts["m0"],
                           pts["vol0"], pts["hl"], pts["be"], pts["J"])
            obj.set_grains(grains["q0"], grains["q"], grains["v"], grains["r"], grains["M0"],
                           grains["fixed"])
        ref.set_points(pts["q0"], pts["q"], pts["v"], pts["m"], pts["vol"], pts["m0"],
                       pts["vol0"], pts["hl"], pts["be"], pts["J"])
        ref.set_grains(grains["q0"], grains["q"], grains["v"], grains["r"], grains["M0"],
                       grains["fixed"])
