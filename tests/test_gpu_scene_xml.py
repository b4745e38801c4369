"""Scenes read from XML (the reference's schema) run on the device exactly as
the same scenes built from the library's scene dicts: the files are
written here from the library's scenes with every number in full
precision, read back by libhybridgrains_gb300.scene_xml and stepped
beside the originals."""
import numpy as np
import pytest

import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import hybrid, scene_xml, scenes

pytestmark = pytest.mark.gpu


def f(x):
    return repr(float(x))


def step(dt):
    """A time step as the reference's rational form ("1 / n")."""
    n = round(1.0 / dt)
    assert 1.0 / float(n) == dt
    return "1 / %d" % n


def pair(v):
    return "%s %s" % (f(v[0]), f(v[1]))


def mpm_xml(cfg, basis="Standard"):
    planes = "".join(
        '<static_plane x="%s" n="%s" boundary_behavior="%s"/>\n'
        % (pair(x), pair(n), "sticking" if st else "sliding") for (x, n, st, _lb) in cfg["planes"])
    return ('<mpmgrains2d>\n<grid min="%s" max="%s" cell_width="%s"/>\n'
            '<integrator dt="%s" alpha="%s" shape_function_order="1" '
            'shape_function_category="%s"/>\n'
            '<material shear_modulus="%s" bulk_modulus="%s" alpha="%s"/>\n'
            '<rectangle min="%s" max="%s" density="%s" cell_samples_per_dim="%d" vel="0 0" '
            'omega="0"/>\n<near_earth_gravity f="%s"/>\n%s</mpmgrains2d>\n'
            % (pair(cfg["grid_min"]), pair(cfg["grid_max"]), f(cfg["h"]), step(cfg["dt"]),
               f(cfg["flip_alpha"]), basis, f(cfg["shear_modulus"]), f(cfg["bulk_modulus"]),
               f(cfg["dp_alpha"]), pair(cfg["rect_min"]), pair(cfg["rect_max"]), f(cfg["rho"]),
               cfg["samples_per_dim"], pair(scenes.GRAVITY), planes))


def dem_xml(sc, dp, planes, cell_scale=1.0, dt=1e-6, rho=2600.0):
    rs = sorted(set(sc["r"].tolist()))
    gi = {r: k for k, r in enumerate(rs)}
    rho = np.full(len(sc["r"]), rho)
    out = ['<rigidbody2d_scene>',
           '<collision_detection broadphase="spatial_grid" cell_scale="%s" '
           'bandwidth_reduction="none"/>' % f(cell_scale),
           '<penalty_impact_map dt="%s" kn="%s" kt="%s" gamman="%s" gammat="%s" mu="%s"/>'
           % (step(dt), f(dp["kn"]), f(dp["kt"]), f(dp["gamman"]), f(dp["gammat"]), f(dp["mu"])),
           '<near_earth_gravity f="%s"/>' % pair(scenes.GRAVITY)]
    out += ['<static_plane x="%s" n="%s"/>' % (pair(x), pair(n)) for (x, n) in planes]
    out += ['<geometry type="circle" r="%s"/>' % f(r) for r in rs]
    for k in range(len(sc["r"])):
        out.append('<rigid_body x="%s %s" theta="%s" v="%s %s" omega="%s" rho="%s" geo_idx="%d" '
                   'fixed="%d"/>' % (f(sc["q"][k, 0]), f(sc["q"][k, 1]), f(sc["q"][k, 2]),
                                     f(sc["v"][k, 0]), f(sc["v"][k, 1]), f(sc["v"][k, 2]),
                                     f(rho[k]), gi[sc["r"][k]], sc["fixed"][k]))
    out.append('</rigidbody2d_scene>')
    return "\n".join(out)


def test_xml_column_steps_like_the_library_scene(ctx):
    cfg = scenes.mpm_column("column_12800")
    cx = scene_xml.read_mpm(mpm_xml(cfg))
    p = scenes.seed_column_points(cfg)
    for prec in (hg.FP64, hg.MIXED):
        a = scene_xml.make_mpm(ctx, cx, precision=prec)
        b = hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
                   cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
                   cfg["planes"], precision=prec, capacity=len(p["m"]))
        b.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])
        a.flow(cfg["dt"], 50)
        b.flow(cfg["dt"], 50)
        sa, sb = a.download(), b.download()
        assert a.status() == 0 and b.status() == 0
        # the P2G sums are atomics in either precision: the same state up to
        # the order of those sums
        if prec == hg.FP64:
            for k in ("q", "v", "be", "J"):
                assert np.allclose(sa[k], sb[k], rtol=1e-10, atol=1e-13), k
        else:
            assert np.abs(sa["q"] - sb["q"]).max() < 1e-9
        a.close()
        b.close()


def test_xml_dem_steps_like_the_library_scene(ctx):
    sc = scenes.dem_column(n=600, per_row=30)
    dp = scenes.dem_params()
    planes = [((0.0, 0.0), (0.0, 1.0)), ((0.0, 0.0), (1.0, 0.0))]
    d = scene_xml.read_dem(dem_xml(sc, dp, planes, cell_scale=1.1))
    assert np.array_equal(d["q"], sc["q"]) and np.array_equal(d["r"], sc["r"])
    assert np.array_equal(d["m"], sc["m"]) and np.array_equal(d["I"], sc["I"])
    a = scene_xml.make_dem(ctx, d)
    b = hg.DEM(ctx, scenes.GRAVITY, dp["kn"], dp["kt"], dp["gamman"], dp["gammat"], dp["mu"],
               planes, cell_scale=1.1, capacity=len(sc["r"]))
    b.upload(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"])
    a.flow(d["dt"], 300)
    b.flow(d["dt"], 300)
    (qa, va), (qb, vb) = a.download(), b.download()
    assert a.status() == 0 and b.status() == 0
    assert np.array_equal(qa, qb) and np.array_equal(va, vb)  # the FP64 step is bit-exact


def test_xml_hybrid_runs_like_the_library_scene(ctx, tmp_path):
    scene = scenes.hybrid_column(scale=0.02)
    cfg, zs, rs = scene["mpm"], scene["zones"], scene["resampling"]
    planes = [(x, n) for (x, n, _st, _lb) in cfg["planes"]]
    (tmp_path / "mpm.xml").write_text(mpm_xml(cfg, basis="uGIMP"))
    (tmp_path / "dem.xml").write_text(dem_xml(scene["dem"], scene["dem_params"], planes))
    (tmp_path / "hybrid.xml").write_text(
        '<hybridgrains2d_scene>\n<discrete_sim file_name="dem.xml"/>\n'
        '<continuum_sim file_name="mpm.xml"/>\n<time_step dt="%s"/>\n<end_time t="1"/>\n'
        '<integrator_style style="prediction_correction_advection_node_node"/>\n'
        '<coupling_force rzoneHalfThickness="%s" demRMean="%s" demRStd="%s" '
        'avoidAVoidFreq="%d" phiThreshold="%s" rzoneLevelSet="%s" phi_window_size="%s" '
        'phi_samples_per_cell_side="%d" level_set_cell_width="%s" rho_dem="%s" '
        'homogenize_stress="1" homogenize_velocity="1"/>\n</hybridgrains2d_scene>\n'
        % (step(cfg["dt"]), f(zs["rzone_half_thickness"]), f(rs["dem_r_mean"]), f(rs["dem_r_std"]),
           rs["avoid_a_void_freq"], f(zs["phi_threshold"]), f(zs["rzone_level_set"]),
           f(zs["phi_window_size"]), zs["phi_samples_per_cell_side"],
           f(zs["level_set_cell_width"]), f(rs["rho_dem"])))
    sx = scene_xml.read_hybrid(str(tmp_path / "hybrid.xml"))
    a = hybrid.HybridSim(ctx, sx)
    b = hybrid.HybridSim(ctx, scene)
    a.step(210)  # the initial resampling and the one after 200 steps
    b.step(210)
    assert a.resamplings == b.resamplings >= 2
    sa, sb = a.mpm.download(), b.mpm.download()
    (qa, _), (qb, _) = a.dem.download(), b.dem.download()
    assert a.mpm.status() == 0 and a.dem.status() == 0
    # the MPM half sums with atomics (see above); the grains follow within that
    assert np.allclose(sa["q"], sb["q"], rtol=0, atol=1e-12)
    assert np.allclose(qa, qb, rtol=0, atol=1e-12)
