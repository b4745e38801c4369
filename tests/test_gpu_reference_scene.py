"""The reference's own hybrid column-collapse scene (assets/hybridgrains2dnew/
column-collapse: 6,694 disks, 615 of them fixed, over a uGIMP MPM column in
CGS units) run by the library from scene files. The files are written here
from the fixtures tests/golden/make_column_collapse_assets.py made from the
reference's XML, read back by scene_xml and stepped by hybrid.HybridSim
through three resampling intervals, with the MPM bulk in FP64 and in mixed
precision."""
import json
import os

import numpy as np
import pytest

from libhybridgrains_gb300 import cli, frames, hybrid, scene_xml

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def num(x):
    return repr(float(x))


def pair(v):
    return "%s %s" % (num(v[0]), num(v[1]))


def write_scene(d):
    with open(os.path.join(GOLDEN, "column_collapse_scene.json")) as f:
        sc = json.load(f)
    z = np.load(os.path.join(GOLDEN, "column_collapse_dem.npz"))
    m, dm, hy = sc["mpm"], sc["dem"], sc["hybrid"]
    dt = "1 / %d" % round(1.0 / hy["dt"])
    planes = "".join('<static_plane x="%s" n="%s" boundary_behavior="%s"/>\n'
                     % (pair(p["x"]), pair(p["n"]), "sticking" if p["sticking"] else "sliding")
                     for p in m["planes"])
    with open(os.path.join(d, "mpm.xml"), "w") as f:
        f.write('<mpmgrains2d>\n<grid min="%s" max="%s" cell_width="%s"/>\n'
                '<integrator dt="%s" alpha="%s" shape_function_order="1" '
                'shape_function_category="%s"/>\n'
                '<material shear_modulus="%s" bulk_modulus="%s" alpha="%s"/>\n'
                '<rectangle min="%s" max="%s" density="%s" cell_samples_per_dim="%d" vel="0 0" '
                'omega="0"/>\n<near_earth_gravity f="%s"/>\n%s</mpmgrains2d>\n'
                % (pair(m["grid_min"]), pair(m["grid_max"]), num(m["cell_width"]), dt,
                   num(m["flip_alpha"]), m["basis"], num(m["shear_modulus"]),
                   num(m["bulk_modulus"]), num(m["dp_alpha"]), pair(m["rect_min"]),
                   pair(m["rect_max"]), num(m["density"]), m["samples_per_dim"],
                   pair(m["gravity"]), planes))
    radii = sorted(set(z["r"].tolist()))
    gi = {r: k for k, r in enumerate(radii)}
    body = ['<rigid_body x="%s %s" theta="%s" v="0 0" omega="0" rho="%s" geo_idx="%d" '
            'fixed="%d"/>' % (num(x), num(y), num(t), num(rho), gi[r], fx)
            for x, y, t, r, rho, fx in zip(z["x"], z["y"], z["theta"], z["r"], z["rho"],
                                           z["fixed"])]
    with open(os.path.join(d, "dem.xml"), "w") as f:
        f.write('<rigidbody2d_scene>\n<collision_detection broadphase="spatial_grid" '
                'cell_scale="%s" bandwidth_reduction="cuthill_mckee"/>\n'
                '<penalty_impact_map dt="%s" kn="%s" gamman="%s" kt="%s" gammat="%s" mu="%s"/>\n'
                '<near_earth_gravity f="%s"/>\n%s%s\n%s\n</rigidbody2d_scene>\n'
                % (num(dm["cell_scale"]), dt, num(dm["kn"]), num(dm["gamman"]), num(dm["kt"]),
                   num(dm["gammat"]), num(dm["mu"]), pair(dm["gravity"]),
                   "".join('<static_plane x="%s" n="%s"/>\n' % (pair(p["x"]), pair(p["n"]))
                           for p in dm["planes"]),
                   "\n".join('<geometry type="circle" r="%s"/>' % num(r) for r in radii),
                   "\n".join(body)))
    with open(os.path.join(d, "hybrid.xml"), "w") as f:
        f.write('<hybridgrains2d_scene>\n<discrete_sim file_name="dem.xml"/>\n'
                '<continuum_sim file_name="mpm.xml"/>\n<time_step dt="%s"/>\n'
                '<end_time t="%s"/>\n<integrator_type type="coupled"/>\n'
                '<integrator_style style="prediction_correction_advection_node_node"/>\n'
                '<coupling_force rzoneHalfThickness="%s" demRMean="%s" demRStd="%s" '
                'avoidAVoidFreq="%d" phiThreshold="%s" rzoneLevelSet="%s" phi_window_size="%s" '
                'phi_samples_per_cell_side="%d" level_set_cell_width="%s" rho_dem="%s" '
                'homogenize_stress="%d" homogenize_velocity="%d"/>\n</hybridgrains2d_scene>\n'
                % (dt, num(hy["end_time"]), num(hy["rzone_half_thickness"]),
                   num(hy["dem_r_mean"]), num(hy["dem_r_std"]), hy["avoid_a_void_freq"],
                   num(hy["phi_threshold"]), num(hy["rzone_level_set"]),
                   num(hy["phi_window_size"]), hy["phi_samples_per_cell_side"],
                   num(hy["level_set_cell_width"]), num(hy["rho_dem"]),
                   hy["homogenize_stress"], hy["homogenize_velocity"]))
    return sc, z


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reference_column_collapse_runs(ctx, tmp_path, precision):
    import libhybridgrains_gb300 as hg
    sc, z = write_scene(str(tmp_path))
    scene = scene_xml.read_hybrid(str(tmp_path / "hybrid.xml"))
    assert scene["dt"] == sc["hybrid"]["dt"] and len(scene["dem"]["r"]) == len(z["r"]) == 6694
    assert int(scene["dem"]["fixed"].sum()) == 615 and scene["mpm"]["basis"] == "ugimp"
    sim = hybrid.HybridSim(ctx, scene, precision=hg.MIXED if precision == "mixed" else hg.FP64)
    sim.step(250)  # resamplings at iterations 0, 100 and 200
    assert sim.resamplings >= 3
    assert sim.mpm.status() == 0 and sim.dem.status() == 0
    st = sim.mpm.download()
    q3, v3 = sim.dem.download()
    assert len(st["q"]) > 0 and len(q3) > 0
    assert np.isfinite(st["q"]).all() and np.isfinite(q3).all()
    # fixed grains (the rough floor) stay where they are
    fixed = sim.G["fixed"].astype(bool)
    assert fixed.sum() > 0 and np.array_equal(q3[fixed], sim.G["q0"][fixed])
    # nothing leaves the domain in 250 steps of 1 us: speeds stay far below
    # the 40 cm a disk would need
    assert np.abs(v3[~fixed, :2]).max() < 1e3 and np.abs(st["v"]).max() < 1e3


def test_reference_column_collapse_cli(tmp_path):
    write_scene(str(tmp_path))
    out = tmp_path / "out"
    # 1000080 / 2160 = 463 steps per output; 0.0005 s is 501 steps
    assert cli.main(["hybridgrains2d", str(tmp_path / "hybrid.xml"), "-e", "0.0005",
                     "-o", str(out), "-f", "2160", "--precision", "mixed", "-q"]) == 0
    names = sorted(os.listdir(str(out)))
    assert names == ["config_0.npz", "config_1.npz"]
    f = frames.read(str(out / "config_1.npz"))
    assert int(f["global_iteration"]) == 463 and str(f["sim_type"]) == "hybrid2d"
