"""Scene files in the reference's XML schema (mpmgrains2d, rigidbody2d,
hybridgrains2d) read by libhybridgrains_gb300.scene_xml, on the CPU.

The scenes below are small ones written for these tests in the reference's
element and attribute names; where the reference checkout is present, its
column-collapse scene is also read and compared with the fixtures that
tests/golden/make_column_collapse_assets.py made from it."""
import math
import os
from fractions import Fraction

import numpy as np
import pytest

from libhybridgrains_gb300 import scene_xml as sx
from libhybridgrains_gb300 import scenes

HERE = os.path.dirname(os.path.abspath(__file__))

MPM_XML = """<mpmgrains2d>
  <end_time t="0.5"/>
  <grid min="0.0 0.0" max="1.0 0.5" cell_width="0.005"/>
  <integrator dt="1 / 100000" alpha="0.999" shape_function_order="1"/>
  <material shear_modulus="384615.4" bulk_modulus="833333.3" alpha="0.3266"/>
  <rectangle min="0.1 0.0" max="0.3 0.4" density="1550" cell_samples_per_dim="2" vel="0.0 0.0" omega="0.0"/>
  <near_earth_gravity f="0.0 -1.0"/>
  <near_earth_gravity f="0.0 -9.81"/>
  <static_plane x="0.0 0.0" n="0.0 1.0" boundary_behavior="sticking"/>
  <static_plane x="0.0 0.0" n="1.0 0.0" boundary_behavior="sticking"/>
  <static_plane x="1.0 0.0" n="-1.0 0.0" boundary_behavior="sliding"/>
</mpmgrains2d>"""


def test_mpm_scene_fields():
    c = sx.read_mpm(MPM_XML)
    assert c["grid_min"] == (0.0, 0.0) and c["grid_max"] == (1.0, 0.5) and c["h"] == 0.005
    assert c["dt_rational"].numerator == 1 and c["dt_rational"].denominator == 100000
    assert c["dt"] == 1.0 / 100000.0
    assert c["flip_alpha"] == 0.999 and c["basis"] == "linear"
    assert c["shear_modulus"] == 384615.4 and c["dp_alpha"] == 0.3266
    assert c["gravity"] == (0.0, -9.81)  # the last near_earth_gravity wins
    assert c["end_time"] == 0.5
    assert [p[2] for p in c["planes"]] == [True, True, False]
    assert all(p[3] == -math.inf for p in c["planes"])
    assert c["rect_min"] == (0.1, 0.0) and c["rho"] == 1550.0 and c["samples_per_dim"] == 2


def test_mpm_seeding_matches_the_column_scene():
    # the 12,800-point column: same points as the library's column scene
    c = sx.read_mpm(MPM_XML)
    p = sx.seed_points(c)
    cfg = scenes.mpm_column("column_12800")
    ref = scenes.seed_column_points(cfg)
    assert len(p["m"]) == 12800
    assert np.array_equal(p["q"], ref["q"])
    assert np.array_equal(p["m"], ref["m"]) and np.array_equal(p["hl"], ref["hl"])
    assert np.array_equal(p["v"], np.zeros((12800, 2)))


def test_mpm_rectangle_velocity_and_spin():
    text = MPM_XML.replace('vel="0.0 0.0" omega="0.0"', 'vel="0.5 -0.25" omega="2.0 7.0"')
    p = sx.seed_points(sx.read_mpm(text))
    xc, yc = 0.2, 0.2
    # v + omega (z x arm): omega read as the first token, as a stream reads it
    exp = np.stack([0.5 - 2.0 * (p["q"][:, 1] - yc), -0.25 + 2.0 * (p["q"][:, 0] - xc)], axis=1)
    assert np.array_equal(p["v"], exp)


def test_mpm_lower_bound_ends_the_plane_test():
    # pointInsidePlane returns "outside" at the first plane whose lower bound
    # is above the point, before later planes are looked at
    text = MPM_XML.replace('<static_plane x="0.0 0.0" n="0.0 1.0" boundary_behavior="sticking"/>',
                           '<static_plane x="0.0 0.0" n="0.0 1.0" boundary_behavior="sticking" '
                           'lower_bound="0.2"/>'
                           '<static_plane x="0.25 0.0" n="1.0 0.0" boundary_behavior="sliding"/>')
    c = sx.read_mpm(text)
    assert c["planes"][0][3] == 0.2
    q = sx.seed_points(c)["q"]
    # below y = 0.2 the test stops at the first plane: points left of x = 0.25
    # stay; above it the plane x >= 0.25 removes them
    low, high = q[q[:, 1] < 0.2], q[q[:, 1] > 0.2]
    assert (low[:, 0] < 0.25).any()
    assert not (high[:, 0] < 0.25).any()


def test_mpm_multiple_rectangles_in_file_order():
    text = MPM_XML.replace(
        '<near_earth_gravity f="0.0 -1.0"/>',
        '<rectangle min="0.5 0.0" max="0.6 0.1" density="1000" cell_samples_per_dim="1" '
        'vel="1.0 0.0" omega="0.0"/><near_earth_gravity f="0.0 -1.0"/>')
    c = sx.read_mpm(text)
    p = sx.seed_points(c)
    assert len(c["rectangles"]) == 2 and len(p["m"]) == 12800 + 400
    tail = slice(12800, None)
    assert (p["q"][tail, 0] > 0.5).all() and (p["v"][tail, 0] == 1.0).all()
    assert p["hl"][-1] == 0.0025 and p["m"][-1] == 1000.0 * 0.005 * 0.005


def test_dem_scene_static_drums():
    # loadStaticDrums (RigidBody2DSceneParser.cpp:541-585)
    d = sx.read_dem(DEM_XML.replace('<near_earth_gravity f="0.0 -9.0"/>',
                                    '<near_earth_gravity f="0.0 -9.0"/>'
                                    '<static_drum x="0.5 0.25" r="0.2"/>'
                                    '<static_drum x="1 2" r="3 4"/>'))
    assert d["drums"] == [((0.5, 0.25), 0.2), ((1.0, 2.0), 3.0)]
    assert sx.read_dem(DEM_XML)["drums"] == []


@pytest.mark.parametrize("old,new,msg", [
    ('<material shear_modulus="384615.4" bulk_modulus="833333.3" alpha="0.3266"/>', "",
     "material"),
    ('shape_function_order="1"', 'shape_function_order="3"', "third-order"),
    ('shape_function_order="1"', 'shape_function_order="2"', "1 or 3"),
    ('alpha="0.999"', 'alpha="1.5"', "alpha"),
    ('dt="1 / 100000"', 'dt="-1 / 100000"', "positive"),
    ('boundary_behavior="sliding"', 'boundary_behavior="slippy"', "sticking or sliding"),
    ('max="0.3 0.4" density', 'max="0.3 0.6" density', "above the simulation grid"),
    ('min="0.1 0.0" max', 'min="0.1 -0.1" max', "below the simulation grid"),
    ('vel="0.0 0.0"', 'vel="0.0"', "2 scalars"),
    ('<mpmgrains2d>', '<mpmgrains3d>', "root node"),
])
def test_mpm_scene_errors(old, new, msg):
    text = MPM_XML.replace(old, new)
    if new.startswith("<mpmgrains3d"):
        text = text.replace("</mpmgrains2d>", "</mpmgrains3d>")
    with pytest.raises(sx.SceneError, match=msg):
        sx.seed_points(sx.read_mpm(text))


def test_rationals_like_the_reference():
    assert sx.rational("1 / 1000080") == Fraction(1, 1000080)
    assert sx.rational("0.000001") == Fraction(1, 1000000)
    assert sx.rational("3") == 3
    assert sx.rational(" 0.5 ") == Fraction(1, 2) and sx.rational("-2 / 4") == Fraction(-1, 2)
    for bad in ("1/2/3", "1.5/2", "1..2", "x", "1e-06", "1/0", "."):
        with pytest.raises(sx.SceneError):
            sx.rational(bad)


DEM_XML = """<rigidbody2d_scene>
  <camera center="0 0" scale="1" fps="60" render_at_fps="1" locked="0"/>
  <collision_detection broadphase="spatial_grid" cell_scale="1.1" bandwidth_reduction="none"/>
  <penalty_impact_map dt="0.000001" kn="100000" gamman="0.5" kt="28571.4" gammat="0.5" mu="0.5"/>
  <near_earth_gravity f="0.0 -9.0"/>
  <near_earth_gravity f="0.5 -0.81"/>
  <static_plane x="0 0" n="0 2"/>
  <geometry type="circle" r="0.001"/>
  <geometry type="box" r="0.01 0.02"/>
  <geometry type="circle" r="0.0011"/>
  <rigid_body x="0.01 0.002" theta="0.1" v="0.0 -1.0" omega="3.0" rho="2600" geo_idx="0" fixed="1"/>
  <rigid_body x="0.02 0.002" theta="0.0" v="1.0 0.0" omega="0.0" rho="2600" geo_idx="2"/>
  <!-- <rigid_body x="0.03 0.002" theta="0.0" v="0 0" omega="0" rho="2600" geo_idx="0"/> -->
  <rigid_body x="0.03 0.004" theta="0.0" v="0.0 0.0" omega="0.0" rho="1000" geo_idx="0" fixed="0"/>
</rigidbody2d_scene>"""


def test_dem_scene_fields():
    d = sx.read_dem(DEM_XML)
    assert d["q"].shape == (3, 3) and d["q"][0].tolist() == [0.01, 0.002, 0.1]
    assert d["v"][0].tolist() == [0.0, -1.0, 3.0]
    assert d["r"].tolist() == [0.001, 0.0011, 0.001]
    assert d["fixed"].tolist() == [1, 0, 0]
    # CircleGeometry::massAndInertia, left to right
    m = d["rho"] * math.pi * d["r"] * d["r"]
    assert np.array_equal(d["m"], m) and np.array_equal(d["I"], 0.5 * m * d["r"] * d["r"])
    assert d["gravity"] == (0.5, -9.81)  # the forces add
    assert d["dt"] == 1e-6 and d["kn"] == 100000.0 and d["mu"] == 0.5
    assert d["cell_scale"] == 1.1 and d["planes"] == [((0.0, 0.0), (0.0, 2.0))]


@pytest.mark.parametrize("old,new,msg", [
    ('geo_idx="2"', 'geo_idx="1"', "box bodies"),
    ('geo_idx="2"', 'geo_idx="5"', "out of range"),
    ('fixed="1"', 'fixed="2"', "boolean"),
    ('<near_earth_gravity f="0.0 -9.0"/>', '<static_drum x="0 0" r="0"/>', "static_drum"),
    ('<near_earth_gravity f="0.0 -9.0"/>', '<planar_portal/>', "planar_portal"),
    ('<penalty_impact_map dt="0.000001" kn="100000" gamman="0.5" kt="28571.4" gammat="0.5" '
     'mu="0.5"/>', "", "penalty_impact_map"),
    ('broadphase="spatial_grid"', 'broadphase="all_pairs"', "spatial_grid"),
    ('cell_scale="1.1"', 'cell_scale="0"', "positive"),
    ('kn="100000"', 'kn="-1"', "non-negative"),
])
def test_dem_scene_errors(old, new, msg):
    with pytest.raises(sx.SceneError, match=msg):
        sx.read_dem(DEM_XML.replace(old, new))


HYBRID_XML = """<hybridgrains2d_scene>
  <discrete_sim file_name="grains.xml"/>
  <continuum_sim file_name="continuum.xml"/>
  <time_step dt="1 / 1000000"/>
  <end_time t="1.0"/>
  <integrator_type type="coupled"/>
  <integrator_style style="prediction_correction_advection_node_node"/>
  <coupling_force rzoneHalfThickness="0.00125" demRMean="0.001" avoidAVoidFreq="200"
      level_set_cell_width="0.0025" phi_window_size="0.00435" phi_samples_per_cell_side="1"
      homogenize_stress="1" homogenize_velocity="0"/>
</hybridgrains2d_scene>"""


def test_hybrid_scene(tmp_path):
    (tmp_path / "grains.xml").write_text(DEM_XML)
    (tmp_path / "continuum.xml").write_text(MPM_XML)
    (tmp_path / "hybrid.xml").write_text(HYBRID_XML)
    s = sx.read_hybrid(str(tmp_path / "hybrid.xml"))
    assert s["dt"] == 1e-6 and s["mpm"]["dt"] == 1e-6 and s["end_time"] == 1.0
    assert len(s["dem"]["r"]) == 3 and s["mpm"]["h"] == 0.005
    z, r = s["zones"], s["resampling"]
    # the values given, and the parser's defaults for the others
    assert z["rzone_half_thickness"] == 0.00125 and z["level_set_cell_width"] == 0.0025
    assert z["phi_threshold"] == 0.5 and z["rzone_level_set"] == 0.0
    assert z["allow_direct_transitions"] is False
    assert r["avoid_a_void_freq"] == 200 and r["dem_r_mean"] == 0.001 and r["dem_r_std"] == 0.0
    assert r["rho_dem"] == 0.96
    assert r["homogenize_stress"] is True and r["homogenize_velocity"] is False
    assert r["newly_inserted_continuum_stress_free"] is False
    assert s["dem_params"]["planes"] == [((0.0, 0.0), (0.0, 2.0))]
    (tmp_path / "hybrid.xml").write_text(HYBRID_XML.replace(
        "prediction_correction_advection_node_node", "iterative"))
    with pytest.raises(sx.SceneError, match="node-node"):
        sx.read_hybrid(str(tmp_path / "hybrid.xml"))


def _reference_column_collapse():
    import __graft_entry__
    root = os.environ.get("HG_REFERENCE_ROOT") or __graft_entry__.REFERENCE_CHECKOUT
    d = os.path.join(root, "assets", "hybridgrains2dnew", "column-collapse")
    if not os.path.exists(os.path.join(d, "hybrid.xml")):
        pytest.skip("reference checkout absent")
    return d


def test_reference_column_collapse_matches_the_fixtures():
    import json
    d = _reference_column_collapse()
    s = sx.read_hybrid(os.path.join(d, "hybrid.xml"))
    with open(os.path.join(HERE, "golden", "column_collapse_scene.json")) as f:
        fx = json.load(f)
    z = np.load(os.path.join(HERE, "golden", "column_collapse_dem.npz"))
    dem, mpm = s["dem"], s["mpm"]
    assert np.array_equal(dem["q"][:, 0], z["x"]) and np.array_equal(dem["q"][:, 1], z["y"])
    assert np.array_equal(dem["q"][:, 2], z["theta"]) and np.array_equal(dem["r"], z["r"])
    assert np.array_equal(dem["fixed"], z["fixed"]) and np.array_equal(dem["rho"], z["rho"])
    fm, fd = fx["mpm"], fx["dem"]
    assert list(mpm["grid_min"]) == fm["grid_min"] and mpm["h"] == fm["cell_width"]
    assert mpm["basis"] == "ugimp" and fm["basis"] == "uGIMP"
    assert mpm["dp_alpha"] == fm["dp_alpha"] and mpm["flip_alpha"] == fm["flip_alpha"]
    assert [list(p[1]) for p in mpm["planes"]] == [p["n"] for p in fm["planes"]]
    for k in ("kn", "kt", "gamman", "gammat", "mu", "dt", "cell_scale"):
        assert dem[k] == fd[k]
    assert s["dt"] == fx["hybrid"]["dt"]
    assert s["zones"]["rzone_half_thickness"] == fx["hybrid"]["rzone_half_thickness"]
    assert s["resampling"]["avoid_a_void_freq"] == fx["hybrid"]["avoid_a_void_freq"]
    assert len(sx.seed_points(mpm)["m"]) == 7936


def test_reference_hourglass_is_outside_this_path():
    d = os.path.join(os.path.dirname(_reference_column_collapse()), "hourglass")
    with pytest.raises(sx.SceneError, match="box bodies"):
        sx.read_hybrid(os.path.join(d, "hybrid.xml"))
