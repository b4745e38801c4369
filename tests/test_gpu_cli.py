"""The command-line drivers on the device: an MPM scene run with frames and
numbered snapshots, resumed from a snapshot to the same end; a DEM and a
hybrid scene run with frames (libhybridgrains_gb300.cli)."""
import glob
import os

import numpy as np
import pytest

from libhybridgrains_gb300 import cli, frames, reference_format as rf

pytestmark = pytest.mark.gpu

MPM = """<mpmgrains2d>
  <end_time t="0.001"/>
  <grid min="0.0 0.0" max="1.0 0.5" cell_width="0.005"/>
  <integrator dt="1 / 100000" alpha="0.999" shape_function_order="1"/>
  <material shear_modulus="384615.4" bulk_modulus="833333.3" alpha="0.3266"/>
  <rectangle min="0.1 0.0" max="0.3 0.4" density="1550" cell_samples_per_dim="2" vel="0 0" omega="0"/>
  <near_earth_gravity f="0.0 -9.81"/>
  <static_plane x="0.0 0.0" n="0.0 1.0" boundary_behavior="sticking"/>
  <static_plane x="0.0 0.0" n="1.0 0.0" boundary_behavior="sticking"/>
  <static_plane x="1.0 0.0" n="-1.0 0.0" boundary_behavior="sticking"/>
</mpmgrains2d>"""


def test_mpm_cli_frames_snapshots_and_resume(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    (tmp_path / "mpm.xml").write_text(MPM)
    out = tmp_path / "out"
    # 100 steps, an output every 10 (10 kHz at dt 1e-5): frames 0..10
    assert cli.main(["mpmgrains2d", "mpm.xml", "-o", str(out), "-f", "10000", "-s", "1",
                     "--precision", "fp64", "-q"]) == 0
    names = sorted(os.path.basename(p) for p in glob.glob(str(out / "config_*.npz")))
    assert names == ["config_%02d.npz" % k for k in range(11)]
    f0, f10 = frames.read(str(out / "config_00.npz")), frames.read(str(out / "config_10.npz"))
    assert int(f10["iteration"]) == 100 and float(f10["time"]) == pytest.approx(1e-3)
    assert f0["q"].shape == (2, 12800) and int(f0["npoints"]) == 12800
    assert f10["q"][1].min() >= 0.0 and (f10["q"] != f0["q"]).any()
    snaps = sorted(glob.glob(str(out / "serial_*.bin")))
    assert len(snaps) == 11
    state, run = rf.read_mpm_snapshot(str(out / "serial_05.bin"))
    assert run["iteration"] == 50 and run["steps_per_save"] == 10 and run["output_frame"] == 5
    assert np.array_equal(state["points"]["q"], frames.read(str(out / "config_05.npz"))["q"].T)
    # resume from frame 5: frames 5..10 are written again
    final = f10["q"].copy()
    os.remove(str(out / "config_10.npz"))
    assert cli.main(["mpmgrains2d", "-r", str(out / "serial_05.bin"), "-o", str(out),
                     "--precision", "fp64", "-q"]) == 0
    again = frames.read(str(out / "config_10.npz"))
    assert int(again["iteration"]) == 100
    # the same steps from the same state (P2G atomics: up to their order)
    assert np.allclose(again["q"], final, rtol=0, atol=1e-12)
    # -s 0 overwrites serial.bin in the working directory
    assert cli.main(["mpmgrains2d", "mpm.xml", "-e", "0.0002", "-s", "0", "-q"]) == 0
    state, run = rf.read_mpm_snapshot(str(tmp_path / "serial.bin"))
    assert run["iteration"] == 20 and run["overwrite_snapshots"] is True


DEM = """<rigidbody2d_scene>
  <collision_detection broadphase="spatial_grid" cell_scale="1.1" bandwidth_reduction="none"/>
  <penalty_impact_map dt="1 / 1000000" kn="100000" gamman="0.5" kt="28571.4" gammat="0.5" mu="0.5"/>
  <end_time t="0.0005"/>
  <near_earth_gravity f="0.0 -9.81"/>
  <static_plane x="0 0" n="0 1"/>
  <geometry type="circle" r="0.001"/>
  %s
</rigidbody2d_scene>"""


def test_dem_cli_frames(tmp_path):
    bodies = "\n".join('<rigid_body x="%r %r" theta="0" v="0 0" omega="0" rho="2600" '
                       'geo_idx="0"/>' % (0.0025 * (k % 10), 0.0012 + 0.0025 * (k // 10))
                       for k in range(60))
    (tmp_path / "dem.xml").write_text(DEM % bodies)
    out = tmp_path / "out"
    assert cli.main(["rigidbody2d", str(tmp_path / "dem.xml"), "-o", str(out), "-f", "10000",
                     "-i", "-q"]) == 0
    names = sorted(glob.glob(str(out / "config_*.npz")))
    assert len(names) == 6  # 500 steps, an output every 100
    f = frames.read(names[-1])
    assert str(f["sim_type"]) == "rigidbody2d" and int(f["iteration"]) == 500
    q = f["discrete/q"].reshape(-1, 3)
    assert q.shape == (60, 3) and np.isfinite(q).all() and q[:, 1].min() > 0.0


def test_hybrid_cli_frames(tmp_path):
    from test_gpu_scene_xml import dem_xml, mpm_xml, step, f as num
    from libhybridgrains_gb300 import scenes
    scene = scenes.hybrid_column(scale=0.02)
    cfg, zs, rs = scene["mpm"], scene["zones"], scene["resampling"]
    planes = [(x, n) for (x, n, _st, _lb) in cfg["planes"]]
    (tmp_path / "mpm.xml").write_text(mpm_xml(cfg, basis="uGIMP"))
    (tmp_path / "dem.xml").write_text(dem_xml(scene["dem"], scene["dem_params"], planes))
    (tmp_path / "hybrid.xml").write_text(
        '<hybridgrains2d_scene><discrete_sim file_name="dem.xml"/>'
        '<continuum_sim file_name="mpm.xml"/><time_step dt="%s"/><end_time t="0.00021"/>'
        '<integrator_style style="prediction_correction_advection_node_node"/>'
        '<coupling_force rzoneHalfThickness="%s" demRMean="%s" demRStd="%s" avoidAVoidFreq="%d" '
        'phiThreshold="%s" rzoneLevelSet="%s" phi_window_size="%s" phi_samples_per_cell_side="%d" '
        'level_set_cell_width="%s" rho_dem="%s" homogenize_stress="1" homogenize_velocity="1"/>'
        '</hybridgrains2d_scene>'
        % (step(cfg["dt"]), num(zs["rzone_half_thickness"]), num(rs["dem_r_mean"]),
           num(rs["dem_r_std"]), rs["avoid_a_void_freq"], num(zs["phi_threshold"]),
           num(zs["rzone_level_set"]), num(zs["phi_window_size"]),
           zs["phi_samples_per_cell_side"], num(zs["level_set_cell_width"]), num(rs["rho_dem"])))
    out = tmp_path / "out"
    assert cli.main(["hybridgrains2d", str(tmp_path / "hybrid.xml"), "-o", str(out),
                     "-f", "10000", "-q"]) == 0
    names = sorted(glob.glob(str(out / "config_*.npz")))
    assert len(names) == 3  # iterations 0, 100, 200; the run ends at 210
    f = frames.read(names[-1])
    assert str(f["sim_type"]) == "hybrid2d" and int(f["global_iteration"]) == 200
    n = int(f["continuum/npoints"])
    assert f["continuum/q"].shape == (2, n) and np.isfinite(f["continuum/q"]).all()
    assert len(f["discrete/grid_node_masses"]) == len(f["continuum/grid_node_masses"])
    assert f["discrete/grid_node_masses"].sum() > 0.0
