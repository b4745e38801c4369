"""The command-line drivers' host logic (libhybridgrains_gb300.cli) on the
CPU: the output schedule, the exit iteration, file names and argument
errors, against the reference CLI's rules (mpmgrains2d_cli.cpp)."""
import math
from fractions import Fraction

import pytest

from libhybridgrains_gb300 import cli


def test_steps_per_save_must_be_an_integer():
    assert cli.steps_per_save(Fraction(1, 100000), 0) == 1
    assert cli.steps_per_save(Fraction(1, 100000), 100) == 1000
    assert cli.steps_per_save(Fraction(1, 1000080), 240) == 4167
    with pytest.raises(cli.CLIError, match="integer number of timesteps"):
        cli.steps_per_save(Fraction(1, 1000080), 7)


def exit_by_loop(start, end, dt):
    # the reference's loop, one step at a time
    i = start
    while not (i * dt >= end):
        i += 1
    return i


@pytest.mark.parametrize("end,dt", [(2.0, 1.0 / 1000080), (0.01, 1e-5), (0.3, 0.1),
                                    (1e-3, 3e-6), (0.5, 1e-5), (1.0, 1.0 / 3.0)])
def test_final_iteration_is_the_loops_exit(end, dt):
    for start in (0, 7):
        assert cli.final_iteration(start, end, dt) == exit_by_loop(start, end, dt)
    past = exit_by_loop(0, end, dt) + 5
    assert cli.final_iteration(past, end, dt) == past  # resumed past the end: no steps


def test_run_loop_outputs_and_chunks():
    steps, outs = [], []
    n = cli.run_loop(0, 95, 10, steps.append, outs.append)
    assert outs == list(range(0, 91, 10)) and n == 10
    assert sum(steps) == 95 and steps[-1] == 5 and all(k <= 10 for k in steps)
    # resumed at a multiple: that output is written again, as the reference does
    steps, outs = [], []
    cli.run_loop(40, 60, 10, steps.append, outs.append)
    assert outs == [40, 50, 60] and steps == [10, 10]
    # resumed off a multiple: the first chunk ends on the next one
    steps, outs = [], []
    cli.run_loop(43, 60, 10, steps.append, outs.append)
    assert outs == [50, 60] and steps == [7, 10]
    steps, outs = [], []
    cli.run_loop(0, 3, 1, steps.append, outs.append)
    assert outs == [0, 1, 2, 3] and steps == [1, 1, 1]


def test_widths_names_and_precision():
    # 1 + ceil(end / dt) / steps-per-output, in digits
    assert cli.save_number_width(0.01, 1e-5, 10) == len(str(1 + 1000 // 10))
    assert cli.save_number_width(2.0, 1.0 / 1000080, 4167) == len(str(1 + math.ceil(2.0 * 1000080) // 4167))
    assert cli.frame_name("out", "config", 7, 4, "npz").endswith("config_0007.npz")
    assert cli.frame_name("", "serial", 12, 3, "bin") == "serial_012.bin"
    assert cli.display_precision(Fraction(1, 1000000), "0.000001") == 6
    assert cli.display_precision(Fraction(1, 2000), "0.0005") == 4
    assert cli.display_precision(Fraction(1, 1000080), "1 / 1000080") == 6


SCENE = """<mpmgrains2d>
  <grid min="0.0 0.0" max="1.0 0.5" cell_width="0.005"/>
  <integrator dt="1 / 100000" alpha="0.999" shape_function_order="1"/>
  <material shear_modulus="384615.4" bulk_modulus="833333.3" alpha="0.3266"/>
  <rectangle min="0.1 0.0" max="0.3 0.4" density="1550" cell_samples_per_dim="2" vel="0 0" omega="0"/>
  <static_plane x="0.0 0.0" n="0.0 1.0" boundary_behavior="sticking"/>
</mpmgrains2d>"""


def test_argument_errors_before_any_device_work(tmp_path, capsys):
    path = tmp_path / "mpm.xml"
    path.write_text(SCENE)
    # no end time in the scene and none given
    assert cli.main(["mpmgrains2d", str(path), "-q"]) == 1
    assert "end_time" in capsys.readouterr().err
    # an output rate that does not divide the step
    assert cli.main(["mpmgrains2d", str(path), "-e", "0.01", "-f", "30000", "-q"]) == 1
    assert "integer number of timesteps" in capsys.readouterr().err
    assert cli.main(["mpmgrains2d", str(path), "-e", "-1", "-q"]) == 1
    assert "positive" in capsys.readouterr().err
    assert cli.main(["mpmgrains2d", "-q"]) == 1
    assert "Usage" in capsys.readouterr().err
    with pytest.raises(SystemExit):
        cli.main(["mpmgrains2d", str(path), "-s", "2"])
    with pytest.raises(SystemExit):  # -r and -s are MPM options only
        cli.main(["rigidbody2d", str(path), "-r", "serial.bin"])
