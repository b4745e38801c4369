"""Command-line drivers with the reference's three CLIs' options.

    python -m libhybridgrains_gb300.cli mpmgrains2d scene.xml [-r file] [-e end] [-o dir]
                                                              [-f Hz] [-s 0|1]
    python -m libhybridgrains_gb300.cli rigidbody2d scene.xml [-i] [-e end] [-o dir] [-f Hz]
    python -m libhybridgrains_gb300.cli hybridgrains2d hybrid.xml [-i] [-e end] [-o dir] [-f Hz]

Each runs a scene file to its end time on the GPU, as mpmgrains2d_cli,
rigidbody2d_cli and hybridgrains2d_cli do (mpmgrains2d_cli.cpp:275-555,
rigidbody2d_cli.cpp, hybridgrains2d_cli.cpp):

* ``-f`` sets the output rate in Hz; the steps per output, 1 / (dt f), must
  be an integer, as an exact rational (without ``-f`` every step is output);
* the loop outputs at iteration 0 and after every step whose iteration is a
  multiple of the steps per output, and stops at the first iteration i with
  i dt >= the end time (both in doubles);
* ``-o dir`` writes each output as ``dir/config_<frame>.npz``, the frame
  number zero-padded to the width of 1 + ceil(end / dt) / steps-per-output,
  with the reference's HDF5 dataset names (HDF5 is not available: see
  ``frames``);
* ``-s 0`` (MPM) serialises the run to ``serial.bin`` at every output,
  ``-s 1`` to ``serial_<frame>.bin`` beside the frames, in the reference's
  byte layout (``reference_format``); ``-r file`` resumes such a snapshot,
  with its own end time, output rate and frame counter;
* ``-i`` (impulses) is accepted and, as in the reference's CLIs, writes
  nothing more.

The reference's hybrid and penalty-map states do not serialise
(HybridIntegratorState.cpp:67-85, PenaltyImpactFrictionMap.cpp:1155-1158);
``-s`` and ``-r`` are MPM options here for that reason (the library's own
checkpoint files cover the other objects). Between outputs the GPU steps
in one call, so that repeated steps replay as CUDA graphs.
"""
import argparse
import math
import os
import sys
from fractions import Fraction


class CLIError(Exception):
    """An invalid command line or run configuration (the reference prints
    the message and exits with EXIT_FAILURE)."""


def steps_per_save(dt, frequency):
    """mpmgrains2d_cli.cpp:516-531: 1 / (dt f) as an exact rational; it must
    be an integer. Without an output rate every step is output."""
    if not frequency:
        return 1
    x = Fraction(1) / (Fraction(dt) * int(frequency))
    if x.denominator != 1:
        raise CLIError("Timestep and output frequency do not yield an integer number of "
                       "timesteps for data output.")
    return int(x.numerator)


def num_digits(n):
    """MathUtilities::computeNumDigits: decimal digits of n (1 for 0)."""
    return len(str(int(n)))


def save_number_width(end_time, dt, sps):
    """1 + ceil(end / dt) / steps-per-output (unsigned division), in digits."""
    return num_digits(1 + int(math.ceil(end_time / dt)) // sps)


def final_iteration(start, end_time, dt):
    """The first iteration i >= start with i dt >= end_time in doubles (the
    loop's exit test, mpmgrains2d_cli.cpp:294-299)."""
    i = max(int(start), int(math.floor(end_time / dt)) - 2)
    while i * dt < end_time:
        i += 1
    # the estimate may overshoot only if start is already past the end
    while i > start and (i - 1) * dt >= end_time:
        i -= 1
    return i


def run_loop(start, stop, sps, step, export):
    """Outputs at ``start`` (when a multiple of sps) and at every multiple of
    sps reached while stepping to ``stop``; ``step(k)`` advances k steps,
    ``export(iteration)`` writes one output. Returns the outputs written."""
    it, outputs = int(start), 0
    if it % sps == 0:
        export(it)
        outputs += 1
    while it < stop:
        k = min(sps - it % sps, stop - it)
        step(k)
        it += k
        if it % sps == 0:
            export(it)
            outputs += 1
    return outputs


def display_precision(dt, dt_string):
    """computeTimestepDisplayPrecision (mpmgrains2d_cli.cpp:77-91): the
    digits after the point of the dt string, else of std::fixed (6)."""
    s = dt_string if dt_string and "." in dt_string else "%f" % float(dt)
    return len(s) - s.index(".") - 1


def frame_name(directory, stem, frame, width, ext):
    """generateOutputFileName: <dir>/<stem>_<frame zero-padded>.<ext>."""
    name = "%s_%0*d.%s" % (stem, width, frame, ext)
    return os.path.join(directory, name) if directory else name


def _common(p, resume=True, snapshots=True, impulses=False):
    p.add_argument("scene", nargs="?", help="XML scene file")
    if impulses:
        p.add_argument("-i", "--impulses", action="store_true",
                       help="accepted for compatibility; writes nothing more")
    if resume:
        p.add_argument("-r", "--resume", metavar="file",
                       help="resume from a serialized snapshot")
    p.add_argument("-e", "--end", type=float, metavar="scalar",
                   help="override the end time of the scene file")
    p.add_argument("-o", "--output_dir", metavar="dir", help="write outputs to this directory")
    p.add_argument("-f", "--frequency", type=int, default=0, metavar="integer",
                   help="output rate in Hz; ignored without an output directory")
    if snapshots:
        p.add_argument("-s", "--serialize_snapshots", type=int, choices=(0, 1), metavar="bool",
                       help="0: overwrite serial.bin at every output; 1: a new snapshot each")
    p.add_argument("--precision", choices=("fp64", "mixed"), default=None,
                   help="arithmetic of the MPM / DEM step (default: mixed MPM, fp64 DEM "
                        "and fp64 hybrid bulk)")
    p.add_argument("--device", type=int, default=0)
    p.add_argument("-q", "--quiet", action="store_true")


def _end_time(args, scene_end):
    if args.end is not None:
        if not args.end > 0.0:
            raise CLIError("Value for -e/--end must be a positive scalar.")
        return args.end
    if not math.isfinite(scene_end):
        raise CLIError("the scene has no end_time; give -e/--end")
    return scene_end


def _say(args, *msg):
    if not args.quiet:
        print(*msg, flush=True)


def _precision(args, default):
    import libhybridgrains_gb300 as hg
    if args.precision is None:
        return default
    return hg.FP64 if args.precision == "fp64" else hg.MIXED


def run_mpm(args):
    """mpmgrains2d_cli: an MPM scene, or a snapshot with -r."""
    import numpy as np
    import libhybridgrains_gb300 as hg
    from . import frames, reference_format as rf, scene_xml
    if args.resume:
        state, run = rf.read_mpm_snapshot(args.resume)
        p = state["points"]
        host = dict(m=p["m"], vol=p["volume"], hl=p["hl"], q0=p["q0"])
        cfg = dict(h=state["grid"]["cell_width"], shear_modulus=state["shear_modulus"],
                   bulk_modulus=state["bulk_modulus"], dp_alpha=state["dp_alpha"],
                   flip_alpha=state["flip_alpha"], gravity=tuple(state["gravity"]),
                   planes=[(x, n, b == rf.STICKING, lb) for (x, n, b, lb) in state["planes"]])
        dt_r = Fraction(int(run["dt"][0]), int(run["dt"][1]))
        it0, end = int(run["iteration"]), float(run["end_time"])
        sps, frame = int(run["steps_per_save"]) or 1, int(run["output_frame"])
        width, prec = int(run["save_number_width"]), int(run["dt_string_precision"])
        snapshots, overwrite = bool(run["serialize_snapshots"]), bool(run["overwrite_snapshots"])
    else:
        if not args.scene:
            raise CLIError("Usage: mpmgrains2d xml_scene_file_name [options]")
        cfg = scene_xml.read_mpm(args.scene)
        pts = scene_xml.seed_points(cfg)
        host = dict(m=pts["m"], vol=pts["vol"], hl=pts["hl"], q0=pts["q"].copy())
        dt_r, it0, frame = cfg["dt_rational"], 0, 0
        end = _end_time(args, cfg["end_time"])
        sps = steps_per_save(dt_r, args.frequency)
        width = save_number_width(end, float(dt_r.numerator) / float(dt_r.denominator), sps)
        prec = display_precision(dt_r, cfg["dt_string"])
        snapshots = args.serialize_snapshots is not None
        overwrite = not bool(args.serialize_snapshots)
    dt = float(dt_r.numerator) / float(dt_r.denominator)
    stop = final_iteration(it0, end, dt)
    ctx = hg.Context(args.device)
    if args.resume:
        mpm = rf.device_from_snapshot(ctx, state, precision=_precision(args, hg.MIXED))
    else:
        mpm = scene_xml.make_mpm(ctx, cfg, precision=_precision(args, hg.MIXED), points=pts)
    out = args.output_dir
    if out:
        os.makedirs(out, exist_ok=True)
    counter = [frame]
    _say(args, "Simulation stats:\n  Material Point Count: %d\n  Time-Step: %s\n  End Time: %g\n"
         "  Steps: %d to %d, output every %d" % (len(host["m"]), dt_r, end, it0, stop, sps))

    def export(it):
        f = counter[0]
        if out:
            path = frame_name(out, "config", f, width, "npz")
            _say(args, "Saving state at time %.*f to %s" % (prec, it * dt, path))
            frames.write(path, {"timestep": np.array(dt), "iteration": np.array(it, np.uint32),
                                "time": np.array(dt * it), "git_hash": np.array("")},
                         frames.mpm_frame(mpm, cfg, host["m"], host["vol"], host["hl"], prefix=""))
        if snapshots:
            path = "serial.bin" if overwrite else frame_name(out, "serial", f, width, "bin")
            state = rf.snapshot_from_device(mpm, cfg, host["m"], host["vol"], host["hl"],
                                            host["q0"])
            rf.write_mpm_snapshot(path, state, dict(
                iteration=it, dt=(dt_r.numerator, dt_r.denominator), end_time=end,
                steps_per_save=sps, output_frame=f, dt_string_precision=prec,
                save_number_width=width, serialize_snapshots=True,
                overwrite_snapshots=overwrite))
        counter[0] += 1

    def step(k):
        mpm.flow(dt, k)
        st = mpm.status()
        if st:
            raise CLIError("device status word %#x after iteration stepping" % st)

    n = run_loop(it0, stop, sps, step, export)
    _say(args, "Simulation complete at time %.*f (%d outputs). Exiting." % (prec, stop * dt, n))
    return 0


def run_dem(args):
    """rigidbody2d_cli: circles under the penalty impact-friction map."""
    import numpy as np
    import libhybridgrains_gb300 as hg
    from . import frames, scene_xml
    if not args.scene:
        raise CLIError("Usage: rigidbody2d xml_scene_file_name [options]")
    d = scene_xml.read_dem(args.scene)
    dt_r = d["dt_rational"]
    dt = float(dt_r.numerator) / float(dt_r.denominator)
    end = _end_time(args, d["end_time"])
    sps = steps_per_save(dt_r, args.frequency)
    width = save_number_width(end, dt, sps)
    prec = display_precision(dt_r, d["dt_string"])
    stop = final_iteration(0, end, dt)
    ctx = hg.Context(args.device)
    dem = scene_xml.make_dem(ctx, d, precision=_precision(args, hg.FP64))
    out = args.output_dir
    if out:
        os.makedirs(out, exist_ok=True)
    counter = [0]
    _say(args, "Simulation stats:\n  Bodies: %d\n  Time-Step: %s\n  End Time: %g"
         % (len(d["r"]), dt_r, end))

    def export(it):
        if out:
            path = frame_name(out, "config", counter[0], width, "npz")
            _say(args, "Saving state at time %.*f to %s" % (prec, it * dt, path))
            frames.write(path, {"timestep": np.array(dt), "iteration": np.array(it, np.uint32),
                                "time": np.array(dt * it), "git_hash": np.array(""),
                                "sim_type": np.array("rigidbody2d")},
                         frames.dem_frame(dem, d["r"], d["m"], d["fixed"]))
        counter[0] += 1

    def step(k):
        dem.flow(dt, k)
        st = dem.status()
        if st:
            raise CLIError("device status word %#x" % st)

    n = run_loop(0, stop, sps, step, export)
    _say(args, "Simulation complete at time %.*f (%d outputs). Exiting." % (prec, stop * dt, n))
    return 0


def run_hybrid(args):
    """hybridgrains2d_cli with the node-node integrator and the resampling
    interval (hybrid.HybridSim)."""
    import numpy as np
    import libhybridgrains_gb300 as hg
    from . import frames, hybrid, scene_xml
    if not args.scene:
        raise CLIError("Usage: hybridgrains2d xml_scene_file_name [options]")
    scene = scene_xml.read_hybrid(args.scene)
    dt_r = scene["dt_rational"]
    dt = float(dt_r.numerator) / float(dt_r.denominator)
    end = _end_time(args, scene["end_time"])
    sps = steps_per_save(dt_r, args.frequency)
    width = save_number_width(end, dt, sps)
    prec = display_precision(dt_r, None)
    stop = final_iteration(0, end, dt)
    ctx = hg.Context(args.device)
    sim = hybrid.HybridSim(ctx, scene, precision=_precision(args, hg.FP64))
    out = args.output_dir
    if out:
        os.makedirs(out, exist_ok=True)
    counter = [0]

    def export(it):
        if out:
            path = frame_name(out, "config", counter[0], width, "npz")
            _say(args, "Saving state at time %.*f to %s" % (prec, it * dt, path))
            c = sim.hyb.coupling() if sim.started else None
            P, G = sim.P, sim.G
            frames.write(
                path, {"global_timestep": np.array(dt),
                       "global_iteration": np.array(it, np.uint32),
                       "global_time": np.array(float(it * dt_r)), "git_hash": np.array(""),
                       "sim_type": np.array("hybrid2d")},
                frames.dem_frame(sim.dem, G["r"], G["M0"][:, 0] * G["w"], G["fixed"]),
                frames.mpm_frame(sim.mpm, sim.cfg, P["m0"] * P["w"], P["vol0"] * P["w"],
                                 P["hl"], prefix="continuum",
                                 hybrid_factors=None if c is None else c["homog_factor"]),
                {"discrete/grid_node_masses": (np.zeros(sim.mpm.nnodes) if c is None
                                               else c["dem_mass_grid"])})
        counter[0] += 1

    def step(k):
        sim.step(k)
        st = sim.mpm.status() | sim.dem.status()
        if st:
            raise CLIError("device status word %#x" % st)

    n = run_loop(0, stop, sps, step, export)
    _say(args, "Simulation complete at time %.*f (%d outputs, %d resamplings). Exiting."
         % (prec, stop * dt, n, sim.resamplings))
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m libhybridgrains_gb300.cli",
                                 description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="sim", required=True)
    _common(sub.add_parser("mpmgrains2d", help="MPM scene (mpmgrains2d_cli)"))
    _common(sub.add_parser("rigidbody2d", help="DEM scene (rigidbody2d_cli)"),
            resume=False, snapshots=False, impulses=True)
    _common(sub.add_parser("hybridgrains2d", help="hybrid scene (hybridgrains2d_cli)"),
            resume=False, snapshots=False, impulses=True)
    args = ap.parse_args(argv)
    run = {"mpmgrains2d": run_mpm, "rigidbody2d": run_dem, "hybridgrains2d": run_hybrid}
    try:
        return run[args.sim](args)
    except (CLIError, ValueError) as e:
        print(str(e), file=sys.stderr)
        return 1


if __name__ == "__main__":
    sys.exit(main())
