"""Benchmark: mixed-precision MPM step on the 2,000,000-point column.

One "step" is one ExplicitIntegrator::flow step (mpmgrains2d) of the
2,000,000-point granular column on a 2048 x 1024 grid (h = 1 mm, dt = 2e-6 s),
the large mixed-precision configuration. Prints one JSON line:

  value      particle-steps/s of the MIXED path with the particle state resident
             in HBM (all ranks together);
  e2e        the same metric through the public C ABI with host buffers: every
             step uploads the particle state from pinned host memory, steps and
             downloads it again;
  fp64       the plain FP64 GPU step on the same workload, and the one-step
             grid-velocity error of the MIXED path against it;
  roofline   the fused G2P/P2G kernel's algorithmic bytes / measured kernel time
             against the measured HBM copy bandwidth;
  cpu_baseline  the CPU oracle (FP64 restatement of the reference, OpenMP
             over the host cores) on a bounded sample of the same workload.

``--impl reference`` times the CPU oracle alone on the same workload (the
reference itself needs Eigen and RapidXML, which are not available, so its
own build cannot run).

The line also carries the batched serving loop (``serving``), the DEM column
and a 1,000,000-disk pile (``dem``), the hybrid column (``hybrid``) and the
column with the uGIMP basis (``ugimp``).
Multi-GPU runs are replicas: every rank steps its own copy of the scene.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s mixed vs FP64 GPU at stated error; batched p50/p99 latency"
UNIT = "particle-steps/s"
# Algorithmic bytes of one fused G2P/P2G launch, with the per-unit figures of
# the reference algorithm's two particle passes: P2G reads 48 B per point
# (position 16, velocity 8, mass 4, volume 4, J 4, be_bar 12) and writes 20 B
# per active node (mass, momentum, force); G2P reads 40 B and writes 40 B per
# point and reads 16 B per active node (velocity, acceleration). The fused
# kernel reads each point once, so it moves fewer bytes than this
# (FUSED_MIN_* below, and the ncu DRAM traffic in profiles/).
BYTES_PER_PARTICLE = 48 + 80
BYTES_PER_ACTIVE_NODE = 20 + 16
FUSED_MIN_BYTES_PER_PARTICLE = 90  # u 16+16, v 8+8, (m, V) 8, strain 16+16, flags 1+1
FUSED_MIN_BYTES_PER_ACTIVE_NODE = 36


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([s.strip() for s in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        sm = [float(s[1]) for s in self.samples if len(s) > 8 and s[1].replace(".", "").isdigit()]
        smax = [float(s[2]) for s in self.samples if len(s) > 8 and s[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            if len(s) > 8:
                for k, name in enumerate(names):
                    if s[5 + k].lower().startswith("active"):
                        reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def scene():
    from libhybridgrains_gb300 import scenes
    cfg = scenes.mpm_column("column_2M")
    pts = scenes.seed_column_points(cfg)
    return cfg, pts


def make_mpm(ctx, cfg, precision, n):
    import libhybridgrains_gb300 as hg
    from libhybridgrains_gb300 import scenes
    return hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
                  cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
                  cfg["planes"], precision=precision, capacity=n)


def cpu_oracle_rate(cfg, pts, steps, threads):
    """Oracle (FP64, OpenMP) particle-steps/s on `steps` steps of the scene."""
    import oracle
    from libhybridgrains_gb300 import scenes
    o = oracle.MPM(cfg["grid_min"], cfg["grid_max"], cfg["h"],
                   shear_modulus=cfg["shear_modulus"], bulk_modulus=cfg["bulk_modulus"],
                   dp_alpha=cfg["dp_alpha"], flip_alpha=cfg["flip_alpha"],
                   gravity=scenes.GRAVITY, threads=threads)
    for (x, n, st, lb) in cfg["planes"]:
        o.add_plane(x, n, st, lb)
    o.set_particles(pts["q"], pts["v"], pts["m"], pts["vol"], pts["hl"])
    o.step(cfg["dt"], 1)  # warm-up (allocates the per-thread grids)
    t0 = time.perf_counter()
    o.step(cfg["dt"], steps)
    dt = time.perf_counter() - t0
    return len(pts["m"]) * steps / dt, dt


def barrier_max(value, world):
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def init_dist(world):
    if world <= 1:
        return
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group("gloo")


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args, rank, world):
    """CPU oracle alone (the reference's own CPU path cannot be built here)."""
    if rank != 0:
        return
    cfg, pts = scene()
    threads = os.cpu_count() or 1
    # Each timed step is one full step of the workload; the number of timed
    # steps is capped so that the run stays within about a minute.
    _, one = cpu_oracle_rate(cfg, pts, 1, threads)
    steps = max(1, min(args.steps, int(60.0 / max(one, 1e-3))))
    rate, secs = cpu_oracle_rate(cfg, pts, steps, threads)
    line = {"metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": "column_2M: 2,000,000-point MPM granular column, 2048x1024 "
                                   "grid, h=1 mm, dt=2e-6 s", "particles": len(pts["m"])},
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d steps of the 2,000,000-point column (%.1f s)"
                                       % (steps, secs)},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local):
    import libhybridgrains_gb300 as hg
    from libhybridgrains_gb300 import build as gbuild
    from libhybridgrains_gb300 import scenes as hg_scenes
    gbuild.build()
    ctx = hg.Context(local)
    cfg, pts = scene()
    n = len(pts["m"])
    dt = cfg["dt"]

    # ---- resident MIXED step ------------------------------------------------
    mix = make_mpm(ctx, cfg, hg.MIXED, n)
    mix.upload(pts["q"], pts["v"], pts["m"], pts["vol"], pts["hl"])
    # launch shapes of the two kernels chosen on this scene (the tuning steps
    # count as warm-up)
    tune = mix.autotune(dt, args.tune_steps) if args.tune_steps > 0 else None
    mix.flow(dt, args.warmup)
    ctx.synchronize()
    barrier(world)
    launches0 = hg.kernel_launch_count()
    with ClockSampler(local) as clk:
        ctx.timer_begin()
        mix.flow(dt, args.steps)
        ms = ctx.timer_end()
    launches = hg.kernel_launch_count() - launches0
    barrier(world)
    ms = barrier_max(ms, world)
    value = n * args.steps * world / (ms * 1e-3)
    status = mix.status()
    G = mix.grid()
    n_active = int((G["mass"] > 0).sum())
    # Per-kernel durations for the roofline: the timed steps replay 16-step
    # CUDA graphs, which carry no events, so the column runs again from the
    # same start with CUDA events around each launch (each interval also holds
    # the gap to the neighbouring launch) over two fixed windows of a
    # 10,000-step run, whatever --steps is: steps 0-2,000 (the column at
    # rest) and 8,000-10,000 (flowing, more points on the plastic branch).
    mix.upload(pts["q"], pts["v"], pts["m"], pts["vol"], pts["hl"])
    windows = []
    for start, length in ((0, args.roofline_window), (args.roofline_span - args.roofline_window,
                                                      args.roofline_window)):
        done = sum(w["start"] + w["steps"] for w in windows[-1:])
        if start > done:
            mix.flow(dt, start - done)
        mix.profile(True)
        mix.flow(dt, length)
        f_ms, u_ms, k = mix.profile_read()
        mix.profile(False)
        windows.append({"start": start, "steps": k, "g2p2g_us": 1e3 * f_ms / max(k, 1),
                        "grid_update_us": 1e3 * u_ms / max(k, 1)})
    g2p2g_ms = sum(w["g2p2g_us"] * w["steps"] for w in windows) * 1e-3
    update_ms = sum(w["grid_update_us"] * w["steps"] for w in windows) * 1e-3
    prof_steps = sum(w["steps"] for w in windows)
    status |= mix.status()

    # ---- plain FP64 GPU step on the same workload ------------------------------
    fp64 = None
    if args.fp64_steps > 0:
        f64 = make_mpm(ctx, cfg, hg.FP64, n)
        f64.upload(pts["q"], pts["v"], pts["m"], pts["vol"], pts["hl"])
        f64.flow(dt, 3)
        fsteps = args.fp64_steps
        barrier(world)
        ctx.timer_begin()
        f64.flow(dt, fsteps)
        fms = ctx.timer_end()
        fp64_value = n * fsteps * world / (barrier_max(fms, world) * 1e-3)
        # one-step grid-velocity error of MIXED against FP64 from the same state
        st = f64.download()
        chk = make_mpm(ctx, cfg, hg.MIXED, n)
        chk.upload(st["q"], st["v"], pts["m"], pts["vol"], pts["hl"], st["be"], st["J"], st["jh"])
        chk.flow(dt, 1)
        f64.flow(dt, 1)
        Gm, Gf = chk.grid(), f64.grid()
        act = Gf["mass"] > 0
        vel_err = float(np.linalg.norm(Gm["vel"][act] - Gf["vel"][act]) /
                        max(np.linalg.norm(Gf["vel"][act]), 1e-300))
        fp64 = {"value": fp64_value, "unit": UNIT, "steps": fsteps,
                "ms_per_step": fms / fsteps, "speedup_mixed_over_fp64": value / fp64_value,
                "grid_velocity_rel_error": vel_err,
                "error_state": "after %d FP64 steps from rest" % (fsteps + 3)}
        del chk, f64

    # ---- the uGIMP basis (the reference's shipped scenes use it) --------------------
    ugimp = None
    if args.ugimp_steps >= 0:
        cu = dict(cfg, grid_min=(cfg["grid_min"][0] - 4 * cfg["h"],
                                 cfg["grid_min"][1] - 4 * cfg["h"]))
        rates = {}
        usteps = args.ugimp_steps if args.ugimp_steps > 0 else args.steps
        for name, prec, k in (("mixed", hg.MIXED, usteps), ("fp64", hg.FP64, 5)):
            mu_ = hg.MPM(ctx, cu["grid_min"], cu["grid_max"], cu["h"], cu["shear_modulus"],
                         cu["bulk_modulus"], cu["dp_alpha"], cu["flip_alpha"],
                         hg_scenes.GRAVITY,
                         cu["planes"], basis=hg.UGIMP, precision=prec, capacity=n)
            mu_.upload(pts["q"], pts["v"], pts["m"], pts["vol"], pts["hl"])
            utune = None
            if prec == hg.MIXED and args.tune_steps > 0:
                utune = mu_.autotune(dt, args.tune_steps)
            mu_.flow(dt, 3)
            ctx.synchronize()
            ctx.timer_begin()
            mu_.flow(dt, k)
            ums = ctx.timer_end()
            rates[name] = {"value": n * k / (ums * 1e-3), "ms_per_step": ums / k, "steps": k,
                           "status": mu_.status()}
            if prec == hg.MIXED:
                # the fused uGIMP kernel against the same per-unit bytes as
                # the linear one, event-timed over the next window of steps
                ua = int((mu_.grid()["mass"] > 0).sum())
                mu_.profile(True)
                mu_.flow(dt, args.roofline_window)
                f_ms, u_ms, kk = mu_.profile_read()
                mu_.profile(False)
                per = f_ms * 1e-3 / max(kk, 1)
                ub = n * BYTES_PER_PARTICLE + ua * BYTES_PER_ACTIVE_NODE
                rates[name].update(
                    launch_shape=utune, active_nodes=ua, status=mu_.status(),
                    of_linear_step_time=(ums / k) / (ms / args.steps),
                    roofline={"kernel": "kxu_step", "algorithmic_bytes": ub,
                              "kernel_ms": per * 1e3, "grid_update_ms": u_ms / max(kk, 1),
                              "achieved_gbs": ub / per / 1e9,
                              "timing": "CUDA events around each launch, %d steps after the "
                                        "timed ones" % kk})
            mu_.close()
        ugimp = {"workload": "column_2M with the uGIMP basis (half-width h/4), grid extended by "
                             "4 cells below and left", **rates,
                 "speedup_mixed_over_fp64": rates["mixed"]["value"] / rates["fp64"]["value"]}

    # ---- end to end through the C ABI with host buffers --------------------------
    e2e = None
    if args.e2e_steps > 0:
        import torch
        host = {k: torch.empty(v.shape, dtype=torch.float64, pin_memory=True).numpy()
                for k, v in (("q", pts["q"]), ("v", pts["v"]), ("m", pts["m"]),
                             ("vol", pts["vol"]))}
        for k in ("q", "v", "m", "vol"):
            host[k][...] = pts[k]
        host["be"] = torch.empty((n, 4), dtype=torch.float64, pin_memory=True).numpy()
        host["be"][...] = [1.0, 0.0, 0.0, 1.0]
        host["J"] = torch.ones(n, dtype=torch.float64, pin_memory=True).numpy()
        host["jh"] = torch.zeros(n, dtype=torch.int32, pin_memory=True).numpy()
        e2 = make_mpm(ctx, cfg, hg.MIXED, n)

        def one():
            e2.upload(host["q"], host["v"], host["m"], host["vol"], None, host["be"], host["J"],
                      host["jh"])
            e2.flow(dt, 1)
            e2.download_into(host["q"], host["v"], host["be"], host["J"], host["jh"])

        one()
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            one()
        e2e_s = barrier_max(time.perf_counter() - t0, world)
        h2d = n * (16 + 16 + 8 + 8 + 32 + 8 + 4)
        d2h = n * (16 + 16 + 32 + 8 + 4)
        e2e = {"value": n * args.e2e_steps * world / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "steps": args.e2e_steps, "ms_per_step": 1e3 * e2e_s / args.e2e_steps}
        del e2

    batch = None
    if args.batch_steps > 0 and args.batch_scenes > 0:
        batch = run_batch(args, ctx, value / world, world)
    serve = None
    if args.serve_requests > 0:
        serve = run_serving(args, ctx, rank, world)
    dem = None
    if args.dem_steps > 0:
        dem = run_dem(args, ctx)
    hyb = None
    if args.hybrid_steps > 0:
        hyb = run_hybrid(args, ctx)
    c0 = None
    if args.c0_steps > 0 and world == 1:
        c0 = run_column_12800(args, ctx)

    if rank != 0:
        return
    peaks = measured_peaks()
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    alg_bytes = n * BYTES_PER_PARTICLE + n_active * BYTES_PER_ACTIVE_NODE
    per_launch_s = (g2p2g_ms * 1e-3) / max(prof_steps, 1)
    achieved = alg_bytes / per_launch_s / 1e9
    traffic = ncu_dram_pct = None  # from the committed ncu summary of this kernel
    tpath = os.path.join(ROOT, "profiles", "kx_g2p2g_column_2M.md")
    if os.path.exists(tpath):
        import re
        with open(tpath) as f:
            text = f.read()
        mt = re.search(r"traffic_bytes_per_launch = (\d+)", text)
        if mt:
            traffic = int(mt.group(1))
        mt = re.search(r"dram_throughput_pct = ([0-9.]+)", text)
        if mt:
            ncu_dram_pct = float(mt.group(1))
    fused_min = n * FUSED_MIN_BYTES_PER_PARTICLE + n_active * FUSED_MIN_BYTES_PER_ACTIVE_NODE

    cpu = None
    if world == 1 and args.cpu_steps > 0:
        threads = os.cpu_count() or 1
        rate, secs = cpu_oracle_rate(cfg, pts, args.cpu_steps, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "%d steps of the 2,000,000-point column (%.1f s)" % (args.cpu_steps, secs)}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 positions)",
        "data": "synthetic",
        "config": {"workload": "column_2M: 2,000,000-point MPM granular column, 2048x1024 grid, "
                               "h=1 mm, dt=2e-6 s, linear basis, mixed precision",
                   "particles": n, "grid_cells": [2048, 1024], "active_nodes": n_active,
                   "l2": "inputs larger than L2 (particle state 180 MB per step)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "launch_shape": tune},
        "fp64": fp64,
        "ugimp": ugimp,
        "roofline": {"bound": "hbm", "kernel": "kx_g2p2g", "achieved": achieved, "peak": peak,
                     "peak_source": peak_src, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "algorithmic_bytes": alg_bytes,
                     "fused_min_bytes": fused_min,
                     "frac_fused_min": fused_min / per_launch_s / 1e9 / peak,
                     "ncu_dram_throughput_pct": ncu_dram_pct,
                     "kernel_ms": per_launch_s * 1e3,
                     "grid_update_ms": update_ms / max(prof_steps, 1),
                     "windows": windows,
                     "timing": "CUDA events around each launch, steps 0-%d and %d-%d of a "
                               "%d-step run from rest (the mean of both windows)"
                               % (args.roofline_window,
                                  args.roofline_span - args.roofline_window,
                                  args.roofline_span, args.roofline_span)},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "batch": batch,
        "serving": serve,
        "dem": dem,
        "hybrid": hyb,
        "column_12800": c0,
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "status_word": status,
    }
    print(json.dumps(line), flush=True)


def run_dem(args, ctx):
    """DEM column (10,000 disks, hex pitch 2.2 mm, r U[0.9, 1.1] mm, seed
    12345, rho 2600, kn 1e5, mu 0.5, floor plane, dt 1e-6 s): disk-steps/s on
    the GPU (FP64, bit-exact with the oracle) and the oracle on one host core
    (the reference's penalty map is serial)."""
    import libhybridgrains_gb300 as hg
    import oracle
    from libhybridgrains_gb300 import scenes
    sc = scenes.dem_column()
    dp = scenes.dem_params()
    planes = [((0.0, 0.0), (0.0, 1.0))]
    n = len(sc["r"])
    d = hg.DEM(ctx, scenes.GRAVITY, dp["kn"], dp["kt"], dp["gamman"], dp["gammat"], dp["mu"],
               planes, capacity=n)
    d.upload(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"])
    dt = 1.0e-6
    d.flow(dt, 20)
    ctx.synchronize()
    l0 = hg.kernel_launch_count()
    ctx.timer_begin()
    d.flow(dt, args.dem_steps)
    ms = ctx.timer_end()
    launches = hg.kernel_launch_count() - l0
    contacts = d.num_contacts()
    o = oracle.DEM(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"], scenes.GRAVITY,
                   dp["kn"], dp["kt"], dp["gamman"], dp["gammat"], dp["mu"], 1.0)
    for (x, nn) in planes:
        o.add_plane(x, nn)
    o.step(dt, 1)
    t0 = time.perf_counter()
    csteps = max(1, args.dem_cpu_steps)
    o.step(dt, csteps)
    cs = time.perf_counter() - t0
    gpu_rate = n * args.dem_steps / (ms * 1e-3)
    # per disk-step 128 B, per contact 40 B (FP64 figures of the scope table)
    alg = n * 128 + contacts * 40
    # the HG_PRECISION_MIXED step on the same column (FP32 contact law)
    dm = hg.DEM(ctx, scenes.GRAVITY, dp["kn"], dp["kt"], dp["gamman"], dp["gammat"], dp["mu"],
                planes, capacity=n, precision=hg.MIXED)
    dm.upload(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"])
    dm.flow(dt, 20)
    ctx.synchronize()
    ctx.timer_begin()
    dm.flow(dt, args.dem_steps)
    msm = ctx.timer_end()
    mixed = {"disk_steps_per_s": n * args.dem_steps / (msm * 1e-3),
             "us_per_step": 1e3 * msm / args.dem_steps}
    dm.close()
    large = None
    if args.dem_large_disks > 0:
        # the same lattice at a size where the step is no longer launch-bound
        nl = args.dem_large_disks
        sl = scenes.dem_column(n=nl, per_row=1000)
        large = {"workload": "%d disks, the same lattice 1000 per row, dt 1e-5 s" % nl,
                 "steps": args.dem_large_steps}
        for name, prec in (("fp64", hg.FP64), ("mixed", hg.MIXED)):
            dl = hg.DEM(ctx, scenes.GRAVITY, dp["kn"], dp["kt"], dp["gamman"], dp["gammat"],
                        dp["mu"], planes, capacity=nl, contact_capacity=4 * nl, precision=prec)
            dl.upload(sl["q"], sl["v"], sl["r"], sl["m"], sl["I"], sl["fixed"])
            dl.flow(1.0e-5, 200)
            ctx.synchronize()
            ctx.timer_begin()
            dl.flow(1.0e-5, args.dem_large_steps)
            msl = ctx.timer_end()
            ncl = dl.num_contacts()
            # algorithmic bytes per step: FP64 128 B per disk + 40 per contact,
            # mixed 88 + 24 (the scope table's per-unit figures)
            per_disk, per_contact = (128, 40) if prec == hg.FP64 else (88, 24)
            algl = nl * per_disk + ncl * per_contact
            achl = algl / (msl * 1e-3 / args.dem_large_steps) / 1e9
            peak = measured_peaks().get("hbm_gbs") or 6800.0
            large[name] = {"disk_steps_per_s": nl * args.dem_large_steps / (msl * 1e-3),
                           "us_per_step": 1e3 * msl / args.dem_large_steps,
                           "contacts": ncl, "status": dl.status(),
                           "algorithmic_bytes_per_step": algl, "achieved_gbs": achl,
                           "hbm_frac": achl / peak}
            dl.close()
    dense = run_dem_dense(args, ctx) if args.dem_dense_steps > 0 else None
    return {"workload": "DEM column: 10,000 disks, hex pitch 2.2 mm, r U[0.9,1.1] mm, dt 1e-6 s, "
                        "FP64 penalty contacts with friction history",
            "dense": dense,
            "disk_steps_per_s": gpu_rate, "us_per_step": 1e3 * ms / args.dem_steps,
            "steps": args.dem_steps, "contacts": contacts,
            "launches_per_step": launches / args.dem_steps,
            "algorithmic_bytes_per_step": alg,
            "achieved_gbs": alg / (ms * 1e-3 / args.dem_steps) / 1e9,
            "cpu_baseline": {"value": n * csteps / cs, "unit": "disk-steps/s", "cores": 1,
                             "kind": "port", "sample": "%d steps of the same column (%.1f s)" %
                             (csteps, cs)},
            "mixed": mixed, "large": large}


def run_dem_dense(args, ctx):
    """The DEM column's disks compacted to a 1.9 mm hex pitch between a floor
    and two walls (scenes.dem_packed: about 2.8 contacts per disk, so the
    contact law carries the load), at 10,000 and 1,000,000 disks, FP64
    (bit-exact with the oracle) and mixed precision; disk-steps/s, contacts
    per disk and algorithmic bandwidth against the measured HBM copy rate.
    The oracle times the 10,000-disk case on one host core (the reference's
    penalty map is serial)."""
    import libhybridgrains_gb300 as hg
    import oracle
    from libhybridgrains_gb300 import scenes
    dp = scenes.dem_params()
    peak = measured_peaks().get("hbm_gbs") or 6800.0
    dt = 1.0e-6
    out = {"workload": "disks of the DEM column on a 1.9 mm hex pitch (r U[0.9,1.1] mm, seed "
                       "12345) between a floor and two walls, dt 1e-6 s, 200 settling steps "
                       "before timing"}
    for label, n, per_row, steps in (("10k", 10000, 100, args.dem_dense_steps),
                                     ("1M", 1000000, 1000, args.dem_dense_large_steps)):
        if steps <= 0:
            continue
        sc = scenes.dem_packed(n=n, per_row=per_row)
        case = {"disks": n, "steps": steps}
        for name, prec in (("fp64", hg.FP64), ("mixed", hg.MIXED)):
            d = hg.DEM(ctx, scenes.GRAVITY, dp["kn"], dp["kt"], dp["gamman"], dp["gammat"],
                       dp["mu"], sc["planes"], capacity=n, contact_capacity=4 * n,
                       precision=prec)
            d.upload(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"])
            d.flow(dt, 200)
            ctx.synchronize()
            l0 = hg.kernel_launch_count()
            ctx.timer_begin()
            d.flow(dt, steps)
            ms = ctx.timer_end()
            launches = hg.kernel_launch_count() - l0
            nc = d.num_contacts()
            per_disk, per_contact = (128, 40) if prec == hg.FP64 else (88, 24)
            alg = n * per_disk + nc * per_contact
            ach = alg / (ms * 1e-3 / steps) / 1e9
            case[name] = {"disk_steps_per_s": n * steps / (ms * 1e-3),
                          "us_per_step": 1e3 * ms / steps, "contacts": nc,
                          "contacts_per_disk": nc / n, "launches_per_step": launches / steps,
                          "algorithmic_bytes_per_step": alg, "achieved_gbs": ach,
                          "hbm_frac": ach / peak, "status": d.status()}
            d.close()
        if label == "10k" and args.dem_cpu_steps > 0:
            o = oracle.DEM(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"],
                           scenes.GRAVITY, dp["kn"], dp["kt"], dp["gamman"], dp["gammat"],
                           dp["mu"], 1.0)
            for (x, nn) in sc["planes"]:
                o.add_plane(x, nn)
            o.step(dt, 1)
            csteps = max(1, args.dem_cpu_steps)
            t0 = time.perf_counter()
            o.step(dt, csteps)
            cs = time.perf_counter() - t0
            case["cpu_baseline"] = {"value": n * csteps / cs, "unit": "disk-steps/s",
                                    "cores": 1, "kind": "port",
                                    "sample": "%d steps of the same packing (%.1f s)"
                                              % (csteps, cs)}
        out[label] = case
    return out


def run_hybrid(args, ctx):
    """Hybrid column (100,000 material points under 20,000 disks, uGIMP,
    node-node coupling, resampling every 200 steps on the host): steps/s of
    the whole loop, with the share of the host resampling, with the MPM bulk
    in FP64 (the reference's arithmetic) and in mixed precision (FP32 bulk,
    FP64 positions)."""
    import libhybridgrains_gb300 as hg
    from libhybridgrains_gb300 import hybrid, scenes

    def run(precision):
        sim = hybrid.HybridSim(ctx, scenes.hybrid_column(), precision=precision)
        sim.step(1)  # initial resampling and one step
        ctx.synchronize()
        t0 = time.perf_counter()
        rs0 = sim.resamplings
        host = [0.0]
        orig = sim._resample

        def timed():
            ctx.synchronize()
            t = time.perf_counter()
            orig()
            host[0] += time.perf_counter() - t
        sim._resample = timed
        phases0 = dict(sim.host_s)
        st0 = len(sim.stats)
        sim.step(args.hybrid_steps)
        ctx.synchronize()
        wall = time.perf_counter() - t0
        n, nd = sim.counts()
        phases = {k: sim.host_s[k] - phases0[k] for k in phases0}
        # inside the resampling proper, summed over the timed intervals
        inner = {k: sum(x[k] for x in sim.stats[st0:]) for k in
                 ("ms_insert_grains", "ms_insert_points", "ms_point_grids", "ms_quantities",
                  "ms_delete", "points_inserted", "grains_inserted", "points_deleted",
                  "grains_deleted")}
        out = {"steps": args.hybrid_steps, "steps_per_s": args.hybrid_steps / wall,
               "ms_per_step": 1e3 * wall / args.hybrid_steps,
               "resamplings": sim.resamplings - rs0, "resampling_host_s": host[0],
               "resampling_host_s_by_phase": phases,
               "resampler_by_phase": inner,
               "resampling_share": host[0] / wall,
               "device_ms_per_step": 1e3 * (wall - host[0]) / args.hybrid_steps,
               "points": n, "disks": nd, "status": [sim.mpm.status(), sim.dem.status()]}
        return out

    fp64 = run(hg.FP64)
    mixed = run(hg.MIXED)
    cpu = None
    if args.hybrid_cpu_steps > 0:
        cpu = hybrid_cpu_baseline(args.hybrid_cpu_steps)
    return dict(fp64, workload="hybrid column: 100,000 MPM points (h 2.5 mm, uGIMP) under "
                               "20,000 disks, node-node coupling, homogenised stress and "
                               "velocity, resampling every 200 steps, dt 1e-6 s; top level: "
                               "FP64 MPM bulk", mixed=mixed, cpu_baseline=cpu)


def hybrid_cpu_baseline(steps):
    """The oracle's node-node step (HybridGrains2DSim.cpp:116-220 restated in
    FP64: MPM with OpenMP over the host cores, the penalty map serial as in
    the reference) on the hybrid column's scene before its first resampling,
    with the coupling band's grains weighted 1/2. The resampling interval is
    host code on both sides (this library's is a restatement of the
    reference's), so the baseline times the device-side step only."""
    import oracle
    from libhybridgrains_gb300 import scenes
    scene = scenes.hybrid_column()
    cfg, sc, dp = scene["mpm"], scene["dem"], scene["dem_params"]
    p = scenes.seed_column_points(cfg)
    threads = os.cpu_count() or 1
    cm = oracle.MPM(cfg["grid_min"], cfg["grid_max"], cfg["h"], basis=1,
                    shear_modulus=cfg["shear_modulus"], bulk_modulus=cfg["bulk_modulus"],
                    dp_alpha=cfg["dp_alpha"], flip_alpha=cfg["flip_alpha"],
                    gravity=scenes.GRAVITY, threads=threads)
    for (x, n, st, lb) in cfg["planes"]:
        cm.add_plane(x, n, st, lb)
    cm.set_particles(p["q"], p["v"], p["m"], p["vol"], p["hl"])
    cd = oracle.DEM(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"], scenes.GRAVITY,
                    dp["kn"], dp["kt"], dp["gamman"], dp["gammat"], dp["mu"], 1.0)
    for (x, n, _st, _lb) in cfg["planes"]:
        cd.add_plane(x, n)
    cd.set_weights(np.where(sc["q"][:, 1] < cfg["rect_max"][1], 0.5, 1.0))
    ch = oracle.Hybrid(cm, cd)
    ch.step(cfg["dt"], 1, homogenize_stress=True, homogenize_velocity=True)
    t0 = time.perf_counter()
    ch.step(cfg["dt"], steps, homogenize_stress=True, homogenize_velocity=True)
    secs = time.perf_counter() - t0
    return {"value": steps / secs, "unit": "hybrid steps/s", "cores": threads, "kind": "port",
            "sample": "%d node-node steps of the hybrid column, 100,000 points and 20,000 "
                      "disks, before resampling (%.1f s)" % (steps, secs)}


def run_column_12800(args, ctx):
    """The 12,800-point MPM column (1.0 x 0.5 m domain, h = 5 mm, dt 1e-5 s)
    on the GPU in mixed precision and FP64, and the oracle (FP64, OpenMP over
    the host cores) on a sample of the same steps: particle-steps/s each."""
    import libhybridgrains_gb300 as hg
    import oracle
    from libhybridgrains_gb300 import scenes
    cfg = scenes.mpm_column("column_12800")
    pts = scenes.seed_column_points(cfg)
    n = len(pts["m"])
    out = {"workload": "column_12800: 12,800-point MPM granular column, 200x100 grid, h=5 mm, "
                       "dt=1e-5 s, sticking floor and walls", "particles": n,
           "steps": args.c0_steps}
    for name, prec in (("mixed", hg.MIXED), ("fp64", hg.FP64)):
        m = make_mpm(ctx, cfg, prec, n)
        m.upload(pts["q"], pts["v"], pts["m"], pts["vol"], pts["hl"])
        m.flow(cfg["dt"], 20)
        ctx.synchronize()
        ctx.timer_begin()
        m.flow(cfg["dt"], args.c0_steps)
        ms = ctx.timer_end()
        out[name] = {"value": n * args.c0_steps / (ms * 1e-3), "unit": UNIT,
                     "ms_per_step": ms / args.c0_steps, "status": m.status()}
        m.close()
    threads = os.cpu_count() or 1
    rate, secs = cpu_oracle_rate(cfg, pts, args.c0_cpu_steps, threads)
    out["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                           "sample": "%d steps of the same column (%.1f s)"
                                     % (args.c0_cpu_steps, secs)}
    return out


def gather_parts(part, world):
    """Every rank's summary_parts (one object per rank)."""
    if world <= 1:
        return [part]
    import torch.distributed as dist
    out = [None] * world
    dist.all_gather_object(out, part)
    return out


def run_batch(args, ctx, single_rate, world=1):
    """The requests of the serving section (seed 2024) as MIXED scenes all
    resident in one batch: whole steps timed with CUDA events over
    --batch-steps steps (16-step graph chunks), the per-phase split from the
    profiled per-step path, and the same scenes stepped one at a time through
    their own graphs. The point-step rate is compared with the 2M column's
    (single_rate, this run's headline value per GPU)."""
    import libhybridgrains_gb300 as hg
    from libhybridgrains_gb300 import scenes as hg_scenes
    from libhybridgrains_gb300 import serving
    reqs = serving.column_requests(n=args.batch_scenes, rate=args.serve_rate,
                                   steps=args.serve_steps, seed=2024)
    b = hg.Batch(ctx, max_members=len(reqs))
    members = []
    for r in reqs:
        c = r.cfg
        m = hg.MPM(ctx, c["grid_min"], c["grid_max"], c["h"], c["shear_modulus"],
                   c["bulk_modulus"], c["dp_alpha"], c["flip_alpha"], hg_scenes.GRAVITY,
                   c["planes"], capacity=r.npoints)
        m.seed_rectangle_device(c["rect_min"], c["rect_max"], c["rho"], c["samples_per_dim"])
        b.add(m, r.dt)
        members.append((m, r.dt))
    npts = sum(r.npoints for r in reqs)
    tune = b.autotune(args.tune_steps) if args.tune_steps > 0 else None
    b.step(max(args.warmup, 16))
    ctx.synchronize()
    barrier(world)
    ctx.timer_begin()
    b.step(args.batch_steps)
    ms = barrier_max(ctx.timer_end(), world)
    b.profile(True)
    b.step(32)
    prof = b.profile_read()
    b.profile(False)
    status = max(m.status() for m, _ in members)
    b.close()
    # the same scenes one at a time, each through its own step graphs
    for m, dt in members:
        m.flow(dt, 16)
    ctx.synchronize()
    alone_ms = 0.0
    for m, dt in members:
        ctx.timer_begin()
        m.flow(dt, args.batch_alone_steps)
        alone_ms += ctx.timer_end()
    for m, _ in members:
        m.close()
    rate = npts * args.batch_steps / (ms * 1e-3)
    steps = max(prof["steps"], 1)
    return {
        "workload": "the %d serving requests (seed 2024; points log-U[2e3,2e5], aspect "
                    "U[0.5,4]) as MIXED scenes, all resident in one batch" % len(reqs),
        "scenes": len(reqs), "points": npts, "steps": args.batch_steps,
        "ms_per_step": ms / args.batch_steps,
        "particle_steps_per_s": rate,
        "of_single_scene_rate": rate / single_rate,
        "single_scene_rate": single_rate,
        "per_step_profile_ms": {"fused": prof["fused_ms"] / steps,
                                "update": prof["update_ms"] / steps,
                                "resort": prof["resort_ms"] / steps,
                                "table": prof["table_ms"] / steps},
        "one_at_a_time": {"steps": args.batch_alone_steps,
                          "particle_steps_per_s": npts * args.batch_alone_steps
                          / (alone_ms * 1e-3)},
        "launch_shape": tune,
        "status": int(status),
    }


def run_serving(args, ctx, rank=0, world=1):
    """Batched serving of column-collapse requests: Poisson arrivals with
    continuous batching (latency), the same requests all queued at once
    (saturated throughput) and served one scene at a time (baseline). With
    several ranks each serves its share of the requests on its own GPU
    (serving.shard_requests) and the figures cover all of them."""
    from libhybridgrains_gb300 import serving

    def copies(reqs, at_once=False):
        return [r.copy(0.0 if at_once else None) for r in reqs]

    budget = int(args.serve_budget_gb * 2**30)
    all_reqs = serving.column_requests(n=args.serve_requests, rate=args.serve_rate,
                                       steps=args.serve_steps, seed=2024)
    reqs = serving.shard_requests(all_reqs, rank, world)
    be = serving.DeviceBackend(ctx, max_members=min(256, args.serve_requests))
    # warm-up: a few short requests (library load, pools)
    serving.Server(be, budget).run(copies(serving.column_requests(n=8, rate=1e3, steps=200,
                                                                   seed=7)))
    launches0 = __import__("libhybridgrains_gb300").kernel_launch_count()
    barrier(world)
    srv = serving.Server(be, budget, max_members=min(256, args.serve_requests))
    live = srv.run(copies(reqs))
    poisson = serving.summary_of_parts(gather_parts(serving.summary_parts(live, srv.makespan),
                                                    world))
    launches = __import__("libhybridgrains_gb300").kernel_launch_count() - launches0
    barrier(world)
    srv2 = serving.Server(be, budget, max_members=min(256, args.serve_requests))
    sat_reqs = srv2.run(copies(reqs, at_once=True))
    saturated = serving.summary_of_parts(
        gather_parts(serving.summary_parts(sat_reqs, srv2.makespan), world))
    be.shutdown()
    alone = copies(reqs)
    barrier(world)
    alone_s = barrier_max(serving.run_one_at_a_time(ctx, alone), world)
    cpu = serving_cpu_baseline(all_reqs, args) if (args.serve_cpu_requests > 0 and rank == 0) \
        else None
    psteps = float(sum(r.npoints * r.steps for r in all_reqs))
    dsteps = float(sum(r.ndisks * r.steps for r in all_reqs))
    diff = barrier_max(max((serving.frame_diff(a[1], b[1])
                            for r1, r2 in zip(live, alone) for a, b in zip(r1.frames, r2.frames)),
                           default=0.0), world)
    return {
        "workload": "%d column-collapse requests, Poisson arrivals %.0f/s (seed 2024), points "
                    "log-U[2e3,2e5], aspect U[0.5,4], friction angle U[20,40] deg, a DEM pile "
                    "of U[0,0.2] x the point count in disks, %d steps, a frame (positions) "
                    "every 100 steps" % (len(all_reqs), args.serve_rate, args.serve_steps),
        "ranks": world,
        "disks": int(sum(r.ndisks for r in all_reqs)),
        "p50_latency_s": poisson["p50_latency_s"], "p99_latency_s": poisson["p99_latency_s"],
        "max_latency_s": poisson["max_latency_s"],
        "p99_admission_wait_s": poisson["p99_admission_wait_s"],
        "makespan_s": poisson["makespan_s"],
        "particle_steps_per_s": poisson["particle_steps_per_s"],
        "disk_steps_per_s": poisson["disk_steps_per_s"],
        "peak_members": srv.peak_members, "peak_resident_bytes": srv.peak_resident,
        "hbm_budget_bytes": budget, "gpu_launches": launches,
        "saturated": {"particle_steps_per_s": saturated["particle_steps_per_s"],
                      "disk_steps_per_s": saturated["disk_steps_per_s"],
                      "requests_per_s": saturated["requests_per_s"],
                      "p50_latency_s": saturated["p50_latency_s"],
                      "p99_latency_s": saturated["p99_latency_s"],
                      "makespan_s": saturated["makespan_s"]},
        "one_at_a_time": {"particle_steps_per_s": psteps / alone_s,
                          "disk_steps_per_s": dsteps / alone_s,
                          "requests_per_s": len(all_reqs) / alone_s, "seconds": alone_s},
        "batched_over_one_at_a_time": saturated["particle_steps_per_s"] * alone_s / psteps,
        "dem_precision": "mixed (FP32 contact law, FP64 positions and pair differences)",
        "cpu_baseline": cpu,
        "max_frame_front_diff_m": diff,
    }


def serving_cpu_baseline(reqs, args):
    """The serving mix run one scene at a time on the CPU: the oracle (FP64;
    the column with OpenMP over the host cores, its DEM pile serially, as the
    reference runs them) steps each of the first few requests in arrival order
    for a sample of its steps; a request's time is scaled to its full step
    count. Reports requests/s and particle-steps/s of that sequential serving."""
    import oracle
    from libhybridgrains_gb300 import scenes, serving
    threads = os.cpu_count() or 1
    sample = sorted(reqs, key=lambda r: r.arrival)[:args.serve_cpu_requests]
    total_s = 0.0
    psteps = 0.0
    for r in sample:
        c = r.cfg
        pts = scenes.seed_column_points(c)
        o = oracle.MPM(c["grid_min"], c["grid_max"], c["h"], shear_modulus=c["shear_modulus"],
                       bulk_modulus=c["bulk_modulus"], dp_alpha=c["dp_alpha"],
                       flip_alpha=c["flip_alpha"], gravity=scenes.GRAVITY, threads=threads)
        for (x, n, st, lb) in c["planes"]:
            o.add_plane(x, n, st, lb)
        o.set_particles(pts["q"], pts["v"], pts["m"], pts["vol"], pts["hl"])
        od = None
        if r.ndisks > 0:
            pl = serving.dem_pile(r, 0)
            dp = scenes.dem_params()
            od = oracle.DEM(pl["q"], pl["v"], pl["r"], pl["m"], pl["I"], pl["fixed"],
                            scenes.GRAVITY, dp["kn"], dp["kt"], dp["gamman"], dp["gammat"],
                            dp["mu"], 1.0)
            od.add_plane((0.0, 0.0), (0.0, 1.0))
        k = min(args.serve_cpu_steps, r.steps)
        t0 = time.perf_counter()
        o.step(r.dt, k)
        if od is not None:
            od.step(r.dt, k)
        total_s += (time.perf_counter() - t0) * r.steps / k
        psteps += float(r.npoints) * r.steps
    return {"value": len(sample) / total_s, "unit": "requests/s", "cores": threads,
            "kind": "port", "particle_steps_per_s": psteps / total_s,
            "sample": "the first %d requests in arrival order, %d of their steps each, scaled "
                      "to their 2,000 steps (%.1f s of CPU work)"
                      % (len(sample), args.serve_cpu_steps,
                         total_s * args.serve_cpu_steps / 2000.0)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-steps", type=int, default=10)
    ap.add_argument("--fp64-steps", type=int, default=10)
    ap.add_argument("--dem-steps", type=int, default=2000)
    ap.add_argument("--hybrid-steps", type=int, default=1000)
    ap.add_argument("--hybrid-cpu-steps", type=int, default=20)
    ap.add_argument("--c0-steps", type=int, default=1000)
    ap.add_argument("--c0-cpu-steps", type=int, default=200)
    ap.add_argument("--serve-cpu-requests", type=int, default=4)
    ap.add_argument("--serve-cpu-steps", type=int, default=100)
    ap.add_argument("--dem-cpu-steps", type=int, default=200)
    ap.add_argument("--tune-steps", type=int, default=20)
    ap.add_argument("--roofline-span", type=int, default=10000)
    ap.add_argument("--roofline-window", type=int, default=2000)
    ap.add_argument("--ugimp-steps", type=int, default=0,
                    help="steps of the uGIMP column (0: as many as --steps, <0: skip)")
    ap.add_argument("--dem-large-disks", type=int, default=1000000)
    ap.add_argument("--dem-large-steps", type=int, default=200)
    ap.add_argument("--dem-dense-steps", type=int, default=2000)
    ap.add_argument("--dem-dense-large-steps", type=int, default=200)
    ap.add_argument("--batch-scenes", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=400)
    ap.add_argument("--batch-alone-steps", type=int, default=64)
    ap.add_argument("--serve-requests", type=int, default=256)
    ap.add_argument("--serve-rate", type=float, default=50.0)
    ap.add_argument("--serve-steps", type=int, default=2000)
    ap.add_argument("--serve-budget-gb", type=float, default=64.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()
    init_dist(world)
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
