"""Small fixed workloads for kernel profilers (ncu launch lists and captures).

    python -m libhybridgrains_gb300.profile_cases dem --disks 1000000 --steps 12
    python -m libhybridgrains_gb300.profile_cases dem --disks 10000 --per-row 100 --steps 12
    python -m libhybridgrains_gb300.profile_cases dem --disks 1000000 --packed --steps 12 \
        [--precision mixed]
    python -m libhybridgrains_gb300.profile_cases hybrid --steps 6 [--precision mixed]
    python -m libhybridgrains_gb300.profile_cases column --steps 8 [--basis ugimp]
    python -m libhybridgrains_gb300.profile_cases batch --scenes 256 --steps 8
    python -m libhybridgrains_gb300.profile_cases e2e --steps 8

Each case builds its scene, runs one warm-up step, then ``--steps`` steps one
call per step (so that every kernel is a separate launch a profiler can
select), synchronises and prints the wall time per step and the status words.
The DEM case is the DEM column's lattice (1000 disks per row unless
--per-row says otherwise; dt 1e-5 s), or with --packed the same disks
compacted to a 1.9 mm pitch between a floor and two walls (about 2.5
contacts per disk; dt 1e-6 s);
the hybrid case is the hybrid column (100,000 points under 20,000 disks)
after its initial resampling; the column case is the 2,000,000-point MIXED
column (with --basis ugimp on a grid 4 cells wider below and left, as the
bench runs it); the batch case is the serving mix (the first --scenes requests of
seed 2024) as MIXED scenes in one batch; the e2e case is the bench's end-to-end
step on the 2,000,000-point column: the state in the reference's layouts in
page-locked host memory, uploaded, stepped once and downloaded again each
step.
"""
import argparse
import time


def main(argv=None):
    import libhybridgrains_gb300 as hg
    from libhybridgrains_gb300 import scenes, serving

    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["dem", "hybrid", "column", "batch", "e2e"])
    ap.add_argument("--scenes", type=int, default=256, help="batch: serving requests")
    ap.add_argument("--basis", choices=("linear", "ugimp"), default="linear",
                    help="column: the MPM basis")
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--disks", type=int, default=1000000)
    ap.add_argument("--per-row", type=int, default=1000, help="DEM lattice disks per row")
    ap.add_argument("--packed", action="store_true",
                    help="DEM: the compacted lattice (scenes.dem_packed)")
    ap.add_argument("--precision", choices=("fp64", "mixed"), default="fp64",
                    help="the hybrid case's MPM bulk; the packed DEM case's contact law")
    args = ap.parse_args(argv)
    ctx = hg.Context(0)
    if args.case == "dem":
        if args.packed:
            sc = scenes.dem_packed(n=args.disks, per_row=args.per_row)
            dp = scenes.dem_params()
            obj = hg.DEM(ctx, scenes.GRAVITY, dp["kn"], dp["kt"], dp["gamman"], dp["gammat"],
                         dp["mu"], sc["planes"], capacity=args.disks,
                         contact_capacity=4 * args.disks,
                         precision=hg.MIXED if args.precision == "mixed" else hg.FP64)
            ddt = 1.0e-6
        else:
            sc = scenes.dem_column(n=args.disks, per_row=args.per_row)
            obj = serving.dem_for_piles(ctx, args.disks)
            ddt = 1.0e-5
        obj.upload(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"])

        def step():
            obj.flow(ddt, 1)
        status = obj.status
    elif args.case == "hybrid":
        from libhybridgrains_gb300.hybrid import HybridSim
        sim = HybridSim(ctx, scenes.hybrid_column(),
                        precision=hg.MIXED if args.precision == "mixed" else hg.FP64)
        sim.step(1)

        def step():
            sim.hyb.step(sim.dt, 1, *sim.hom)

        def status():
            return sim.mpm.status(), sim.dem.status()
    elif args.case == "batch":
        reqs = serving.column_requests(n=args.scenes, seed=2024)
        obj = hg.Batch(ctx, max_members=len(reqs))
        members = []
        for r in reqs:
            c = r.cfg
            m = hg.MPM(ctx, c["grid_min"], c["grid_max"], c["h"], c["shear_modulus"],
                       c["bulk_modulus"], c["dp_alpha"], c["flip_alpha"], scenes.GRAVITY,
                       c["planes"], capacity=r.npoints)
            m.seed_rectangle_device(c["rect_min"], c["rect_max"], c["rho"], c["samples_per_dim"])
            obj.add(m, r.dt)
            members.append(m)

        def step():
            obj.step(1)

        def status():
            return max(m.status() for m in members)
    elif args.case == "e2e":
        import numpy as np
        cfg = scenes.mpm_column("column_2M")
        p = scenes.seed_column_points(cfg)
        n = len(p["m"])
        host = {k: hg.pinned(p[k].shape) for k in ("q", "v", "m", "vol")}
        for k in host:
            host[k][...] = p[k]
        host["be"] = hg.pinned((n, 4))
        host["be"][...] = [1.0, 0.0, 0.0, 1.0]
        host["J"] = hg.pinned(n)
        host["J"][...] = 1.0
        host["jh"] = hg.pinned(n, np.int32)
        host["jh"][...] = 0
        obj = hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
                     cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
                     cfg["planes"], precision=hg.MIXED, capacity=n)

        def step():
            obj.upload(host["q"], host["v"], host["m"], host["vol"], None, host["be"],
                       host["J"], host["jh"])
            obj.flow(cfg["dt"], 1)
            obj.download_into(host["q"], host["v"], host["be"], host["J"], host["jh"])
        status = obj.status
    else:
        cfg = scenes.mpm_column("column_2M")
        p = scenes.seed_column_points(cfg)
        basis = hg.LINEAR
        if args.basis == "ugimp":
            basis = hg.UGIMP
            cfg = dict(cfg, grid_min=(cfg["grid_min"][0] - 4 * cfg["h"],
                                      cfg["grid_min"][1] - 4 * cfg["h"]))
        obj = hg.MPM(ctx, cfg["grid_min"], cfg["grid_max"], cfg["h"], cfg["shear_modulus"],
                     cfg["bulk_modulus"], cfg["dp_alpha"], cfg["flip_alpha"], scenes.GRAVITY,
                     cfg["planes"], basis=basis, capacity=len(p["m"]))
        obj.upload(p["q"], p["v"], p["m"], p["vol"], p["hl"])

        def step():
            obj.flow(cfg["dt"], 1)
        status = obj.status
    step()
    ctx.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    ctx.synchronize()
    ms = 1e3 * (time.perf_counter() - t0) / max(args.steps, 1)
    print("%s: %d steps, %.3f ms/step (one call per step), status %s" %
          (args.case, args.steps, ms, status()))


if __name__ == "__main__":
    main()
