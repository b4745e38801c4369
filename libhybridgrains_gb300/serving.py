"""Serving loop: many column-collapse requests on one GPU, continuously batched.

No counterpart in the reference (its CLIs run one scene per process). A
request is a granular-column scene that runs ``steps`` MPM steps and returns
a frame every ``frame_every`` steps. The loop

* admits arrived requests first come, first served while their device
  footprint (``hg_mpm_estimate_bytes``) fits the budget and a batch slot is
  free; a request that does not fit waits at the head of the queue;
* creates each admitted scene on the device from its geometry (no host
  point data) and keeps it resident;
* steps all resident scenes together
  (``hg_batch_step``: one grid-update and one fused G2P/P2G launch per step);
* admits new requests at chunk boundaries (every ``frame_every`` steps), at
  most ``admit_per_chunk`` per chunk, so work that arrives while others run
  joins the running batch;
* queues each frame's copy to page-locked host memory and a fence behind the
  chunk, and hands frames over once the fence is done, keeping at most
  ``depth`` chunks queued on the device;
* records for each request its arrival, admission and completion times.

The scheduling is separate from the device (``Backend``) so that admission
and ordering can be tested without a GPU.
"""
import collections
import math
import time

import numpy as np

from . import scenes


class Request:
    __slots__ = ("rid", "arrival", "cfg", "npoints", "steps", "frame_every", "dt",
                 "admitted", "finished", "frames", "footprint", "issued")

    def __init__(self, rid, arrival, cfg, npoints, steps=2000, frame_every=100, dt=1.0e-5):
        self.rid = rid
        self.arrival = arrival
        self.cfg = cfg
        self.npoints = npoints
        self.steps = steps
        self.frame_every = frame_every
        self.dt = dt
        self.admitted = None
        self.finished = None
        self.frames = []  # per frame: (step, run-out x of the front)
        self.footprint = 0
        self.issued = 0   # frames queued on the device

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival


def column_requests(n=256, rate=50.0, seed=2024, steps=2000, frame_every=100,
                    nmin=2.0e3, nmax=2.0e5):
    """Seeded request stream: exponential inter-arrival gaps at ``rate``/s,
    aspect ratio U[0.5, 4], point count log-uniform in [nmin, nmax],
    friction angle U[20, 40] degrees."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=n)
    arrivals = np.cumsum(gaps) - gaps[0]
    out = []
    for i in range(n):
        aspect = rng.uniform(0.5, 4.0)
        npts = math.exp(rng.uniform(math.log(nmin), math.log(nmax)))
        phi = rng.uniform(20.0, 40.0)
        cfg = scenes.serving_column(npts, aspect, phi)
        npoints = len(scenes.seed_column_points(cfg)["m"])
        out.append(Request(i, float(arrivals[i]), cfg, npoints, steps, frame_every,
                           cfg["dt"]))
    return out


class Backend:
    """Device operations the loop needs (implemented by DeviceBackend)."""

    def footprint(self, req):
        raise NotImplementedError

    def open(self, req):  # create the scene and join the batch
        raise NotImplementedError

    def step(self, nsteps):
        raise NotImplementedError

    def frame(self, req, slot):  # queue a frame copy into slot
        raise NotImplementedError

    def leave(self, req):  # leave the batch (state stays until close)
        raise NotImplementedError

    def fence(self):
        raise NotImplementedError

    def fence_done(self, f):
        raise NotImplementedError

    def fence_wait(self, f):
        raise NotImplementedError

    def read_frame(self, req, slot):  # after the fence: the frame's summary
        raise NotImplementedError

    def close(self, req):  # release device state and host buffers
        raise NotImplementedError


class Server:
    def __init__(self, backend, budget_bytes, max_members=256, depth=3, admit_per_chunk=16,
                 clock=time.perf_counter, sleep=time.sleep):
        self.b = backend
        self.budget = int(budget_bytes)
        self.max_members = max_members
        self.depth = depth
        # scenes created per chunk: creation overlaps with the chunks queued
        # on the device instead of delaying the first one
        self.admit_per_chunk = admit_per_chunk
        self.clock = clock
        self.sleep = sleep
        self.resident = 0
        self.peak_resident = 0
        self.peak_members = 0
        self.chunks = 0

    def run(self, requests):
        """Serve ``requests`` (arrival times in seconds from the start);
        returns them with admission/completion times and frames filled in."""
        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        pending.reverse()  # pop() gives the earliest
        waiting = collections.deque()
        active = []        # admitted, still stepping
        inflight = collections.deque()  # (fence, [(req, frame_no, step)], finished reqs)
        closing = []       # (fence, req): left the batch, closed once fence done
        t0 = self.clock()
        for r in requests:
            r.footprint = self.b.footprint(r)
            if r.footprint > self.budget:
                raise ValueError(f"request {r.rid} needs {r.footprint} bytes, "
                                 f"over the budget of {self.budget}")
        chunk = None
        while pending or waiting or active or inflight:
            now = self.clock() - t0
            while pending and pending[-1].arrival <= now:
                waiting.append(pending.pop())
            # admission: FIFO, by footprint and free slots
            admitted = 0
            while waiting and len(active) < self.max_members and admitted < self.admit_per_chunk \
                    and self.resident + waiting[0].footprint <= self.budget:
                admitted += 1
                r = waiting.popleft()
                self.b.open(r)
                r.admitted = self.clock() - t0
                active.append(r)
                self.resident += r.footprint
            self.peak_resident = max(self.peak_resident, self.resident)
            self.peak_members = max(self.peak_members, len(active))
            if active:
                fe = active[0].frame_every
                if chunk is None:
                    chunk = fe
                # keep at most depth chunks queued on the device
                while len(inflight) >= self.depth:
                    self._retire(inflight.popleft(), t0, closing, wait=True)
                self.b.step(chunk)
                self.chunks += 1
                frames, done = [], []
                for r in active:
                    k = r.issued
                    r.issued += 1
                    step = (k + 1) * chunk
                    self.b.frame(r, k % (self.depth + 1))
                    frames.append((r, k, step))
                    if step >= r.steps:
                        done.append(r)
                for r in done:
                    active.remove(r)
                    self.b.leave(r)
                f = self.b.fence()
                inflight.append((f, frames, done))
            # hand over every chunk the device has finished
            while inflight and (self.b.fence_done(inflight[0][0]) or not active):
                self._retire(inflight.popleft(), t0, closing, wait=True)
            self._close_finished(closing)
            if not active and not inflight and not waiting and pending:
                gap = pending[-1].arrival - (self.clock() - t0)
                if gap > 0:
                    self.sleep(gap)
        for f, r in closing:
            self.b.fence_wait(f)
            self.b.close(r)
        self.makespan = self.clock() - t0
        return requests

    def _retire(self, item, t0, closing, wait):
        f, frames, done = item
        if wait:
            self.b.fence_wait(f)
        for (r, k, step) in frames:
            r.frames.append((step, self.b.read_frame(r, k % (self.depth + 1))))
        now = self.clock() - t0
        for r in done:
            r.finished = now
            self.resident -= r.footprint
            closing.append((f, r))

    def _close_finished(self, closing):
        keep = []
        for f, r in closing:
            if self.b.fence_done(f):
                self.b.close(r)
            else:
                keep.append((f, r))
        closing[:] = keep


def summary(requests, makespan):
    lat = np.array([r.latency for r in requests])
    wait = np.array([r.admitted - r.arrival for r in requests])
    psteps = float(sum(r.npoints * r.steps for r in requests))
    return dict(requests=len(requests), p50_latency_s=float(np.percentile(lat, 50)),
                p99_latency_s=float(np.percentile(lat, 99)),
                max_latency_s=float(lat.max()),
                p50_admission_wait_s=float(np.percentile(wait, 50)),
                p99_admission_wait_s=float(np.percentile(wait, 99)),
                makespan_s=makespan, particle_steps=psteps,
                particle_steps_per_s=psteps / makespan,
                requests_per_s=len(requests) / makespan)


class DeviceBackend(Backend):
    """The loop on one GPU: MIXED MPM scenes in one hg_batch."""

    def __init__(self, ctx, max_members=256, depth=3):
        from . import Batch  # noqa: WPS433 (package import cycle)
        self.ctx = ctx
        self.batch = Batch(ctx, max_members)
        self.depth = depth
        self.state = {}
        self.pool = collections.defaultdict(list)  # page-locked buffers by size class
        self.owner = {}

    def _buf(self, shape):
        """A page-locked view of the given shape, from a pool of buffers whose
        row counts are powers of two (scenes of similar size share them)."""
        from . import pinned
        rows = shape[0]
        cls = 1 << max(rows - 1, 1).bit_length()
        key = (cls,) + tuple(shape[1:])
        free = self.pool[key]
        base = free.pop() if free else pinned(key)
        view = base[:rows]
        self.owner[id(view)] = (key, base)
        return view

    def _give(self, view):
        key, base = self.owner.pop(id(view))
        self.pool[key].append(base)

    def footprint(self, req):
        from . import mpm_estimate_bytes
        c = req.cfg
        return mpm_estimate_bytes(c["grid_min"], c["grid_max"], c["h"], req.npoints)

    def open(self, req):
        from . import MPM
        c = req.cfg
        m = MPM(self.ctx, c["grid_min"], c["grid_max"], c["h"], c["shear_modulus"],
                c["bulk_modulus"], c["dp_alpha"], c["flip_alpha"], scenes.GRAVITY,
                c["planes"], capacity=req.npoints)
        # points generated on the device from the request's geometry
        m.seed_rectangle_device(c["rect_min"], c["rect_max"], c["rho"], c["samples_per_dim"])
        frames = [self._buf((req.npoints, 2)) for _ in range(self.depth + 1)]
        self.batch.add(m, req.dt)
        self.state[req.rid] = dict(m=m, frames=frames)

    def step(self, nsteps):
        self.batch.step(nsteps)

    def frame(self, req, slot):
        s = self.state[req.rid]
        s["m"].frame_async(s["frames"][slot], None)

    def leave(self, req):
        self.batch.remove(self.state[req.rid]["m"])

    def fence(self):
        return self.ctx.fence()

    def fence_done(self, f):
        return self.ctx.fence_done(f)

    def fence_wait(self, f):
        self.ctx.fence_wait(f)

    def read_frame(self, req, slot):
        q = self.state[req.rid]["frames"][slot]
        return float(q[:, 0].max())  # run-out: front position

    def close(self, req):
        s = self.state.pop(req.rid)
        s["m"].close()
        for a in s["frames"]:
            self._give(a)

    def shutdown(self):
        self.batch.close()


def run_one_at_a_time(ctx, requests):
    """The same requests served one after another, each scene alone
    (hg_mpm_step per frame interval, frame read synchronously); returns
    wall seconds."""
    from . import MPM
    t0 = time.perf_counter()
    for r in requests:
        c = r.cfg
        m = MPM(ctx, c["grid_min"], c["grid_max"], c["h"], c["shear_modulus"],
                c["bulk_modulus"], c["dp_alpha"], c["flip_alpha"], scenes.GRAVITY,
                c["planes"], capacity=r.npoints)
        m.seed_rectangle_device(c["rect_min"], c["rect_max"], c["rho"], c["samples_per_dim"])
        q = np.zeros((r.npoints, 2))
        for k in range(r.steps // r.frame_every):
            m.flow(r.dt, r.frame_every)
            m.download_into(q=q)
            r.frames.append(((k + 1) * r.frame_every, float(q[:, 0].max())))
        m.close()
    return time.perf_counter() - t0

