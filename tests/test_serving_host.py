"""Serving loop scheduling on the host, with a fake device.

The fake device advances a virtual clock by a cost per point-step when a
chunk is stepped and completes fences in order, so the test checks the
loop's own rules without a GPU: admission in arrival order only while the
device footprints fit the budget, no more members than batch slots, every
request gets steps/frame_every frames in order, frames are read only after
their fence, and no request finishes before it arrives.
"""
import numpy as np
import pytest

from libhybridgrains_gb300 import serving


class FakeDevice(serving.Backend):
    def __init__(self, clock, cost=1e-9):
        self.clock = clock
        self.cost = cost
        self.members = {}
        self.fences = []      # (fence id, virtual completion time)
        self.busy_until = 0.0
        self.written = {}     # (rid, slot) -> fence id that covers the copy
        self.opened, self.closed = [], []
        self.max_members = 0
        self.pending_frames = []

    def footprint(self, req):
        return req.npoints * 100

    def open(self, req):
        self.members[req.rid] = req
        self.opened.append(req.rid)
        self.max_members = max(self.max_members, len(self.members))

    def step(self, nsteps):
        work = sum(r.npoints for r in self.members.values()) * nsteps * self.cost
        self.busy_until = max(self.busy_until, self.clock.t) + work

    def frame(self, req, slot):
        self.pending_frames.append((req.rid, slot))

    def leave(self, req):
        del self.members[req.rid]

    def fence(self):
        f = len(self.fences)
        self.fences.append(self.busy_until)
        for key in self.pending_frames:
            self.written[key] = f
        self.pending_frames = []
        return f

    def fence_done(self, f):
        return self.fences[f] <= self.clock.t

    def fence_wait(self, f):
        self.clock.t = max(self.clock.t, self.fences[f])

    def read_frame(self, req, slot):
        f = self.written[(req.rid, slot)]
        assert self.fence_done(f), "frame read before its fence"
        return float(f)

    def close(self, req):
        assert req.rid not in self.members
        self.closed.append(req.rid)


class Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 1e-6  # host work per call
        return self.t

    def sleep(self, s):
        self.t += s


def requests(n=40, seed=3):
    rng = np.random.default_rng(seed)
    arr = np.cumsum(rng.exponential(0.02, size=n))
    out = []
    for i in range(n):
        npts = int(np.exp(rng.uniform(np.log(2e3), np.log(2e5))))
        out.append(serving.Request(i, float(arr[i]), None, npts, steps=2000, frame_every=100))
    return out


@pytest.mark.parametrize("budget_points,slots", [(10**9, 256), (400_000, 256), (10**9, 3)])
def test_admission_order_budget_and_frames(budget_points, slots):
    clock = Clock()
    dev = FakeDevice(clock)
    reqs = requests()
    srv = serving.Server(dev, budget_points * 100, max_members=slots, depth=3, clock=clock,
                         sleep=clock.sleep)
    srv.run(reqs)
    assert dev.opened == sorted(dev.opened)            # first come, first served
    assert sorted(dev.closed) == list(range(len(reqs)))
    assert srv.peak_resident <= budget_points * 100
    assert dev.max_members <= slots
    for r in reqs:
        assert r.admitted >= r.arrival
        assert r.finished >= r.admitted
        assert [s for s, _ in r.frames] == list(range(100, 2001, 100))
        fences = [f for _, f in r.frames]
        assert fences == sorted(fences)
    s = serving.summary(reqs, srv.makespan)
    assert s["p99_latency_s"] >= s["p50_latency_s"] > 0


def test_request_over_budget_is_rejected():
    clock = Clock()
    reqs = requests(3)
    srv = serving.Server(FakeDevice(clock), 100, clock=clock, sleep=clock.sleep)
    with pytest.raises(ValueError):
        srv.run(reqs)


def test_column_request_stream_is_seeded():
    a = serving.column_requests(n=8, seed=5, steps=200)
    b = serving.column_requests(n=8, seed=5, steps=200)
    assert [r.npoints for r in a] == [r.npoints for r in b]
    assert [r.arrival for r in a] == [r.arrival for r in b]
    assert all(1500 <= r.npoints <= 2.5e5 for r in a)
    assert a[0].arrival == 0.0
