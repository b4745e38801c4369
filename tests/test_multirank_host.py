"""The multi-GPU path on the host (world size 2, gloo on CPU, no GPU): the
bench's max-over-ranks timing, the serving loop's request sharding and the
pooled latency figures. Scenes are independent, so ranks exchange only
these figures."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def fake_run(reqs, t0=0.0):
    # deterministic admission and completion times in place of a device run
    for k, r in enumerate(reqs):
        r.admitted = r.arrival + 0.01 * (k % 3)
        r.finished = r.admitted + 0.1 + 0.001 * r.rid
    return t0 + max(r.finished for r in reqs)


def worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from libhybridgrains_gb300 import serving
    everything = serving.column_requests(n=12, rate=100.0, seed=5, nmax=5e3)
    mine = serving.shard_requests(everything, rank, world)
    makespan = fake_run(mine)
    parts = bench.gather_parts(serving.summary_parts(mine, makespan), world)
    merged = serving.summary_of_parts(parts)
    slowest = bench.barrier_max(float(rank + 1), world)
    out.put((rank, [r.rid for r in mine], merged, slowest))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_share_the_requests_and_pool_the_figures():
    from libhybridgrains_gb300 import serving
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ids0, m0, s0), (r1, ids1, m1, s1) = res
    assert sorted(ids0 + ids1) == list(range(12)) and not set(ids0) & set(ids1)
    assert s0 == s1 == 2.0  # max over ranks
    assert m0 == m1  # every rank pools the same figures
    # the pooled figures equal one process serving every request
    everything = serving.column_requests(n=12, rate=100.0, seed=5, nmax=5e3)
    shards = [serving.shard_requests(everything, r, 2) for r in range(2)]
    spans = [fake_run(s) for s in shards]
    assert m0["requests"] == 12 and m0["makespan_s"] == max(spans)
    lat = sorted(r.latency for s in shards for r in s)
    assert m0["max_latency_s"] == lat[-1]
    assert m0["particle_steps"] == sum(r.npoints * r.steps for r in everything)
