"""The DEM shim of INTEGRATION.md (an ImpactFrictionMap subclass over the C
ABI) driven as the reference's hybrid loop drives the penalty map.

tests/integration/dem_shim_driver.cpp runs the shim through three stages: two
weighted steps; host edits of velocities and positions (as the coupling
makes after every DEM step) and two more steps; bodies removed through
removeBodies / deleteCacheEntries and two added through addBody /
enlargeCache (as the resampling step does) and two more steps. The FP64 DEM
is bit-exact, so:

* stages 1 and 2 equal the CPU oracle given the same edits, bit for bit (a
  shim that ignored the host's edits would differ);
* stage 3 equals the library driven directly (upload_relabel with the same
  renumbering), bit for bit.
"""
import os
import struct
import subprocess

import numpy as np
import pytest

import oracle
import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import build, scenes

from integration import shims

pytestmark = pytest.mark.gpu

DT = 1.0e-6


def scene():
    sc = scenes.dem_column(n=600, per_row=30)
    sc["v"][:, 1] = -2.0
    return sc


def run_driver(tmp_path, sc, dp):
    exe, r = shims.build_dem_driver(tmp_path, os.path.dirname(build.build()))
    assert r.returncode == 0, r.stderr
    n = len(sc["r"])
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(struct.pack("<q", n))
        f.write(np.array([DT, dp["kn"], dp["kt"], dp["gamman"], dp["gammat"], dp["mu"],
                          scenes.GRAVITY[0], scenes.GRAVITY[1]], dtype="<f8").tobytes())
        for k in ("q", "v", "r", "m", "I"):
            f.write(np.ascontiguousarray(sc[k], dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(sc["fixed"], dtype=np.uint8).tobytes())
    out = tmp_path / "out.bin"
    r = subprocess.run([exe, str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    data = out.read_bytes()
    stages, pos = [], 0
    for _ in range(3):
        (m,) = struct.unpack_from("<q", data, pos)
        pos += 8
        q = np.frombuffer(data, "<f8", 3 * m, pos).reshape(m, 3)
        pos += 24 * m
        v = np.frombuffer(data, "<f8", 3 * m, pos).reshape(m, 3)
        pos += 24 * m
        stages.append((q, v))
    return stages


def edit(q, v):
    q, v = q.copy(), v.copy()
    i = np.arange(len(q))
    v[i % 5 == 0, 1] = -0.1
    q[i % 7 == 0, 0] += 1.0e-5
    return q, v


def test_dem_shim_follows_host_edits_and_body_changes(ctx, tmp_path):
    sc = scene()
    dp = scenes.dem_params()
    n = len(sc["r"])
    stages = run_driver(tmp_path, sc, dp)
    ones = np.ones(n)

    # stages 1 and 2 against the oracle
    c = oracle.DEM(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"], scenes.GRAVITY,
                   dp["kn"], dp["kt"], dp["gamman"], dp["gammat"], dp["mu"], 1.0)
    c.add_plane((0.0, 0.0), (0.0, 1.0))
    c.set_weights(ones)
    c.step(DT, 2, weighted=True)
    q1, v1 = c.state()
    assert np.array_equal(stages[0][0], q1) and np.array_equal(stages[0][1], v1)
    qe, ve = edit(q1, v1)
    c.set_state(qe, ve)
    c.step(DT, 2, weighted=True)
    q2, v2 = c.state()
    assert np.array_equal(stages[1][0], q2) and np.array_equal(stages[1][1], v2)
    assert len(c.contacts()) > 0

    # stage 3 against the library driven directly
    g = hg.DEM(ctx, scenes.GRAVITY, dp["kn"], dp["kt"], dp["gamman"], dp["gammat"], dp["mu"],
               [((0.0, 0.0), (0.0, 1.0))], capacity=n + 16, contact_capacity=8 * (n + 16))
    g.upload(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["fixed"])
    g.set_weights(ones)
    g.flow_with_weights(DT, 2)
    qd, vd = g.download()
    g.set_state(*edit(qd, vd))
    g.flow_with_weights(DT, 2)
    qd, vd = g.download()
    keep = np.arange(n) % 11 != 3
    old_to_new = np.where(keep, np.cumsum(keep) - 1, -1).astype(np.int32)
    add_q = np.array([[0.5, 0.5, 0.0], [0.6, 0.5, 0.0]])
    g.upload_relabel(np.concatenate([qd[keep], add_q]),
                     np.concatenate([vd[keep], np.zeros((2, 3))]),
                     np.concatenate([sc["r"][keep], [1.0e-3, 1.0e-3]]),
                     np.concatenate([sc["m"][keep], sc["m"][:1], sc["m"][:1]]),
                     np.concatenate([sc["I"][keep], sc["I"][:1], sc["I"][:1]]),
                     np.zeros(keep.sum() + 2, dtype=np.uint8), old_to_new)
    g.set_weights(np.ones(keep.sum() + 2))
    g.flow_with_weights(DT, 2)
    q3, v3 = g.download()
    assert len(stages[2][0]) == keep.sum() + 2
    assert np.array_equal(stages[2][0], q3) and np.array_equal(stages[2][1], v3)
    assert g.num_contacts() > 0
    assert g.status() == 0
