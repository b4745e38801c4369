"""Checkpoint files: device state blobs and host arrays in one file.

The reference's CLIs snapshot with ``-s`` and resume with ``-r`` through a
chain of ``serialize()`` calls behind a magic number (MPM 9035768,
mpmgrains2d_cli.cpp:44, 154-247; hybrid 8675309, hybridgrains2d_cli.cpp:45,
242-334), and the hybrid chain exits in HybridIntegratorState::serialize
(HybridIntegratorState.cpp:67-85). Here a checkpoint holds what the device
objects export (``hg_*_state_save``: sorted particle records, the next step's
accumulators, the DEM contact history, the interval's homogenised fields), the
resampler's random streams and the host-side arrays of a hybrid simulation,
so that a simulation resumed from it continues as the saved one would.

File layout: the 8 bytes ``HGCKPT\\x00\\x01``, a little-endian uint64 header
length, a UTF-8 JSON header ``{"entries": [{"name", "dtype", "shape",
"offset", "bytes"}, ...], "meta": {...}}`` and the entries' bytes, each at an
8-byte aligned offset from the start of the payload.
"""
import json
import struct

import numpy as np

MAGIC = b"HGCKPT\x00\x01"


def write(path, arrays, meta=None):
    """Writes ``arrays`` (name -> numpy array) and a JSON-serialisable
    ``meta`` dict."""
    entries, off = [], 0
    items = [(k, np.ascontiguousarray(v)) for k, v in arrays.items()]
    for name, a in items:
        entries.append(dict(name=name, dtype=a.dtype.str, shape=list(a.shape), offset=off,
                            bytes=int(a.nbytes)))
        off += (a.nbytes + 7) & ~7
    head = json.dumps(dict(entries=entries, meta=meta or {})).encode()
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(struct.pack("<Q", len(head)))
        f.write(head)
        for (name, a), e in zip(items, entries):
            f.write(a.tobytes())
            f.write(b"\0" * (((a.nbytes + 7) & ~7) - a.nbytes))


def read(path):
    """Returns (arrays, meta) of a checkpoint file."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != MAGIC:
        raise ValueError(f"{path} is not a checkpoint file")
    (hlen,) = struct.unpack_from("<Q", data, 8)
    if 16 + hlen > len(data):
        raise ValueError(f"{path} is truncated")
    head = json.loads(data[16:16 + hlen].decode())
    base = 16 + hlen
    arrays = {}
    for e in head["entries"]:
        start = base + e["offset"]
        if start + e["bytes"] > len(data):
            raise ValueError(f"{path} is truncated")
        a = np.frombuffer(data, dtype=np.dtype(e["dtype"]), count=int(np.prod(e["shape"])),
                          offset=start)
        arrays[e["name"]] = a.reshape(e["shape"]).copy()
    return arrays, head["meta"]


def save_objects(path, meta=None, **objects):
    """Checkpoints device objects (anything with ``state()``: MPM, DEM,
    Hybrid) under their keyword names."""
    write(path, {k: o.state() for k, o in objects.items()}, meta)


def load_objects(path, **objects):
    """Restores device objects saved by ``save_objects`` (each created with
    the same grid, capacities at least the saved counts); returns meta."""
    arrays, meta = read(path)
    for k, o in objects.items():
        if k not in arrays:
            raise KeyError(f"{path} holds no state for {k!r}")
        o.load_state(arrays[k])
    return meta
