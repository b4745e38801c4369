"""The reference's MPM snapshot format (serial.bin of mpmgrains2d_cli), host
only: field offsets written out by hand for a two-point scene, a round trip
of every field, and the refusals of damaged files."""
import struct

import numpy as np
import pytest

from libhybridgrains_gb300 import reference_format as rf


def two_point_state():
    rng = np.random.default_rng(3)
    n, cc = 2, (3, 2)
    nn = (cc[0] + 1) * (cc[1] + 1)
    pts = dict(q0=rng.normal(size=(n, 2)), q=rng.normal(size=(n, 2)), v=rng.normal(size=(n, 2)),
               m=rng.uniform(1, 2, n), volume=rng.uniform(1, 2, n), m0=rng.uniform(1, 2, n),
               volume0=rng.uniform(1, 2, n), weight=rng.uniform(size=n), hl=rng.uniform(size=n),
               be_bar=rng.normal(size=(n, 4)), J=rng.uniform(0.9, 1.1, n),
               sigma=rng.normal(size=(n, 4)), vel_grad=rng.normal(size=(n, 4)),
               just_homogenized=np.array([0, 1], dtype=np.int32),
               always_fixed=np.array([False, True]),
               kinematically_scripted=np.array([True, False]))
    grid = dict(min=(0.0, -0.5), max=(0.3, 0.5), cell_width=0.1, cell_count=cc,
                mass=rng.uniform(size=nn), momentum=rng.normal(size=(nn, 2)),
                momentum_new=rng.normal(size=(nn, 2)), force=rng.normal(size=(nn, 2)),
                velocity=rng.normal(size=(nn, 2)), acceleration=rng.normal(size=(nn, 2)),
                homog_factor=rng.uniform(size=nn), hybridized=np.arange(nn, dtype=np.int32))
    state = dict(points=pts, grid=grid, planes=[((0.0, 0.0), (0.0, 1.0), rf.STICKING, -np.inf),
                                                ((0.3, 0.0), (-1.0, 0.0), rf.SLIDING, 0.25)],
                 shear_modulus=3.8e5, bulk_modulus=8.3e5, dp_alpha=0.37, gravity=(0.0, -981.0),
                 flip_alpha=0.999, basis=rf.BASIS_UGIMP)
    run = dict(git_revision="abc123", iteration=77, dt=(1, 1000080), end_time=2.5,
               steps_per_save=10, output_frame=7, dt_string_precision=6, save_number_width=5,
               serialize_snapshots=True, overwrite_snapshots=False)
    return state, run


def test_layout_by_hand():
    state, run = two_point_state()
    b = rf.encode_mpm_snapshot(state, run)
    p = state["points"]
    o = 0
    assert struct.unpack_from("<I", b, o)[0] == 9035768
    o += 4
    assert struct.unpack_from("<Q", b, o)[0] == 6 and b[o + 8:o + 14] == b"abc123"
    o += 14
    assert struct.unpack_from("<I", b, o)[0] == 2  # npoints
    o += 4
    # q0: column count then the 2 x 2 column-major data
    assert struct.unpack_from("<q", b, o)[0] == 2
    assert np.array_equal(np.frombuffer(b, "<f8", 4, o + 8), p["q0"].reshape(-1))
    o += 8 + 32
    o += 2 * (8 + 32)  # q, v
    for k in ("m", "volume", "m0", "volume0", "weight", "hl"):
        assert struct.unpack_from("<q", b, o)[0] == 2
        assert np.array_equal(np.frombuffer(b, "<f8", 2, o + 8), p[k])
        o += 8 + 16
    assert struct.unpack_from("<Q", b, o)[0] == 2  # be_bar count
    assert np.array_equal(np.frombuffer(b, "<f8", 8, o + 8), p["be_bar"].reshape(-1))
    o += 8 + 64
    o += 8 + 16  # J
    o += 2 * (8 + 64)  # sigma, vel_grad
    assert struct.unpack_from("<q2i", b, o) == (2, 0, 1)  # just_homogenized
    o += 16
    assert struct.unpack_from("<Q2B", b, o) == (2, 0, 1)  # always_fixed
    o += 10
    assert struct.unpack_from("<Q2B", b, o) == (2, 1, 0)  # kinematically_scripted
    o += 10
    assert struct.unpack_from("<5d2I", b, o) == (0.0, -0.5, 0.3, 0.5, 0.1, 3, 2)
    nn = 12
    o += 48
    o += (8 + 8 * nn) + 5 * (8 + 16 * nn) + (8 + 8 * nn)
    assert struct.unpack_from("<q", b, o)[0] == nn
    assert np.array_equal(np.frombuffer(b, "<i4", nn, o + 8), np.arange(nn))
    o += 8 + 4 * nn
    assert struct.unpack_from("<Q", b, o)[0] == 2
    o += 8
    assert struct.unpack_from("<4did", b, o) == (0.0, 0.0, 0.0, 1.0, 1, -np.inf)
    o += 2 * 44
    assert struct.unpack_from("<6di", b, o) == (3.8e5, 8.3e5, 0.37, 0.0, -981.0, 0.999, 2)
    o += 52
    assert struct.unpack_from("<I2qd4I2?", b, o) == (77, 1, 1000080, 2.5, 10, 7, 6, 5, True, False)
    o += 4 + 16 + 8 + 16 + 2
    assert o == len(b)


def test_round_trip(tmp_path):
    state, run = two_point_state()
    for with_dir in (False, True):
        run["output_dir"] = "frames"
        path = tmp_path / "serial.bin"
        rf.write_mpm_snapshot(path, state, run, with_output_dir=with_dir)
        s2, r2 = rf.read_mpm_snapshot(path, with_output_dir=with_dir)
        for k, v in state["points"].items():
            assert np.array_equal(np.asarray(s2["points"][k]).reshape(np.shape(v)), v), k
        for k, v in state["grid"].items():
            assert np.array_equal(np.asarray(s2["grid"][k]).reshape(np.shape(v)), v), k
        assert [(tuple(a), tuple(b_), c, d) for a, b_, c, d in s2["planes"]] == \
            [(tuple(a), tuple(b_), c, d) for a, b_, c, d in state["planes"]]
        for k in ("shear_modulus", "bulk_modulus", "dp_alpha", "flip_alpha", "basis"):
            assert s2[k] == state[k]
        assert tuple(s2["gravity"]) == state["gravity"]
        for k, v in run.items():
            if k != "output_dir" or with_dir:
                assert (tuple(r2[k]) if k == "dt" else r2[k]) == v, k


def test_damaged_files_are_refused():
    state, run = two_point_state()
    b = rf.encode_mpm_snapshot(state, run)
    with pytest.raises(ValueError):
        rf.decode_mpm_snapshot(b"\0" + b[1:])
    with pytest.raises(ValueError):
        rf.decode_mpm_snapshot(b[:-3])
    with pytest.raises(ValueError):
        rf.decode_mpm_snapshot(b + b"\0")
    with pytest.raises(ValueError):  # the HDF5 build's layout read as the other
        rf.decode_mpm_snapshot(rf.encode_mpm_snapshot(state, run, with_output_dir=True))


def test_cauchy_stress_matches_the_constitutive_formula():
    rng = np.random.default_rng(8)
    n = 50
    a = rng.normal(scale=0.1, size=(n, 3))
    be = np.stack([1 + a[:, 0], a[:, 1], a[:, 1], 1 + a[:, 2]], axis=1)
    be /= np.sqrt(be[:, 0] * be[:, 3] - be[:, 1] * be[:, 2])[:, None]  # det 1
    J = rng.uniform(0.95, 1.05, n)
    jh = (rng.uniform(size=n) < 0.2).astype(np.int32)
    s = rf.cauchy_stress(be, J, jh, 3.0, 7.0)
    for i in range(n):
        B = be[i].reshape(2, 2, order="F") * J[i]
        Jt = np.sqrt(np.linalg.det(B))
        Bb = B / Jt
        tau = 7.0 * 0.5 * (Jt + 1) * (Jt - 1) * np.eye(2) + 3.0 * (Bb - np.trace(Bb) / 2 * np.eye(2))
        exp = np.zeros(4) if (J[i] > 1 or jh[i]) else (tau / J[i]).reshape(-1, order="F")
        assert np.allclose(s[i], exp, rtol=1e-12, atol=1e-12)
