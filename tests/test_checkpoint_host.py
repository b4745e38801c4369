"""Checkpoint container and the resampler's random-stream state (host only,
no GPU)."""
import numpy as np
import pytest

import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import checkpoint, scenes


def test_container_round_trip(tmp_path):
    p = tmp_path / "c.hgckpt"
    arrays = dict(blob=np.arange(13, dtype=np.uint8), q=np.random.default_rng(1).normal(size=(5, 2)),
                  jh=np.array([1, 0, 1], dtype=np.int32), empty=np.zeros(0))
    checkpoint.write(p, arrays, dict(counter=3, stats=[{"a": 1}]))
    back, meta = checkpoint.read(p)
    assert meta == dict(counter=3, stats=[{"a": 1}])
    assert set(back) == set(arrays)
    for k in arrays:
        assert back[k].dtype == arrays[k].dtype and np.array_equal(back[k], arrays[k])
    data = p.read_bytes()
    (p.parent / "bad").write_bytes(b"XXXX" + data[4:])
    with pytest.raises(ValueError):
        checkpoint.read(p.parent / "bad")
    (p.parent / "short").write_bytes(data[:-8])
    with pytest.raises(ValueError):
        checkpoint.read(p.parent / "short")


def resampler():
    sc = scenes.hybrid_column(scale=0.05)
    cfg, zs, rs = sc["mpm"], sc["zones"], sc["resampling"]
    h = cfg["h"]
    nx = int(round((cfg["grid_max"][0] - cfg["grid_min"][0]) / h))
    ny = int(round((cfg["grid_max"][1] - cfg["grid_min"][1]) / h))
    zargs = (cfg["grid_min"], h, (nx, ny), zs["level_set_cell_width"], zs["phi_window_size"],
             zs["phi_samples_per_cell_side"], zs["phi_threshold"], zs["rzone_level_set"],
             zs["rzone_half_thickness"], zs["allow_direct_transitions"])
    return hg.Resampler(zargs, cfg["grid_max"], 1, h / 2, cfg["rho"], rs["dem_r_mean"],
                        rs["dem_r_std"], rs["rho_dem"], cfg["bulk_modulus"], cfg["shear_modulus"],
                        rs["newly_inserted_continuum_stress_free"], rs["homogenize_stress"],
                        rs["homogenize_velocity"])


def draws(r, k=700):
    # past one MT19937 block (624 words) and an odd number of normal draws
    return ([r.random_u32() for _ in range(k)], [r.random_f32() for _ in range(9)],
            [r.random_radius() for _ in range(7)])


def test_resampler_random_streams_resume():
    a = resampler()
    draws(a, 100)
    blob = a.rng_state()
    expect = draws(a)
    b = resampler()
    b.load_rng_state(blob)
    assert draws(b) == expect
    with pytest.raises(hg.HGError):
        b.load_rng_state(blob[:40])
    bad = blob.copy()
    bad[0] ^= 1
    with pytest.raises(hg.HGError):
        b.load_rng_state(bad)
