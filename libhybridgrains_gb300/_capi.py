"""ctypes binding of libhg_gpu.so (include/hg_gpu.h).

Loading fails loudly: there is no CPU fallback. ``load()`` raises when the
shared library is missing or does not export the declared entry points.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# HG_GPU_VARIANT=bounds selects the bounds-checking build
LIB_PATH = (os.path.join(HERE, "_build_bounds", "libhg_gpu_bounds.so")
            if os.environ.get("HG_GPU_VARIANT") == "bounds"
            else os.path.join(HERE, "_build", "libhg_gpu.so"))

HG_MAX_PLANES = 8
HG_MAX_DRUMS = 8
HG_DEM_KIND_PLANE, HG_DEM_KIND_CIRCLE, HG_DEM_KIND_KINEMATIC, HG_DEM_KIND_DRUM = 0, 1, 2, 3
HG_DEM_RECORD_WIDTH = 22
HG_STATIC_PAIRS_MAX_BOXES = 16384
HG_STATIC_PAIRS_MAX_PAIRS = 262144
HG_MAX_BATCH = 1024

STATUS = {0: "HG_OK", 1: "HG_ERR_INVALID_ARGUMENT", 2: "HG_ERR_CUDA", 3: "HG_ERR_OUT_OF_MEMORY",
          4: "HG_ERR_CAPACITY", 5: "HG_ERR_UNSUPPORTED", 6: "HG_ERR_DEVICE_STATUS"}

HG_STATUS_NONFINITE = 1 << 0
HG_STATUS_OUT_OF_GRID = 1 << 1
HG_STATUS_CONTACT_OVERFLOW = 1 << 2
HG_STATUS_CELL_OVERFLOW = 1 << 3


class MpmPlane(ctypes.Structure):
    _fields_ = [("x", ctypes.c_double * 2), ("n", ctypes.c_double * 2),
                ("sticking", ctypes.c_int32), ("pad_", ctypes.c_int32),
                ("lower_bound", ctypes.c_double)]


class MpmDesc(ctypes.Structure):
    _fields_ = [("grid_min", ctypes.c_double * 2), ("grid_max", ctypes.c_double * 2),
                ("cell_width", ctypes.c_double), ("basis", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("shear_modulus", ctypes.c_double),
                ("bulk_modulus", ctypes.c_double), ("dp_alpha", ctypes.c_double),
                ("flip_alpha", ctypes.c_double), ("gravity", ctypes.c_double * 2),
                ("num_planes", ctypes.c_int32), ("pad_", ctypes.c_int32),
                ("planes", MpmPlane * HG_MAX_PLANES), ("capacity", ctypes.c_int64)]


class DemPlane(ctypes.Structure):
    _fields_ = [("x", ctypes.c_double * 2), ("n", ctypes.c_double * 2)]


class DemDrum(ctypes.Structure):
    _fields_ = [("x", ctypes.c_double * 2), ("r", ctypes.c_double)]


class ZonesDesc(ctypes.Structure):
    _fields_ = [("mpm_grid_min", ctypes.c_double * 2), ("mpm_cell_width", ctypes.c_double),
                ("mpm_cells", ctypes.c_int32 * 2), ("level_set_cell_width", ctypes.c_double),
                ("allow_direct_transitions", ctypes.c_int32),
                ("phi_samples_per_cell_side", ctypes.c_int32), ("phi_window_size", ctypes.c_double),
                ("phi_threshold", ctypes.c_double), ("rzone_level_set", ctypes.c_double),
                ("rzone_half_thickness", ctypes.c_double)]


class ResamplerDesc(ctypes.Structure):
    _fields_ = [("zones", ZonesDesc), ("mpm_grid_max", ctypes.c_double * 2),
                ("basis", ctypes.c_int32), ("newly_inserted_continuum_stress_free", ctypes.c_int32),
                ("initial_particle_size", ctypes.c_double), ("material_density", ctypes.c_double),
                ("dem_r_mean", ctypes.c_double), ("dem_r_std", ctypes.c_double),
                ("rho_dem", ctypes.c_double), ("kappa", ctypes.c_double), ("mu", ctypes.c_double),
                ("homogenize_stress", ctypes.c_int32), ("homogenize_velocity", ctypes.c_int32)]


class ResamplerStats(ctypes.Structure):
    _fields_ = [("points_inserted", ctypes.c_int64), ("grains_inserted", ctypes.c_int64),
                ("points_deleted", ctypes.c_int64), ("grains_deleted", ctypes.c_int64),
                ("ms_insert_grains", ctypes.c_double), ("ms_insert_points", ctypes.c_double),
                ("ms_point_grids", ctypes.c_double), ("ms_quantities", ctypes.c_double),
                ("ms_delete", ctypes.c_double)]


HG_TUNE_CANDIDATES = 4


class LaunchShape(ctypes.Structure):
    _fields_ = [("fused_ctas_per_sm", ctypes.c_int32), ("update_ctas_per_sm", ctypes.c_int32)]


class TuneReport(ctypes.Structure):
    _fields_ = [("candidates", ctypes.c_int32), ("tried", LaunchShape * HG_TUNE_CANDIDATES),
                ("fused_ms", ctypes.c_double * HG_TUNE_CANDIDATES),
                ("update_ms", ctypes.c_double * HG_TUNE_CANDIDATES), ("chosen", LaunchShape),
                ("step_ms", (ctypes.c_double * HG_TUNE_CANDIDATES) * HG_TUNE_CANDIDATES),
                ("steps", ctypes.c_int64)]


class DemDesc(ctypes.Structure):
    _fields_ = [("gravity", ctypes.c_double * 2), ("kn", ctypes.c_double),
                ("kt", ctypes.c_double), ("gamman", ctypes.c_double),
                ("gammat", ctypes.c_double), ("mu", ctypes.c_double),
                ("cell_scale", ctypes.c_double), ("num_planes", ctypes.c_int32),
                ("pad_", ctypes.c_int32), ("planes", DemPlane * HG_MAX_PLANES),
                ("capacity", ctypes.c_int64), ("contact_capacity", ctypes.c_int64),
                ("precision", ctypes.c_int32), ("num_drums", ctypes.c_int32),
                ("drums", DemDrum * HG_MAX_DRUMS)]


_P = ctypes.c_void_p
_PP = ctypes.POINTER(ctypes.c_void_p)
_D = ctypes.POINTER(ctypes.c_double)
_I32 = ctypes.POINTER(ctypes.c_int32)
_I64 = ctypes.POINTER(ctypes.c_int64)
_U8 = ctypes.POINTER(ctypes.c_uint8)
_U32 = ctypes.POINTER(ctypes.c_uint32)
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_dbl = ctypes.c_double

# name -> argument types (every function returns hg_status unless listed in _RET)
SIGNATURES = {
    "hg_context_create": [_i32, _PP],
    "hg_context_destroy": [_P],
    "hg_context_synchronize": [_P],
    "hg_status_string": [_i32],
    "hg_last_error": [],
    "hg_kernel_launch_count": [],
    "hg_set_host_threads": [_i32],
    "hg_context_timer_begin": [_P],
    "hg_context_timer_end": [_P, _D],
    "hg_mpm_create": [_P, ctypes.POINTER(MpmDesc), _PP],
    "hg_mpm_destroy": [_P],
    "hg_mpm_grid_info": [_P, _D, _D, _I32],
    "hg_mpm_seed_rectangle": [_P, _D, _D, _dbl, _i32, _D, _dbl, _i64, _D, _D, _D, _D, _D, _I64],
    "hg_mpm_upload": [_P, _i64, _D, _D, _D, _D, _D, _D, _D, _I32, _U8],
    "hg_mpm_download": [_P, _D, _D, _D, _D, _I32],
    "hg_mpm_num_particles": [_P, _I64],
    "hg_mpm_step": [_P, _dbl, _i32],
    "hg_mpm_phase0": [_P],
    "hg_mpm_phase1": [_P, _dbl],
    "hg_mpm_phase2": [_P, _dbl],
    "hg_mpm_download_grid": [_P, _D, _D, _D, _D, _D, _D],
    "hg_mpm_cell_index": [_P, _I32],
    "hg_mpm_status": [_P, _U32],
    "hg_mpm_clear_status": [_P],
    "hg_mpm_rebin_count": [_P, _I64],
    "hg_mpm_profile": [_P, _i32],
    "hg_mpm_profile_read": [_P, _D, _D, _I64],
    "hg_context_fence": [_P, _I64],
    "hg_context_fence_done": [_P, _i64, _I32],
    "hg_context_fence_wait": [_P, _i64],
    "hg_context_device_bytes": [_P, _I64],
    "hg_host_alloc": [_i64, _PP],
    "hg_host_free": [_P],
    "hg_mpm_seed_rectangle_device": [_P, _D, _D, _dbl, _i32, _D, _dbl, _I64],
    "hg_mpm_upload_async": [_P, _i64, _D, _D, _D, _D, _D, _D, _D, _I32, _U8],
    "hg_mpm_frame_async": [_P, _D, _D],
    "hg_mpm_estimate_bytes": [ctypes.POINTER(MpmDesc), _I64],
    "hg_batch_create": [_P, _i32, _PP],
    "hg_batch_destroy": [_P],
    "hg_batch_add": [_P, _P, _dbl],
    "hg_batch_remove": [_P, _P],
    "hg_batch_size": [_P, _I32],
    "hg_batch_step": [_P, _i32],
    "hg_batch_stats": [_P, _I64, _I64, _I64, _D, _D],
    "hg_batch_profile": [_P, _i32],
    "hg_batch_profile_read": [_P, _D, _D, _D, _D, _I64],
    "hg_mpm_autotune": [_P, _dbl, _i32, ctypes.POINTER(TuneReport)],
    "hg_mpm_launch_shape": [_P, ctypes.POINTER(LaunchShape)],
    "hg_mpm_set_launch_shape": [_P, ctypes.POINTER(LaunchShape)],
    "hg_batch_autotune": [_P, _i32, ctypes.POINTER(TuneReport)],
    "hg_batch_launch_shape": [_P, ctypes.POINTER(LaunchShape)],
    "hg_tune_save": [ctypes.c_char_p],
    "hg_tune_load": [ctypes.c_char_p],
    "hg_tune_clear": [],
    "hg_dem_set_concurrent": [_P, _i32],
    "hg_dem_wait_context": [_P],
    "hg_dem_join": [_P],
    "hg_mpm_state_bytes": [_P, _I64],
    "hg_mpm_state_save": [_P, _P, _i64],
    "hg_mpm_state_load": [_P, _P, _i64],
    "hg_dem_state_bytes": [_P, _I64],
    "hg_dem_state_save": [_P, _P, _i64],
    "hg_dem_state_load": [_P, _P, _i64],
    "hg_hybrid_state_bytes": [_P, _I64],
    "hg_hybrid_state_save": [_P, _P, _i64],
    "hg_hybrid_state_load": [_P, _P, _i64],
    "hg_resampler_rng_bytes": [_P, _I64],
    "hg_resampler_rng_save": [_P, _P, _i64],
    "hg_resampler_rng_load": [_P, _P, _i64],
    "hg_zones_create": [ctypes.POINTER(ZonesDesc), _PP],
    "hg_zones_destroy": [_P],
    "hg_zones_update": [_P, _i64, _D, _D, _U8, _i64, _D],
    "hg_zones_grid_info": [_P, _I32, _I32],
    "hg_zones_fields": [_P, _D, _D, _I32, _I32],
    "hg_zones_set_labels": [_P, _I32],
    "hg_zones_list": [_P, _i32, _i64, _D, _I32, _I64],
    "hg_zones_to_delete": [_P, _i32, _i64, _D, _i32, _U8, _i64, _I32, _I64],
    "hg_zones_weights": [_P, _i32, _i64, _D, _i32, _D],
    "hg_zones_boundary_samples": [_P, _I64],
    "hg_zones_disk_box_area": [_dbl, _dbl, _dbl, _dbl, _dbl, _dbl, _dbl],
    "hg_resampler_create": [ctypes.POINTER(ResamplerDesc), _PP],
    "hg_resampler_destroy": [_P],
    "hg_resampler_set_points": [_P, _i64, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, _I32, _U8],
    "hg_resampler_set_grains": [_P, _i64, _D, _D, _D, _D, _D, _U8],
    "hg_resampler_set_homogenized": [_P, _D, _D],
    "hg_resampler_run": [_P, _P],
    "hg_resampler_counts": [_P, _I64, _I64, ctypes.POINTER(ResamplerStats)],
    "hg_resampler_get_points": [_P, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, _I32, _U8],
    "hg_resampler_get_grains": [_P, _D, _D, _D, _D, _D, _D, _U8, _I32],
    "hg_resampler_dem_map_size": [_P, _I64],
    "hg_resampler_random_u32": [_P],
    "hg_resampler_random_f32": [_P],
    "hg_resampler_random_radius": [_P],
    "hg_dem_create": [_P, ctypes.POINTER(DemDesc), _PP],
    "hg_dem_upload_relabel": [_P, _i64, _D, _D, _D, _D, _D, _U8, _i64, _I32],
    "hg_dem_edit_async": [_P, _i64, _I32, _i64, _D, _D, _D, _D, _D, _U8],
    "hg_dem_frame_async": [_P, _D, _D],
    "hg_dem_num_bodies": [_P, _I64],
    "hg_dem_destroy": [_P],
    "hg_dem_upload": [_P, _i64, _D, _D, _D, _D, _D, _U8],
    "hg_dem_set_weights": [_P, _D],
    "hg_dem_set_state": [_P, _D, _D],
    "hg_dem_download": [_P, _D, _D],
    "hg_dem_step": [_P, _dbl, _i32, _i32],
    "hg_dem_num_contacts": [_P, _I64],
    "hg_dem_download_contacts": [_P, _i64, _D, _I64],
    "hg_dem_status": [_P, _U32],
    "hg_dem_candidate_pairs": [_P, _i64, _D, _D, _i64, _I32, _I64],
    "hg_dem_candidate_pairs_static": [_P, _i64, _D, _D, _i64, _I32, _I64],
    "hg_hybrid_create": [_P, _P, _P, _PP],
    "hg_hybrid_destroy": [_P],
    "hg_hybrid_step": [_P, _dbl, _i32, _i32],
    "hg_hybrid_clear_homogenized": [_P],
    "hg_hybrid_num_packed": [_P, _I64, _I64],
    "hg_hybrid_download": [_P, _I32, _I32, _D, _D, _D, _D, _D, _D, _D],
}
_RET = {"hg_status_string": ctypes.c_char_p, "hg_last_error": ctypes.c_char_p,
        "hg_zones_disk_box_area": ctypes.c_double,
        "hg_resampler_random_u32": ctypes.c_uint32, "hg_resampler_random_f32": ctypes.c_float,
        "hg_resampler_random_radius": ctypes.c_double,
        "hg_kernel_launch_count": ctypes.c_int64}

_lib = None


def declared_symbols():
    """Names of the entry points declared in include/hg_gpu.h."""
    import re
    hdr = os.path.join(os.path.dirname(HERE), "include", "hg_gpu.h")
    with open(hdr) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(hg_[a-z0-9_]+)\s*\(", text)))


def load(path=None):
    """Load libhg_gpu.so and bind every declared entry point; raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError("libhg_gpu.so not built (%s): run __graft_entry__.build() or "
                           "python libhybridgrains_gb300/build.py" % path)
    lib = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RET.get(name, ctypes.c_int32)
    _lib = lib
    return lib


class HGError(RuntimeError):
    def __init__(self, fn, status, msg):
        super().__init__("%s failed: %s (%s)" % (fn, STATUS.get(status, status), msg))
        self.status = status


def check(fn, *args):
    """Call an hg_* entry point and raise HGError on a non-zero status."""
    lib = load()
    st = getattr(lib, fn)(*args)
    if st != 0:
        msg = lib.hg_last_error()
        raise HGError(fn, st, msg.decode() if msg else "")
    return st
