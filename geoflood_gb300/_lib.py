"""ctypes binding of ``libgeoflood_gb300.so`` (the C ABI in include/geoflood_gb300.h).

The library is the only compute path: if it is missing this module raises
instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libgeoflood_gb300.so"

GF_OK = 0
GF_MAX_MANNING = 4
GF_MAX_PHYS = 1024

STATUS_NAMES = {
    0: "GF_OK", -1: "GF_ERR_ARG", -2: "GF_ERR_CUDA", -3: "GF_ERR_NOMEM",
    -4: "GF_ERR_DEVICE", -5: "GF_ERR_STATE", -6: "GF_ERR_UNSUPPORTED",
}


class gf_qad_task(C.Structure):
    _fields_ = [("fine", C.c_int), ("coarse", C.c_int), ("side", C.c_int), ("ox", C.c_int),
                ("oy", C.c_int)]


class gf_phys(C.Structure):
    _fields_ = [
        ("grav", C.c_double),
        ("dry_tolerance", C.c_double),
        ("sea_level", C.c_double),
        ("friction_depth", C.c_double),
        ("manning_coefficient", C.c_double * GF_MAX_MANNING),
        ("manning_break", C.c_double * GF_MAX_MANNING),
        ("num_manning", C.c_int),
        ("friction_forcing", C.c_int),
        ("variable_friction", C.c_int),
        ("friction_index", C.c_int),
        ("order", C.c_int),
        ("transverse", C.c_int),
        ("mthlim", C.c_int * 3),
        ("src_term", C.c_int),
        ("maxcfl_cap", C.c_double),
    ]


class gf_region(C.Structure):
    _fields_ = [("x_low", C.c_double), ("x_hi", C.c_double), ("y_low", C.c_double),
                ("y_hi", C.c_double), ("t_low", C.c_double), ("t_hi", C.c_double),
                ("min_level", C.c_int), ("max_level", C.c_int)]


class gf_refine(C.Structure):
    _fields_ = [("wave_tolerance", C.c_double), ("speed_tolerance", C.c_double * 8),
                ("num_speed_tolerance", C.c_int), ("deep_depth", C.c_double),
                ("max_level_deep", C.c_int), ("max_velocity_depth_product", C.c_double),
                ("num_flowgrades", C.c_int), ("flowgradevalue", C.c_double * 4),
                ("flowgradevariable", C.c_int * 4), ("flowgradetype", C.c_int * 4),
                ("flowgrademinlevel", C.c_int * 4), ("num_regions", C.c_int),
                ("regions", gf_region * 16)]


class gf_transfer(C.Structure):
    _fields_ = [("kind", C.c_int), ("coarse", C.c_int), ("fine", C.c_int), ("code", C.c_int),
                ("ox", C.c_int), ("oy", C.c_int)]


GF_SERVER_MAX_LANES = 4
SCEN_QUEUED, SCEN_ACTIVE, SCEN_DONE, SCEN_FAILED, SCEN_CANCELLED = 0, 1, 2, 3, 4
SCEN_STATE_NAMES = {0: "queued", 1: "active", 2: "done", 3: "failed", 4: "cancelled"}


class gf_scenario(C.Structure):
    _fields_ = [("mx", C.c_int), ("npx", C.c_int), ("npy", C.c_int), ("maux", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("xlower", C.c_double),
                ("ylower", C.c_double), ("q", C.c_void_p), ("aux", C.c_void_p),
                ("q_out", C.c_void_p), ("phys", gf_phys), ("mthbc", C.c_int * 4),
                ("hydro_side", C.c_int * 4), ("nhydro", C.c_int), ("hydro_time", C.c_void_p),
                ("hydro_hu", C.c_void_p), ("hydro_width", C.c_double), ("hydro_x0", C.c_double),
                ("hydro_y0", C.c_double), ("t_final", C.c_double), ("nout", C.c_int),
                ("initial_dt", C.c_double), ("desired_cfl", C.c_double),
                ("max_cfl", C.c_double)]


class gf_server_opts(C.Structure):
    _fields_ = [("hbm_budget", C.c_size_t), ("max_active", C.c_int), ("nlanes", C.c_int),
                ("lane_cells", C.c_longlong * GF_SERVER_MAX_LANES), ("priority", C.c_int),
                ("backfill", C.c_int), ("reserve_sms", C.c_int), ("mixed_update", C.c_int),
                ("cull_dry", C.c_int), ("split_sizes", C.c_int)]


class gf_scenario_info(C.Structure):
    _fields_ = [("state", C.c_int), ("lane", C.c_int), ("steps", C.c_longlong),
                ("rejects", C.c_longlong), ("cell_updates", C.c_longlong), ("t", C.c_double),
                ("dt", C.c_double), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double), ("max_cfl_seen", C.c_double),
                ("device_bytes", C.c_size_t)]


class gf_server_stats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("admitted", C.c_longlong), ("done", C.c_longlong),
                ("rounds", C.c_longlong), ("launches", C.c_longlong),
                ("cell_updates", C.c_longlong), ("bytes_in_use", C.c_size_t),
                ("bytes_peak", C.c_size_t), ("active", C.c_int), ("queued", C.c_int)]


class gf_forest_opts(C.Structure):
    _fields_ = [("mx", C.c_int), ("maux", C.c_int), ("nbx", C.c_int), ("nby", C.c_int),
                ("minlevel", C.c_int), ("maxlevel", C.c_int), ("x0", C.c_double),
                ("y0", C.c_double), ("dx0", C.c_double), ("dy0", C.c_double),
                ("phys_slot", C.c_int), ("mthbc", C.c_int * 4), ("regrid_interval", C.c_int),
                ("max_patches", C.c_int), ("refine", gf_refine), ("subcycle", C.c_int)]


class gf_forest_stats(C.Structure):
    _fields_ = [("steps", C.c_longlong), ("rejects", C.c_longlong), ("regrids", C.c_longlong),
                ("cell_updates", C.c_longlong), ("t", C.c_double), ("dt", C.c_double),
                ("max_cfl_seen", C.c_double), ("npatch", C.c_int), ("npatch_max", C.c_int),
                ("levels_used", C.c_int)]


class gf_forest_batch_stats(C.Structure):
    _fields_ = [("rounds", C.c_longlong), ("epochs", C.c_longlong), ("regrids", C.c_longlong),
                ("launches", C.c_longlong), ("cell_updates", C.c_longlong),
                ("s_rounds", C.c_double), ("s_regrid", C.c_double), ("s_epoch", C.c_double)]


class gf_forest_request(C.Structure):
    _fields_ = [("opts", gf_forest_opts), ("phys", gf_phys), ("fields", C.c_void_p),
                ("topo", C.c_void_p), ("qinit", C.c_int), ("nhydro", C.c_int),
                ("hydro_time", C.c_void_p), ("hydro_hu", C.c_void_p), ("hydro_side", C.c_int * 4),
                ("hydro_width", C.c_double), ("hydro_x0", C.c_double), ("hydro_y0", C.c_double),
                ("t_final", C.c_double), ("nout", C.c_int), ("initial_dt", C.c_double),
                ("desired_cfl", C.c_double), ("max_cfl", C.c_double)]


class gf_fserver_opts(C.Structure):
    _fields_ = [("hbm_budget", C.c_size_t), ("max_active", C.c_int), ("backfill", C.c_int),
                ("lane_cells", C.c_longlong * 2), ("reserve_sms", C.c_int)]


class gf_forest_request_info(C.Structure):
    _fields_ = [("state", C.c_int), ("steps", C.c_longlong), ("rejects", C.c_longlong),
                ("regrids", C.c_longlong), ("cell_updates", C.c_longlong), ("t", C.c_double),
                ("dt", C.c_double), ("max_cfl_seen", C.c_double), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_done", C.c_double), ("npatch", C.c_int),
                ("npatch_max", C.c_int), ("footprint", C.c_size_t), ("device_bytes", C.c_size_t),
                ("lane", C.c_int)]


class gf_fserver_stats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("admitted", C.c_longlong), ("done", C.c_longlong),
                ("failed", C.c_longlong), ("lane_admitted", C.c_longlong * 4),
                ("iterations", C.c_longlong), ("epochs", C.c_longlong),
                ("rounds", C.c_longlong), ("launches", C.c_longlong), ("regrids", C.c_longlong),
                ("cell_updates", C.c_longlong), ("sub_steps", C.c_longlong),
                ("s_admit", C.c_double), ("s_epoch", C.c_double),
                ("s_rounds", C.c_double), ("s_regrid", C.c_double), ("bytes_in_use", C.c_size_t),
                ("bytes_peak", C.c_size_t), ("active", C.c_int), ("queued", C.c_int),
                ("held", C.c_int)]


GF_MAX_TILES = 12


class gf_tile_result(C.Structure):
    _fields_ = [("mx", C.c_int), ("nvariant", C.c_int), ("threads", C.c_int * GF_MAX_TILES),
                ("band", C.c_int * GF_MAX_TILES), ("cluster", C.c_int * GF_MAX_TILES),
                ("throughput", C.c_double * GF_MAX_TILES),
                ("latency_us", C.c_double * GF_MAX_TILES), ("best_throughput", C.c_int),
                ("best_latency", C.c_int)]


XFER_AVG_FACE, XFER_AVG_CORNER, XFER_INTERP_FACE = 0, 1, 2
XFER_INTERP_CORNER, XFER_INTERP2FINE, XFER_AVG2COARSE = 3, 4, 5

_dp = C.POINTER(C.c_double)
_vp = C.c_void_p

# (name, restype, argtypes) for every exported entry point.
SIGNATURES = [
    ("gf_phys_default", None, [C.POINTER(gf_phys)]),
    ("gf_ctx_create", C.c_int, [C.c_int, C.POINTER(_vp)]),
    ("gf_ctx_destroy", None, [_vp]),
    ("gf_ctx_last_error", C.c_char_p, [_vp]),
    ("gf_ctx_set_phys", C.c_int, [_vp, C.c_int, C.POINTER(gf_phys)]),
    ("gf_patch_update", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                  C.c_double, C.c_double, C.c_double, _dp, _dp, _dp]),
    ("gf_patch_update_batch", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                        _dp, _dp, C.c_double, C.c_double, C.POINTER(_dp),
                                        C.POINTER(_dp), _dp, _dp]),
    ("gf_step_buffer_create", C.c_int, [_vp, C.c_int, C.POINTER(_vp)]),
    ("gf_step_buffer_destroy", None, [_vp]),
    ("gf_step_buffer_update", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                        _dp, _dp, _dp]),
    ("gf_level_create", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(_vp)]),
    ("gf_level_destroy", None, [_vp]),
    ("gf_level_set_geometry", C.c_int, [_vp, _dp, _dp, C.POINTER(C.c_int)]),
    ("gf_level_upload", C.c_int, [_vp, _dp, _dp]),
    ("gf_level_download", C.c_int, [_vp, _dp]),
    ("gf_level_download_aux", C.c_int, [_vp, _dp]),
    ("gf_level_step", C.c_int, [_vp, C.c_double, C.c_double, _dp]),
    ("gf_level_step_host", C.c_int, [_vp, _dp, C.c_double, C.c_double, _dp]),
    ("gf_level_set_pipeline", C.c_int, [_vp, C.c_int]),
    ("gf_level_step_async", C.c_int, [_vp, C.c_double, C.c_double]),
    ("gf_level_sync", C.c_int, [_vp, _dp]),
    ("gf_ctx_stream", C.c_int, [_vp, C.POINTER(_vp)]),
    ("gf_ctx_set_fp_contract", C.c_int, [_vp, C.c_int]),
    ("gf_ctx_set_mixed_update", C.c_int, [_vp, C.c_int]),
    ("gf_level_patch_cfl", C.c_int, [_vp, _dp]),
    ("gf_level_set_layout", C.c_int, [_vp, C.POINTER(C.c_int), _dp, _dp]),
    ("gf_level_set_bc", C.c_int, [_vp, C.POINTER(C.c_int)]),
    ("gf_level_set_hydrograph", C.c_int, [_vp, C.c_int, _dp, _dp, C.POINTER(C.c_int), C.c_double,
                                          C.c_double, C.c_double]),
    ("gf_level_ghost_fill", C.c_int, [_vp, C.c_double]),
    ("gf_level_ghost_fill_async", C.c_int, [_vp, C.c_double]),
    ("gf_measure_fp64_rates", C.c_int, [C.c_int, _dp]),
    ("gf_level_transfer", C.c_int, [_vp, _vp, C.c_int, C.POINTER(gf_transfer)]),
    ("gf_level_timeinterp", C.c_int, [_vp, _vp, _vp, C.c_double]),
    ("gf_level_qad", C.c_int, [_vp, _vp, C.c_int, C.POINTER(gf_qad_task), C.c_double, _dp]),
    ("gf_level_tag4refinement", C.c_int, [_vp, C.POINTER(gf_refine), C.c_int, C.c_int, C.c_int,
                                          C.c_double, C.POINTER(C.c_int)]),
    ("gf_level_tag4coarsening", C.c_int, [_vp, C.POINTER(gf_refine), C.c_int,
                                          C.POINTER(C.c_int), C.c_int, C.c_int, C.c_int,
                                          C.c_double, C.POINTER(C.c_int)]),
    ("gf_patch_update_noalloc", C.c_int, [C.c_int, C.POINTER(gf_phys), C.c_int, C.c_int, C.c_int,
                                          C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_double,
                                          C.c_void_p, C.c_void_p, _dp, _dp, C.c_void_p]),
    ("gf_level_device_planes", C.c_int, [_vp, C.POINTER(_dp), C.POINTER(_dp)]),
    ("gf_forest_opts_default", None, [C.POINTER(gf_forest_opts)]),
    ("gf_forest_create", C.c_int, [_vp, C.POINTER(gf_forest_opts), _dp, C.POINTER(_vp)]),
    ("gf_forest_destroy", None, [_vp]),
    ("gf_forest_set_hydrograph", C.c_int, [_vp, C.c_int, _dp, _dp, C.POINTER(C.c_int),
                                           C.c_double, C.c_double, C.c_double]),
    ("gf_forest_init", C.c_int, [_vp]),
    ("gf_forest_ghost_fill", C.c_int, [_vp, C.c_double]),
    ("gf_forest_step", C.c_int, [_vp, C.c_double, C.c_double, _dp]),
    ("gf_forest_accept", C.c_int, [_vp, C.c_int]),
    ("gf_forest_regrid", C.c_int, [_vp, C.c_double, C.POINTER(C.c_int)]),
    ("gf_forest_run", C.c_int, [_vp, C.c_double, C.c_int, C.c_double, C.c_double, C.c_double,
                                C.c_int, C.POINTER(gf_forest_stats)]),
    ("gf_forest_get_stats", C.c_int, [_vp, C.POINTER(gf_forest_stats)]),
    ("gf_forest_npatch", C.c_int, [_vp]),
    ("gf_forest_patches", C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                    C.POINTER(C.c_int)]),
    ("gf_forest_download", C.c_int, [_vp, _dp]),
    ("gf_forest_download_aux", C.c_int, [_vp, _dp]),
    ("gf_forest_upload", C.c_int, [_vp, _dp]),
    ("gf_forest_batch_run", C.c_int, [C.POINTER(_vp), C.c_int, C.c_double, C.c_int, C.c_double,
                                      C.c_double, C.c_double, C.POINTER(gf_forest_batch_stats)]),
    ("gf_topo_create", C.c_int, [C.POINTER(_vp)]),
    ("gf_topo_destroy", None, [_vp]),
    ("gf_topo_set_missing", C.c_int, [_vp, C.c_double]),
    ("gf_topo_read_file", C.c_int, [_vp, C.c_char_p, C.c_int]),
    ("gf_topo_read_data", C.c_int, [_vp, C.c_char_p]),
    ("gf_topo_add_grid", C.c_int, [_vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                   C.c_double, _dp]),
    ("gf_topo_count", C.c_int, [_vp]),
    ("gf_topo_grid_info", C.c_int, [_vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), _dp, _dp,
                                    _dp, _dp, _dp, _dp, _dp]),
    ("gf_topo_covered_area", C.c_int, [_vp, C.c_double, C.c_double, C.c_double, C.c_double, _dp]),
    ("gf_topo_raster", C.c_int, [_vp, _vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                 C.c_double, C.c_double, C.c_double, C.c_double, _dp]),
    ("gf_forest_set_topo", C.c_int, [_vp, _vp, C.c_int]),
    ("gf_write_ascii_frame", C.c_int, [C.c_char_p, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int,
                                       _dp, _dp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                       C.POINTER(C.c_int), _dp, _dp, _dp, _dp]),
    ("gf_sample_gauge", C.c_int, [C.c_int, C.c_int, _dp, _dp, C.c_double, C.c_double, C.c_double,
                                  C.c_double, C.c_double, C.c_double, C.c_double, _dp]),
    ("gf_write_gauge_header", C.c_int, [C.c_char_p, C.c_int, C.c_double, C.c_double]),
    ("gf_write_gauge_rows", C.c_int, [C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_int), _dp, _dp]),
    ("gf_read_gauges_data", C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      _dp, _dp, _dp, _dp, _dp]),
    ("gf_forest_write_ascii", C.c_int, [_vp, C.c_char_p, C.c_int]),
    ("gf_forest_set_output", C.c_int, [_vp, C.c_char_p, C.c_int]),
    ("gf_forest_set_gauges", C.c_int, [_vp, C.c_int, C.POINTER(C.c_int), _dp, _dp, _dp, _dp, _dp]),
    ("gf_forest_sample_gauges", C.c_int, [_vp, C.c_double]),
    ("gf_forest_flush_gauges", C.c_int, [_vp]),
    ("gf_autotune", C.c_int, [_vp, C.c_int, C.POINTER(gf_tile_result)]),
    ("gf_tile_count", C.c_int, [C.c_int]),
    ("gf_tile_get", C.c_int, [C.c_int, C.c_int]),
    ("gf_tile_set", C.c_int, [C.c_int, C.c_int, C.c_int]),
    ("gf_server_opts_default", None, [C.POINTER(gf_server_opts)]),
    ("gf_server_create", C.c_int, [C.c_int, C.POINTER(gf_server_opts), C.POINTER(_vp)]),
    ("gf_server_destroy", None, [_vp]),
    ("gf_server_last_error", C.c_char_p, [_vp]),
    ("gf_scenario_footprint", C.c_size_t, [C.POINTER(gf_scenario)]),
    ("gf_server_submit", C.c_int, [_vp, C.POINTER(gf_scenario), C.POINTER(C.c_longlong)]),
    ("gf_server_pump", C.c_int, [_vp, C.POINTER(C.c_int)]),
    ("gf_server_start", C.c_int, [_vp]),
    ("gf_server_stop", C.c_int, [_vp]),
    ("gf_server_wait", C.c_int, [_vp, C.c_longlong, C.c_double]),
    ("gf_server_poll", C.c_int, [_vp, C.c_longlong, C.POINTER(gf_scenario_info)]),
    ("gf_server_cancel", C.c_int, [_vp, C.c_longlong]),
    ("gf_server_stats_get", C.c_int, [_vp, C.POINTER(gf_server_stats)]),
    ("gf_server_clock", C.c_double, [_vp]),
    ("gf_forest_footprint", C.c_size_t, [C.POINTER(gf_forest_opts)]),
    ("gf_probe_bounded_wait", C.c_int, [C.c_int, C.c_int, C.c_uint, C.POINTER(C.c_int), _dp]),
    ("gf_fserver_opts_default", None, [C.POINTER(gf_fserver_opts)]),
    ("gf_fserver_create", C.c_int, [C.c_int, C.POINTER(gf_fserver_opts), C.POINTER(_vp)]),
    ("gf_fserver_destroy", None, [_vp]),
    ("gf_fserver_last_error", C.c_char_p, [_vp]),
    ("gf_fserver_ctx", _vp, [_vp]),
    ("gf_fserver_submit", C.c_int, [_vp, C.POINTER(gf_forest_request), C.POINTER(C.c_longlong)]),
    ("gf_fserver_pump", C.c_int, [_vp, C.POINTER(C.c_int)]),
    ("gf_fserver_start", C.c_int, [_vp]),
    ("gf_fserver_stop", C.c_int, [_vp]),
    ("gf_fserver_wait", C.c_int, [_vp, C.c_longlong, C.c_double]),
    ("gf_fserver_poll", C.c_int, [_vp, C.c_longlong, C.POINTER(gf_forest_request_info)]),
    ("gf_fserver_cancel", C.c_int, [_vp, C.c_longlong]),
    ("gf_fserver_forest", C.c_int, [_vp, C.c_longlong, C.POINTER(_vp)]),
    ("gf_fserver_download", C.c_int, [_vp, C.c_longlong, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.POINTER(C.c_int), C.POINTER(C.c_int), _dp, _dp]),
    ("gf_fserver_release", C.c_int, [_vp, C.c_longlong]),
    ("gf_fserver_stats_get", C.c_int, [_vp, C.POINTER(gf_fserver_stats)]),
    ("gf_fserver_clock", C.c_double, [_vp]),
]

_lib = None


def load() -> C.CDLL:
    """Load the CUDA library; raise if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"{LIB_PATH.name} is not built; run geoflood_gb300.build.build() "
            "(the CUDA library is the only compute path)")
    lib = C.CDLL(str(LIB_PATH))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def dptr(a: np.ndarray | None):
    """Pointer to a C-contiguous float64 array (or NULL)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], "need contiguous float64"
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_int))
