"""ctypes binding of ``libgpuocean_gb300.so`` (declared in ``include/gpuocean_gb300.h``).

The library is built in-tree (``python -m gpuocean_gb300.build_lib``).  There
is no fallback: if it is missing, every simulator call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgpuocean_gb300.so")

c_int, c_float, c_void_p, c_size_t = ctypes.c_int, ctypes.c_float, ctypes.c_void_p, ctypes.c_size_t
c_fp = ctypes.POINTER(ctypes.c_float)
c_i64 = ctypes.c_int64


class GocDriftWindDesc(ctypes.Structure):
    """Mirror of ``GocDriftWindDesc`` in include/gpuocean_gb300.h."""
    _fields_ = [("x_current", c_void_p), ("x_next", c_void_p), ("y_current", c_void_p), ("y_next", c_void_p),
                ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("wind_drift_factor", c_float)]


class GocCdklmParams(ctypes.Structure):
    """Mirror of ``GocCdklmParams`` in include/gpuocean_gb300.h."""
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
        ("dx", c_float), ("dy", c_float), ("g", c_float), ("r", c_float),
        ("theta", c_float), ("desing_eps", c_float), ("flux_slope_eps", c_float),
        ("depth_cutoff", c_float), ("flux_balancer", c_float), ("rho_o", c_float),
        ("wind_stress_factor", c_float),
        ("rk_order", ctypes.c_int32), ("one_dimensional", ctypes.c_int32),
        ("bc_north", ctypes.c_int32), ("bc_east", ctypes.c_int32),
        ("bc_south", ctypes.c_int32), ("bc_west", ctypes.c_int32),
        ("land_value", c_float),
        ("coriolis_f", c_void_p), ("coriolis_nx", ctypes.c_int32), ("coriolis_ny", ctypes.c_int32),
        ("coriolis_cell", c_void_p), ("coriolis_cell_pitch", ctypes.c_int32),
        ("angle", c_void_p), ("angle_nx", ctypes.c_int32), ("angle_ny", ctypes.c_int32),
        ("wind_x_cur", c_void_p), ("wind_x_next", c_void_p),
        ("wind_x_nx", ctypes.c_int32), ("wind_x_ny", ctypes.c_int32),
        ("wind_y_cur", c_void_p), ("wind_y_next", c_void_p),
        ("wind_y_nx", ctypes.c_int32), ("wind_y_ny", ctypes.c_int32),
        ("wind_t", c_float),
        ("atm_p_cur", c_void_p), ("atm_p_next", c_void_p),
        ("atm_p_nx", ctypes.c_int32), ("atm_p_ny", ctypes.c_int32),
        ("atm_p_t", c_float),
    ]


# name -> (restype, argtypes)
SIGNATURES = {
    "goc_version": (c_int, []),
    "goc_last_error": (c_int, [ctypes.c_char_p, c_int]),
    "goc_device_count": (c_int, [ctypes.POINTER(c_int)]),
    "goc_set_device": (c_int, [c_int]),
    "goc_device_synchronize": (c_int, []),
    "goc_malloc": (c_int, [ctypes.POINTER(c_void_p), c_size_t]),
    "goc_free": (c_int, [c_void_p]),
    "goc_host_alloc": (c_int, [ctypes.POINTER(c_void_p), c_size_t]),
    "goc_host_free": (c_int, [c_void_p]),
    "goc_memset_async": (c_int, [c_void_p, c_int, c_size_t, c_void_p]),
    "goc_memcpy_h2d_async": (c_int, [c_void_p, c_void_p, c_size_t, c_void_p]),
    "goc_memcpy_d2h_async": (c_int, [c_void_p, c_void_p, c_size_t, c_void_p]),
    "goc_memcpy_d2d_async": (c_int, [c_void_p, c_void_p, c_size_t, c_void_p]),
    "goc_stream_create": (c_int, [ctypes.POINTER(c_void_p)]),
    "goc_stream_destroy": (c_int, [c_void_p]),
    "goc_stream_synchronize": (c_int, [c_void_p]),
    "goc_event_create": (c_int, [ctypes.POINTER(c_void_p)]),
    "goc_event_destroy": (c_int, [c_void_p]),
    "goc_event_record": (c_int, [c_void_p, c_void_p]),
    "goc_stream_fan_out": (c_int, [c_void_p, c_void_p, c_int]),
    "goc_stream_fan_in": (c_int, [c_void_p, c_void_p, c_int]),
    "goc_event_elapsed_ms": (c_int, [c_void_p, c_void_p, ctypes.POINTER(c_float)]),
    "goc_graph_begin_capture": (c_int, [c_void_p]),
    "goc_graph_end_capture": (c_int, [c_void_p, ctypes.POINTER(c_void_p)]),
    "goc_graph_launch": (c_int, [c_void_p, c_void_p]),
    "goc_graph_destroy": (c_int, [c_void_p]),
    "goc_kernel_launch_count": (c_i64, []),
    "goc_cdklm_rk2_step": (c_int, [ctypes.POINTER(GocCdklmParams), c_float,
                                   c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int,
                                   c_void_p, c_int, c_void_p, c_int, c_void_p]),
    "goc_cdklm_rk2_steps": (c_int, [ctypes.POINTER(GocCdklmParams), c_void_p, c_int] + [c_void_p] * 6 +
                            [c_int, c_void_p, c_int, c_void_p, c_int, c_void_p]),
    "goc_cdklm_rk2_step_stage": (c_int, [ctypes.POINTER(GocCdklmParams), c_float] + [c_void_p] * 9 +
                                 [c_int, c_void_p, c_int, c_void_p, c_int, c_void_p]),
    "goc_cdklm_stage": (c_int, [ctypes.POINTER(GocCdklmParams), c_float, c_int,
                                c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p, c_int, c_void_p]),
    "goc_cell_texture": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_int, c_void_p]),
    "goc_periodic_ghosts": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    "goc_bathymetry_init": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_float,
                                    c_void_p, c_int, c_void_p, c_int, c_void_p]),
    "goc_max_dt_partials": (c_int, [c_int, c_int]),
    "goc_max_dt": (c_int, [c_int, c_int, c_float, c_float, c_float, c_void_p, c_void_p, c_void_p, c_int,
                           c_void_p, c_int, c_float, c_void_p, c_int, c_void_p, c_void_p]),
    "goc_max_dt_noalloc_capacity": (c_int, []),
    "goc_max_dt_noalloc": (c_int, [c_int, c_int, c_float, c_float, c_float, c_void_p, c_void_p, c_void_p, c_int,
                                   c_void_p, c_int, c_float, c_void_p, c_void_p]),
    "goc_cdklm_vjp_partials": (c_int, [c_int, c_int]),
    "goc_cdklm_rk2_step_members": (c_int, [ctypes.POINTER(GocCdklmParams), c_float] + [c_void_p] * 9 +
                                   [c_int, ctypes.c_longlong, c_int, c_int, c_void_p, c_int, c_void_p, c_int, c_void_p]),
    "goc_cdklm_stage_vjp_members": (c_int, [ctypes.POINTER(GocCdklmParams), c_float, c_int] + [c_void_p] * 18 +
                                    [c_int, ctypes.c_longlong, c_int, c_int, c_void_p, c_int, c_void_p, c_int,
                                     c_void_p, c_void_p]),
    "goc_cdklm_stage_vjp": (c_int, [ctypes.POINTER(GocCdklmParams), c_float, c_int] + [c_void_p] * 18 +
                            [c_int, c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p]),
    "goc_cdklm_stage_vjp_out": (c_int, [ctypes.POINTER(GocCdklmParams), c_float, c_int] + [c_void_p] * 21 +
                                [c_int, c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p]),
    "goc_cdklm_stage_vjp_members_out": (c_int, [ctypes.POINTER(GocCdklmParams), c_float, c_int] + [c_void_p] * 21 +
                                        [c_int, ctypes.c_longlong, c_int, c_int, c_void_p, c_int, c_void_p, c_int,
                                         c_void_p, c_void_p]),
    "goc_drift": (c_int, [c_int, c_int, c_float, c_float, c_float, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int,
                          c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_int, c_float,
                          c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_float, c_float, c_void_p]),
    "goc_drift_vjp": (c_int, [c_int, c_int, c_float, c_float, c_float, c_int, c_int, c_void_p, c_void_p, c_void_p,
                              c_int, c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_int, c_void_p, c_int, c_float,
                              c_void_p, c_void_p, c_void_p, c_void_p]),
    "goc_drift_enforce_boundary": (c_int, [c_float, c_float, c_int, c_int, c_int, c_void_p, c_int, c_void_p]),
    "goc_sponge_boundary": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_int, c_float,
                                    c_void_p]),
    "goc_kl_table_floats": (ctypes.c_longlong, [c_int, c_int, c_void_p]),
    "goc_kl_perturb": (c_int, [c_void_p, c_int, c_int, c_float, c_float, c_float, c_int, c_void_p, c_void_p, c_void_p,
                               c_int, c_void_p, c_int, c_int, c_int, c_void_p]),
    "goc_kl_batch_create": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    "goc_kl_batch_destroy": (c_int, [c_void_p]),
    "goc_kl_batch_seed": (c_int, [c_void_p, ctypes.c_ulonglong, c_void_p]),
    "goc_kl_batch_generate": (c_int, [c_void_p, c_void_p, c_int, c_void_p]),
    "goc_kl_batch_set_rollers": (c_int, [c_void_p, c_void_p, c_int, c_void_p]),
    "goc_kl_batch_set_random": (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
    "goc_kl_batch_perturb": (c_int, [c_void_p, c_void_p, c_float, c_int, c_void_p]),
    "goc_ensemble_drifter_rows": (c_int, [c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "goc_ensemble_gather_drifters": (c_int, [c_void_p, c_void_p, c_void_p]),
    "goc_ensemble_scatter_observations": (c_int, [c_void_p, c_void_p, c_void_p]),
    "goc_observe_underlying_flow": (c_int, [c_int, c_int, c_float, c_float, c_int, c_int, c_void_p, c_int, c_void_p,
                                            c_int, c_void_p, c_int, c_float, c_int, c_void_p, c_int, c_void_p, c_int,
                                            c_void_p]),
    "goc_ensemble_observe": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int, ctypes.c_longlong, c_int, c_void_p,
                                     c_void_p]),
    "goc_ensemble_moments": (c_int, [c_void_p, c_int, c_int, c_int, c_float, c_int, c_void_p, c_void_p, c_void_p]),
    "goc_ml_combine": (c_int, [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p]),
    "goc_ensemble_create": (c_int, [c_void_p, c_int, c_int, ctypes.POINTER(c_void_p)]),
    "goc_ensemble_destroy": (c_int, [c_void_p]),
    "goc_ensemble_size": (c_int, [c_void_p, ctypes.POINTER(c_int), ctypes.POINTER(c_int)]),
    "goc_ensemble_staging_errors": (c_int, [c_void_p, ctypes.POINTER(c_int)]),
    "goc_ensemble_tma_status": (c_int, [c_void_p, ctypes.POINTER(c_int), ctypes.POINTER(ctypes.c_longlong),
                                        ctypes.POINTER(c_int)]),
    "goc_selftest_wait_timeout": (c_int, [ctypes.c_double, ctypes.POINTER(c_int), ctypes.POINTER(ctypes.c_double)]),
    "goc_ensemble_set_schedule": (c_int, [c_void_p, c_fp, ctypes.POINTER(c_int), c_void_p]),
    "goc_ensemble_rk2_substep": (c_int, [c_void_p, c_int, c_void_p]),
    "goc_ensemble_end_block": (c_int, [c_void_p, c_int, c_void_p]),
    "goc_ensemble_tile_shape_count": (c_int, []),
    "goc_ensemble_tile_shape": (c_int, [c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int)]),
    "goc_ensemble_set_tile_shape": (c_int, [c_void_p, c_int]),
    "goc_ensemble_get_tile_shape": (c_int, [c_void_p, ctypes.POINTER(c_int)]),
    "goc_ensemble_get_member": (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
    "goc_ensemble_max_dt": (c_int, [c_void_p, c_void_p, c_void_p]),
    "goc_ensemble_set_drifters": (c_int, [c_void_p, c_void_p, ctypes.POINTER(c_int), c_float, c_void_p]),
    "goc_ensemble_set_drift_wind": (c_int, [c_void_p, c_void_p, c_void_p]),
    "goc_ensemble_set_wind_times": (c_int, [c_void_p, c_void_p, c_void_p]),
    "goc_lcg_fill": (c_int, [c_int, c_int, c_int, c_void_p, c_int, c_void_p, c_int, c_int, c_void_p]),
    "goc_xorwow_state_bytes": (c_size_t, [c_int]),
    "goc_xorwow_init": (c_int, [c_void_p, c_int, ctypes.c_ulonglong, c_void_p]),
    "goc_xorwow_normal": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int, c_void_p]),
    "goc_soar": (c_int, [c_void_p, c_float, c_int, c_void_p]),
    "goc_perturb_ocean": (c_int, [c_void_p, c_int, c_int, c_float, c_float, c_void_p, c_void_p, c_void_p, c_int,
                                  c_void_p, c_int, c_float, c_int, c_void_p]),
    "goc_noise_batch_create": (c_int, [c_void_p, c_void_p, ctypes.POINTER(c_void_p)]),
    "goc_noise_batch_destroy": (c_int, [c_void_p]),
    "goc_noise_batch_perturb": (c_int, [c_void_p, c_void_p, c_float, c_int, c_void_p]),
    "goc_noise_batch_field": (c_int, [c_void_p, c_void_p, c_float, c_int, c_void_p]),
    "goc_ensemble_set_block_noise": (c_int, [c_void_p, c_void_p, c_int]),
    "goc_ensemble_set_noise_mask": (c_int, [c_void_p, c_void_p, c_void_p]),
    "goc_noise_batch_seed": (c_int, [c_void_p, ctypes.c_ulonglong, c_void_p]),
    "goc_noise_batch_generate": (c_int, [c_void_p, c_void_p, c_int, c_void_p]),
}

_lib = None
_lock = threading.Lock()


class GocError(RuntimeError):
    """A C-ABI call returned a non-zero status."""


def load():
    """Load the shared library (once) and attach the declared signatures."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise GocError(
                f"{LIB_PATH} is missing: build it with `python -m gpuocean_gb300.build_lib` "
                "(the CUDA library is required; there is no CPU fallback)")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(512)
    load().goc_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        raise GocError(f"{what or 'gpuocean_gb300'} failed ({rc}): {last_error()}")


def call(name: str, *args) -> None:
    """Call a status-returning entry point and raise on failure."""
    check(getattr(load(), name)(*args), name)
