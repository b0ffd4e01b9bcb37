"""The C-ABI library loads and exports every entry point the header declares."""
import ctypes
import os
import re

from gpuocean_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "gpuocean_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(goc_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "goc_cdklm_rk2_step" in names and "goc_max_dt" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_params_struct_matches_header_fields():
    text = open(HEADER).read()
    body = text[text.index("typedef struct GocCdklmParams"):text.index("} GocCdklmParams;")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = re.findall(r"\*?\s*([a-z_0-9]+)\s*[,;]", body.split("{", 1)[1])
    assert [f[0] for f in _lib.GocCdklmParams._fields_] == names


def test_argument_validation_without_gpu():
    # validation happens before any CUDA call
    lib = _lib.load()
    p = _lib.GocCdklmParams()
    p.nx, p.ny = 0, 4
    rc = lib.goc_cdklm_rk2_step(ctypes.byref(p), 1.0, None, None, None, None, None, None, 64, None, 64, None, 64, None)
    assert rc == -1 and "nx, ny" in _lib.last_error()
    assert lib.goc_max_dt_partials(256, 256) == 8 * 32
    rc = lib.goc_max_dt(8, 8, 1.0, 1.0, 9.8, None, None, None, 48, None, 48, 1e20, None, 0, None, None)
    assert rc == -1


def test_new_entry_points_validate_without_gpu():
    """Observation, statistics, KL and sponge entries reject bad arguments
    before any CUDA call."""
    import numpy as np
    lib = _lib.load()
    # observation operator: empty grid, bad pitch; zero drifters is a no-op
    assert lib.goc_observe_underlying_flow(0, 4, 1.0, 1.0, 2, 2, None, 0, None, 0, None, 0, 1.0, 3, None, 8, None, 8,
                                           None) == -1
    assert lib.goc_observe_underlying_flow(4, 4, 1.0, 1.0, 2, 2, None, 0, 1, 4, 1, 4, 1.0, 3, 1, 8, 1, 8, None) == -1
    assert "pitch" in _lib.last_error()
    assert lib.goc_observe_underlying_flow(4, 4, 1.0, 1.0, 2, 2, None, 0, None, 0, None, 0, 1.0, 0, None, 8, None, 8,
                                           None) == 0
    # ensemble statistics need a handle; the multi-level assembly checks its levels
    assert lib.goc_ensemble_observe(None, 0, 1, 1, 8, 0, 1, 1, None) == -1
    assert lib.goc_ensemble_moments(None, 0, 1, 0, 0.0, 0, 1, 1, None) == -1
    fine = (ctypes.c_void_p * 2)(1, 1)
    coarse = (ctypes.c_void_p * 2)(None, 1)
    nx = np.array([6, 13], np.int32)   # 13 is not twice 6
    ny = np.array([4, 8], np.int32)
    assert lib.goc_ml_combine(2, fine, coarse, nx.ctypes.data, ny.ctypes.data, 3, 1, None) == -1
    assert "coarsened" in _lib.last_error()
    assert lib.goc_ml_combine(9, fine, coarse, nx.ctypes.data, ny.ctypes.data, 3, 1, None) == -1
    # KL: table size from the basis; empty basis ranges are rejected
    from gpuocean_gb300.SWEsimulators.ModelErrorKL import GocKLDesc
    d = GocKLDesc()
    d.basis_x_start, d.basis_x_end, d.basis_y_start, d.basis_y_end = 2, 8, 1, 7
    assert lib.goc_kl_table_floats(512, 300, ctypes.byref(d)) == 2 * 7 * (514 + 302)
    d.basis_y_end = 0
    assert lib.goc_kl_table_floats(512, 300, ctypes.byref(d)) < 0
    assert lib.goc_kl_perturb(ctypes.byref(d), 8, 8, 1.0, 1.0, 1.0, 1, 1, None, None, 48, None, 0, 0, 0, None) == -1
    # sponges: flow relaxation needs exterior data, linear interpolation sponge cells
    cells = np.array([4, 0, 4, 0], np.int32)
    assert lib.goc_sponge_boundary(8, 8, 3, 1, 3, 1, cells.ctypes.data, 1, 1, 1, 48, None, None, 2, None, None, 2,
                                   0.0, None) == -1
    assert "exterior" in _lib.last_error()
    cells0 = np.zeros(4, np.int32)
    assert lib.goc_sponge_boundary(8, 8, 4, 1, 4, 1, cells0.ctypes.data, 1, 1, 1, 48, None, None, 2, None, None, 2,
                                   0.0, None) == -1
    big = np.array([99, 0, 0, 0], np.int32)
    assert lib.goc_sponge_boundary(8, 8, 4, 1, 1, 1, big.ctypes.data, 1, 1, 1, 48, None, None, 2, None, None, 2,
                                   0.0, None) == -1


def test_step_run_and_tma_entries_validate_without_gpu():
    """The multi-step entry, the TMA status query and the wait self-test
    reject bad arguments before any CUDA call."""
    import numpy as np
    lib = _lib.load()
    p = _lib.GocCdklmParams()
    p.nx, p.ny, p.dx, p.dy, p.g, p.rk_order = 8, 8, 1.0, 1.0, 9.81, 2
    p.theta, p.desing_eps, p.flux_slope_eps, p.depth_cutoff, p.flux_balancer = 1.3, 0.1, 0.1, 1e-5, 0.8
    p.bc_north = p.bc_east = p.bc_south = p.bc_west = 1
    p.land_value = 1e20
    # one-value textures (validation checks the pointers and sizes, it does not read them)
    for name in ("coriolis_f", "angle", "wind_x_cur", "wind_x_next", "wind_y_cur", "wind_y_next", "atm_p_cur",
                 "atm_p_next"):
        setattr(p, name, 16)
    for name in ("coriolis", "angle", "wind_x", "wind_y", "atm_p"):
        setattr(p, name + "_nx", 1)
        setattr(p, name + "_ny", 1)
    dts = np.full(3, 1.0, np.float32)
    # null buffers
    rc = lib.goc_cdklm_rk2_steps(ctypes.byref(p), dts.ctypes.data, 3, None, None, None, None, None, None, 48,
                                 None, 52, None, 48, None)
    assert rc == -1 and "null buffer" in _lib.last_error()
    # negative step count / missing dt list / negative dt
    rc = lib.goc_cdklm_rk2_steps(ctypes.byref(p), None, 2, 1, 1, 1, 2, 2, 2, 48, 1, 52, 1, 48, None)
    assert rc == -1 and "step list" in _lib.last_error()
    rc = lib.goc_cdklm_rk2_steps(ctypes.byref(p), dts.ctypes.data, -1, 1, 1, 1, 2, 2, 2, 48, 1, 52, 1, 48, None)
    assert rc == -1 and "step list" in _lib.last_error()
    bad = np.array([1.0, -1.0], np.float32)
    rc = lib.goc_cdklm_rk2_steps(ctypes.byref(p), bad.ctypes.data, 2, 1, 1, 1, 2, 2, 2, 48, 1, 52, 1, 48, None)
    assert rc == -1 and "dt 1" in _lib.last_error()
    # the two buffer sets must differ
    rc = lib.goc_cdklm_rk2_steps(ctypes.byref(p), dts.ctypes.data, 3, 1, 1, 1, 1, 1, 1, 48, 1, 52, 1, 48, None)
    assert rc == -1 and "differ" in _lib.last_error()
    assert lib.goc_ensemble_tma_status(None, None, None, None) == -1
    timed_out, waited = ctypes.c_int(), ctypes.c_double()
    assert lib.goc_selftest_wait_timeout(0.0, ctypes.byref(timed_out), ctypes.byref(waited)) == -1
    assert lib.goc_selftest_wait_timeout(5000.0, ctypes.byref(timed_out), ctypes.byref(waited)) == -1
