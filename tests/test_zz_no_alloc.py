"""The allocation-free CFL entry point against the one that takes caller scratch.

goc_max_dt_noalloc exists for callers that cannot allocate device memory on
their step path (a host model that owns all device memory through its own
pool, or a loop that must not pay cudaMalloc's implicit synchronisation):
its partial minima live in a scratch array inside the library.  This file is
collected last so that a failure here cannot hide the other tests.
"""
import ctypes

import numpy as np
import pytest

from gpuocean_gb300 import _lib

pytestmark = pytest.mark.gpu


class _Dev:
    """A device buffer made through the C ABI."""

    def __init__(self, host):
        self.host = np.ascontiguousarray(host, dtype=np.float32)
        p = ctypes.c_void_p()
        _lib.call("goc_malloc", ctypes.byref(p), ctypes.c_size_t(max(4, self.host.nbytes)))
        self.ptr = p.value
        _lib.call("goc_memcpy_h2d_async", self.ptr, self.host.ctypes.data, ctypes.c_size_t(self.host.nbytes), None)

    def free(self):
        _lib.load().goc_free(self.ptr)


def _state(nx, ny, seed, depth):
    rng = np.random.default_rng(seed)
    shape = (ny + 4, nx + 4)
    eta = 0.5 * rng.standard_normal(shape)
    hu = 3.0 * rng.standard_normal(shape)
    hv = 3.0 * rng.standard_normal(shape)
    Hm = depth + rng.uniform(0.0, 5.0, shape)
    return [_Dev(a) for a in (eta, hu, hv, Hm)]


def _dt(nx, ny, bufs, noalloc):
    lib = _lib.load()
    eta, hu, hv, Hm = bufs
    pitch = 4 * (nx + 4)
    out = _Dev(np.zeros(1))
    if noalloc:
        rc = lib.goc_max_dt_noalloc(nx, ny, 100.0, 120.0, 9.81, eta.ptr, hu.ptr, hv.ptr, pitch, Hm.ptr, pitch,
                                    ctypes.c_float(1e20), out.ptr, None)
        scratch = None
    else:
        n = lib.goc_max_dt_partials(nx, ny)
        scratch = _Dev(np.zeros(n))
        rc = lib.goc_max_dt(nx, ny, 100.0, 120.0, 9.81, eta.ptr, hu.ptr, hv.ptr, pitch, Hm.ptr, pitch,
                            ctypes.c_float(1e20), scratch.ptr, n, out.ptr, None)
    _lib.check(rc, "max dt")
    res = np.zeros(1, dtype=np.float32)
    _lib.call("goc_memcpy_d2h_async", res.ctypes.data, out.ptr, ctypes.c_size_t(4), None)
    _lib.call("goc_device_synchronize")
    out.free()
    if scratch is not None:
        scratch.free()
    return res[0]


def test_noalloc_matches_scratch_entry_point_twice_in_a_row():
    _lib.call("goc_set_device", 0)
    # first call on a large grid with a small limit, second on a smaller
    # grid: the second must not see the first call's partial minima
    big = (700, 650, 1, 4.0)
    small = (90, 70, 2, 50.0)
    for nx, ny, seed, depth in (big, small):
        bufs = _state(nx, ny, seed, depth)
        want = _dt(nx, ny, bufs, noalloc=False)
        got = _dt(nx, ny, bufs, noalloc=True)
        # the CFL tests compare dt bit for bit
        assert got == want, (nx, ny, got, want)
        assert 0.0 < got < 1e5
        for b in bufs:
            b.free()


def test_noalloc_rejects_grids_beyond_its_scratch():
    lib = _lib.load()
    cap = lib.goc_max_dt_noalloc_capacity()
    assert cap == 65536
    nx, ny = 32 * 512, 8 * 129     # 66048 reduction blocks
    assert lib.goc_max_dt_partials(nx, ny) > cap
    rc = lib.goc_max_dt_noalloc(nx, ny, 1.0, 1.0, 9.81, None, None, None, 4 * (nx + 4), None, 4 * (nx + 4),
                                ctypes.c_float(1e20), None, None)
    assert rc == -1 and "built-in scratch holds 65536" in _lib.last_error()
