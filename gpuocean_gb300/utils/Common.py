"""Device runtime and data layer: the drop-in counterpart of GPU Ocean's ``utils/Common.py``.

Replaces the PyCUDA-based classes of the reference (U/ = src/gpuocean/utils):

* ``CUDAContext``                U/Common.py:284-512 (no JIT: kernels are prebuilt for sm_103a)
* ``CUDAArray2D``                U/Common.py:516-644 (tight pitch float32 device arrays)
* ``SWEDataArakawaA``            U/Common.py:774-831 (double-buffered state)
* ``BoundaryConditions``         U/Common.py:920-1046
* ``BoundaryConditionsData``     U/Common.py:1051-1117 (exterior data of the sponges)
* ``BoundaryConditionsArakawaA`` U/Common.py:1121-1404 (periodic ghosts, flow relaxation, linear interpolation)
* ``Bathymetry``                 U/Common.py:1408-1561

Device memory, streams and copies go through the library's C ABI.
"""
from __future__ import annotations

import ctypes
import logging
import time

import numpy as np

from .. import _lib


class Stream:
    """A CUDA stream owned by the library (replaces ``pycuda.driver.Stream``)."""

    def __init__(self):
        h = ctypes.c_void_p()
        _lib.call("goc_stream_create", ctypes.byref(h))
        self.handle = h.value

    def synchronize(self):
        _lib.call("goc_stream_synchronize", self.handle)

    def release(self):
        if self.handle:
            _lib.load().goc_stream_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class Timer:
    """Context manager that logs wall time (U/Common.py:52-68)."""

    def __init__(self, tag, log_level=logging.DEBUG):
        self.tag = tag
        self.log_level = log_level
        self.logger = logging.getLogger(__name__)

    def __enter__(self):
        self.start = time.time()
        return self

    def __exit__(self, *args):
        self.secs = time.time() - self.start
        self.msecs = self.secs * 1000
        self.logger.log(self.log_level, "%s: %f ms", self.tag, self.msecs)


class CUDAContext:
    """Selects the GPU.  The reference's JIT cache is not needed: all kernels
    are compiled ahead of time for sm_103a into ``libgpuocean_gb300.so``."""

    def __init__(self, device=0, context_flags=None, use_cache=True, autotuning=True):
        self.logger = logging.getLogger(__name__)
        self.device = int(device)
        lib = _lib.load()
        n = ctypes.c_int(0)
        _lib.check(lib.goc_device_count(ctypes.byref(n)), "goc_device_count")
        if self.device >= n.value:
            raise RuntimeError(f"CUDA device {self.device} requested, {n.value} available")
        _lib.call("goc_set_device", self.device)

    def synchronize(self):
        _lib.call("goc_device_synchronize")

    def __str__(self):
        return f"CUDAContext(device={self.device})"


class DevicePtr:
    """Raw device allocation; ``.gpudata``/``.ptr`` give the address as an int."""

    def __init__(self, nbytes):
        p = ctypes.c_void_p()
        _lib.call("goc_malloc", ctypes.byref(p), ctypes.c_size_t(int(nbytes)))
        self.ptr = p.value or 0
        self.nbytes = int(nbytes)

    @property
    def gpudata(self):
        return self.ptr

    def free(self):
        if self.ptr:
            _lib.load().goc_free(self.ptr)
            self.ptr = 0

    def __int__(self):
        return self.ptr


def _stream_handle(stream):
    if stream is None:
        return None
    return getattr(stream, "handle", stream)


class CUDAArray2D:
    """2D float32 (or float64/uint64) device array with halo, tight pitch."""

    def __init__(self, gpu_stream, nx, ny, halo_x, halo_y, data, asymHalo=None,
                 double_precision=False, integers=False):
        self.double_precision = double_precision
        self.integers = integers
        host = np.asarray(data)
        if integers:
            host = np.ascontiguousarray(host, dtype=np.uint64)
        elif double_precision:
            host = np.ascontiguousarray(host, dtype=np.float64)
        else:
            host = self.convert_to_float32(host)
        self.nx, self.ny = int(nx), int(ny)
        self.nx_halo = self.nx + 2 * int(halo_x)
        self.ny_halo = self.ny + 2 * int(halo_y)
        if asymHalo is not None and len(asymHalo) == 4:
            self.nx_halo = self.nx + asymHalo[1] + asymHalo[3]
            self.ny_halo = self.ny + asymHalo[0] + asymHalo[2]
        assert host.shape[1] == self.nx_halo, str(host.shape[1]) + " vs " + str(self.nx_halo)
        assert host.shape[0] == self.ny_halo, str(host.shape[0]) + " vs " + str(self.ny_halo)
        self.bytes_per_float = host.itemsize
        self.dtype = host.dtype
        self.pitch = np.int32(self.nx_halo * self.bytes_per_float)
        self.data = DevicePtr(self.nx_halo * self.ny_halo * self.bytes_per_float)
        self.holds_data = True
        self.mask = data.mask if np.ma.is_masked(data) else None
        self.upload(gpu_stream, data)

    @property
    def ptr(self):
        return self.data.ptr

    def upload(self, gpu_stream, data):
        if not self.holds_data:
            raise RuntimeError("The buffer has been freed before upload is called")
        if np.ma.is_masked(data):
            self.mask = data.mask
        if self.integers:
            host = np.ascontiguousarray(np.asarray(data), dtype=np.uint64)
        elif self.double_precision:
            host = np.ascontiguousarray(np.asarray(data), dtype=np.float64)
        else:
            host = self.convert_to_float32(np.asarray(data))
        assert host.shape == (self.ny_halo, self.nx_halo), str(host.shape) + " vs " + str((self.ny_halo, self.nx_halo))
        assert host.itemsize == self.bytes_per_float
        _lib.call("goc_memcpy_h2d_async", self.data.ptr, host.ctypes.data, ctypes.c_size_t(host.nbytes),
                  _stream_handle(gpu_stream))
        # the host array must outlive the asynchronous copy
        _lib.call("goc_stream_synchronize", _stream_handle(gpu_stream))

    def copyBuffer(self, gpu_stream, buffer):
        if not self.holds_data:
            raise RuntimeError("The buffer has been freed before copying buffer")
        if not buffer.holds_data:
            raise RuntimeError("The provided buffer is either not allocated, or has been freed before copying buffer")
        assert buffer.nx_halo == self.nx_halo and buffer.ny_halo == self.ny_halo
        assert buffer.bytes_per_float == self.bytes_per_float
        _lib.call("goc_memcpy_d2d_async", self.data.ptr, buffer.data.ptr,
                  ctypes.c_size_t(self.bytes_per_float * self.nx_halo * self.ny_halo), _stream_handle(gpu_stream))

    def download(self, gpu_stream):
        if not self.holds_data:
            raise RuntimeError("CUDA buffer has been freed")
        host = np.empty((self.ny_halo, self.nx_halo), dtype=self.dtype)
        _lib.call("goc_memcpy_d2h_async", host.ctypes.data, self.data.ptr, ctypes.c_size_t(host.nbytes),
                  _stream_handle(gpu_stream))
        _lib.call("goc_stream_synchronize", _stream_handle(gpu_stream))
        if self.mask is not None:
            host = np.ma.array(host, mask=self.mask)
        return host

    def release(self):
        if self.holds_data:
            self.data.free()
            self.holds_data = False

    @staticmethod
    def convert_to_float32(data):
        # native float32 in C order (the device copy takes the raw bytes, so a
        # big-endian array, as NetCDF files hold, is converted too)
        if data.dtype != np.dtype(np.float32) or np.isfortran(data) or not data.flags.c_contiguous:
            return np.ascontiguousarray(data, dtype=np.float32)
        return data


class SWEDataArakawaA:
    """Double-buffered (eta, hu, hv) on an Arakawa A grid.

    ``h0/hu0/hv0`` always hold the latest state.  After a fused RK2 step the
    other set holds the previous time step.
    """

    def __init__(self, gpu_stream, nx, ny, halo_x, halo_y, h0, hu0, hv0):
        self.h0 = CUDAArray2D(gpu_stream, nx, ny, halo_x, halo_y, h0)
        self.hu0 = CUDAArray2D(gpu_stream, nx, ny, halo_x, halo_y, hu0)
        self.hv0 = CUDAArray2D(gpu_stream, nx, ny, halo_x, halo_y, hv0)
        self.h1 = CUDAArray2D(gpu_stream, nx, ny, halo_x, halo_y, h0)
        self.hu1 = CUDAArray2D(gpu_stream, nx, ny, halo_x, halo_y, hu0)
        self.hv1 = CUDAArray2D(gpu_stream, nx, ny, halo_x, halo_y, hv0)

    def swap(self):
        self.h1, self.h0 = self.h0, self.h1
        self.hu1, self.hu0 = self.hu0, self.hu1
        self.hv1, self.hv0 = self.hv0, self.hv1

    def download(self, gpu_stream):
        return self.h0.download(gpu_stream), self.hu0.download(gpu_stream), self.hv0.download(gpu_stream)

    def downloadPrevTimestep(self, gpu_stream):
        return self.h1.download(gpu_stream), self.hu1.download(gpu_stream), self.hv1.download(gpu_stream)

    def release(self):
        for a in (self.h0, self.hu0, self.hv0, self.h1, self.hu1, self.hv1):
            a.release()


class BoundaryConditions:
    """Boundary flags: 1 wall, 2 periodic, 3 flow relaxation, 4 linear interpolation.

    Flags 3 and 4 are sponge boundaries: spongeCells gives, per side, the
    rows or columns of the array (ghost cells included) that the sponge spans.
    """

    def __init__(self, north=1, east=1, south=1, west=1,
                 spongeCells={'north': 0, 'south': 0, 'east': 0, 'west': 0}):
        self.north = np.int32(north)
        self.east = np.int32(east)
        self.south = np.int32(south)
        self.west = np.int32(west)
        self.spongeCells = {k: np.int32(v) for k, v in spongeCells.items()}
        assert not ((self.north == 2 or self.south == 2) and (self.north != self.south)), \
            'The given periodic boundary conditions are not periodically (north/south)'
        assert not ((self.east == 2 or self.west == 2) and (self.east != self.west)), \
            'The given periodic boundary conditions are not periodically (east/west)'

    def get(self):
        raise NotImplementedError("get() implementation changed! Change calling code")

    def getBCDict(self):
        return {'north': self.north, 'south': self.south, 'east': self.east, 'west': self.west}

    def getSponge(self):
        return self.spongeCells

    def isDefault(self):
        return self.north == 1 and self.east == 1 and self.south == 1 and self.west == 1

    def isSponge(self):
        return any(v in (3, 4) for v in (self.north, self.east, self.south, self.west))

    def isPeriodicNorthSouth(self):
        return self.north == 2 and self.south == 2

    def isPeriodicEastWest(self):
        return self.east == 2 and self.west == 2

    def isPeriodic(self):
        return self.isPeriodicEastWest() and self.isPeriodicNorthSouth()

    @staticmethod
    def _toString(cond):
        return {1: "Wall", 2: "Periodic", 3: "Flow_Relaxation_Scheme",
                4: "Open_Linear_Interpolation"}.get(int(cond), "Invalid_:|")

    def __str__(self):
        return ("north: " + self._toString(self.north) + ", east: " + self._toString(self.east)
                + ", south: " + self._toString(self.south) + ", west: " + self._toString(self.west)
                + ", spongeCells: " + str({k: int(v) for k, v in self.spongeCells.items()}))

    @classmethod
    def fromstring(cls, bc_string):
        """The boundary conditions of their text form (as __str__ writes it and
        as simulator files store it, U/Common.py:1010-1045)."""
        import re
        flags = {"Wall": 1, "Periodic": 2, "Flow_Relaxation_Scheme": 3, "Open_Linear_Interpolation": 4}
        side = {}
        for name in ("north", "east", "south", "west"):
            m = re.search(name + r"\s*:\s*([A-Za-z_:|]+)", bc_string)
            side[name] = flags.get(m.group(1).rstrip(",") if m else "", -1)
        sponge = {"north": 0, "south": 0, "east": 0, "west": 0}
        m = re.search(r"spongeCells\s*:\s*\{([^}]*)\}", bc_string)
        if m:
            for key, val in re.findall(r"'?(north|south|east|west)'?\s*:\s*(?:np\.int\d+\()?(-?\d+)", m.group(1)):
                sponge[key] = int(val)
        return cls(north=side["north"], east=side["east"], south=side["south"], west=side["west"],
                   spongeCells=sponge)


class SingleBoundaryConditionData:
    """Exterior solution along one side over time (U/Common.py:1040-1078):
    lists of 1D float32 arrays h, hu, hv, one per time stamp."""

    def __init__(self, h=None, hu=None, hv=None):
        self.h = [np.zeros(2, dtype=np.float32)] if h is None else h
        self.hu = [np.zeros(2, dtype=np.float32)] if hu is None else hu
        self.hv = [np.zeros(2, dtype=np.float32)] if hv is None else hv
        self.numSteps = len(self.h)
        self.shape = self.h[0].shape
        for i in range(self.numSteps):
            for a in (self.h[i], self.hu[i], self.hv[i]):
                assert a.shape == self.shape, str(self.shape) + " vs " + str(a.shape)
                assert a.dtype == np.float32, "boundary data needs to be of type np.float32"

    def __str__(self):
        return str(self.numSteps) + " steps, each " + str(self.shape)


class BoundaryConditionsData:
    """Exterior solution for the sponge boundaries over time (U/Common.py:1081-1117)."""

    def __init__(self, t=None, north=None, south=None, east=None, west=None):
        self.t = [0]
        self.numSteps = 1
        self.north = north or SingleBoundaryConditionData()
        self.south = south or SingleBoundaryConditionData()
        self.east = east or SingleBoundaryConditionData()
        self.west = west or SingleBoundaryConditionData()
        if t is not None:
            self.t = t
            self.numSteps = len(t)
        for data in (self.north, self.south, self.east, self.west):
            assert data.numSteps == self.numSteps, "Wrong timesteps " + str(data.numSteps) + " vs " + str(self.numSteps)
        assert self.north.h[0].shape == self.south.h[0].shape, "Wrong shape of north vs south"
        assert self.east.h[0].shape == self.west.h[0].shape, "Wrong shape of east vs west"

    def __str__(self):
        return ("Steps=" + str(self.numSteps) + ", [north=" + str(self.north) + "], [south=" + str(self.south)
                + "], [east=" + str(self.east) + "], [west=" + str(self.west) + "]")


class BoundaryConditionsArakawaA:
    """Ghost and sponge cells of an (eta, hu, hv) triple (U/Common.py:1120-1400):
    periodic images (flag 2), flow relaxation towards exterior data (flag 3)
    and linear interpolation (flag 4), north-south first, then east-west."""

    def __init__(self, gpu_ctx, gpu_stream, nx, ny, halo_x, halo_y, boundary_conditions,
                 bc_data=None, block_width=16, block_height=16):
        self.boundary_conditions = boundary_conditions
        self.nx, self.ny = np.int32(nx), np.int32(ny)
        self.halo_x, self.halo_y = np.int32(halo_x), np.int32(halo_y)
        self.bc_data = BoundaryConditionsData() if bc_data is None else bc_data
        bc = boundary_conditions
        sp = bc.spongeCells
        self.sponge_cells = np.array([sp.get('north', 0), sp.get('east', 0), sp.get('south', 0), sp.get('west', 0)],
                                     dtype=np.int32)
        self.bc_timestamps = [None, None]
        self.bc_t = np.float32(0.0)
        self.ns_nx = int(self.bc_data.north.h[0].shape[0])
        self.ew_ny = int(self.bc_data.east.h[0].shape[0])
        self.frs = 3 in (int(bc.north), int(bc.south), int(bc.east), int(bc.west))
        self.bc_ns = [None, None]
        self.bc_ew = [None, None]
        if bc.isSponge():
            z_ns = np.zeros((2, self.ns_nx, 3), np.float32)
            z_ew = np.zeros((self.ew_ny, 2, 3), np.float32)
            self.bc_ns = [CUDAArray2D(gpu_stream, 3 * self.ns_nx, 2, 0, 0, z_ns.reshape(2, -1)) for _ in range(2)]
            self.bc_ew = [CUDAArray2D(gpu_stream, 6, self.ew_ny, 0, 0, z_ew.reshape(self.ew_ny, -1)) for _ in range(2)]

    def update_bc_values(self, gpu_stream, t):
        """Time interpolation of the exterior data for the flow relaxation
        scheme (U/Common.py:1193-1308)."""
        if not self.frs:
            return
        data = self.bc_data
        t_max_index = len(data.t) - 1
        t0_index = max(0, np.searchsorted(data.t, t) - 1)
        t1_index = min(t_max_index, np.searchsorted(data.t, t))
        new_t0, new_t1 = data.t[t0_index], data.t[t1_index]
        old_t0, old_t1 = self.bc_timestamps
        self.bc_timestamps = [new_t0, new_t1]

        def pack_ns(d, i):
            return np.transpose(np.vstack((np.squeeze(d.h[i]), np.squeeze(d.hu[i]), np.squeeze(d.hv[i]))))

        def pack_ew(d, i):
            return np.transpose(np.vstack((np.squeeze(d.h[i]), np.squeeze(d.hu[i]), np.squeeze(d.hv[i]))))

        for slot, (old, new, idx) in enumerate(((old_t0, new_t0, t0_index), (old_t1, new_t1, t1_index))):
            if new != old:
                ns = np.stack([pack_ns(data.south, idx), pack_ns(data.north, idx)]).astype(np.float32)
                ew = np.stack([pack_ew(data.west, idx), pack_ew(data.east, idx)], axis=1).astype(np.float32)
                self.bc_ns[slot].upload(gpu_stream, np.ascontiguousarray(ns.reshape(2, -1)))
                self.bc_ew[slot].upload(gpu_stream, np.ascontiguousarray(ew.reshape(self.ew_ny, -1)))
        elapsed = t - new_t0
        interval = max(1.0e-10, (new_t1 - new_t0))
        self.bc_t = np.float32(max(0.0, min(1.0, elapsed / interval)))

    def _sponge(self, gpu_stream, h, u, v, north, east, south, west):
        ns0, ns1 = (a.ptr if a is not None else None for a in self.bc_ns)
        ew0, ew1 = (a.ptr if a is not None else None for a in self.bc_ew)
        _lib.call("goc_sponge_boundary", int(self.nx), int(self.ny), int(north), int(east), int(south), int(west),
                  self.sponge_cells.ctypes.data, h.ptr, u.ptr, v.ptr, int(h.pitch), ns0, ns1, self.ns_nx,
                  ew0, ew1, self.ew_ny, ctypes.c_float(self.bc_t), _stream_handle(gpu_stream))

    def boundaryCondition(self, gpu_stream, h, u, v):
        bc = self.boundary_conditions
        n, e, s, w = int(bc.north), int(bc.east), int(bc.south), int(bc.west)
        if n == 2:
            _lib.call("goc_periodic_ghosts", int(self.nx), int(self.ny), 2, 1, h.ptr, u.ptr, v.ptr, int(h.pitch),
                      _stream_handle(gpu_stream))
        elif n in (3, 4) or s in (3, 4):
            self._sponge(gpu_stream, h, u, v, n, 1, s, 1)
        if e == 2:
            _lib.call("goc_periodic_ghosts", int(self.nx), int(self.ny), 1, 2, h.ptr, u.ptr, v.ptr, int(h.pitch),
                      _stream_handle(gpu_stream))
        elif e in (3, 4) or w in (3, 4):
            self._sponge(gpu_stream, h, u, v, 1, e, 1, w)

    def release(self):
        for a in self.bc_ns + self.bc_ew:
            if a is not None:
                a.release()


class Bathymetry:
    """Corner depths Bi (ny+5, nx+5) and cell means Bm (ny+4, nx+4) on the device."""

    def __init__(self, gpu_ctx, gpu_stream, nx, ny, halo_x, halo_y, Bi_host,
                 boundary_conditions=BoundaryConditions(), block_width=16, block_height=16):
        self.gpu_stream = gpu_stream
        self.nx, self.ny = np.int32(nx), np.int32(ny)
        self.halo_x, self.halo_y = np.int32(halo_x), np.int32(halo_y)
        self.halo_nx = np.int32(nx + 2 * halo_x)
        self.halo_ny = np.int32(ny + 2 * halo_y)
        self.boundary_conditions = boundary_conditions
        self.mask_value = np.float32(1.0e20)
        self.use_mask = False
        if np.ma.is_masked(Bi_host):
            Bi_host = Bi_host.copy().filled(self.mask_value).astype(np.float32)
            self.use_mask = True
        BiShapeY, BiShapeX = Bi_host.shape
        assert BiShapeX == nx + 1 + 2 * halo_x and BiShapeY == ny + 1 + 2 * halo_y, \
            "Wrong size of bottom bathymetry, should be defined on cell intersections, not cell centers. " + \
            str((BiShapeX, BiShapeY)) + " vs " + str((nx + 1 + 2 * halo_x, ny + 1 + 2 * halo_y))
        self.Bi = CUDAArray2D(gpu_stream, nx + 1, ny + 1, halo_x, halo_y, np.asarray(Bi_host))
        self.Bm = CUDAArray2D(gpu_stream, nx, ny, halo_x, halo_y,
                              np.zeros((self.halo_ny, self.halo_nx), dtype=np.float32))
        bc = boundary_conditions
        _lib.call("goc_bathymetry_init", int(nx), int(ny), int(bc.north), int(bc.east), int(bc.south),
                  int(bc.west), ctypes.c_float(self.mask_value), self.Bi.ptr, int(self.Bi.pitch),
                  self.Bm.ptr, int(self.Bm.pitch), _stream_handle(gpu_stream))

    def download(self, gpu_stream):
        Bm_cpu = self.Bm.download(gpu_stream)
        Bi_cpu = self.Bi.download(gpu_stream)
        if self.use_mask:
            Bi_cpu = np.ma.array(data=Bi_cpu, mask=(Bi_cpu == self.mask_value), fill_value=0.0)
            Bm_cpu = np.ma.array(data=Bm_cpu, mask=(Bm_cpu == self.mask_value), fill_value=0.0)
        return Bi_cpu, Bm_cpu

    def release(self):
        self.Bm.release()
        self.Bi.release()
