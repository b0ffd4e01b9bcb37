"""Base class of the simulators (counterpart of ``SWEsimulators/Simulator.py:44-430``).

Holds the common parameters, the stream, the forcing textures and the state
download/upload/copy interface.
"""
from __future__ import annotations

import logging

import numpy as np

from ..utils import Common


class Simulator:
    def __init__(self, gpu_ctx, nx, ny, ghost_cells_x, ghost_cells_y, dx, dy, dt, g, f, r, A, t,
                 theta, rk_order, coriolis_beta, y_zero_reference_cell, wind, atmospheric_pressure,
                 write_netcdf, ignore_ghostcells, offset_x, offset_y, comm, block_width, block_height,
                 local_particle_id=0):
        self.gpu_stream = Common.Stream()
        self.logger = logging.getLogger(__name__)
        self.gpu_ctx = gpu_ctx
        self.nx = np.int32(nx)
        self.ny = np.int32(ny)
        self.ghost_cells_x = np.int32(ghost_cells_x)
        self.ghost_cells_y = np.int32(ghost_cells_y)
        self.dx = np.float32(dx)
        self.dy = np.float32(dy)
        self.dt = dt
        self.g = np.float32(g)
        self.f = np.float32(f)
        self.r = np.float32(r)
        self.coriolis_beta = np.float32(coriolis_beta)
        self.wind_stress = wind
        if self.wind_stress.stress_u is None or self.wind_stress.stress_v is None:
            self.wind_stress.compute_wind_stress_from_wind()
        self.atmospheric_pressure = atmospheric_pressure
        self.y_zero_reference_cell = np.float32(y_zero_reference_cell)
        self.offset_x, self.offset_y = offset_x, offset_y
        self.t = t
        self.num_iterations = 0
        self.A = 'NA' if A is None else np.float32(A)
        self.theta = 'NA' if theta is None else np.float32(theta)
        self.rk_order = 'NA' if rk_order is None else np.int32(rk_order)
        self.hasDrifters = False
        self.drifters = None
        self.drifter_t = self.t
        self.model_error = None
        self.hasCrossProductDrifter = False
        self.CrossProductDrifter = None
        self.write_netcdf = write_netcdf
        self.ignore_ghostcells = ignore_ghostcells
        self.sim_writer = None
        self.comm = comm
        self.local_particle_id = local_particle_id
        self.local_size = (block_width, block_height, 1)
        self.global_size = (int(np.ceil(self.nx / float(block_width))), int(np.ceil(self.ny / float(block_height))))

        # forcing textures (current and next time level)
        ws = self.wind_stress
        self.wind_stress_timestamps = {}
        t0, t1 = self._interval(ws.t)
        s = self.gpu_stream
        self.wind_stress_x_current_arr = Common.CUDAArray2D(s, ws.stress_u[t0].shape[1], ws.stress_u[t0].shape[0], 0, 0, ws.stress_u[t0])
        self.wind_stress_y_current_arr = Common.CUDAArray2D(s, ws.stress_v[t0].shape[1], ws.stress_v[t0].shape[0], 0, 0, ws.stress_v[t0])
        self.wind_stress_x_next_arr = Common.CUDAArray2D(s, ws.stress_u[t1].shape[1], ws.stress_u[t1].shape[0], 0, 0, ws.stress_u[t1])
        self.wind_stress_y_next_arr = Common.CUDAArray2D(s, ws.stress_v[t1].shape[1], ws.stress_v[t1].shape[0], 0, 0, ws.stress_v[t1])
        ap = self.atmospheric_pressure
        self.atmospheric_pressure_timestamps = {}
        t0, t1 = self._interval(ap.t)
        self.atmospheric_pressure_current_arr = Common.CUDAArray2D(s, ap.P[t0].shape[1], ap.P[t0].shape[0], 0, 0, ap.P[t0])
        self.atmospheric_pressure_next_arr = Common.CUDAArray2D(s, ap.P[t1].shape[1], ap.P[t1].shape[0], 0, 0, ap.P[t1])

    def _interval(self, times):
        t_max_index = len(times) - 1
        t0 = max(0, np.searchsorted(times, self.t) - 1)
        t1 = min(t_max_index, np.searchsorted(times, self.t))
        return t0, t1

    def _update_forcing(self, times, stamps, key, uploads):
        """Time interpolation weight of a forcing, uploading new levels when the
        time interval changes (S/Simulator.py:183-288)."""
        t0, t1 = self._interval(times)
        new_t0, new_t1 = times[t0], times[t1]
        old = stamps.get(key, [None, None])
        stamps[key] = [new_t0, new_t1]
        if new_t0 != old[0]:
            uploads(t0, "current")
        if new_t1 != old[1]:
            uploads(t1, "next")
        elapsed = self.t - new_t0
        interval = max(1.0e-10, (new_t1 - new_t0))
        return max(0.0, min(1.0, elapsed / interval))

    def update_wind_stress(self, kernel_module=None):
        ws = self.wind_stress

        def up(i, which):
            if which == "current":
                self.wind_stress_x_current_arr.upload(self.gpu_stream, ws.stress_u[i])
                self.wind_stress_y_current_arr.upload(self.gpu_stream, ws.stress_v[i])
            else:
                self.wind_stress_x_next_arr.upload(self.gpu_stream, ws.stress_u[i])
                self.wind_stress_y_next_arr.upload(self.gpu_stream, ws.stress_v[i])
        return self._update_forcing(ws.t, self.wind_stress_timestamps, "step", up)

    def update_atmospheric_pressure(self, kernel_module=None):
        ap = self.atmospheric_pressure

        def up(i, which):
            arr = self.atmospheric_pressure_current_arr if which == "current" else self.atmospheric_pressure_next_arr
            arr.upload(self.gpu_stream, ap.P[i])
        return self._update_forcing(ap.t, self.atmospheric_pressure_timestamps, "step", up)

    def __del__(self):
        try:
            self.cleanUp()
        except Exception:
            pass

    def cleanUp(self):
        pass

    def closeNetCDF(self):
        if self.write_netcdf and self.sim_writer is not None:
            self.sim_writer.__exit__(0, 0, 0)
            self.write_netcdf = False

    def attachDrifters(self, drifters):
        self.drifters = drifters
        self.hasDrifters = True
        self.drifters.setGPUStream(self.gpu_stream)
        self.drifter_t = self.t

    def attachCrossProductDrifters(self, drifter_list, sim_list):
        assert len(drifter_list) == len(sim_list), "Same number of drifter objects and partner simulations needed!"
        self.hasCrossProductDrifter = True
        self.CrossProductDrifter = drifter_list
        for d in self.CrossProductDrifter:
            d.setGPUStream(self.gpu_stream)
        self.CPsims = sim_list
        self.CPdrifter_t = self.t

    def download(self, interior_domain_only=False):
        eta, hu, hv = self.gpu_data.download(self.gpu_stream)
        if interior_domain_only:
            n, e, s, w = self.interior_domain_indices
            return eta[s:n, w:e], hu[s:n, w:e], hv[s:n, w:e]
        return eta, hu, hv

    def downloadPrevTimestep(self):
        return self.gpu_data.downloadPrevTimestep(self.gpu_stream)

    def copyState(self, otherSim):
        assert type(otherSim) is type(self), "A simulator can only copy the state from another simulator of the same class."
        assert (self.ny, self.nx) == (otherSim.ny, otherSim.nx), "Simulators differ in computational domain."
        for a, b in ((self.gpu_data.h0, otherSim.gpu_data.h0), (self.gpu_data.hu0, otherSim.gpu_data.hu0),
                     (self.gpu_data.hv0, otherSim.gpu_data.hv0), (self.gpu_data.h1, otherSim.gpu_data.h1),
                     (self.gpu_data.hu1, otherSim.gpu_data.hu1), (self.gpu_data.hv1, otherSim.gpu_data.hv1)):
            a.copyBuffer(self.gpu_stream, b)
        self.wind_stress = otherSim.wind_stress
        if otherSim.hasDrifters and self.hasDrifters:
            self.drifters.setDrifterPositions(otherSim.drifters.getDrifterPositions())
            self.drifters.setObservationPosition(otherSim.drifters.getObservationPosition())

    def upload(self, eta0, hu0, hv0, eta1=None, hu1=None, hv1=None):
        self.gpu_data.h0.upload(self.gpu_stream, eta0)
        self.gpu_data.hu0.upload(self.gpu_stream, hu0)
        self.gpu_data.hv0.upload(self.gpu_stream, hv0)
        if eta1 is None:
            eta1, hu1, hv1 = eta0, hu0, hv0
        self.gpu_data.h1.upload(self.gpu_stream, eta1)
        self.gpu_data.hu1.upload(self.gpu_stream, hu1)
        self.gpu_data.hv1.upload(self.gpu_stream, hv1)
        self.bc_kernel.update_bc_values(self.gpu_stream, self.t)
        self.bc_kernel.boundaryCondition(self.gpu_stream, self.gpu_data.h0, self.gpu_data.hu0, self.gpu_data.hv0)
