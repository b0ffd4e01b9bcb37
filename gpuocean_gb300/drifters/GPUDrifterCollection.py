"""Drifters advected on the GPU (drop-in for ``drifters/GPUDrifterCollection.py:34-253``).

Positions live on the device as a (N+1) x 2 float32 array (the last row is
the observation); ``drift`` is one launch of the library's drift kernel.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .. import _lib
from ..utils import Common, WindStress
from .BaseDrifterCollection import BaseDrifterCollection


class GPUDrifterCollection(BaseDrifterCollection):
    def __init__(self, gpu_ctx, numDrifters, observation_variance=0.01, boundaryConditions=None,
                 initialization_cov_drifters=None, domain_size_x=1.0, domain_size_y=1.0, gpu_stream=None,
                 initialize=False, wind=None, wind_drift_factor=0.0, block_width=64):
        super().__init__(numDrifters, observation_variance=observation_variance,
                         boundaryConditions=boundaryConditions, domain_size_x=domain_size_x,
                         domain_size_y=domain_size_y)
        self.gpu_ctx = gpu_ctx
        self.block_width = block_width
        self.block_height = 1
        self.wind = wind if wind is not None else WindStress.WindStress()
        self.wind_drift_factor = np.float32(wind_drift_factor)
        # the drift kernel reads both wind components with the x texture's
        # size (as the reference's does, K/driftKernels.cu:155-156): textures
        # of different sizes would be read out of bounds
        if self.wind_drift_factor and any(np.shape(u) != np.shape(v)
                                          for u, v in zip(self.wind.wind_u, self.wind.wind_v)):
            raise ValueError("wind drift needs wind_u and wind_v textures of the same shape")
        self.gpu_stream = gpu_stream if gpu_stream is not None else Common.Stream()
        self.sensitivity = 1.0
        self.driftersHost = np.zeros((self.getNumDrifters() + 1, 2), dtype=np.float32)
        self.driftersDevice = Common.CUDAArray2D(self.gpu_stream, 2, self.getNumDrifters() + 1, 0, 0,
                                                 self.driftersHost)
        t0, t1 = 0, 0
        self.wind_timestamps = {}
        s = self.gpu_stream
        w = self.wind
        self.wind_x_current_arr = Common.CUDAArray2D(s, w.wind_u[t0].shape[1], w.wind_u[t0].shape[0], 0, 0, w.wind_u[t0])
        self.wind_y_current_arr = Common.CUDAArray2D(s, w.wind_v[t0].shape[1], w.wind_v[t0].shape[0], 0, 0, w.wind_v[t0])
        self.wind_x_next_arr = Common.CUDAArray2D(s, w.wind_u[t1].shape[1], w.wind_u[t1].shape[0], 0, 0, w.wind_u[t1])
        self.wind_y_next_arr = Common.CUDAArray2D(s, w.wind_v[t1].shape[1], w.wind_v[t1].shape[0], 0, 0, w.wind_v[t1])
        if self.wind_drift_factor:
            self.update_wind(0.0)
        if initialize:
            self.uniformly_distribute_drifters(initialization_cov_drifters=initialization_cov_drifters)

    def copy(self):
        c = GPUDrifterCollection(self.gpu_ctx, self.getNumDrifters(), observation_variance=self.observation_variance,
                                 boundaryConditions=self.boundaryConditions, domain_size_x=self.domain_size_x,
                                 domain_size_y=self.domain_size_y, gpu_stream=self.gpu_stream,
                                 block_width=self.block_width)
        c.setDrifterPositions(self.getDrifterPositions())
        c.setObservationPosition(self.getObservationPosition())
        return c

    def update_wind(self, t):
        """Bring the current / next wind textures to the interval of time t
        and return the time weight of t in it (D/GPUDrifterCollection.py:
        138-174)."""
        t0, t1 = self.wind_interval(t)
        self.load_wind_interval(t0, t1)
        return self.wind_weight(t, t0, t1)

    def wind_interval(self, t, side="left"):
        """Indices of the wind time stamps around t.  At a time stamp itself
        side "left" gives the interval that ends there (as update_wind
        chooses), "right" the one that starts there; both give t the same
        wind (weight 1 of the one, weight 0 of the other)."""
        last = len(self.wind.t) - 1
        k = int(np.searchsorted(self.wind.t, t, side=side))
        return max(0, k - 1), min(last, k)

    def load_wind_interval(self, t0, t1):
        w = self.wind
        new_t0, new_t1 = w.t[t0], w.t[t1]
        old = self.wind_timestamps.get("drift", [None, None])
        self.wind_timestamps["drift"] = [new_t0, new_t1]
        if new_t0 != old[0]:
            self.wind_x_current_arr.upload(self.gpu_stream, w.wind_u[t0])
            self.wind_y_current_arr.upload(self.gpu_stream, w.wind_v[t0])
        if new_t1 != old[1]:
            self.wind_x_next_arr.upload(self.gpu_stream, w.wind_u[t1])
            self.wind_y_next_arr.upload(self.gpu_stream, w.wind_v[t1])

    def wind_weight(self, t, t0, t1):
        new_t0, new_t1 = self.wind.t[t0], self.wind.t[t1]
        return max(0.0, min(1.0, (t - new_t0) / max(1.0e-10, (new_t1 - new_t0))))

    def setDrifterPositions(self, newDrifterPositions):
        allpos = np.concatenate((np.asarray(newDrifterPositions, dtype=np.float32),
                                 np.array([self.getObservationPosition()], dtype=np.float32)), axis=0)
        self.driftersDevice.upload(self.gpu_stream, allpos)

    def setObservationPosition(self, newObservationPosition):
        allpos = np.concatenate((self.getDrifterPositions(), np.array([newObservationPosition], dtype=np.float32)))
        self.driftersDevice.upload(self.gpu_stream, allpos)

    def setSensitivity(self, sensitivity):
        self.sensitivity = sensitivity

    def getDrifterPositions(self):
        return self.driftersDevice.download(self.gpu_stream)[:-1, :]

    def getObservationPosition(self):
        return self.driftersDevice.download(self.gpu_stream)[self.obs_index, :]

    def driftFromSim(self, sim, dt):
        self.drift(sim.gpu_data.h0, sim.gpu_data.hu0, sim.gpu_data.hv0, sim.bathymetry.Bm, sim.nx, sim.ny, sim.t,
                   sim.dx, sim.dy, dt, np.int32(2), np.int32(2))

    def drift(self, eta, hu, hv, Hm, nx, ny, t, dx, dy, dt, x_zero_ref, y_zero_ref):
        wind_t = np.float32(self.update_wind(t)) if self.wind_drift_factor else np.float32(0.0)
        bc = self.boundaryConditions
        _lib.call("goc_drift", int(nx), int(ny), ctypes.c_float(dx), ctypes.c_float(dy), ctypes.c_float(dt),
                  int(x_zero_ref), int(y_zero_ref), eta.ptr, hu.ptr, hv.ptr, int(eta.pitch), Hm.ptr, int(Hm.pitch),
                  int(bc.isPeriodicNorthSouth()), int(bc.isPeriodicEastWest()), int(self.getNumDrifters()),
                  self.driftersDevice.ptr, int(self.driftersDevice.pitch), ctypes.c_float(self.sensitivity),
                  self.wind_x_current_arr.ptr, self.wind_x_next_arr.ptr, self.wind_y_current_arr.ptr,
                  self.wind_y_next_arr.ptr, int(self.wind_x_current_arr.nx_halo), int(self.wind_x_current_arr.ny_halo),
                  ctypes.c_float(wind_t), ctypes.c_float(self.wind_drift_factor), self.gpu_stream.handle)

    def setGPUStream(self, gpu_stream):
        self.gpu_stream = gpu_stream

    def cleanUp(self):
        for a in ("driftersDevice", "wind_x_current_arr", "wind_y_current_arr", "wind_x_next_arr", "wind_y_next_arr"):
            arr = getattr(self, a, None)
            if arr is not None:
                arr.release()
        self.gpu_ctx = None

    def enforceBoundaryConditions(self):
        bc = self.boundaryConditions
        if bc.isPeriodicNorthSouth() or bc.isPeriodicEastWest():
            _lib.call("goc_drift_enforce_boundary", ctypes.c_float(self.domain_size_x),
                      ctypes.c_float(self.domain_size_y), int(bc.isPeriodicNorthSouth()),
                      int(bc.isPeriodicEastWest()), int(self.numDrifters), self.driftersDevice.ptr,
                      int(self.driftersDevice.pitch), self.gpu_stream.handle)
