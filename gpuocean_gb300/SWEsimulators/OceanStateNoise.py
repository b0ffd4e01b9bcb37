"""SOAR model error of the ocean state (drop-in for ``SWEsimulators/OceanStateNoise.py:40-475``).

A coarse N(0,1) field is correlated with a SOAR covariance (5x5 stencil,
cutoff 2), optionally up-sampled bicubically by an odd factor, and added to
eta together with the geostrophically balanced momentum.  Random numbers
come from the GPU generators or are injected with ``setRandomNumbers``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .. import _lib
from ..utils import Common, RandomNumbers, config


class GocNoiseDesc(ctypes.Structure):
    """Mirror of ``GocNoiseDesc`` in include/gpuocean_gb300.h."""
    _fields_ = [
        ("coarse_nx", ctypes.c_int32), ("coarse_ny", ctypes.c_int32),
        ("coarse_dx", ctypes.c_float), ("coarse_dy", ctypes.c_float),
        ("soar_q0", ctypes.c_float), ("soar_L", ctypes.c_float),
        ("periodic_ns", ctypes.c_int32), ("periodic_ew", ctypes.c_int32),
        ("interpolation_factor", ctypes.c_int32),
        ("offset_i", ctypes.c_int32), ("offset_j", ctypes.c_int32),
        ("random", ctypes.c_void_p), ("random_pitch", ctypes.c_int32),
        ("coarse", ctypes.c_void_p), ("coarse_pitch", ctypes.c_int32),
        ("f", ctypes.c_float), ("beta", ctypes.c_float), ("g", ctypes.c_float),
        ("north_x", ctypes.c_float), ("north_y", ctypes.c_float),
        ("coriolis_f", ctypes.c_void_p), ("coriolis_nx", ctypes.c_int32), ("coriolis_ny", ctypes.c_int32),
    ]


class OceanStateNoise:
    def __init__(self, gpu_ctx, gpu_stream, nx, ny, dx, dy, boundaryConditions, staggered,
                 soar_q0=None, soar_L=None, interpolation_factor=1, use_lcg=False, xorwow_seed=None,
                 np_seed=None, angle=None, coriolis_f=None, block_width=16, block_height=16,
                 strict_odd_factor=True):
        if staggered:
            raise NotImplementedError("staggered grids (FBL/CTCS) are not part of this package")
        self.use_lcg = use_lcg
        self.random_state = np.random.RandomState()
        self.gpu_ctx = gpu_ctx
        self.gpu_stream = gpu_stream
        self.nx, self.ny = np.int32(nx), np.int32(ny)
        self.dx, self.dy = np.float32(dx), np.float32(dy)
        self.staggered = 0
        self.cutoff = np.int32(config.soar_cutoff)
        # the reference accepts odd factors only (S/OceanStateNoise.py:98); the
        # bicubic transfer here is defined for any factor, which
        # strict_odd_factor=False allows
        if strict_odd_factor:
            assert interpolation_factor > 0 and interpolation_factor % 2 == 1, \
                'interpolation_factor must be a positive odd integer'
        assert interpolation_factor > 0, 'interpolation_factor must be positive'
        self.periodicNorthSouth = np.int32(boundaryConditions.isPeriodicNorthSouth())
        if self.periodicNorthSouth:
            assert ny % interpolation_factor == 0, 'ny must be divisible by the interpolation factor'
        self.periodicEastWest = np.int32(boundaryConditions.isPeriodicEastWest())
        if self.periodicEastWest:
            assert nx % interpolation_factor == 0, 'nx must be divisible by the interpolation factor'
        self.interpolation_factor = np.int32(interpolation_factor)
        self.coarse_nx = np.int32(np.ceil(nx / self.interpolation_factor))
        self.coarse_ny = np.int32(np.ceil(ny / self.interpolation_factor))
        self.coarse_dx = np.float32(dx * self.interpolation_factor)
        self.coarse_dy = np.float32(dy * self.interpolation_factor)
        self.rand_ghost_cells_x = np.int32(0 if self.periodicEastWest else 2 + self.cutoff)
        self.rand_ghost_cells_y = np.int32(0 if self.periodicNorthSouth else 2 + self.cutoff)
        self.rand_nx = np.int32(self.coarse_nx + 2 * self.rand_ghost_cells_x)
        self.rand_ny = np.int32(self.coarse_ny + 2 * self.rand_ghost_cells_y)
        self.rng = RandomNumbers.RandomNumbers(gpu_ctx, gpu_stream, self.rand_nx, self.rand_ny, use_lcg=use_lcg,
                                               seed=np_seed, xorwow_seed=xorwow_seed,
                                               block_width=block_width, block_height=block_height)
        self.seed_ny = np.int32(self.rand_ny)
        self.seed_nx = np.int32(np.ceil(self.rand_nx / 2))
        self.floatMax = self.rng.floatMax
        self.host_seed = self.rng.host_seed if use_lcg else None
        self.soar_q0 = np.float32(self.dx / 100000) if soar_q0 is None else np.float32(soar_q0)
        self.soar_L = np.float32(0.75 * self.coarse_dx) if soar_L is None else np.float32(soar_L)
        self.random_numbers_host = np.zeros((self.rand_ny, self.rand_nx), dtype=np.float32)
        self.random_numbers = Common.CUDAArray2D(gpu_stream, self.rand_nx, self.rand_ny, 0, 0, self.random_numbers_host)
        self.coarse_buffer_host = np.zeros((self.coarse_ny + 4, self.coarse_nx + 4), dtype=np.float32)
        self.coarse_buffer = Common.CUDAArray2D(gpu_stream, self.coarse_nx, self.coarse_ny, 2, 2, self.coarse_buffer_host)
        if coriolis_f is None:
            coriolis_f = np.array([[0]], dtype=np.float32)
        if isinstance(coriolis_f, Common.CUDAArray2D):
            self.coriolis_f_arr = coriolis_f
        else:
            self.coriolis_f_arr = Common.CUDAArray2D(gpu_stream, coriolis_f.shape[1], coriolis_f.shape[0], 0, 0,
                                                     coriolis_f)
        if angle is None:
            angle = np.array([[0]], dtype=np.float32)
        if isinstance(angle, Common.CUDAArray2D):
            self.angle_arr = angle
            a0 = float(angle.download(gpu_stream).flat[0])
        else:
            self.angle_arr = Common.CUDAArray2D(gpu_stream, angle.shape[1], angle.shape[0], 0, 0, angle)
            a0 = float(np.asarray(angle).flat[0])
        # the north vector of the noise kernels is taken from the first angle value
        self.north = (np.float32(np.sin(a0)), np.float32(np.cos(a0)))
        self.local_size = (block_width, block_height, 1)

    @classmethod
    def fromsim(cls, sim, soar_q0=None, soar_L=None, interpolation_factor=1, use_lcg=False, xorwow_seed=None,
                block_width=16, block_height=16, strict_odd_factor=True):
        return cls(sim.gpu_ctx, sim.gpu_stream, sim.nx, sim.ny, sim.dx, sim.dy, sim.boundary_conditions, False,
                   soar_q0=soar_q0, soar_L=soar_L, interpolation_factor=interpolation_factor,
                   angle=sim.angle_arr, coriolis_f=sim.coriolis_f_arr, use_lcg=use_lcg, xorwow_seed=xorwow_seed,
                   block_width=block_width, block_height=block_height, strict_odd_factor=strict_odd_factor)

    def cleanUp(self, do_gc=True):
        for a in ("random_numbers", "coarse_buffer"):
            arr = getattr(self, a, None)
            if arr is not None:
                arr.release()
        if getattr(self, "rng", None) is not None:
            self.rng.cleanUp()

    def __del__(self):
        try:
            self.cleanUp()
        except Exception:
            pass

    # ------------------------------------------------------------------
    def getSeed(self):
        return self.rng.getSeed()

    def resetSeed(self):
        self.rng.resetSeed()

    def getRandomNumbers(self):
        return self.random_numbers.download(self.gpu_stream)

    def setRandomNumbers(self, random_numbers):
        """Inject a (rand_ny, rand_nx) field of N(0,1) draws (host array)."""
        self.random_numbers.upload(self.gpu_stream, np.asarray(random_numbers, dtype=np.float32))

    def getCoarseBuffer(self):
        return self.coarse_buffer.download(self.gpu_stream)

    def generateNormalDistribution(self):
        self.rng.generateNormalDistribution(self.random_numbers)

    def generateUniformDistribution(self):
        self.rng.generateUniformDistribution(self.random_numbers)

    def _obtain_coarse_grid_offset(self, fine_index_i, fine_index_j):
        default_offset = self.interpolation_factor // 2
        offset_i, offset_j = 0, 0
        if fine_index_i is not None:
            offset_i = -int(fine_index_i % self.interpolation_factor - default_offset)
        if fine_index_j is not None:
            offset_j = -int(fine_index_j % self.interpolation_factor - default_offset)
        return offset_i, offset_j

    def descriptor(self, f, beta, g, offset_i=0, offset_j=0, q0_scale=1.0):
        d = GocNoiseDesc()
        d.coarse_nx, d.coarse_ny = int(self.coarse_nx), int(self.coarse_ny)
        d.coarse_dx, d.coarse_dy = float(self.coarse_dx), float(self.coarse_dy)
        d.soar_q0 = float(np.float32(self.soar_q0 * q0_scale))
        d.soar_L = float(self.soar_L)
        d.periodic_ns, d.periodic_ew = int(self.periodicNorthSouth), int(self.periodicEastWest)
        d.interpolation_factor = int(self.interpolation_factor)
        d.offset_i, d.offset_j = int(offset_i), int(offset_j)
        d.random, d.random_pitch = self.random_numbers.ptr, int(self.random_numbers.pitch)
        d.coarse, d.coarse_pitch = self.coarse_buffer.ptr, int(self.coarse_buffer.pitch)
        d.f, d.beta, d.g = float(np.float32(f)), float(np.float32(beta)), float(np.float32(g))
        d.north_x, d.north_y = float(self.north[0]), float(self.north[1])
        d.coriolis_f = self.coriolis_f_arr.ptr
        d.coriolis_nx, d.coriolis_ny = int(self.coriolis_f_arr.nx_halo), int(self.coriolis_f_arr.ny_halo)
        return d

    def perturbSim(self, sim, q0_scale=1.0, update_random_field=True, perturbation_scale=1.0,
                   perpendicular_scale=0.0, align_with_cell_i=None, align_with_cell_j=None, stream=None):
        self.perturbOceanState(sim.gpu_data.h0, sim.gpu_data.hu0, sim.gpu_data.hv0, sim.bathymetry.Bi,
                               sim.f, beta=sim.coriolis_beta, g=sim.g, y0_reference_cell=sim.y_zero_reference_cell,
                               ghost_cells_x=sim.ghost_cells_x, ghost_cells_y=sim.ghost_cells_y, q0_scale=q0_scale,
                               update_random_field=update_random_field, perturbation_scale=perturbation_scale,
                               perpendicular_scale=perpendicular_scale, align_with_cell_i=align_with_cell_i,
                               align_with_cell_j=align_with_cell_j, land_mask_value=sim.bathymetry.mask_value,
                               stream=stream)

    def perturbSimSimilarAs(self, sim, modelError, perturbation_scale=1.0):
        """Perturb `sim` with the random field of another noise object (the
        coarse/fine partner of a multi-level pair)."""
        self.random_numbers.copyBuffer(self.gpu_stream, modelError.random_numbers)
        self.perturbSim(sim, update_random_field=False, perturbation_scale=perturbation_scale)

    def perturbOceanState(self, eta, hu, hv, H, f, beta=0.0, g=9.81, y0_reference_cell=0, ghost_cells_x=0,
                          ghost_cells_y=0, q0_scale=1.0, update_random_field=True, perturbation_scale=1.0,
                          perpendicular_scale=0.0, align_with_cell_i=None, align_with_cell_j=None,
                          land_mask_value=np.float32(1.0e20), stream=None):
        """SOAR field from the random numbers, then the balanced perturbation of
        the interior (S/OceanStateNoise.py:356-459)."""
        if perpendicular_scale > 0:
            raise NotImplementedError("perpendicular random fields (IEWPF) are not part of this package")
        if ghost_cells_x != 2 or ghost_cells_y != 2:
            raise NotImplementedError("the state must carry two ghost cells per side")
        st = Common._stream_handle(stream if stream is not None else self.gpu_stream)
        if update_random_field:
            self.generateNormalDistribution()
        oi, oj = self._obtain_coarse_grid_offset(align_with_cell_i, align_with_cell_j)
        d = self.descriptor(f, beta, g, oi, oj, q0_scale)
        _lib.call("goc_soar", ctypes.byref(d), ctypes.c_float(perturbation_scale), 0, st)
        _lib.call("goc_perturb_ocean", ctypes.byref(d), int(self.nx), int(self.ny), ctypes.c_float(self.dx),
                  ctypes.c_float(self.dy), eta.ptr, hu.ptr, hv.ptr, int(eta.pitch), H.ptr, int(H.pitch),
                  ctypes.c_float(land_mask_value), 1, st)
