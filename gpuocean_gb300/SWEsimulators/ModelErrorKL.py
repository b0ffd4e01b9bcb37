"""Karhunen-Loeve model error (drop-in for ``SWEsimulators/ModelErrorKL.py:38-463``).

A perturbation of eta is sampled from sine and cosine basis functions on the
unit square, m^-decay n^-decay sin(2 pi m y) sin(2 pi n x) (and cosines),
weighted with N(0,1) draws and shifted by random "rollers"; hu and hv get
the geostrophically balanced perturbation.  The device evaluates the
separable sum from per-column and per-row tables (``goc_kl_perturb``) instead
of all 2 Nx Ny transcendental terms per cell.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .. import _lib
from ..utils import Common, RandomNumbers


class GocKLDesc(ctypes.Structure):
    """Mirror of ``GocKLDesc`` in include/gpuocean_gb300.h."""
    _fields_ = [
        ("basis_x_start", ctypes.c_int32), ("basis_x_end", ctypes.c_int32),
        ("basis_y_start", ctypes.c_int32), ("basis_y_end", ctypes.c_int32),
        ("include_cos", ctypes.c_int32), ("include_sin", ctypes.c_int32),
        ("kl_decay", ctypes.c_float), ("kl_scaling", ctypes.c_float),
        ("roll_x_sin", ctypes.c_float), ("roll_y_sin", ctypes.c_float),
        ("roll_x_cos", ctypes.c_float), ("roll_y_cos", ctypes.c_float),
        ("random", ctypes.c_void_p), ("random_pitch", ctypes.c_int32),
        ("f", ctypes.c_float), ("beta", ctypes.c_float), ("g", ctypes.c_float),
        ("north_x", ctypes.c_float), ("north_y", ctypes.c_float),
        ("coriolis_f", ctypes.c_void_p), ("coriolis_nx", ctypes.c_int32), ("coriolis_ny", ctypes.c_int32),
        ("table", ctypes.c_void_p),
    ]


class ModelErrorKL:
    def __init__(self, gpu_ctx, gpu_stream, nx, ny, dx, dy, boundary_conditions,
                 kl_decay=1.2, kl_scaling=1.0, include_cos=True, include_sin=True,
                 basis_x_start=1, basis_y_start=1, basis_x_end=10, basis_y_end=10,
                 use_lcg=False, xorwow_seed=None, np_seed=None,
                 angle=np.array([[0]], dtype=np.float32), coriolis_f=np.array([[0]], dtype=np.float32),
                 block_width=16, block_height=16):
        self.use_lcg = use_lcg
        self.random_state = np.random.RandomState()
        self.gpu_ctx = gpu_ctx
        self.gpu_stream = gpu_stream
        self.nx, self.ny = np.int32(nx), np.int32(ny)
        self.dx, self.dy = np.float32(dx), np.float32(dy)
        self.boundary_conditions = boundary_conditions
        self.kl_decay = np.float32(kl_decay)
        self.kl_scaling = np.float32(kl_scaling)
        self.include_cos = np.int32(include_cos)
        self.include_sin = np.int32(include_sin)
        self.basis_x_start, self.basis_y_start = np.int32(basis_x_start), np.int32(basis_y_start)
        self.basis_x_end, self.basis_y_end = np.int32(basis_x_end), np.int32(basis_y_end)
        self.np_rng = np.random.default_rng(seed=np_seed)
        self.roll_x_sin = self.roll_y_sin = self.roll_x_cos = self.roll_y_cos = 0.0
        self.N_basis_x = np.int32(self.basis_x_end - self.basis_x_start + 1)
        self.N_basis_y = np.int32(self.basis_y_end - self.basis_y_start + 1)
        # one normal per basis function: sine rows first, then cosine rows
        self.rand_nx = np.int32(self.N_basis_x)
        self.rand_ny = np.int32(self.N_basis_y * 2)
        self.rng = RandomNumbers.RandomNumbers(gpu_ctx, gpu_stream, self.rand_nx, self.rand_ny, use_lcg=use_lcg,
                                               seed=np_seed, xorwow_seed=xorwow_seed,
                                               block_width=block_width, block_height=block_height)
        self.seed_ny = np.int32(self.rand_ny)
        self.seed_nx = np.int32(np.ceil(self.rand_nx / 2))
        self.floatMax = self.rng.floatMax
        self.host_seed = self.rng.host_seed if use_lcg else None
        self.random_numbers_host = np.zeros((self.rand_ny, self.rand_nx), dtype=np.float32)
        self.random_numbers = Common.CUDAArray2D(gpu_stream, self.rand_nx, self.rand_ny, 0, 0,
                                                 self.random_numbers_host)
        if isinstance(coriolis_f, Common.CUDAArray2D):
            self.coriolis_f_arr = coriolis_f
        else:
            coriolis_f = np.atleast_2d(np.asarray(coriolis_f, dtype=np.float32))
            self.coriolis_f_arr = Common.CUDAArray2D(gpu_stream, coriolis_f.shape[1], coriolis_f.shape[0], 0, 0,
                                                     coriolis_f)
        if isinstance(angle, Common.CUDAArray2D):
            self.angle_arr = angle
            a0 = float(angle.download(gpu_stream).flat[0])
        else:
            angle = np.atleast_2d(np.asarray(angle, dtype=np.float32))
            self.angle_arr = Common.CUDAArray2D(gpu_stream, angle.shape[1], angle.shape[0], 0, 0, angle)
            a0 = float(angle.flat[0])
        # the noise kernels take the north vector from the first angle value
        # (as for the SOAR noise)
        self.north = (np.float32(np.sin(a0)), np.float32(np.cos(a0)))
        self.local_size = (block_width, block_height, 1)
        probe = self._desc(0.0, 0.0, 9.81)
        self.table = Common.DevicePtr(4 * _lib.load().goc_kl_table_floats(int(nx), int(ny), ctypes.byref(probe)))

    @classmethod
    def fromsim(cls, sim, kl_decay=1.2, kl_scaling=1.0, include_cos=True, include_sin=True,
                basis_x_start=1, basis_y_start=1, basis_x_end=10, basis_y_end=10,
                use_lcg=False, xorwow_seed=None, np_seed=None, block_width=16, block_height=16):
        return cls(sim.gpu_ctx, sim.gpu_stream, sim.nx, sim.ny, sim.dx, sim.dy, sim.boundary_conditions,
                   kl_decay=kl_decay, kl_scaling=kl_scaling, include_cos=include_cos, include_sin=include_sin,
                   basis_x_start=basis_x_start, basis_y_start=basis_y_start,
                   basis_x_end=basis_x_end, basis_y_end=basis_y_end,
                   angle=sim.angle_arr, coriolis_f=sim.coriolis_f_arr,
                   use_lcg=use_lcg, xorwow_seed=xorwow_seed, np_seed=np_seed,
                   block_width=block_width, block_height=block_height)

    def cleanUp(self, do_gc=True):
        if getattr(self, "rng", None) is not None:
            self.rng.cleanUp()
        for a in ("random_numbers",):
            arr = getattr(self, a, None)
            if arr is not None:
                arr.release()
        if getattr(self, "table", None) is not None:
            self.table.free()
        self.boundary_conditions = None

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

    def generateNormalDistribution(self):
        self.rng.generateNormalDistribution(self.random_numbers)

    def setRandomNumbers(self, random_numbers):
        assert random_numbers.shape == self.random_numbers_host.shape, \
            "Wrong shape of random numbers: " + str(random_numbers.shape) + " vs " + str(self.random_numbers_host.shape)
        self.random_numbers_host[:, :] = random_numbers[:, :]
        self.random_numbers.upload(self.gpu_stream, self.random_numbers_host)

    def _setRollers(self, roll_x_sin, roll_y_sin, roll_x_cos, roll_y_cos):
        """Rollers in [0, 1]; missing ones are drawn from the model error's
        own generator in the order x_sin, y_sin, x_cos, y_cos
        (S/ModelErrorKL.py:277-300)."""
        if roll_x_sin is None:
            roll_x_sin = self.np_rng.uniform()
        if roll_y_sin is None:
            roll_y_sin = self.np_rng.uniform()
        if roll_x_cos is None:
            roll_x_cos = self.np_rng.uniform()
        if roll_y_cos is None:
            roll_y_cos = self.np_rng.uniform()
        for r, name in ((roll_x_sin, "roll_x_sin"), (roll_y_sin, "roll_y_sin"), (roll_x_cos, "roll_x_cos"),
                        (roll_y_cos, "roll_y_cos")):
            assert isinstance(r, (float, int, np.float32)) and 0 <= r <= 1, \
                "illegal type/value of " + name + ": " + str(r)
        self.roll_x_sin, self.roll_y_sin = roll_x_sin, roll_y_sin
        self.roll_x_cos, self.roll_y_cos = roll_x_cos, roll_y_cos

    def _desc(self, f, beta, g):
        d = GocKLDesc()
        d.basis_x_start, d.basis_x_end = int(self.basis_x_start), int(self.basis_x_end)
        d.basis_y_start, d.basis_y_end = int(self.basis_y_start), int(self.basis_y_end)
        d.include_cos, d.include_sin = int(self.include_cos), int(self.include_sin)
        d.kl_decay, d.kl_scaling = float(self.kl_decay), float(self.kl_scaling)
        d.roll_x_sin, d.roll_y_sin = float(np.float32(self.roll_x_sin)), float(np.float32(self.roll_y_sin))
        d.roll_x_cos, d.roll_y_cos = float(np.float32(self.roll_x_cos)), float(np.float32(self.roll_y_cos))
        rn = getattr(self, "random_numbers", None)
        if rn is not None:
            d.random, d.random_pitch = rn.ptr, int(rn.pitch)
        d.f, d.beta, d.g = float(np.float32(f)), float(np.float32(beta)), float(np.float32(g))
        d.north_x, d.north_y = float(self.north[0]), float(self.north[1])
        d.coriolis_f = self.coriolis_f_arr.ptr
        d.coriolis_nx, d.coriolis_ny = int(self.coriolis_f_arr.nx_halo), int(self.coriolis_f_arr.ny_halo)
        t = getattr(self, "table", None)
        d.table = t.ptr if t is not None else None
        return d

    def _refresh(self, random_numbers, update_random_field, stream):
        if random_numbers is not None:
            assert isinstance(random_numbers, (Common.CUDAArray2D, np.ndarray)), \
                "random numbers should be a CUDA 2D array or a numpy array, but is " + str(type(random_numbers))
            if isinstance(random_numbers, Common.CUDAArray2D):
                self.random_numbers.copyBuffer(stream, random_numbers)
            else:
                self.random_numbers.upload(stream, np.asarray(random_numbers, dtype=np.float32))
        elif update_random_field:
            self.generateNormalDistribution()

    # ------------------------------------------------------------------
    def perturbEtaSim(self, sim, perturbation_scale=1.0, update_random_field=True, random_numbers=None,
                      roll_x_sin=None, roll_y_sin=None, roll_x_cos=None, roll_y_cos=None, stream=None):
        self.perturbEta(sim.gpu_data.h0, update_random_field=update_random_field, random_numbers=random_numbers,
                        roll_x_sin=roll_x_sin, roll_y_sin=roll_y_sin, roll_x_cos=roll_x_cos, roll_y_cos=roll_y_cos,
                        perturbation_scale=perturbation_scale, stream=stream)

    def perturbEta(self, eta, update_random_field=True, random_numbers=None, roll_x_sin=None, roll_y_sin=None,
                   roll_x_cos=None, roll_y_cos=None, perturbation_scale=1.0, stream=None):
        """KL perturbation added to the interior of eta only (kl_sample_eta)."""
        stream = self.gpu_stream if stream is None else stream
        self._refresh(random_numbers, update_random_field, stream)
        self._setRollers(roll_x_sin, roll_y_sin, roll_x_cos, roll_y_cos)
        d = self._desc(0.0, 0.0, 9.81)
        _lib.call("goc_kl_perturb", ctypes.byref(d), int(self.nx), int(self.ny), ctypes.c_float(self.dx),
                  ctypes.c_float(self.dy), ctypes.c_float(perturbation_scale), 1, eta.ptr, None, None,
                  int(eta.pitch), None, 0, 0, 0, Common._stream_handle(stream))

    def perturbSim(self, sim, perturbation_scale=1.0, update_random_field=True, random_numbers=None,
                   roll_x_sin=None, roll_y_sin=None, roll_x_cos=None, roll_y_cos=None, stream=None):
        self.perturbOceanState(sim.gpu_data.h0, sim.gpu_data.hu0, sim.gpu_data.hv0, sim.bathymetry.Bi,
                               sim.dx, sim.dy, sim.f, beta=sim.coriolis_beta, g=sim.g,
                               y0_reference_cell=sim.y_zero_reference_cell,
                               update_random_field=update_random_field, perturbation_scale=perturbation_scale,
                               land_mask_value=sim.bathymetry.mask_value, random_numbers=random_numbers,
                               roll_x_sin=roll_x_sin, roll_y_sin=roll_y_sin, roll_x_cos=roll_x_cos,
                               roll_y_cos=roll_y_cos, stream=stream,
                               periodic=(sim.boundary_conditions.isPeriodicNorthSouth(),
                                         sim.boundary_conditions.isPeriodicEastWest()))

    def perturbOceanState(self, eta, hu, hv, H, dx, dy, f, beta=0.0, g=9.81, y0_reference_cell=0,
                          update_random_field=True, perturbation_scale=1.0, land_mask_value=np.float32(1.0e20),
                          random_numbers=None, roll_x_sin=None, roll_y_sin=None, roll_x_cos=None, roll_y_cos=None,
                          stream=None, periodic=(False, False)):
        """KL perturbation of eta plus the balanced hu, hv (kl_sample_ocean_state,
        S/ModelErrorKL.py:365-449).  ``periodic`` (north-south, east-west)
        also writes the periodic ghost images of the perturbed cells."""
        stream = self.gpu_stream if stream is None else stream
        self._refresh(random_numbers, update_random_field, stream)
        self._setRollers(roll_x_sin, roll_y_sin, roll_x_cos, roll_y_cos)
        d = self._desc(f, beta, g)
        _lib.call("goc_kl_perturb", ctypes.byref(d), int(self.nx), int(self.ny), ctypes.c_float(dx),
                  ctypes.c_float(dy), ctypes.c_float(perturbation_scale), 0, eta.ptr, hu.ptr, hv.ptr,
                  int(eta.pitch), H.ptr, int(H.pitch), int(bool(periodic[0])), int(bool(periodic[1])),
                  Common._stream_handle(stream))

    def perturbSimSimilarAs(self, simToPerturb, simSource=None, modelError=None, stream=None, perturbation_scale=1.0):
        """Perturb with another model error's normals and rollers (the coarse
        partner of a multi-level pair, S/ModelErrorKL.py:451-463)."""
        assert simSource is not None or modelError is not None, \
            "Please provide either simSource or modelError input arguments"
        assert simSource is None or modelError is None, \
            "Please provide only one of simSource or modelError, not both."
        if simSource is not None:
            modelError = simSource.model_error
        self.perturbSim(simToPerturb, perturbation_scale=perturbation_scale, random_numbers=modelError.random_numbers,
                        roll_x_cos=modelError.roll_x_cos, roll_y_cos=modelError.roll_y_cos,
                        roll_x_sin=modelError.roll_x_sin, roll_y_sin=modelError.roll_y_sin, stream=stream)

    def batch_descriptor(self, sim):
        """Descriptor of this model error on `sim` for the batched engine."""
        return self._desc(sim.f, sim.coriolis_beta, sim.g)
