"""Random number generation on the GPU (counterpart of ``utils/RandomNumbers.py:39-185``).

Two generators, as in the reference: an LCG with one uint64 seed per pair
of numbers (seeded from ``numpy.random.RandomState(seed)``) and curand's
XORWOW (the default).  ``setRandomNumbers`` injects host-drawn normals.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .. import _lib
from . import Common


class RandomNumbers:
    def __init__(self, gpu_ctx, gpu_stream, nx, ny, use_lcg=False, seed=None, xorwow_seed=None,
                 block_width=16, block_height=16):
        self.use_lcg = use_lcg
        self.gpu_stream = gpu_stream
        self.random_state = np.random.RandomState(seed=seed)
        self.nx, self.ny = np.int32(nx), np.int32(ny)
        self.seed_ny = np.int32(self.ny)
        self.seed_nx = np.int32(np.ceil(self.nx / 2))
        self.floatMax = 2147483648.0
        self.host_seed = None
        self.seed = None
        self.states = None
        if self.use_lcg:
            self.host_seed = (self.random_state.rand(self.seed_ny, self.seed_nx) * self.floatMax).astype(np.uint64)
            self.seed = Common.CUDAArray2D(gpu_stream, self.seed_nx, self.seed_ny, 0, 0, self.host_seed, integers=True)
        else:
            if xorwow_seed is None:
                xorwow_seed = seed if seed is not None else np.random.randint(0, 2 ** 31 - 1)
            n = int(self.nx) * int(self.ny)
            self.states = Common.DevicePtr(_lib.load().goc_xorwow_state_bytes(n))
            _lib.call("goc_xorwow_init", self.states.ptr, n, ctypes.c_ulonglong(int(xorwow_seed)),
                      Common._stream_handle(gpu_stream))

    def cleanUp(self):
        if self.seed is not None:
            self.seed.release()
            self.seed = None
        if self.states is not None:
            self.states.free()
            self.states = None

    def __del__(self):
        try:
            self.cleanUp()
        except Exception:
            pass

    def getSeed(self):
        assert self.use_lcg, "getSeed is only valid if LCG is used as pseudo-random generator."
        return self.seed.download(self.gpu_stream)

    def resetSeed(self):
        assert self.use_lcg, "resetSeed is only valid if LCG is used as pseudo-random generator."
        self.host_seed = (self.random_state.rand(self.seed_ny, self.seed_nx) * self.floatMax).astype(np.uint64)
        self.seed.upload(self.gpu_stream, self.host_seed)

    def _check(self, arr):
        assert (arr.ny, arr.nx) == (self.ny, self.nx), \
            "expected random_numbers with shape " + str((self.ny, self.nx)) + " but got " + str((arr.ny, arr.nx))

    def _lcg(self, random_numbers, normal):
        _lib.call("goc_lcg_fill", int(self.seed_nx), int(self.seed_ny), int(self.nx), self.seed.ptr,
                  int(self.seed.pitch), random_numbers.ptr, int(random_numbers.pitch), int(normal),
                  Common._stream_handle(self.gpu_stream))

    def generateNormalDistribution(self, random_numbers):
        self._check(random_numbers)
        if self.use_lcg:
            self._lcg(random_numbers, True)
        else:
            _lib.call("goc_xorwow_normal", self.states.ptr, int(self.nx), int(self.ny), random_numbers.ptr,
                      int(random_numbers.pitch), Common._stream_handle(self.gpu_stream))

    def generateUniformDistribution(self, random_numbers):
        self._check(random_numbers)
        if not self.use_lcg:
            raise NotImplementedError("uniform draws are provided by the LCG generator (use_lcg=True)")
        self._lcg(random_numbers, False)
