"""The reference's own CUDA kernels, run on the GPU as a second oracle.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module.

``oracle/build_ref.py`` compiles the reference kernel sources
(``src/gpuocean/gpu_kernels/*.cu`` of GPU Ocean) unchanged to sm_103a cubins
under ``oracle/_ref/``, with the ``#define`` sets and nvcc options that the
reference's Python host passes to PyCUDA for each configuration listed in
``REF_CONFIGS``.  This module loads those cubins through the CUDA driver API
(ctypes on ``libcuda``) and replays the reference host's launch sequences:

* ``RefCDKLM16``: ``CDKLM16.__init__`` bathymetry set-up
  (U/Common.py:1408-1491: intersection BC kernels + initBm), the dry clamp of
  eta0 (S/CDKLM16.py:320-321), the RK2 step sequence of ``CDKLM16.step``
  (S/CDKLM16.py:477-584: stage 0, ghost fill of the stage buffer, stage 1,
  optional model error, ghost fill), ``callKernel`` (:688-723) and
  ``updateDt`` (:814-841).
* ``RefNoise.perturb``: ``OceanStateNoise.perturbOceanState``
  (S/OceanStateNoise.py:380-459) on injected normals: SOAR into the coarse
  buffer, then bicubicInterpolation (factor > 1) or geostrophicBalance.
* ``RefDrifters.drift``: ``GPUDrifterCollection.drift``
  (D/GPUDrifterCollection.py:198-233); ``enforce_boundary`` runs
  ``enforceBoundaryConditions`` (:240-253), which ``drift`` itself does not.

Paths: S/ = src/gpuocean/SWEsimulators, U/ = src/gpuocean/utils,
D/ = src/gpuocean/drifters, K/ = src/gpuocean/gpu_kernels.

Memory is allocated in the device's primary context (the one the CUDA
runtime uses), so buffers can be compared with the product's directly.
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

# ---------------------------------------------------------------------------
# configurations: the #defines the reference host would emit
# ---------------------------------------------------------------------------

CDKLM_FLAGS = ["--ftz=true", "--prec-div=false", "--prec-sqrt=false", "--fmad=false"]   # S/CDKLM16.py:277-281
NOISE_FLAGS = ["--use_fast_math", "--maxrregcount=32"]                                   # S/OceanStateNoise.py:214-217


def _f(x):
    return "{:.12f}f".format(float(np.float32(x)))


def cdklm_defines(nx, ny, dx, dy, g=9.81, r=0.0, theta=1.8, rk_order=2, coriolis_shape=(1, 1),
                  angle_shape=(1, 1), desing_eps=0.1, flux_slope_eps=0.1, depth_cutoff=1e-5,
                  rho_o=1025.0, wind_stress_factor=1.0, flux_balancer=0.8, block=(12, 32),
                  wind_shape=(1, 1), pressure_shape=(1, 1), direct_lookup=False):
    """S/CDKLM16.py:242-269 (one_dimensional False); texture shapes are (ny, nx)."""
    return {"block_width": block[0], "block_height": block[1],
            "KPSIMULATOR_DESING_EPS": _f(desing_eps), "KPSIMULATOR_FLUX_SLOPE_EPS": _f(flux_slope_eps),
            "KPSIMULATOR_DEPTH_CUTOFF": _f(depth_cutoff), "THETA": _f(theta), "RK_ORDER": int(rk_order),
            "NX": int(nx), "NY": int(ny), "DX": _f(dx), "DY": _f(dy), "GRAV": _f(g), "FRIC": _f(r),
            "RHO_O": _f(rho_o), "WIND_STRESS_FACTOR": _f(wind_stress_factor), "ONE_DIMENSIONAL": 0,
            "FLUX_BALANCER": _f(flux_balancer),
            "CORIOLIS_F_NX": int(coriolis_shape[1]), "CORIOLIS_F_NY": int(coriolis_shape[0]),
            "ANGLE_NX": int(angle_shape[1]), "ANGLE_NY": int(angle_shape[0]),
            "ATMOS_PRES_NX": int(pressure_shape[1]), "ATMOS_PRES_NY": int(pressure_shape[0]),
            "WIND_STRESS_X_NX": int(wind_shape[1]), "WIND_STRESS_X_NY": int(wind_shape[0]),
            "WIND_STRESS_Y_NX": int(wind_shape[1]), "WIND_STRESS_Y_NY": int(wind_shape[0]),
            "USE_DIRECT_LOOKUP": "True" if direct_lookup else "False"}


def noise_defines(coriolis_shape=(1, 1), angle_shape=(1, 1), block=(16, 16), kl_rand=(1, 1)):
    """S/OceanStateNoise.py:206-213; for the KL model error kl_rand = (rand_nx,
    rand_ny) = (Nx, 2 Ny) as S/ModelErrorKL.py:179-187 passes them."""
    return {"block_width": block[0], "block_height": block[1], "kl_rand_nx": kl_rand[0], "kl_rand_ny": kl_rand[1],
            "CORIOLIS_F_NX": int(coriolis_shape[1]), "CORIOLIS_F_NY": int(coriolis_shape[0]),
            "ANGLE_NX": int(angle_shape[1]), "ANGLE_NY": int(angle_shape[0])}


def jet_texture_shape(nx, ny, subsample=10):
    """Shape of the subsampled beta-plane Coriolis texture (S/CDKLM16.py:181-239)."""
    return (max(2, (ny + 4) // subsample), max(2, (nx + 4) // subsample))


# name -> (kernel source file, defines, nvcc options)
REF_CONFIGS = {
    # Gaussian bump, 256 x 256, dx = dy = 200 m, constant f, walls
    "cdklm_bump256": ("CDKLM16_kernel.cu", cdklm_defines(256, 256, 200.0, 200.0), CDKLM_FLAGS),
    # double jet domain, 512 x 300, dx = dy = 5 km, beta-plane texture
    "cdklm_jet512": ("CDKLM16_kernel.cu",
                     cdklm_defines(512, 300, 5000.0, 5000.0, coriolis_shape=jet_texture_shape(512, 300)),
                     CDKLM_FLAGS),
    # mixed physics on an odd grid: friction, RK2, walls
    "cdklm_fric77": ("CDKLM16_kernel.cu", cdklm_defines(77, 45, 150.0, 170.0, r=2.4e-3), CDKLM_FLAGS),
    "max_dt": ("max_dt.cu", {"block_width": 12, "block_height": 32, "NUM_THREADS": 256}, []),
    # BoundaryConditionsArakawaA with default (size-2) boundary data (U/Common.py:1145-1151)
    "boundary": ("boundary_kernels.cu", {"block_width": 16, "block_height": 16, "BC_NS_NX": 2, "BC_NS_NY": 2,
                                         "BC_EW_NX": 2, "BC_EW_NY": 2}, []),
    # Bathymetry's copy, with its dummy sizes (U/Common.py:1452-1459)
    "boundary_bathymetry": ("boundary_kernels.cu", {"block_width": 16, "block_height": 16, "BC_NS_NX": -1,
                                                    "BC_NS_NY": -1, "BC_EW_NX": -1, "BC_EW_NY": -1}, []),
    "init_bm": ("initHm_kernel.cu", {"block_width": 16, "block_height": 16}, []),
    "noise_const": ("ocean_noise.cu", noise_defines(), NOISE_FLAGS),
    "noise_jet512": ("ocean_noise.cu", noise_defines(coriolis_shape=jet_texture_shape(512, 300)), NOISE_FLAGS),
    # the three levels of the multi-level ensemble (2560 km x 1500 km, double jet)
    **{f"cdklm_ml{nx}x{ny}": ("CDKLM16_kernel.cu",
                              cdklm_defines(nx, ny, 2560e3 / nx, 1500e3 / ny, coriolis_shape=jet_texture_shape(nx, ny)),
                              CDKLM_FLAGS)
       for nx, ny in ((128, 64), (256, 128), (512, 256))},
    **{f"noise_ml{nx}x{ny}": ("ocean_noise.cu", noise_defines(coriolis_shape=jet_texture_shape(nx, ny)), NOISE_FLAGS)
       for nx, ny in ((128, 64), (256, 128), (512, 256))},
    # GPUDrifterCollection with the default 1x1 wind (D/GPUDrifterCollection.py:70-76)
    "drift": ("driftKernels.cu", {"block_width": 64, "block_height": 1, "WIND_X_NX": 1, "WIND_X_NY": 1,
                                  "WIND_Y_NX": 1, "WIND_Y_NY": 1}, []),
    # ... and with a 3 x 4 (nx x ny) wind texture for both components
    "drift_wind3x4": ("driftKernels.cu", {"block_width": 64, "block_height": 1, "WIND_X_NX": 3, "WIND_X_NY": 4,
                                          "WIND_Y_NX": 3, "WIND_Y_NY": 4}, []),
    # open boundaries: the reference's sponge test grid (T/schemes/CombinedCDKLM16_test.py:43-56) and
    # boundary kernels for per-cell exterior data along 50 x 70 and 64 x 48 grids
    "cdklm_sponge50x70": ("CDKLM16_kernel.cu", cdklm_defines(50, 70, 200.0, 200.0), CDKLM_FLAGS),
    "boundary_data54x74": ("boundary_kernels.cu", {"block_width": 16, "block_height": 16, "BC_NS_NX": 54,
                                                   "BC_NS_NY": 2, "BC_EW_NX": 2, "BC_EW_NY": 74}, []),
    # time-varying textured wind stress and atmospheric pressure on a 77 x 45 grid
    "cdklm_forcing77": ("CDKLM16_kernel.cu", cdklm_defines(77, 45, 150.0, 170.0, wind_shape=(5, 7),
                                                           pressure_shape=(6, 8)), CDKLM_FLAGS),
    # a rotated grid: north-angle texture of 6 x 5 (nx x ny) values on a 64 x 48 grid
    "cdklm_angle64": ("CDKLM16_kernel.cu", cdklm_defines(64, 48, 500.0, 500.0, angle_shape=(5, 6)), CDKLM_FLAGS),
    # ... with a pressure array of the grid's own size read directly (S/CDKLM16.py:123-133)
    "cdklm_direct77": ("CDKLM16_kernel.cu", cdklm_defines(77, 45, 150.0, 170.0, wind_shape=(5, 7),
                                                          pressure_shape=(49, 81), direct_lookup=True), CDKLM_FLAGS),
    # ModelErrorKL with the default basis (1..10 x 1..10) and with the double-jet case's (2..8 x 1..7)
    "noise_kl10": ("ocean_noise.cu", noise_defines(kl_rand=(10, 20)), NOISE_FLAGS),
    "noise_kl7": ("ocean_noise.cu", noise_defines(kl_rand=(7, 14)), NOISE_FLAGS),
    # OceanNoiseEnsemble's observation kernels, no defines and default options (E/OceanNoiseEnsemble.py:333-339)
    "observation": ("observationKernels.cu", {}, []),
}


def cubin_path(name):
    return os.path.join(REF_DIR, name + ".cubin")


def available(*names):
    """True when the cubins were built (they need the reference sources)."""
    names = names or tuple(REF_CONFIGS)
    return all(os.path.exists(cubin_path(n)) for n in names)


# ---------------------------------------------------------------------------
# CUDA driver API through ctypes
# ---------------------------------------------------------------------------

class Driver:
    _inst = None

    def __init__(self):
        self.lib = ctypes.CDLL("libcuda.so.1")
        L, vp, u64, sz, ui = self.lib, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_size_t, ctypes.c_uint
        L.cuInit.argtypes = [ui]
        L.cuDeviceGet.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.c_int]
        L.cuDevicePrimaryCtxRetain.argtypes = [ctypes.POINTER(vp), ctypes.c_int]
        L.cuCtxSetCurrent.argtypes = [vp]
        L.cuModuleLoad.argtypes = [ctypes.POINTER(vp), ctypes.c_char_p]
        L.cuModuleGetFunction.argtypes = [ctypes.POINTER(vp), vp, ctypes.c_char_p]
        L.cuMemAlloc_v2.argtypes = [ctypes.POINTER(u64), sz]
        L.cuMemFree_v2.argtypes = [u64]
        L.cuMemcpyHtoD_v2.argtypes = [u64, vp, sz]
        L.cuMemcpyDtoH_v2.argtypes = [vp, u64, sz]
        L.cuCtxSynchronize.argtypes = []
        L.cuLaunchKernel.argtypes = [vp, ui, ui, ui, ui, ui, ui, ui, vp, ctypes.POINTER(vp), ctypes.POINTER(vp)]
        self._check(self.lib.cuInit(0), "cuInit")
        dev = ctypes.c_int()
        self._check(self.lib.cuDeviceGet(ctypes.byref(dev), 0), "cuDeviceGet")
        ctx = ctypes.c_void_p()
        self._check(self.lib.cuDevicePrimaryCtxRetain(ctypes.byref(ctx), dev), "cuDevicePrimaryCtxRetain")
        self.ctx = ctx
        self.make_current()
        self.modules = {}

    @classmethod
    def get(cls):
        if cls._inst is None:
            cls._inst = Driver()
        cls._inst.make_current()
        return cls._inst

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUDA driver error {rc}")

    def make_current(self):
        self._check(self.lib.cuCtxSetCurrent(self.ctx), "cuCtxSetCurrent")

    def module(self, name):
        if name not in self.modules:
            mod = ctypes.c_void_p()
            self._check(self.lib.cuModuleLoad(ctypes.byref(mod), cubin_path(name).encode()), "cuModuleLoad " + name)
            self.modules[name] = mod
        return self.modules[name]

    def function(self, module_name, kernel):
        fn = ctypes.c_void_p()
        self._check(self.lib.cuModuleGetFunction(ctypes.byref(fn), self.module(module_name), kernel.encode()),
                    "cuModuleGetFunction " + kernel)
        return fn

    def alloc(self, nbytes):
        p = ctypes.c_uint64()
        self._check(self.lib.cuMemAlloc_v2(ctypes.byref(p), ctypes.c_size_t(max(int(nbytes), 16))), "cuMemAlloc")
        return p.value

    def free(self, ptr):
        self.lib.cuMemFree_v2(ctypes.c_uint64(ptr))

    def upload(self, ptr, host):
        host = np.ascontiguousarray(host)
        self._check(self.lib.cuMemcpyHtoD_v2(ctypes.c_uint64(ptr), host.ctypes.data_as(ctypes.c_void_p),
                                             ctypes.c_size_t(host.nbytes)), "cuMemcpyHtoD")

    def download(self, ptr, shape, dtype=np.float32):
        out = np.empty(shape, dtype=dtype)
        self._check(self.lib.cuMemcpyDtoH_v2(out.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint64(ptr),
                                             ctypes.c_size_t(out.nbytes)), "cuMemcpyDtoH")
        return out

    def synchronize(self):
        self._check(self.lib.cuCtxSynchronize(), "cuCtxSynchronize")

    def launch(self, fn, fmt, grid, block, *args):
        """Launch with PyCUDA's prepared-call argument format (f, i, P)."""
        assert len(fmt) == len(args), (fmt, len(args))
        holders = []
        for c, a in zip(fmt, args):
            if c == "f":
                holders.append(ctypes.c_float(float(a)))
            elif c == "i":
                holders.append(ctypes.c_int32(int(a)))
            elif c == "P":
                holders.append(ctypes.c_uint64(int(a) if a is not None else 0))
            else:
                raise ValueError(c)
        params = (ctypes.c_void_p * len(holders))(*[ctypes.cast(ctypes.pointer(h), ctypes.c_void_p) for h in holders])
        gx, gy = (tuple(grid) + (1,))[:2]
        bx, by, bz = (tuple(block) + (1, 1))[:3]
        self._check(self.lib.cuLaunchKernel(fn, int(gx), int(gy), 1, int(bx), int(by), int(bz), 0, None,
                                            params, None), "cuLaunchKernel")


class Array2D:
    """A tightly pitched float32 device array (CUDAArray2D, U/Common.py:516-559)."""

    def __init__(self, drv, host, dtype=np.float32, pad_rows=0):
        host = np.ascontiguousarray(host, dtype=dtype)
        self.drv, self.shape, self.dtype = drv, host.shape, dtype
        self.pitch = host.shape[1] * host.itemsize
        self.ptr = drv.alloc((host.shape[0] + pad_rows) * self.pitch + 64)
        drv.upload(self.ptr, host)

    def download(self):
        return self.drv.download(self.ptr, self.shape, self.dtype)

    def upload(self, host):
        self.drv.upload(self.ptr, np.ascontiguousarray(host, dtype=self.dtype))

    def free(self):
        if self.ptr:
            self.drv.free(self.ptr)
            self.ptr = 0


def _ceil(a, b):
    return int(math.ceil(a / float(b)))


# ---------------------------------------------------------------------------
# CDKLM16 through the reference kernels
# ---------------------------------------------------------------------------

class RefCDKLM16:
    """CDKLM16 driven by the reference kernels (cubin `config`).

    `ftex` and `angle_tex` are the Coriolis and north-angle textures exactly as
    uploaded (the product's oracle builds them from f, beta and angle the way
    S/CDKLM16.py:147-239 does); `f` is the compensated f the noise uses.
    """

    def __init__(self, config, eta0, hu0, hv0, H, nx, ny, dx, dy, dt, g, f, r, ftex, angle_tex,
                 bc=(1, 1, 1, 1), beta=0.0, courant_number=0.8, block=(12, 32), sponge_cells=(0, 0, 0, 0),
                 bc_data=None, bc_config="boundary", wind=None, pressure=None):
        drv = self.drv = Driver.get()
        self.config = config
        self.nx, self.ny = int(nx), int(ny)
        self.dx, self.dy, self.g = np.float32(dx), np.float32(dy), np.float32(g)
        self.f, self.beta = np.float32(f), np.float32(beta)
        self.bc = tuple(int(b) for b in bc)            # north, east, south, west
        self.courant_number = courant_number
        self.local_size = block
        self.global_size = (_ceil(self.nx, block[0]), _ceil(self.ny, block[1]))
        self.k_step = drv.function(config, "cdklm_swe_2D")
        self.k_bc_ns = drv.function("boundary", "periodicBoundary_NS")
        self.k_bc_ew = drv.function("boundary", "periodicBoundary_EW")
        # open boundaries (U/Common.py:1121-1400): sponge widths (north, east,
        # south, west), exterior data {"t": [...], side: [(h, hu, hv), ...]}
        self.sponge_cells = tuple(int(c) for c in sponge_cells)
        self.bc_config = bc_config
        self.bc_data = bc_data
        self.bc_timestamps = [None, None]
        self.bc_t = np.float32(0.0)
        self.bc_arrays = None
        # time-varying forcing (S/Simulator.py:183-288): (t, [u], [v]) and (t, [P])
        self.wind, self.pressure = wind, pressure
        self.wind_stamps, self.pressure_stamps = [None, None], [None, None]
        self.wind_arrays = self.pressure_arrays = None
        self.k_dt_block = drv.function("max_dt", "per_block_max_dt")
        self.k_dt_reduce = drv.function("max_dt", "max_dt_reduction")
        self.mask_value = np.float32(1.0e20)
        # bathymetry (U/Common.py:1414-1491)
        Hi = np.ma.filled(np.ma.asarray(H).astype(np.float32), self.mask_value) \
            if np.ma.is_masked(H) else np.asarray(H, dtype=np.float32)
        self.Hi = Array2D(drv, Hi)
        self.Hm = Array2D(drv, np.zeros((self.ny + 4, self.nx + 4), np.float32))
        self._bathymetry()
        Hm = self.Hm.download()
        eta0 = np.maximum(np.asarray(eta0, np.float32), -Hm)
        self.h0 = [Array2D(drv, a) for a in (eta0, hu0, hv0)]
        self.h1 = [Array2D(drv, a) for a in (eta0, hu0, hv0)]
        self.ftex = Array2D(drv, np.asarray(ftex, np.float32))
        if wind is not None:
            z = np.zeros_like(np.asarray(wind[1][0], np.float32))
            self.wind_arrays = [Array2D(drv, z) for _ in range(4)]      # x cur, x next, y cur, y next
        if pressure is not None:
            z = np.zeros_like(np.asarray(pressure[1][0], np.float32))
            self.pressure_arrays = [Array2D(drv, z) for _ in range(2)]
        if bc_data is not None:
            ns_n, ew_n = len(bc_data["north"][0][0]), len(bc_data["east"][0][0])
            self.bc_arrays = [Array2D(drv, np.zeros((2, 3 * ns_n), np.float32)) for _ in range(2)] + \
                [Array2D(drv, np.zeros((ew_n, 6), np.float32)) for _ in range(2)]
        self.angle = Array2D(drv, np.asarray(angle_tex, np.float32))
        self.zero = Array2D(drv, np.zeros((1, 1), np.float32))
        nblocks = self.global_size[0] * self.global_size[1]
        self.dt_blocks = Array2D(drv, np.zeros((self.global_size[1], self.global_size[0]), np.float32))
        self.dt_buf = Array2D(drv, np.zeros((1, 1), np.float32))
        self.num_blocks_dt = nblocks
        self.t = 0.0
        self.num_iterations = 0
        self.dt = np.float32(dt)
        if dt <= 0:
            self.updateDt()

    # U/Common.py:1538-1561 and :1484-1491
    def _bathymetry(self):
        drv = self.drv
        bs = (16, 16)
        gs = (_ceil(self.nx + 4 + 1, 16), _ceil(self.ny + 4 + 1, 16))
        n, e, s, w = self.bc
        args = (self.nx, self.ny, 2, 2, self.Hi.ptr, self.Hi.pitch)
        if n == 2 and s == 2:
            drv.launch(drv.function("boundary_bathymetry", "periodic_boundary_intersections_NS"), "iiiiPi", gs, bs, *args)
        elif n == 1 and s == 1:
            drv.launch(drv.function("boundary_bathymetry", "closed_boundary_intersections_NS"), "iiiiPi", gs, bs, *args)
        if e == 2 and w == 2:
            drv.launch(drv.function("boundary_bathymetry", "periodic_boundary_intersections_EW"), "iiiiPi", gs, bs, *args)
        elif n == 1 and s == 1:       # the reference tests north/south here (U/Common.py:1556)
            drv.launch(drv.function("boundary_bathymetry", "closed_boundary_intersections_EW"), "iiiiPi", gs, bs, *args)
        drv.launch(drv.function("init_bm", "initBm"), "iiPifPi", gs, bs, self.nx + 4, self.ny + 4,
                   self.Hi.ptr, self.Hi.pitch, self.mask_value, self.Hm.ptr, self.Hm.pitch)
        drv.synchronize()

    # U/Common.py:1193-1308
    def _update_bc_values(self, t):
        n, e, s, w = self.bc
        if 3 not in (n, e, s, w):
            return
        d = self.bc_data
        tl = d["t"]
        i0 = max(0, np.searchsorted(tl, t) - 1)
        i1 = min(len(tl) - 1, np.searchsorted(tl, t))
        new = [tl[i0], tl[i1]]
        old, self.bc_timestamps = self.bc_timestamps, new

        def row(side, i):
            h, hu, hv = d[side][i]
            return np.transpose(np.vstack((np.squeeze(h), np.squeeze(hu), np.squeeze(hv))))

        for slot, idx in ((0, i0), (1, i1)):
            if new[slot] != old[slot]:
                ns = np.stack([row("south", idx), row("north", idx)]).astype(np.float32)
                ew = np.stack([row("west", idx), row("east", idx)], axis=1).astype(np.float32)
                self.bc_arrays[slot].upload(ns.reshape(2, -1))
                self.bc_arrays[2 + slot].upload(ew.reshape(ew.shape[0], -1))
        self.bc_t = np.float32(max(0.0, min(1.0, (t - new[0]) / max(1.0e-10, new[1] - new[0]))))

    # U/Common.py:1310-1400
    def _boundary(self, Q):
        drv = self.drv
        bs = (16, 16)
        gs = (_ceil(self.nx + 4 + 1, 16), _ceil(self.ny + 4 + 1, 16))
        h, u, v = Q
        n, e, s, w = self.bc
        spn, spe, sps, spw = self.sponge_cells
        st = (h.ptr, h.pitch, u.ptr, u.pitch, v.ptr, v.pitch)
        cfg = self.bc_config
        if n == 2:
            drv.launch(self.k_bc_ns, "iiiiPiPiPi", gs, bs, self.nx, self.ny, 2, 2, *st)
        else:
            if n == 3 or s == 3:
                drv.launch(drv.function(cfg, "flowRelaxationScheme_NS"), "iiiiiiiiPiPiPiPPf", gs, bs, n, s,
                           self.nx, self.ny, 2, 2, spn, sps, *st, self.bc_arrays[0].ptr, self.bc_arrays[1].ptr,
                           self.bc_t)
            if n == 4 or s == 4:
                drv.launch(drv.function(cfg, "linearInterpolation_NS"), "iiiiiiiiPiPiPi", gs, bs, n, s,
                           self.nx, self.ny, 2, 2, spn, sps, *st)
        if e == 2:
            # periodic_boundary_EW(stream, h, v, u) is called with (h, u, v)
            drv.launch(self.k_bc_ew, "iiiiPiPiPi", gs, bs, self.nx, self.ny, 2, 2,
                       h.ptr, h.pitch, v.ptr, v.pitch, u.ptr, u.pitch)
        else:
            if e == 3 or w == 3:
                drv.launch(drv.function(cfg, "flowRelaxationScheme_EW"), "iiiiiiiiPiPiPiPPf", gs, bs, e, w,
                           self.nx, self.ny, 2, 2, spe, spw, *st, self.bc_arrays[2].ptr, self.bc_arrays[3].ptr,
                           self.bc_t)
            if e == 4 or w == 4:
                drv.launch(drv.function(cfg, "linearInterpolation_EW"), "iiiiiiiiPiPiPi", gs, bs, e, w,
                           self.nx, self.ny, 2, 2, spe, spw, *st)

    # S/Simulator.py:183-288
    @staticmethod
    def _forcing_t(tl, t, stamps, upload):
        i0 = max(0, np.searchsorted(tl, t) - 1)
        i1 = min(len(tl) - 1, np.searchsorted(tl, t))
        new = [tl[i0], tl[i1]]
        if new[0] != stamps[0]:
            upload(i0, 0)
        if new[1] != stamps[1]:
            upload(i1, 1)
        stamps[:] = new
        return np.float32(max(0.0, min(1.0, (t - new[0]) / max(1.0e-10, new[1] - new[0]))))

    def _forcing(self):
        wt = pt = np.float32(0.0)
        if self.wind is not None:
            tl, us, vs = self.wind

            def up(i, slot):
                self.wind_arrays[slot].upload(np.asarray(us[i], np.float32))
                self.wind_arrays[2 + slot].upload(np.asarray(vs[i], np.float32))
            wt = self._forcing_t(tl, self.t, self.wind_stamps, up)
        if self.pressure is not None:
            tl, ps = self.pressure

            def up(i, slot):
                self.pressure_arrays[slot].upload(np.asarray(ps[i], np.float32))
            pt = self._forcing_t(tl, self.t, self.pressure_stamps, up)
        return wt, pt

    # S/CDKLM16.py:688-723
    def _call(self, Qin, Qout, local_dt, rk_step, wind_t=0.0, pressure_t=0.0):
        n, e, s, w = self.bc
        bcs = (n << 24) | (s << 16) | (e << 8) | w
        (hi, ui, vi), (ho, uo, vo) = Qin, Qout
        z = self.zero.ptr
        pa = [a.ptr for a in self.pressure_arrays] if self.pressure_arrays else [z, z]
        wa = [a.ptr for a in self.wind_arrays] if self.wind_arrays else [z, z, z, z]
        self.drv.launch(self.k_step, "fiPiPiPiPiPiPiPiPifPPPPfPPPPfi", self.global_size, self.local_size,
                        np.float32(local_dt), rk_step,
                        hi.ptr, hi.pitch, ui.ptr, ui.pitch, vi.ptr, vi.pitch,
                        ho.ptr, ho.pitch, uo.ptr, uo.pitch, vo.ptr, vo.pitch,
                        self.Hi.ptr, self.Hi.pitch, self.Hm.ptr, self.Hm.pitch, self.mask_value,
                        self.ftex.ptr, self.angle.ptr, pa[0], pa[1], np.float32(pressure_t),
                        wa[0], wa[1], wa[2], wa[3], np.float32(wind_t), bcs)

    # S/CDKLM16.py:477-584 (RK2, constant forcing)
    def step(self, t_end, noise=None, drifters=None):
        if self.t == 0:
            self._update_bc_values(self.t)
            self._boundary(self.h0)
        t_now = 0.0
        while t_now < t_end:
            local_dt = np.float32(min(self.dt, np.float32(t_end - t_now)))
            wt, pt = self._forcing()
            self._update_bc_values(self.t)
            self._call(self.h0, self.h1, local_dt, 0, wt, pt)
            self._boundary(self.h1)
            self._call(self.h1, self.h0, local_dt, 1, wt, pt)
            if noise is not None:
                noise.perturb(self)
            self._boundary(self.h0)
            if drifters is not None:
                drifters.drift(self, local_dt)
            self.t += np.float64(local_dt)
            t_now += np.float64(local_dt)
            self.num_iterations += 1
        return self.t

    # S/CDKLM16.py:814-841
    def max_dt(self):
        drv = self.drv
        h, u, v = self.h0
        drv.launch(self.k_dt_block, "iifffPiPiPiPifPi", self.global_size, self.local_size,
                   self.nx, self.ny, self.dx, self.dy, self.g, h.ptr, h.pitch, u.ptr, u.pitch, v.ptr, v.pitch,
                   self.Hm.ptr, self.Hm.pitch, self.mask_value, self.dt_blocks.ptr, self.dt_blocks.pitch)
        drv.launch(self.k_dt_reduce, "iPP", (1, 1), (256, 1, 1), self.num_blocks_dt, self.dt_blocks.ptr,
                   self.dt_buf.ptr)
        return self.dt_buf.download()[0, 0]

    def updateDt(self, courant_number=None):
        c = self.courant_number if courant_number is None else courant_number
        self.dt = np.float32(c * self.max_dt())

    def synchronize(self):
        self.drv.synchronize()

    def download(self):
        self.drv.synchronize()
        return tuple(a.download() for a in self.h0)

    def bathymetry(self):
        return self.Hi.download(), self.Hm.download()

    def free(self):
        for a in (self.wind_arrays or []) + (self.pressure_arrays or []) + (self.bc_arrays or []):
            a.free()
        for a in self.h0 + self.h1 + [self.Hi, self.Hm, self.ftex, self.angle, self.zero, self.dt_blocks,
                                      self.dt_buf]:
            a.free()


# ---------------------------------------------------------------------------
# SOAR model error through the reference kernels
# ---------------------------------------------------------------------------

class RefNoise:
    """OceanStateNoise (S/OceanStateNoise.py:47-459) on injected normals."""

    def __init__(self, config, sim: RefCDKLM16, soar_q0, soar_L, interpolation_factor=1, block=(16, 16)):
        drv = self.drv = Driver.get()
        self.nx, self.ny = sim.nx, sim.ny
        self.dx, self.dy = sim.dx, sim.dy
        self.factor = int(interpolation_factor)
        self.periodic_ns = int(sim.bc[0] == 2)
        self.periodic_ew = int(sim.bc[1] == 2)
        self.coarse_nx = int(np.ceil(self.nx / self.factor))
        self.coarse_ny = int(np.ceil(self.ny / self.factor))
        self.coarse_dx = np.float32(self.dx * self.factor)
        self.coarse_dy = np.float32(self.dy * self.factor)
        gx = 0 if self.periodic_ew else 4
        gy = 0 if self.periodic_ns else 4
        self.rand_nx, self.rand_ny = self.coarse_nx + 2 * gx, self.coarse_ny + 2 * gy
        self.soar_q0 = np.float32(soar_q0)
        self.soar_L = np.float32(soar_L)
        self.block = block
        # the non-periodic SOAR read reaches one row past the random field
        # (clamp(by + j, 0, ny + 8), K/ocean_noise.cu:181-200); a padding row
        # keeps that read inside the allocation; no written value depends on it
        self.random = Array2D(drv, np.zeros((self.rand_ny, self.rand_nx), np.float32), pad_rows=1)
        self.coarse = Array2D(drv, np.zeros((self.coarse_ny + 4, self.coarse_nx + 4), np.float32))
        self.k_soar = drv.function(config, "SOAR")
        self.k_geo = drv.function(config, "geostrophicBalance")
        self.k_bicubic = drv.function(config, "bicubicInterpolation")
        self.pending = []

    def set_random(self, xi):
        assert xi.shape == (self.rand_ny, self.rand_nx), (xi.shape, (self.rand_ny, self.rand_nx))
        self.random.upload(xi)

    def queue(self, draws):
        """Normals to use for the next perturbations, in order (one per call)."""
        self.pending = list(draws)

    # S/OceanStateNoise.py:380-459 (perturbation_scale 1, no perpendicular field,
    # default coarse-grid alignment)
    def perturb(self, sim: RefCDKLM16, perturbation_scale=1.0):
        drv = self.drv
        if self.pending:
            self.set_random(self.pending.pop(0))
        bs = self.block
        gs_soar = (_ceil(self.coarse_nx + 4, bs[0]), _ceil(self.coarse_ny + 4, bs[1]))
        gs = (_ceil(self.nx, bs[0]), _ceil(self.ny, bs[1]))
        drv.launch(self.k_soar, "iifffffiiPiPii", gs_soar, bs, self.coarse_nx, self.coarse_ny,
                   self.coarse_dx, self.coarse_dy, self.soar_q0, self.soar_L, np.float32(perturbation_scale),
                   self.periodic_ns, self.periodic_ew, self.random.ptr, self.random.pitch,
                   self.coarse.ptr, self.coarse.pitch, 0)
        h, u, v = sim.h0
        if self.factor > 1:
            off = 0
            drv.launch(self.k_bicubic, "iiiiffiiiiffiiffffPPPiPiPiPiPif", gs, bs, sim.nx, sim.ny, 2, 2,
                       sim.dx, sim.dy, self.coarse_nx, self.coarse_ny, 2, 2, self.coarse_dx, self.coarse_dy,
                       off, off, sim.g, sim.f, sim.beta, 0.0, sim.ftex.ptr, sim.angle.ptr,
                       self.coarse.ptr, self.coarse.pitch, h.ptr, h.pitch, u.ptr, u.pitch, v.ptr, v.pitch,
                       sim.Hi.ptr, sim.Hi.pitch, sim.mask_value)
        else:
            drv.launch(self.k_geo, "iiffiiffffPPPiPiPiPiPif", gs, bs, sim.nx, sim.ny, sim.dx, sim.dy, 2, 2,
                       sim.g, sim.f, sim.beta, 0.0, sim.ftex.ptr, sim.angle.ptr,
                       self.coarse.ptr, self.coarse.pitch, h.ptr, h.pitch, u.ptr, u.pitch, v.ptr, v.pitch,
                       sim.Hi.ptr, sim.Hi.pitch, sim.mask_value)

    def free(self):
        self.random.free()
        self.coarse.free()


# ---------------------------------------------------------------------------
# drifters through the reference kernels
# ---------------------------------------------------------------------------

def ref_kl_perturb(config, nx, ny, dx, dy, eta, hu, hv, Hi, rns, basis=(1, 10, 1, 10), include_cos=True,
                   include_sin=True, kl_decay=1.2, kl_scaling=1.0, rollers=(0.0, 0.0, 0.0, 0.0), f=1.2e-4,
                   beta=0.0, g=9.81, perturbation_scale=1.0, eta_only=False, land_value=1e20):
    """ModelErrorKL.perturbOceanState / perturbEta through the reference's
    kernels (S/ModelErrorKL.py:313-449): kl_sample_ocean_state on a grid of
    ceil(n / 14) blocks of 16 x 16 (one ghost ring per block), or
    kl_sample_eta on ceil(n / 16) blocks.  1x1 Coriolis (0) and angle (0)
    textures.  Host arrays in, (eta, hu, hv) out."""
    drv = Driver.get()
    arrs = [Array2D(drv, a) for a in (eta, hu, hv)]
    Hi_a = Array2D(drv, Hi)
    r_a = Array2D(drv, rns)
    zero = Array2D(drv, np.zeros((1, 1), np.float32))
    try:
        scale = np.float32(perturbation_scale * np.float32(kl_scaling))
        common = [int(basis[0]), int(basis[1]), int(basis[2]), int(basis[3]), int(include_cos), int(include_sin),
                  np.float32(kl_decay), scale, *[np.float32(r) for r in rollers], r_a.ptr, r_a.pitch]
        if eta_only:
            k = drv.function(config, "kl_sample_eta")
            drv.launch(k, "iiiiiiiiffffffPiPi", (_ceil(nx, 16), _ceil(ny, 16)), (16, 16, 1), int(nx), int(ny),
                       *common, arrs[0].ptr, arrs[0].pitch)
        else:
            k = drv.function(config, "kl_sample_ocean_state")
            drv.launch(k, "iifffffPPiiiiiiffffffPiPiPiPiPif", (_ceil(nx, 14), _ceil(ny, 14)), (16, 16, 1),
                       int(nx), int(ny), np.float32(dx), np.float32(dy), np.float32(g), np.float32(f),
                       np.float32(beta), zero.ptr, zero.ptr, *common, arrs[0].ptr, arrs[0].pitch,
                       arrs[1].ptr, arrs[1].pitch, arrs[2].ptr, arrs[2].pitch, Hi_a.ptr, Hi_a.pitch,
                       np.float32(land_value))
        drv.synchronize()
        return tuple(a.download() for a in arrs)
    finally:
        for a in arrs + [Hi_a, r_a, zero]:
            a.free()


def ref_observe_underlying_flow(nx, ny, dx, dy, hu, hv, positions, H=60.0):
    """observeUnderlyingFlow (K/observationKernels.cu:29-83) on (ny+4, nx+4)
    host arrays, launched as BaseOceanStateEnsemble.observeParticles does
    (E/BaseOceanStateEnsemble.py:117-130: zero reference cells 2, one block of
    num_drifters threads, tight (D, 2) float32 output).  Returns (D, 2)."""
    drv = Driver.get()
    pos = np.ascontiguousarray(positions, dtype=np.float32)
    D = pos.shape[0]
    eta_a = Array2D(drv, np.zeros_like(np.asarray(hu, np.float32)))
    hu_a, hv_a = Array2D(drv, hu), Array2D(drv, hv)
    pos_a = Array2D(drv, pos)
    obs_a = Array2D(drv, np.zeros((D, 2), np.float32))
    try:
        k = drv.function("observation", "observeUnderlyingFlow")
        drv.launch(k, "iiffiiPiPiPifiPiPi", (1, 1), (D, 1, 1), int(nx), int(ny), np.float32(dx), np.float32(dy), 2, 2,
                   eta_a.ptr, eta_a.pitch, hu_a.ptr, hu_a.pitch, hv_a.ptr, hv_a.pitch, np.float32(H), D,
                   pos_a.ptr, pos_a.pitch, obs_a.ptr, obs_a.pitch)
        drv.synchronize()
        return obs_a.download()
    finally:
        for a in (eta_a, hu_a, hv_a, pos_a, obs_a):
            a.free()


class RefDrifters:
    """GPUDrifterCollection (D/GPUDrifterCollection.py:34-253): 1x1 zero wind,
    or (config "drift_wind3x4") wind drift with 3 x 4 wind textures:
    wind = (x_current, x_next, y_current, y_next) arrays of shape (4, 3)."""

    def __init__(self, positions, domain_size_x, domain_size_y, periodic_ns, periodic_ew, config="drift",
                 wind=None, wind_drift_factor=0.0):
        drv = self.drv = Driver.get()
        pos = np.ascontiguousarray(positions, dtype=np.float32)
        self.n = pos.shape[0] - 1
        self.pos = Array2D(drv, pos)
        self.zero = Array2D(drv, np.zeros((1, 1), np.float32))
        self.wind = [Array2D(drv, w) for w in wind] if wind is not None else None
        self.factor = np.float32(wind_drift_factor)
        self.size = (np.float32(domain_size_x), np.float32(domain_size_y))
        self.periodic = (int(periodic_ns), int(periodic_ew))
        self.k_drift = drv.function(config, "passiveDrifterKernel")
        self.k_bc = drv.function(config, "enforceBoundaryConditions")
        self.gs = (_ceil(self.n + 2, 64), 1)       # D/GPUDrifterCollection.py:107-110

    def drift(self, sim: RefCDKLM16, dt, wind_t=0.0):
        h, u, v = sim.h0
        w = [a.ptr for a in self.wind] if self.wind is not None else [self.zero.ptr] * 4
        self.drv.launch(self.k_drift, "iifffiiPiPiPiPiiiiPifPPPPff", self.gs, (64, 1, 1),
                        sim.nx, sim.ny, sim.dx, sim.dy, np.float32(dt), 2, 2,
                        h.ptr, h.pitch, u.ptr, u.pitch, v.ptr, v.pitch, sim.Hm.ptr, sim.Hm.pitch,
                        self.periodic[0], self.periodic[1], self.n, self.pos.ptr, self.pos.pitch,
                        1.0, w[0], w[1], w[2], w[3], np.float32(wind_t), self.factor)

    def enforce_boundary(self):
        self.drv.launch(self.k_bc, "ffiiiPi", self.gs, (64, 1, 1), self.size[0], self.size[1],
                        self.periodic[0], self.periodic[1], self.n, self.pos.ptr, self.pos.pitch)

    def positions(self):
        self.drv.synchronize()
        return self.pos.download()

    def free(self):
        self.pos.free()
        self.zero.free()
        for a in self.wind or []:
            a.free()
