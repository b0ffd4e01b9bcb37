"""CDKLM16 rotating shallow-water simulator on GB300 (drop-in for ``SWEsimulators/CDKLM16.py``).

Same constructor, ``step``, ``download``, ``updateDt`` ... as the reference
(S/ = src/gpuocean/SWEsimulators, S/CDKLM16.py:43-895).  The differences are
in how the work reaches the GPU:

* all kernels are prebuilt for sm_103a and called through ``libgpuocean_gb300``;
  physical parameters are runtime arguments, not ``#define``s;
* an RK2 step is one fused launch (both stages and the periodic ghost fill);
  the two buffer sets are swapped after each step, so ``gpu_data.h0`` is the
  latest state and ``gpu_data.h1`` the previous time step;
* the CFL reduction covers every interior cell.
"""
from __future__ import annotations

import ctypes
import gc
import logging

import numpy as np

from .. import _lib
from ..utils import AtmosphericPressure, Common, WindStress
from .Simulator import Simulator


def subsample_texture(data, factor):
    """Bilinear re-sampling of a texture to (max(2, ny//factor), max(2, nx//factor)).

    Same sample positions as S/CDKLM16.py:181-192; the result is returned in
    [y, x] order, which is how the step kernel reads it.
    """
    from scipy.interpolate import RectBivariateSpline
    ny, nx = data.shape
    dx, dy = 1 / nx, 1 / ny
    spline = RectBivariateSpline(np.linspace(0.5 * dx, 1 - 0.5 * dx, nx),
                                 np.linspace(0.5 * dy, 1 - 0.5 * dy, ny), data.T, kx=1, ky=1)
    new_nx, new_ny = max(2, nx // factor), max(2, ny // factor)
    ndx, ndy = 1 / new_nx, 1 / new_ny
    x_new = np.linspace(0.5 * ndx, 1 - 0.5 * ndx, new_nx)
    y_new = np.linspace(0.5 * ndy, 1 - 0.5 * ndy, new_ny)
    return np.ascontiguousarray(spline(x_new, y_new).T)


def calcCoriolisParams(lat):
    """f and beta of a latitude (rad): f = 2 Omega sin(lat), beta = 2 Omega cos(lat)/a."""
    omega = 7.2921e-5
    a = 6371008.8
    return [2.0 * omega * np.sin(lat), 2.0 * omega * np.cos(lat) / a]


def _reference_cell_f(f, coriolis_beta, dx, dy, angle, gx=2, gy=2):
    """f moved from the grid origin to the first interior cell
    (S/CDKLM16.py:147-149)."""
    north = np.array([np.sin(angle.flat[0]), np.cos(angle.flat[0])])
    return f - coriolis_beta * (gx * dx * north[0] + gy * dy * north[1])


def _unshifted_f(f_stored, beta, dx, dy, gx, gy):
    """The f that the constructor's move to the first interior cell (default
    angle) turns into f_stored, bit for bit (same arithmetic as the
    constructor)."""
    angle = np.array([[0]], dtype=np.float32)
    target = np.float32(f_stored)
    moved = lambda c: np.float32(_reference_cell_f(c, beta, dx, dy, angle, gx, gy))
    cand = float(target) + float(target) - float(moved(float(target)))
    for _ in range(8):
        got = moved(cand)
        if got == target:
            return cand
        cand += float(target) - float(got)
    for _ in range(64):
        got = moved(cand)
        if got == target:
            return cand
        cand = float(np.nextafter(np.float32(cand), np.float32(np.inf if got < target else -np.inf)))
    return cand


class CDKLM16(Simulator):
    """Chertock, Dudzinski, Kurganov & Lukacova-Medvidova (2016) well-balanced
    central-upwind scheme for the rotating shallow-water equations."""

    def __init__(self, gpu_ctx, eta0, hu0, hv0, H, nx, ny, dx, dy, dt, g, f, r,
                 subsample_f=10, angle=np.array([[0]], dtype=np.float32), subsample_angle=10,
                 latitude=None, rho_o=1025.0, t=0.0, theta=1.8, rk_order=2, coriolis_beta=0.0,
                 max_wind_direction_perturbation=0, wind=None, wind_stress_factor=1.0,
                 atmospheric_pressure=None, boundary_conditions=None, boundary_conditions_data=None,
                 model_time_step=None, reportGeostrophicEquilibrium=False, write_netcdf=False,
                 comm=None, local_particle_id=0, super_dir_name=None, netcdf_filename=None,
                 ignore_ghostcells=False, courant_number=0.8, offset_x=0, offset_y=0,
                 flux_slope_eps=1.0e-1, desingularization_eps=1.0e-1, depth_cutoff=1.0e-5,
                 one_dimensional=False, flux_balancer=0.8, block_width=12, block_height=32,
                 num_threads_dt=256, use_direct_lookup=False):
        self.logger = logging.getLogger(__name__)
        assert rk_order in (1, 2, 3), "Only 1st, 2nd and 3rd order Runge Kutta supported"
        if rk_order == 3:
            assert r == 0.0, "3rd order Runge Kutta supported only without friction"
        wind = WindStress.WindStress() if wind is None else wind
        atmospheric_pressure = AtmosphericPressure.AtmosphericPressure() if atmospheric_pressure is None else atmospheric_pressure
        # use_direct_lookup keeps the reference's shape check and nothing
        # more: the reference passes the define as the Python literal True
        # (U/Common.py:478), which the preprocessor's `#if USE_DIRECT_LOOKUP`
        # (K/CDKLM16_kernel.cu:915) evaluates as 0, so its kernel always
        # interpolates the pressure - as this step does
        if use_direct_lookup:
            assert atmospheric_pressure.P[0].shape[0] == ny + 4 and atmospheric_pressure.P[0].shape[1] == nx + 4, \
                "Direct lookup is only supported for same sized grids"
        self.use_direct_lookup = bool(use_direct_lookup)
        boundary_conditions = Common.BoundaryConditions() if boundary_conditions is None else boundary_conditions
        angle = np.asarray(angle)
        ghost_cells_x = ghost_cells_y = 2
        self.boundary_conditions = boundary_conditions
        # compensate f for the reference cell (S/CDKLM16.py:147-149)
        f = _reference_cell_f(f, coriolis_beta, dx, dy, angle, ghost_cells_x, ghost_cells_y)
        self.max_wind_direction_perturbation = max_wind_direction_perturbation
        super().__init__(gpu_ctx, nx, ny, ghost_cells_x, ghost_cells_y, dx, dy, dt, g, f, r, None, t,
                         theta, rk_order, coriolis_beta, 0, wind, atmospheric_pressure, write_netcdf,
                         ignore_ghostcells, offset_x, offset_y, comm, block_width, block_height,
                         local_particle_id=local_particle_id)
        self.interior_domain_indices = np.array([-2, -2, 2, 2])

        # Coriolis texture (S/CDKLM16.py:194-223)
        eta0 = np.asarray(eta0) if not np.ma.isMaskedArray(eta0) else eta0
        if latitude is not None:
            if self.f != 0.0:
                raise RuntimeError("Cannot specify both latitude and f. Make your mind up.")
            coriolis_f, _ = calcCoriolisParams(latitude)
            coriolis_f = np.asarray(coriolis_f, dtype=np.float32)
        elif self.coriolis_beta != 0.0:
            if angle.size != 1:
                raise RuntimeError("non-constant angle cannot be combined with beta plane model (makes no sense)")
            x = np.linspace((-ghost_cells_x + 0.5) * self.dx, (self.nx + ghost_cells_x - 0.5) * self.dx, self.nx + 2 * ghost_cells_x)
            y = np.linspace((-ghost_cells_y + 0.5) * self.dy, (self.ny + ghost_cells_y - 0.5) * self.dy, self.ny + 2 * ghost_cells_x)
            x, y = np.meshgrid(x, y)
            n = x * np.sin(angle.flat[0]) + y * np.cos(angle.flat[0])
            coriolis_f = self.f + self.coriolis_beta * n
        elif np.size(self.f) == 1:
            coriolis_f = np.array([[self.f]], dtype=np.float32)
        elif np.shape(self.f) == eta0.shape:
            coriolis_f = np.array(self.f, dtype=np.float32)
        else:
            raise RuntimeError("The shape of f should match up with eta or be scalar.")
        coriolis_f = np.atleast_2d(coriolis_f)
        if subsample_f and coriolis_f.size >= eta0.size:
            coriolis_f = subsample_texture(coriolis_f, subsample_f)
        self.coriolis_f_arr = Common.CUDAArray2D(self.gpu_stream, coriolis_f.shape[1], coriolis_f.shape[0], 0, 0, coriolis_f)
        if subsample_angle and angle.size >= eta0.size:
            angle = subsample_texture(angle, subsample_angle)
        angle = np.atleast_2d(np.asarray(angle, dtype=np.float32))
        # a north-angle texture: every cell uses its own north vector, so the
        # RK stages run one launch each (goc_cdklm_stage) with the ghost fill
        # between them, as the reference steps
        self.angle_varies = angle.size != 1
        self.angle_arr = Common.CUDAArray2D(self.gpu_stream, angle.shape[1], angle.shape[0], 0, 0, angle)
        # a spatially varying texture is evaluated once per cell centre
        self.coriolis_cell = None
        if coriolis_f.size > 1:
            self.coriolis_cell = Common.CUDAArray2D(self.gpu_stream, nx, ny, 2, 2,
                                                    np.zeros((ny + 4, nx + 4), dtype=np.float32))
            _lib.call("goc_cell_texture", self.coriolis_f_arr.ptr, int(coriolis_f.shape[1]), int(coriolis_f.shape[0]),
                      int(nx), int(ny), self.coriolis_cell.ptr, int(self.coriolis_cell.pitch), self.gpu_stream.handle)

        self.rho_o = np.float32(rho_o)
        self.wind_stress_factor = np.float32(wind_stress_factor)
        self.flux_slope_eps = np.float32(flux_slope_eps)
        self.desingularization_eps = np.float32(desingularization_eps)
        self.depth_cutoff = np.float32(depth_cutoff)
        self.flux_balancer = np.float32(flux_balancer)
        self.one_dimensional = bool(one_dimensional)

        # bathymetry, dry-state clamp and the double-buffered state
        self.bathymetry = Common.Bathymetry(gpu_ctx, self.gpu_stream, nx, ny, ghost_cells_x, ghost_cells_y, H,
                                            boundary_conditions)
        Hm = self.downloadBathymetry()[1]
        eta0 = np.maximum(eta0, -Hm)
        self.gpu_data = Common.SWEDataArakawaA(self.gpu_stream, nx, ny, ghost_cells_x, ghost_cells_y, eta0, hu0, hv0)
        self.gpu_data_extra = None  # third buffer set for RK3

        # CFL reduction buffers
        self.num_threads_dt = num_threads_dt
        n_part = _lib.load().goc_max_dt_partials(int(nx), int(ny))
        if n_part < 0:
            raise ValueError("a %d x %d grid is too large for the CFL reduction" % (nx, ny))
        self.device_dt = Common.DevicePtr(4 * n_part)
        self.num_blocks_dt = np.int32(n_part)
        self.max_dt_buffer = Common.DevicePtr(4)
        self.courant_number = courant_number

        self.reportGeostrophicEquilibrium = np.int32(reportGeostrophicEquilibrium)
        self.constant_equilibrium_depth = np.max(H)
        self.bc_kernel = Common.BoundaryConditionsArakawaA(gpu_ctx, self.gpu_stream, self.nx, self.ny,
                                                           ghost_cells_x, ghost_cells_y, self.boundary_conditions,
                                                           boundary_conditions_data)
        self.model_error = None
        self.model_time_step = model_time_step
        self.total_time_steps = 0
        if model_time_step is None:
            self.model_time_step = self.dt
        self._params = self._make_params()
        if self.dt <= 0:
            self.updateDt()
        if self.write_netcdf:
            from ..utils import SimWriter
            self.sim_writer = SimWriter.SimNetCDFWriter(self, super_dir_name=super_dir_name,
                                                        filename=netcdf_filename,
                                                        ignore_ghostcells=self.ignore_ghostcells,
                                                        offset_x=self.offset_x, offset_y=self.offset_y)

    # ------------------------------------------------------------------
    def _make_params(self):
        p = _lib.GocCdklmParams()
        p.nx, p.ny = int(self.nx), int(self.ny)
        p.dx, p.dy, p.g, p.r = float(self.dx), float(self.dy), float(self.g), float(self.r)
        p.theta = float(self.theta)
        p.desing_eps = float(self.desingularization_eps)
        p.flux_slope_eps = float(self.flux_slope_eps)
        p.depth_cutoff = float(self.depth_cutoff)
        p.flux_balancer = float(self.flux_balancer)
        p.rho_o = float(self.rho_o)
        p.wind_stress_factor = float(self.wind_stress_factor)
        p.rk_order = int(self.rk_order)
        p.one_dimensional = int(self.one_dimensional)
        bc = self.boundary_conditions
        p.bc_north, p.bc_east, p.bc_south, p.bc_west = int(bc.north), int(bc.east), int(bc.south), int(bc.west)
        p.land_value = float(self.bathymetry.mask_value)
        p.coriolis_f = self.coriolis_f_arr.ptr
        p.coriolis_nx, p.coriolis_ny = self.coriolis_f_arr.nx_halo, self.coriolis_f_arr.ny_halo
        if self.coriolis_cell is not None:
            p.coriolis_cell, p.coriolis_cell_pitch = self.coriolis_cell.ptr, int(self.coriolis_cell.pitch)
        p.angle = self.angle_arr.ptr
        p.angle_nx, p.angle_ny = self.angle_arr.nx_halo, self.angle_arr.ny_halo
        p.wind_x_cur, p.wind_x_next = self.wind_stress_x_current_arr.ptr, self.wind_stress_x_next_arr.ptr
        p.wind_x_nx, p.wind_x_ny = self.wind_stress_x_current_arr.nx_halo, self.wind_stress_x_current_arr.ny_halo
        p.wind_y_cur, p.wind_y_next = self.wind_stress_y_current_arr.ptr, self.wind_stress_y_next_arr.ptr
        p.wind_y_nx, p.wind_y_ny = self.wind_stress_y_current_arr.nx_halo, self.wind_stress_y_current_arr.ny_halo
        p.atm_p_cur, p.atm_p_next = self.atmospheric_pressure_current_arr.ptr, self.atmospheric_pressure_next_arr.ptr
        p.atm_p_nx, p.atm_p_ny = self.atmospheric_pressure_current_arr.nx_halo, self.atmospheric_pressure_current_arr.ny_halo
        return p

    @property
    def stream_handle(self):
        return self.gpu_stream.handle

    def cleanUp(self, do_gc=True):
        self.closeNetCDF()
        if getattr(self, "gpu_data", None) is None:
            return
        if self.model_error is not None:
            self.model_error.cleanUp(do_gc=False)
        self.gpu_data.release()
        if self.gpu_data_extra is not None:
            self.gpu_data_extra.release()
        self.bathymetry.release()
        self.bc_kernel.release()
        self.device_dt.free()
        self.max_dt_buffer.free()
        if self.coriolis_cell is not None:
            self.coriolis_cell.release()
        for a in (self.coriolis_f_arr, self.angle_arr, self.wind_stress_x_current_arr, self.wind_stress_y_current_arr,
                  self.wind_stress_x_next_arr, self.wind_stress_y_next_arr, self.atmospheric_pressure_current_arr,
                  self.atmospheric_pressure_next_arr):
            a.release()
        self.gpu_data = None
        self.gpu_ctx = None
        if do_gc:
            gc.collect()

    # ------------------------------------------------------------------
    def _stage(self, src, dst, dt, rk_step, alt=None):
        d = self.gpu_data
        a = alt if alt is not None else (None, None, None)
        _lib.call("goc_cdklm_stage", ctypes.byref(self._params), ctypes.c_float(dt), int(rk_step),
                  src[0].ptr, src[1].ptr, src[2].ptr, dst[0].ptr, dst[1].ptr, dst[2].ptr,
                  a[0].ptr if alt else None, a[1].ptr if alt else None, a[2].ptr if alt else None,
                  int(d.h0.pitch), self.bathymetry.Bi.ptr, int(self.bathymetry.Bi.pitch),
                  self.bathymetry.Bm.ptr, int(self.bathymetry.Bm.pitch), self.stream_handle)

    def _stagewise(self):
        """Whether RK2 runs stage by stage: sponge boundaries act between the
        stages, and a north-angle texture needs the single-stage kernel."""
        return self.boundary_conditions.isSponge() or self.angle_varies

    def _rk_step(self, local_dt):
        d = self.gpu_data
        if self.rk_order == 2 and self._stagewise():
            # sponge boundaries act between the stages (S/CDKLM16.py:519-530):
            # stage by stage, with the boundary kernels on the stage buffer
            self._stage((d.h0, d.hu0, d.hv0), (d.h1, d.hu1, d.hv1), local_dt, 0)
            self.bc_kernel.boundaryCondition(self.gpu_stream, d.h1, d.hu1, d.hv1)
            self._stage((d.h1, d.hu1, d.hv1), (d.h0, d.hu0, d.hv0), local_dt, 1)
        elif self.rk_order == 2:
            _lib.call("goc_cdklm_rk2_step", ctypes.byref(self._params), ctypes.c_float(local_dt),
                      d.h0.ptr, d.hu0.ptr, d.hv0.ptr, d.h1.ptr, d.hu1.ptr, d.hv1.ptr, int(d.h0.pitch),
                      self.bathymetry.Bi.ptr, int(self.bathymetry.Bi.pitch),
                      self.bathymetry.Bm.ptr, int(self.bathymetry.Bm.pitch), self.stream_handle)
            d.swap()
        elif self.rk_order == 1:
            self._stage((d.h0, d.hu0, d.hv0), (d.h1, d.hu1, d.hv1), local_dt, 0)
            d.swap()
            self.bc_kernel.boundaryCondition(self.gpu_stream, d.h0, d.hu0, d.hv0)
        else:
            if self.gpu_data_extra is None:
                eta, hu, hv = self.download()
                self.gpu_data_extra = Common.SWEDataArakawaA(self.gpu_stream, self.nx, self.ny, 2, 2, eta, hu, hv)
            x = self.gpu_data_extra
            q0, q1, q2 = (d.h0, d.hu0, d.hv0), (d.h1, d.hu1, d.hv1), (x.h0, x.hu0, x.hv0)
            self._stage(q0, q1, local_dt, 0)
            self.bc_kernel.boundaryCondition(self.gpu_stream, *q1)
            self._stage(q1, q0, local_dt, 1, alt=q2)
            self.bc_kernel.boundaryCondition(self.gpu_stream, *q2)
            self._stage(q2, q0, local_dt, 2)
            self.bc_kernel.boundaryCondition(self.gpu_stream, *q0)

    def step(self, t_end=0.0, apply_stochastic_term=True, write_now=True, update_dt=False):
        """Advance by ``t_end`` seconds in steps of at most ``self.dt``
        (S/CDKLM16.py:477-584)."""
        if self.t == 0:
            self.bc_kernel.update_bc_values(self.gpu_stream, self.t)
            self.bc_kernel.boundaryCondition(self.gpu_stream, self.gpu_data.h0, self.gpu_data.hu0, self.gpu_data.hv0)
        # nothing between the RK2 steps: the run of steps goes to the library
        # in one call once both forcing weights are 1 (time-independent forcing)
        plain = (not update_dt and self.rk_order == 2 and not self._stagewise()
                 and not (self.model_error is not None and apply_stochastic_term)
                 and not self.hasDrifters and not self.hasCrossProductDrifter
                 and len(self.wind_stress.t) == 1 and len(self.atmospheric_pressure.t) == 1)
        t_now = 0.0
        while t_now < t_end:
            if update_dt:
                self.updateDt()
            local_dt = np.float32(min(self.dt, np.float32(t_end - t_now)))
            self._params.wind_t = float(np.float32(self.update_wind_stress()))
            self._params.atm_p_t = float(np.float32(self.update_atmospheric_pressure()))
            if plain and self._params.wind_t == 1.0 and self._params.atm_p_t == 1.0:
                self._plain_steps(t_now, t_end)
                break
            self.bc_kernel.update_bc_values(self.gpu_stream, self.t)
            self._rk_step(local_dt)
            perturbed = self.model_error is not None and apply_stochastic_term
            if perturbed:
                self.perturbState()
            if perturbed or (self.rk_order == 2 and self._stagewise()):
                self.bc_kernel.boundaryCondition(self.gpu_stream, self.gpu_data.h0, self.gpu_data.hu0,
                                                 self.gpu_data.hv0)
            self.drifterStep(local_dt)
            self.t += np.float64(local_dt)
            t_now += np.float64(local_dt)
            self.num_iterations += 1
        if self.write_netcdf and write_now:
            self.writeState()
        return self.t

    def _plain_steps(self, t_now, t_end):
        """The remaining steps of step(t_end) as one goc_cdklm_rk2_steps call:
        the same dt sequence, time and iteration bookkeeping as the loop."""
        dts = []
        while t_now < t_end:
            local_dt = np.float32(min(self.dt, np.float32(t_end - t_now)))
            dts.append(local_dt)
            t_now += np.float64(local_dt)
        arr = np.asarray(dts, dtype=np.float32)
        d = self.gpu_data
        _lib.call("goc_cdklm_rk2_steps", ctypes.byref(self._params), arr.ctypes.data, len(arr),
                  d.h0.ptr, d.hu0.ptr, d.hv0.ptr, d.h1.ptr, d.hu1.ptr, d.hv1.ptr, int(d.h0.pitch),
                  self.bathymetry.Bi.ptr, int(self.bathymetry.Bi.pitch),
                  self.bathymetry.Bm.ptr, int(self.bathymetry.Bm.pitch), self.stream_handle)
        if len(arr) % 2:
            d.swap()
        for x in arr:
            self.t += np.float64(x)
        self.num_iterations += len(arr)
        return self.t

    # ------------------------------------------------------------------
    def setSOARModelError(self, small_scale_perturbation_amplitude=None, small_scale_perturbation_interpolation_factor=1,
                          use_lcg=False, xorwow_seed=None, block_width_model_error=16, block_height_model_error=16):
        from . import OceanStateNoise
        self.model_error = OceanStateNoise.OceanStateNoise.fromsim(
            self, soar_q0=small_scale_perturbation_amplitude,
            interpolation_factor=small_scale_perturbation_interpolation_factor,
            use_lcg=use_lcg, xorwow_seed=xorwow_seed,
            block_width=block_width_model_error, block_height=block_height_model_error)
        if self.write_netcdf:
            self.sim_writer.writeModelError(self)

    def setKLModelError(self, kl_decay=1.2, kl_scaling=1.0, include_cos=True, include_sin=True,
                        basis_x_start=1, basis_y_start=1, basis_x_end=10, basis_y_end=10,
                        use_lcg=False, xorwow_seed=None, np_seed=None, block_width=16, block_height=16):
        """Karhunen-Loeve model error (S/CDKLM16.py:639-651)."""
        from . import ModelErrorKL
        self.model_error = ModelErrorKL.ModelErrorKL.fromsim(
            self, kl_decay=kl_decay, kl_scaling=kl_scaling, include_cos=include_cos, include_sin=include_sin,
            basis_x_start=basis_x_start, basis_y_start=basis_y_start, basis_x_end=basis_x_end,
            basis_y_end=basis_y_end, use_lcg=use_lcg, xorwow_seed=xorwow_seed, np_seed=np_seed,
            block_width=block_width, block_height=block_height)
        if self.write_netcdf:
            self.sim_writer.writeModelError(self)

    def setKLModelErrorSimilarAs(self, otherSim):
        """The KL model error of another simulator's parameters (S/CDKLM16.py:653-660)."""
        from . import ModelErrorKL
        me = otherSim.model_error
        self.model_error = ModelErrorKL.ModelErrorKL.fromsim(
            self, kl_decay=me.kl_decay, kl_scaling=me.kl_scaling, include_cos=me.include_cos,
            include_sin=me.include_sin, basis_x_start=me.basis_x_start, basis_y_start=me.basis_y_start,
            basis_x_end=me.basis_x_end, basis_y_end=me.basis_y_end, use_lcg=me.use_lcg,
            block_width=me.local_size[0], block_height=me.local_size[1])

    def perturbState(self, perturbation_scale=1.0, update_random_field=True, q0_scale=1):
        if q0_scale != 1:
            perturbation_scale = q0_scale
        if self.model_error is not None:
            self.model_error.perturbSim(self, perturbation_scale=perturbation_scale,
                                        update_random_field=update_random_field)

    def perturbSimilarAs(self, otherSim, perturbation_scale=1.0):
        self.model_error.perturbSimSimilarAs(self, modelError=otherSim.model_error,
                                             perturbation_scale=perturbation_scale)

    def applyBoundaryConditions(self):
        self.bc_kernel.boundaryCondition(self.gpu_stream, self.gpu_data.h0, self.gpu_data.hu0, self.gpu_data.hv0)

    def drifterStep(self, dt):
        if self.hasCrossProductDrifter:
            for d in range(len(self.CrossProductDrifter)):
                if self.CPsims[d] is not None:
                    o = self.CPsims[d]
                    self.CrossProductDrifter[d].drift(o.gpu_data.h0, o.gpu_data.hu0, o.gpu_data.hv0, o.bathymetry.Bm,
                                                      self.nx, self.ny, self.t, self.dx, self.dy, dt,
                                                      np.int32(2), np.int32(2))
                self.CrossProductDrifter[d].drift(self.gpu_data.h0, self.gpu_data.hu0, self.gpu_data.hv0,
                                                  self.bathymetry.Bm, self.nx, self.ny, self.t, self.dx, self.dy, dt,
                                                  np.int32(2), np.int32(2))
            self.CPdrifter_t += dt
        if self.hasDrifters:
            self.drifters.driftFromSim(self, dt)
            self.drifter_t += dt
            return self.drifter_t

    def dataAssimilationStep(self, observation_time, otherSim=None, model_error_final_step=True, write_now=True,
                             courant_number=0.8):
        """Run to ``observation_time`` in blocks of ``model_time_step`` with
        the model error after each block (S/CDKLM16.py:742-806; the plan of
        blocks comes from ``ObservationSchedule.blocks_to_observation``).
        ``otherSim`` (a coarse partner) takes the same blocks and is perturbed
        with this simulator's random field after each of them."""
        from .ObservationSchedule import blocks_to_observation, check_arrival, refresh_dt_after
        plan = blocks_to_observation(observation_time - self.t, self.model_time_step, model_error_final_step)
        sims = (self,) if otherSim is None else (self, otherSim)
        for s in sims:
            s.updateDt(courant_number=courant_number)
        for blk in plan:
            for s in sims:
                s.step(blk.length, apply_stochastic_term=False, write_now=False)
                if blk.perturbation is None:
                    continue
                if s is self:
                    self.perturbState(perturbation_scale=blk.perturbation)
                else:
                    s.perturbSimilarAs(self, perturbation_scale=blk.perturbation)
            self.total_time_steps += 1
            if refresh_dt_after(self.total_time_steps):
                self.updateDt(courant_number=courant_number)
        if self.write_netcdf and write_now:
            self.sim_writer.writeTimestep(self)
        check_arrival(observation_time, self.t)

    def writeState(self):
        if self.write_netcdf:
            self.sim_writer.writeTimestep(self)

    @classmethod
    def fromfilename(cls, gpu_ctx, filename, cont_write_netcdf=True, new_netcdf_filename=None, time0=None):
        """A simulator hot-started from a file of SimNetCDFWriter: its
        parameters and the last written state (or the state at time0)
        (S/CDKLM16.py:403-473).  cont_write_netcdf: write the continued run
        to new_netcdf_filename (generated when None)."""
        from ..utils import SimReader
        reader = SimReader.SimNetCDFReader(filename, ignore_ghostcells=False)
        try:
            name = str(reader.get("simulator_short"))
            assert name == cls.__name__, ("Trying to initialize a " + cls.__name__ +
                                          " simulator with netCDF file based on " + name + " results.")
            H = reader.getH()
            if time0 is None:
                eta0, hu0, hv0, time0 = reader.getLastTimeStep()
            else:
                eta0, hu0, hv0, time0 = reader.getStateAtTime(time0)
            if H.ndim == 3:
                H = H[0]
            dx, dy, beta = reader.get("dx"), reader.get("dy"), reader.get("coriolis_beta")
            # The file holds the simulator's f, already moved to the first
            # interior cell by the constructor (S/CDKLM16.py:147-149), which
            # moves a given f again: hand it the f that moves to the stored one
            # (the reference passes the stored f on and shifts it twice).
            gx, gy = int(reader.get("ghost_cells_west")), int(reader.get("ghost_cells_south"))
            f = _unshifted_f(reader.get("coriolis_force"), beta, dx, dy, gx, gy)
            params = dict(gpu_ctx=gpu_ctx, eta0=eta0, hu0=hu0, hv0=hv0, H=H,
                          nx=int(reader.get("nx")), ny=int(reader.get("ny")),
                          dx=dx, dy=dy, dt=reader.get("dt"), g=reader.get("g"),
                          f=f, r=reader.get("bottom_friction_r"), t=float(time0),
                          theta=reader.get("minmod_theta"), rk_order=int(reader.get("time_integrator")),
                          coriolis_beta=reader.get("coriolis_beta"), write_netcdf=cont_write_netcdf,
                          netcdf_filename=new_netcdf_filename, wind=WindStress.WindStress(),
                          boundary_conditions=reader.getBC())
            if reader.has("model_time_step"):
                params["model_time_step"] = reader.get("model_time_step")
        finally:
            reader.close()
        return cls(**params)

    def setModelErrorFromFile(self, filename, use_lcg=False, xorwow_seed=None):
        """The model error described by the attributes of a simulator file
        (S/CDKLM16.py:600-637)."""
        from ..utils import SimReader
        reader = SimReader.SimNetCDFReader(filename, ignore_ghostcells=False)
        try:
            name = str(reader.get("simulator_short"))
            assert name == self.__class__.__name__, ("Trying to initialize a " + self.__class__.__name__ +
                                                     " simulator with netCDF file based on " + name + " results.")
            if reader.has("small_scale_perturbation"):
                # files of an older writer
                if reader.get("small_scale_perturbation") == "True":
                    self.setSOARModelError(
                        small_scale_perturbation_amplitude=reader.get("small_scale_perturbation_amplitude"),
                        small_scale_perturbation_interpolation_factor=int(
                            reader.get("small_scale_perturbation_interpolation_factor")),
                        use_lcg=use_lcg, xorwow_seed=xorwow_seed)
            elif reader.has("has_model_error") and reader.get("has_model_error") == "True":
                kind = reader.get("model_error_name")
                if kind == "OceanStateNoise":
                    self.setSOARModelError(
                        small_scale_perturbation_amplitude=reader.get("small_scale_perturbation_amplitude"),
                        small_scale_perturbation_interpolation_factor=int(
                            reader.get("small_scale_perturbation_interpolation_factor")),
                        use_lcg=use_lcg, xorwow_seed=xorwow_seed)
                elif kind == "ModelErrorKL":
                    self.setKLModelError(kl_decay=reader.get("kl_decay"), kl_scaling=reader.get("kl_scaling"),
                                         include_cos=reader.get("include_cos") == "True",
                                         include_sin=reader.get("include_sin") == "True",
                                         basis_x_start=int(reader.get("basis_x_start")),
                                         basis_y_start=int(reader.get("basis_y_start")),
                                         basis_x_end=int(reader.get("basis_x_end")),
                                         basis_y_end=int(reader.get("basis_y_end")),
                                         use_lcg=use_lcg, xorwow_seed=xorwow_seed)
        finally:
            reader.close()

    # ------------------------------------------------------------------
    def downloadMaxDt(self):
        """Launch the CFL reduction and return the limit before the Courant factor."""
        d = self.gpu_data
        _lib.call("goc_max_dt", int(self.nx), int(self.ny), ctypes.c_float(self.dx), ctypes.c_float(self.dy),
                  ctypes.c_float(self.g), d.h0.ptr, d.hu0.ptr, d.hv0.ptr, int(d.h0.pitch),
                  self.bathymetry.Bm.ptr, int(self.bathymetry.Bm.pitch), ctypes.c_float(self.bathymetry.mask_value),
                  self.device_dt.ptr, int(self.num_blocks_dt), self.max_dt_buffer.ptr, self.stream_handle)
        out = np.zeros(1, dtype=np.float32)
        _lib.call("goc_memcpy_d2h_async", out.ctypes.data, self.max_dt_buffer.ptr, ctypes.c_size_t(4), self.stream_handle)
        self.gpu_stream.synchronize()
        return out[0]

    def updateDt(self, courant_number=None):
        """dt = courant_number * CFL limit (S/CDKLM16.py:814-841)."""
        if courant_number is None:
            courant_number = self.courant_number
        self.dt = courant_number * self.downloadMaxDt()

    def _getMaxTimestepHost(self, courant_number=0.8):
        eta, hu, hv = self.download(interior_domain_only=True)
        Hm = self.downloadBathymetry()[1][2:-2, 2:-2]
        h = eta + Hm
        gravityWaves = np.sqrt(self.g * h)
        u = hu / h
        v = hv / h
        max_dt = 0.25 * min(self.dx / np.max(np.abs(u) + gravityWaves), self.dy / np.max(np.abs(v) + gravityWaves))
        return courant_number * max_dt

    def downloadBathymetry(self, interior_domain_only=False):
        Bi, Bm = self.bathymetry.download(self.gpu_stream)
        if interior_domain_only:
            Bi = Bi[2:-2 + 1, 2:-2 + 1]
            Bm = Bm[2:-2, 2:-2]
        return [Bi, Bm]

    def getLandMask(self, interior_domain_only=True):
        if self.gpu_data.h0.mask is None:
            return None
        return self.gpu_data.h0.mask[2:-2, 2:-2] if interior_domain_only else self.gpu_data.h0.mask

    def downloadDt(self):
        out = np.zeros(int(self.num_blocks_dt), dtype=np.float32)
        _lib.call("goc_memcpy_d2h_async", out.ctypes.data, self.device_dt.ptr, ctypes.c_size_t(out.nbytes),
                  self.stream_handle)
        self.gpu_stream.synchronize()
        return out
