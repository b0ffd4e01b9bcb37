"""Simulator output to NetCDF files, with the reference's layout.

The reference writes its output and hot-start files with netCDF4
(U/SimWriter.py:35-539, U/ = src/gpuocean/utils): global attributes with the
simulator's parameters (names kept here, so that `CDKLM16.fromfilename` and
the reference's reader find them), dimensions time (unlimited), x, y (cells
with ghost cells) and x_Hi, y_Hi (corners), coordinate variables, the
bathymetry (Hm, Hi), a land mask, the polar-stereographic projection
variable, and per time step eta, hu, hv.  netCDF4 (and HDF5) are not
available here, so this writer produces the same variables and attributes in
the classic NetCDF format (64-bit offset, through scipy.io.netcdf_file), which
netCDF4 readers open as well.  The reference compresses the big variables
(zlib); the classic format has no compression, and the grid-mapping
variable projection_stere has one element instead of none.
"""
from __future__ import annotations

import datetime
import os

import numpy as np
from scipy.io import netcdf_file


def _attr(v):
    # classic NetCDF attributes: numbers and text; booleans are written as
    # text ("True"/"False") as the reference does for its flags
    if isinstance(v, (bool, np.bool_)):
        return str(bool(v))
    if v is None:
        return "None"
    return v


class SimNetCDFWriter:
    """Writes a simulator's state to a NetCDF file after each call of
    writeTimestep (and once at construction).

    sim: the simulator; filename: path without or with ".nc" (generated from
    the simulator name and a time stamp when None, in super_dir_name);
    ignore_ghostcells: write the interior only; offset_x, offset_y: origin of
    the x, y coordinates when ghost cells are ignored.
    """

    def __init__(self, sim, super_dir_name=None, filename=None, num_layers=1, staggered_grid=False,
                 ignore_ghostcells=False, offset_x=0, offset_y=0):
        self.gpu_stream = sim.gpu_stream
        self.ignore_ghostcells = ignore_ghostcells
        self.staggered_grid = staggered_grid
        self.num_layers = num_layers
        if staggered_grid:
            raise NotImplementedError("the staggered-grid layout belongs to simulators this package does not have")
        self.timestamp = datetime.datetime.now().strftime("%Y_%m_%d-%H_%M_%S")
        self.timestamp_short = datetime.datetime.now().strftime("%Y_%m_%d")
        self.simulator_short = str(sim.__class__.__name__)
        self.super_dir_name = super_dir_name if super_dir_name is not None else os.getcwd()
        if not filename:
            self.dir_name = os.path.join(self.super_dir_name, "netcdf_" + self.timestamp_short)
            self.output_file_name = os.path.join(self.dir_name, self.simulator_short + "_" + self.timestamp + ".nc")
        elif os.path.split(filename)[0] == "":
            self.dir_name = os.path.join(self.super_dir_name, "netcdf_" + self.timestamp_short)
            self.output_file_name = os.path.join(self.dir_name, self.simulator_short + "_" + filename + ".nc")
        else:
            self.output_file_name = filename + ".nc"
            self.dir_name = os.path.dirname(filename)
        self.output_file_name = self.output_file_name.replace(".nc.nc", ".nc")
        if self.dir_name:
            os.makedirs(self.dir_name, exist_ok=True)

        nx, ny, dx, dy = int(sim.nx), int(sim.ny), float(sim.dx), float(sim.dy)
        gx, gy = int(sim.ghost_cells_x), int(sim.ghost_cells_y)
        self.Hi, self.Hm = sim.bathymetry.download(self.gpu_stream)
        self.dt = sim.dt

        f = self.ncfile = netcdf_file(self.output_file_name, "w", version=2)
        attrs = {
            "Conventions": "CF-1.4",
            "git_hash": "git info missing...",
            "ignore_ghostcells": str(ignore_ghostcells),
            "num_layers": int(num_layers),
            "staggered_grid": str(staggered_grid),
            "simulator_short": self.simulator_short,
            "boundary_conditions": str(sim.boundary_conditions),
            "boundary_conditions_sponge_mr": str({k: int(v) for k, v in sim.boundary_conditions.getSponge().items()}),
            "time_integrator": int(sim.rk_order),
            "minmod_theta": np.float32(sim.theta),
            "coriolis_force": np.float32(sim.f),
            "coriolis_beta": np.float32(sim.coriolis_beta),
            "y_zero_reference_cell": np.float32(sim.y_zero_reference_cell - 2),
            "eddy_viscosity_coefficient": _attr(sim.A),
            "g": np.float32(sim.g),
            "nx": np.int32(nx),
            "ny": np.int32(ny),
            "dx": np.float32(dx),
            "dy": np.float32(dy),
            "dt": np.float32(sim.dt),
            "auto_dt": "False",
            "bottom_friction_r": np.float32(sim.r),
            "ghost_cells_north": np.int32(gy),
            "ghost_cells_east": np.int32(gx),
            "ghost_cells_south": np.int32(gy),
            "ghost_cells_west": np.int32(gx),
        }
        if sim.wind_stress.source_filename is not None:
            attrs["wind_stress_source"] = str(sim.wind_stress.source_filename)
        for k, v in attrs.items():
            setattr(f, k, v)

        f.createDimension("time", None)
        if not ignore_ghostcells:
            f.createDimension("x", nx + 2 * gx)
            f.createDimension("y", ny + 2 * gy)
        else:
            f.createDimension("x", nx)
            f.createDimension("y", ny)
        f.createDimension("x_Hi", nx + 2 * gx + 1)
        f.createDimension("y_Hi", ny + 2 * gy + 1)

        self.nc_time = f.createVariable("time", "f4", ("time",))
        self.nc_time.units = "seconds since 1970-01-01 00:00:00"
        x = f.createVariable("x", "f4", ("x",))
        y = f.createVariable("y", "f4", ("y",))
        x_Hi = f.createVariable("x_Hi", "f4", ("x_Hi",))
        y_Hi = f.createVariable("y_Hi", "f4", ("y_Hi",))
        for v, name, axis in ((x, "projection_x_coordinate", "X"), (y, "projection_y_coordinate", "Y"),
                              (x_Hi, "projection_x_coordinate", "X"), (y_Hi, "projection_y_coordinate", "Y")):
            v.standard_name = name
            v.axis = axis
            v.units = "meter"
        if not ignore_ghostcells:
            x[:] = np.linspace(-gx * dx + dx / 2.0, (nx + gx) * dx - dx / 2.0, nx + 2 * gx)
            y[:] = np.linspace(-gy * dy + dy / 2.0, (ny + gy) * dy - dy / 2.0, ny + 2 * gy)
        else:
            x[:] = np.linspace(offset_x, nx * dx, nx)
            y[:] = np.linspace(offset_y, ny * dy, ny)
        x_Hi[:] = np.linspace(-gx * dx, (nx + gx) * dx, nx + 2 * gx + 1)
        y_Hi[:] = np.linspace(-gy * dy, (ny + gy) * dy, ny + 2 * gy + 1)

        # the grid-mapping variable is a scalar in the reference's files; scipy
        # mislays the record data of files with a 0-d variable, so it has one
        # element here
        f.createDimension("projection", 1)
        proj = f.createVariable("projection_stere", "i4", ("projection",))
        proj[:] = 0
        proj.grid_mapping_name = "polar_stereographic"
        proj.scale_factor_at_projection_origin = 0.9330127018922193
        proj.straight_vertical_longitude_from_pole = 70.0
        proj.latitude_of_projection_origin = 90.0
        proj.earth_radius = 6371000.0
        proj.proj4 = "+proj=stere +lat_0=90 +lon_0=70 +lat_ts=60 +units=m +a=6.371e+06 +e=0 +no_defs"

        land = f.createVariable("land_binary_mask", "f4", ("y", "x"))
        land.standard_name = "land_binary_mask"
        land.units = "1"
        land[:] = 0.0
        Hm_data = np.ma.getdata(self.Hm)
        Hi_data = np.ma.getdata(self.Hi)
        nc_Hm = f.createVariable("Hm", "f4", ("y", "x"))
        nc_Hm[:] = Hm_data[gy:-gy, gx:-gx] if ignore_ghostcells else Hm_data
        nc_Hi = f.createVariable("Hi", "f4", ("y_Hi", "x_Hi"))
        nc_Hi[:] = Hi_data
        for v in (nc_Hm, nc_Hi):
            v.standard_name = "water_surface_reference_datum_altitude"
            v.grid_mapping = "projection_stere"
            v.coordinates = "y x"
            v.units = "meter"

        self.nc_eta = f.createVariable("eta", "f4", ("time", "y", "x"))
        self.nc_hu = f.createVariable("hu", "f4", ("time", "y", "x"))
        self.nc_hv = f.createVariable("hv", "f4", ("time", "y", "x"))
        self.nc_eta.standard_name = "water_surface_height_above_reference_datum"
        self.nc_hu.standard_name = "x_sea_water_velocity"
        self.nc_hv.standard_name = "y_sea_water_velocity"
        for v, units in ((self.nc_eta, "meter"), (self.nc_hu, "meter second-1"), (self.nc_hv, "meter second-1")):
            v.grid_mapping = "projection_stere"
            v.coordinates = "y x"
            v.units = units
        self.i = 0
        self.writeTimestep(sim)

    def writeModelError(self, sim):
        """Model-error attributes (U/SimWriter.py:388-420): the model time step,
        whether a model error is set, and its parameters."""
        if sim.__class__.__name__ != "CDKLM16":
            return
        f = self.ncfile
        f.model_time_step = np.float32(sim.model_time_step)
        has = sim.model_error is not None
        f.has_model_error = str(has)
        if not has:
            return
        name = sim.model_error.__class__.__name__
        f.model_error_name = name
        me = sim.model_error
        if name == "OceanStateNoise":
            f.small_scale_perturbation_amplitude = np.float32(me.soar_q0)
            f.small_scale_perturbation_interpolation_factor = np.int32(me.interpolation_factor)
        elif name == "ModelErrorKL":
            f.kl_decay = np.float32(me.kl_decay)
            f.kl_scaling = np.float32(me.kl_scaling)
            f.include_cos = str(bool(me.include_cos))
            f.include_sin = str(bool(me.include_sin))
            f.basis_x_start = np.int32(me.basis_x_start)
            f.basis_y_start = np.int32(me.basis_y_start)
            f.basis_x_end = np.int32(me.basis_x_end)
            f.basis_y_end = np.int32(me.basis_y_end)

    def writeTimestep(self, sim):
        """Append the simulator's current state and time."""
        eta, hu, hv = (np.ma.getdata(a) for a in sim.download())
        self.nc_time[self.i] = sim.t
        if self.ignore_ghostcells:
            gx, gy = int(sim.ghost_cells_x), int(sim.ghost_cells_y)
            eta, hu, hv = (a[gy:-gy, gx:-gx] for a in (eta, hu, hv))
        self.nc_eta[self.i] = eta
        self.nc_hu[self.i] = hu
        self.nc_hv[self.i] = hv
        self.i += 1

    def close(self):
        if self.ncfile is not None:
            self.ncfile.close()
            self.ncfile = None

    def __enter__(self):
        return self

    def __exit__(self, exc_type, exc_value, traceback):
        self.close()
