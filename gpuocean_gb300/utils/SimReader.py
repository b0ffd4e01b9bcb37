"""Reading simulator output files written by SimNetCDFWriter.

Mirrors the reference's reader (U/SimReader.py:37-229): global attributes by
name (`get`, `has`), the state at a time step or at a time, the bathymetry
and the boundary conditions.  Files are opened with scipy.io.netcdf_file,
which reads the classic NetCDF formats this package writes; the reference's
own files are netCDF4/HDF5, which need the netCDF4 library (absent here).
The plotting helpers of the reference (animation, info plot) are not
included.
"""
from __future__ import annotations

import numpy as np
from scipy.io import netcdf_file

from . import Common


def _native(a):
    # classic NetCDF stores big-endian values; the simulators upload raw bytes
    a = np.asarray(a)
    return a.astype(a.dtype.newbyteorder("="), copy=True)


def _value(v):
    # attributes come back as bytes (text) or one-element arrays (numbers)
    if isinstance(v, bytes):
        return v.decode()
    a = np.asarray(v)
    if a.ndim == 1 and a.size == 1:
        return a[0]
    return v


class SimNetCDFReader:
    """filename: a NetCDF file of SimNetCDFWriter; ignore_ghostcells: return
    the interior of the state only."""

    def __init__(self, filename, ignore_ghostcells=True):
        self.filename = filename
        self.ignore_ghostcells = ignore_ghostcells
        self.ncfile = netcdf_file(filename, "r", mmap=False)
        self.ghostCells = [int(self.get("ghost_cells_north")), int(self.get("ghost_cells_east")),
                           int(self.get("ghost_cells_south")), int(self.get("ghost_cells_west"))]
        self.staggered_grid = str(self.get("staggered_grid")) == "True"

    def close(self):
        if self.ncfile is not None:
            self.ncfile.close()
            self.ncfile = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get(self, attr):
        """A global attribute, or the text "not found"."""
        if attr in self.ncfile._attributes:
            return _value(self.ncfile._attributes[attr])
        return "not found"

    def has(self, fieldname):
        return fieldname in self.ncfile._attributes or fieldname in self.ncfile.variables

    def printVariables(self):
        for var in self.ncfile.variables:
            print(var)

    def printAttributes(self):
        for attr in self.ncfile._attributes:
            print(attr + "\t--> " + str(self.get(attr)))

    def getNumTimeSteps(self):
        return self.ncfile.variables["time"].shape[0]

    def getBC(self):
        return Common.BoundaryConditions.fromstring(self.get("boundary_conditions"))

    def getTimes(self):
        return _native(self.ncfile.variables["time"][:])

    def _interior(self, a):
        if not self.ignore_ghostcells:
            return a
        n, e, s, w = self.ghostCells
        return a[s:-n, w:-e]

    def getTimeStep(self, index):
        """(eta, hu, hv, time) of time step `index` (negative from the end)."""
        v = self.ncfile.variables
        eta, hu, hv = (self._interior(_native(v[k][index, :, :])) for k in ("eta", "hu", "hv"))
        return eta, hu, hv, np.float32(v["time"][index])

    def getLastTimeStep(self):
        return self.getTimeStep(-1)

    def getH(self):
        v = self.ncfile.variables
        if "H" in v:
            return _native(v["H"][:, :])
        return _native(v["Hm"][:, :]) if self.staggered_grid else _native(v["Hi"][:, :])

    def getHm(self):
        return _native(self.ncfile.variables["Hm"][:, :])

    def getStateAtTime(self, time):
        """The state written at `time` (rounded to a whole second)."""
        time = np.round(time)
        times = self.ncfile.variables["time"]
        for i in range(times.shape[0]):
            if time == times[i]:
                return self.getStateAtTimeStep(i)
        raise RuntimeError("Time " + str(time) + " not in NetCDF file " + self.filename)

    def getStateAtTimeStep(self, index, etaOnly=False):
        v = self.ncfile.variables
        eta = self._interior(_native(v["eta"][index, :, :]))
        if etaOnly:
            return eta, np.float32(v["time"][index])
        hu = self._interior(_native(v["hu"][index, :, :]))
        hv = self._interior(_native(v["hv"][index, :, :]))
        return eta, hu, hv, np.float32(v["time"][index])

    def getEtaAtTimeStep(self, index):
        return self.getStateAtTimeStep(index, etaOnly=True)

    def getAxis(self):
        x = _native(self.ncfile.variables["x"][:])
        y = _native(self.ncfile.variables["y"][:])
        if self.ignore_ghostcells:
            n, e, s, w = self.ghostCells
            x, y = x[w:-e], y[s:-n]
        return x, y

    def getEtaXSlice(self, t, y):
        row = int(y) + int(self.get("ghost_cells_south"))
        return _native(self.ncfile.variables["eta"][t, row, self.ghostCells[3]:-self.ghostCells[1]])
