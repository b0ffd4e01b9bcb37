"""Drifters held and advected on the host (drop-in for
``drifters/CPUDrifterCollection.py:29-232``).

The reference uses this collection where drifters move with velocity fields
that already live on the host - the multi-level drifters, which drift with
the ensemble mean velocity plus a random walk scaled by the ensemble
variance (``MLDrifterCollection``).  Positions are an (N + 1) x 2 float64
array, the last row the observation.  One step for all drifters at once:
cell-centred bilinear interpolation of the given fields, an Euler step and
the periodic wrap of the reference (which wraps y < 0 with the x size, kept
as the reference has it).  Random-walk draws come from numpy's global
generator in the reference's order (per drifter: x, then y).
"""
from __future__ import annotations

import numpy as np

from ..utils import Common
from .BaseDrifterCollection import BaseDrifterCollection


class CPUDrifterCollection(BaseDrifterCollection):
    def __init__(self, numDrifters, observation_variance=0.01, boundaryConditions=None,
                 initialization_cov_drifters=None, domain_size_x=1.0, domain_size_y=1.0, initialize=False):
        super().__init__(numDrifters, observation_variance=observation_variance,
                         boundaryConditions=boundaryConditions if boundaryConditions is not None
                         else Common.BoundaryConditions(),
                         domain_size_x=domain_size_x, domain_size_y=domain_size_y)
        self.positions = np.zeros((self.numDrifters + 1, 2))
        if initialize:
            self.uniformly_distribute_drifters(initialization_cov_drifters=initialization_cov_drifters)

    def copy(self):
        c = CPUDrifterCollection(self.numDrifters, observation_variance=self.observation_variance,
                                 boundaryConditions=self.boundaryConditions, domain_size_x=self.domain_size_x,
                                 domain_size_y=self.domain_size_y)
        c.positions = self.positions.copy()
        return c

    def cleanUp(self):
        pass

    def getDrifterPositions(self):
        return self.positions[:-1, :].copy()

    def getObservationPosition(self):
        return self.positions[-1, :].copy()

    def setDrifterPositions(self, newDrifterPositions):
        np.copyto(self.positions[:-1, :], newDrifterPositions)

    def setObservationPosition(self, newObservationPosition):
        np.copyto(self.positions[-1, :], newObservationPosition)

    # ------------------------------------------------------------------
    @staticmethod
    def _bilinear(field, x0, x1, y0, y1, fx, fy):
        """Cell-centred bilinear value (rows y, columns x) at every drifter."""
        f = np.asarray(field)
        lo = (1 - fx) * f[y0, x0] + fx * f[y0, x1]
        hi = (1 - fx) * f[y1, x0] + fx * f[y1, x1]
        return (1 - fy) * lo + fy * hi

    def _stencil(self, dx, dy, x_zero_ref, y_zero_ref):
        """Lower-left cell, upper cell and weights of every row's position."""
        x, y = self.positions[:, 0], self.positions[:, 1]
        cx = np.floor(x / dx + x_zero_ref).astype(np.int64)
        cy = np.floor(y / dy + y_zero_ref).astype(np.int64)
        frac_x = x / dx - np.floor(x / dx)
        frac_y = y / dy - np.floor(y / dy)
        west, south = frac_x < 0.5, frac_y < 0.5
        x0 = np.where(west, cx - 1, cx)
        y0 = np.where(south, cy - 1, cy)
        fx = np.where(west, frac_x + 0.5, frac_x - 0.5)
        fy = np.where(south, frac_y + 0.5, frac_y - 0.5)
        return x0, x0 + 1, y0, y0 + 1, fx, fy

    def _walk(self, x, y, u, v, u_var, v_var, dt, sensitivity):
        """Euler step plus N(0, var dt^2) displacement per drifter."""
        sx = np.sqrt(u_var) * dt
        sy = np.sqrt(v_var) * dt
        z = np.empty((len(x), 2))
        for i in range(len(x)):
            z[i, 0] = np.random.normal(loc=0, scale=sx[i])
            z[i, 1] = np.random.normal(loc=0, scale=sy[i])
        return x + sensitivity * (u * dt + z[:, 0]), y + sensitivity * (v * dt + z[:, 1])

    def driftFromVelocities(self, u_field, v_field, dx, dy, dt, x_zero_ref=0, y_zero_ref=0, u_var=None,
                            v_var=None, sensitivity=1.0):
        """One Euler step of every drifter (and the observation row) with
        velocities interpolated from (u_field, v_field); {x,y}_zero_ref is the
        cell whose face is at 0.  u_var / v_var (None, scalars or fields) add
        a random walk (D/CPUDrifterCollection.py:99-165)."""
        x0, x1, y0, y1, fx, fy = self._stencil(dx, dy, x_zero_ref, y_zero_ref)
        u = self._bilinear(u_field, x0, x1, y0, y1, fx, fy)
        v = self._bilinear(v_field, x0, x1, y0, y1, fx, fy)
        x, y = self.positions[:, 0], self.positions[:, 1]
        if u_var is None and v_var is None:
            x = x + sensitivity * u * dt
            y = y + sensitivity * v * dt
        else:
            def var_at(var):
                if np.isscalar(var):
                    return np.full(len(x), float(var))
                return np.maximum(0.0, self._bilinear(var, x0, x1, y0, y1, fx, fy))
            x, y = self._walk(x, y, u, v, var_at(u_var), var_at(v_var), dt, sensitivity)
        for i in range(len(x)):
            xi, yi = self._enforceBoundaryConditionsOnPosition(x[i], y[i])
            assert not np.isnan(xi), "new x is NaN after enforcing boundary conditions"
            assert not np.isnan(yi), "new y is NaN after enforcing boundary conditions"
            self.positions[i, 0], self.positions[i, 1] = xi, yi

    def drift(self, eta, hu, hv, Hm, dx, dy, dt, x_zero_ref=0, y_zero_ref=0, u_var=None, v_var=None,
              sensitivity=1.0):
        """Drift with the velocities hu / (eta + Hm), hv / (eta + Hm)."""
        u = hu / (eta + Hm)
        v = hv / (eta + Hm)
        self.driftFromVelocities(u, v, dx, dy, dt, x_zero_ref=x_zero_ref, y_zero_ref=y_zero_ref, u_var=u_var,
                                 v_var=v_var, sensitivity=sensitivity)

    def enforceBoundaryConditions(self):
        """Wrap every row into the domain when both directions are periodic
        (the reference does nothing otherwise)."""
        if self.boundaryConditions.isPeriodicNorthSouth() and self.boundaryConditions.isPeriodicEastWest():
            for i in range(self.getNumDrifters() + 1):
                self.positions[i, 0], self.positions[i, 1] = \
                    self._enforceBoundaryConditionsOnPosition(self.positions[i, 0], self.positions[i, 1])
