"""Drifters of a multi-level ensemble (drop-in for
``drifters/MLDrifterCollection.py:24-176``).

A multi-level ensemble has no member states of its own to drift with; its
drifters move with the multi-level estimate of the mean velocity plus a
random walk scaled by the estimated variance.  Every unique drifter is
represented by ``ensemble_size`` realisations, stored consecutively
(drifter d's realisations are rows d * ensemble_size .. (d + 1) * ensemble_size - 1,
then the observation row).  With the biased walk (the default) each
realisation keeps one standard-normal direction for its whole life, drawn
at construction; otherwise new directions are drawn at every step.
"""
from __future__ import annotations

import numpy as np

from .CPUDrifterCollection import CPUDrifterCollection


class MLDrifterCollection(CPUDrifterCollection):
    def __init__(self, numDrifters, ensemble_size, observation_variance=0.01, boundaryConditions=None,
                 initialization_cov_drifters=None, domain_size_x=1.0, domain_size_y=1.0, use_biased_walk=True):
        super().__init__(numDrifters * ensemble_size, observation_variance=observation_variance,
                         boundaryConditions=boundaryConditions, domain_size_x=domain_size_x,
                         domain_size_y=domain_size_y)
        self.ensemble_size = ensemble_size
        self.num_unique_drifters = numDrifters
        # The reference seeds the realisations from a collection it does not
        # initialise (D/MLDrifterCollection.py:62-72), so every drifter starts
        # at (0, 0) until setDrifterPositions is called; kept for identical
        # results.
        self.positions[:-1, :] = 0.0
        self.use_biased_walk = use_biased_walk
        self.biased_walk_x = None
        self.biased_walk_y = None
        if self.use_biased_walk:
            self.biased_walk_x = np.random.normal(loc=0, scale=1, size=(self.numDrifters + 1))
            self.biased_walk_y = np.random.normal(loc=0, scale=1, size=(self.numDrifters + 1))

    def expandDrifterPositions(self, pos):
        """One position per unique drifter -> that position for each of its
        realisations: (numDrifters, 2) -> (numDrifters * ensemble_size, 2)."""
        return np.repeat(pos, self.ensemble_size, axis=0)

    def getDrifterPositionsForDrifter(self, drifter_index):
        """The (ensemble_size, 2) realisations of one unique drifter."""
        assert drifter_index >= 0, "drifter_index must be positive, but got " + str(drifter_index)
        assert drifter_index < self.num_unique_drifters, \
            "drifter_index must be smaller than number of unique drifters (" + str(self.num_unique_drifters) + \
            "), but got " + str(drifter_index)
        e = self.ensemble_size
        return self.positions[drifter_index * e:(drifter_index + 1) * e, :].copy()

    def getDrifterPositionsForEnsembleMember(self, ensemble_member):
        """Realisation `ensemble_member` of every unique drifter: (numDrifters, 2)."""
        assert ensemble_member >= 0, "ensemble_member must be positive, but got " + str(ensemble_member)
        assert ensemble_member < self.ensemble_size, \
            "drifter_index must be smaller than the ensemble size (" + str(self.ensemble_size) + "), but got " + \
            str(ensemble_member)
        return self.positions[ensemble_member:-1:self.ensemble_size, :].copy()

    def setDrifterPositions(self, newDrifterPositions):
        """Every realisation (numDrifters * ensemble_size rows), or one
        position per unique drifter (copied to all its realisations)."""
        pos = np.asarray(newDrifterPositions)
        if pos.shape[0] == self.numDrifters:
            return super().setDrifterPositions(pos)
        if pos.shape[0] == self.num_unique_drifters:
            return super().setDrifterPositions(self.expandDrifterPositions(pos))

    def drift(self, u_field, v_field, dx, dy, dt, x_zero_ref=0, y_zero_ref=0, u_var=None, v_var=None,
              sensitivity=1.0):
        """One step with the mean velocities (u_field, v_field) and the
        variance fields (u_var, v_var) (D/MLDrifterCollection.py:111-143).  On
        periodic domains the fields get a one-cell periodic halo first, so the
        interpolation reads across the boundary."""
        assert u_var is not None and v_var is not None, \
            "u_var and v_var must be provided for the MLDrifterCollection class to make sense"
        if self.boundaryConditions.isPeriodic() and x_zero_ref == 0 and y_zero_ref == 0:
            u_field, v_field, u_var, v_var = (self._expandPeriodicField(f) for f in (u_field, v_field, u_var, v_var))
            x_zero_ref = y_zero_ref = 1
        self.driftFromVelocities(u_field, v_field, dx, dy, dt, x_zero_ref=x_zero_ref, y_zero_ref=y_zero_ref,
                                 u_var=u_var, v_var=v_var, sensitivity=sensitivity)

    @staticmethod
    def _expandPeriodicField(field):
        """The field with a one-cell halo of its periodic images (corners
        included)."""
        return np.pad(np.asarray(field, dtype=np.float64), 1, mode="wrap")

    def _walk(self, x, y, u, v, u_var, v_var, dt, sensitivity):
        if not self.use_biased_walk:
            return super()._walk(x, y, u, v, u_var, v_var, dt, sensitivity)
        x = x + sensitivity * (u * dt + self.biased_walk_x * np.sqrt(u_var) * dt)
        y = y + sensitivity * (v * dt + self.biased_walk_y * np.sqrt(v_var) * dt)
        return x, y


class DriftTrajectory:
    """Positions of one realisation of every unique drifter over time: the
    part of the reference's observation store (utils/Observation.py, a pandas
    table) that a multi-level ensemble writes and that plots of drift
    trajectories read.  Times are rounded to whole seconds, as there."""

    def __init__(self, jump_limit=100000.0):
        self.times = []
        self.positions = []
        self.obs_errors = []
        self.jump_limit = jump_limit

    def get_num_observations(self):
        return len(self.times)

    def get_num_drifters(self):
        return 0 if not self.positions else self.positions[0].shape[0]

    def add_observation_from_mldrifters(self, t, mldrifters, ensemble_member):
        """Record realisation `ensemble_member` of every unique drifter at time
        t.  Like the reference it also draws (and keeps) a standard-normal
        observation error per coordinate, so numpy's global generator
        advances the same way."""
        rounded = round(t)
        assert rounded not in self.times, "Observation for time " + str(rounded) + " already exists in DataFrame"
        pos = mldrifters.getDrifterPositionsForEnsembleMember(ensemble_member)
        self.obs_errors.append(np.random.normal(size=pos.shape))
        self.times.append(rounded)
        self.positions.append(pos)

    def get_observation_times(self):
        """The recorded times after the first (the first is the start)."""
        return np.array(self.times[1:]) if len(self.times) >= 2 else np.array([])

    def get_drifter_position(self, t):
        """(drifters, 2) positions recorded at time t."""
        rounded = round(t)
        assert self.times.count(rounded) == 1, "Observation for time " + str(rounded) + " does not exists in DataFrame"
        return self.positions[self.times.index(rounded)].copy()

    def get_drifter_path(self, drifter_id, start_t, end_t, in_km=True):
        """The drifter's recorded positions in [start_t, end_t] as a list of
        paths, split where it jumps by more than jump_limit metres (through a
        periodic boundary)."""
        paths, cur = [], []
        for t, pos in zip(self.times, self.positions):
            if t < start_t or t > end_t:
                continue
            p = pos[drifter_id].astype(np.float64)
            if cur and np.hypot(*(p - cur[-1])) > self.jump_limit:
                paths.append(np.array(cur))
                cur = []
            cur.append(p)
        paths.append(np.array(cur).reshape(-1, 2))
        return [p / 1000.0 for p in paths] if in_km else paths

    def to_pickle(self, path):
        import pickle
        with open(path, "wb") as f:
            pickle.dump({"times": self.times, "positions": self.positions, "obs_errors": self.obs_errors}, f)

    def read_pickle(self, path):
        import pickle
        with open(path, "rb") as f:
            d = pickle.load(f)
        self.times, self.positions, self.obs_errors = d["times"], d["positions"], d["obs_errors"]
