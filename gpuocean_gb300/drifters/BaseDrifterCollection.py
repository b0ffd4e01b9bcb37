"""Host-side bookkeeping shared by the drifter collections.

Counterpart of ``drifters/BaseDrifterCollection.py:35-425`` of the reference:
positions of N drifters plus one observation row, periodic distances and
innovations, Gaussian/Cauchy weights, collection mean, resampling and the
regular-grid initialisation.  These are small host-side computations; the
advection itself runs on the GPU (GPUDrifterCollection).
"""
from __future__ import annotations

import numpy as np

from ..utils import Common


class BaseDrifterCollection:
    def __init__(self, numDrifters, observation_variance=0.1, boundaryConditions=None,
                 domain_size_x=1.0, domain_size_y=1.0):
        self.numDrifters = int(numDrifters)
        self.obs_index = self.numDrifters
        self.observation_variance = observation_variance
        self.positions = None
        self.domain_size_x = domain_size_x
        self.domain_size_y = domain_size_y
        self.boundaryConditions = boundaryConditions if boundaryConditions is not None else Common.BoundaryConditions()

    def __del__(self):
        try:
            self.cleanUp()
        except Exception:
            pass

    # abstract
    def getDrifterPositions(self):
        raise NotImplementedError

    def getObservationPosition(self):
        raise NotImplementedError

    def setDrifterPositions(self, newDrifterPositions):
        raise NotImplementedError

    def setObservationPosition(self, newObservationPosition):
        raise NotImplementedError

    def enforceBoundaryConditions(self):
        raise NotImplementedError

    def cleanUp(self):
        pass

    def copy(self):
        raise NotImplementedError

    # gets / sets
    def getNumDrifters(self):
        return self.numDrifters

    def getObservationVariance(self):
        return self.observation_variance

    def getBoundaryConditions(self):
        return self.boundaryConditions

    def getDomainSizeX(self):
        return self.domain_size_x

    def getDomainSizeY(self):
        return self.domain_size_y

    def setBoundaryConditions(self, boundaryConditions):
        self.boundaryConditions = boundaryConditions

    def setDomainSize(self, size_x, size_y):
        self.domain_size_x = size_x
        self.domain_size_y = size_y

    # shared methods
    def uniformly_distribute_drifters(self, initialization_cov_drifters=None):
        """Drifters at the cell centres of a near-square sub-division of the
        domain, optionally perturbed by N(0, cov) (BaseDrifterCollection.py:141-173)."""
        n = self.numDrifters
        sy = int(np.round(np.sqrt(n)))
        sx = int(np.ceil(1.0 * n / sy))
        ids = np.arange(n)
        pos = np.empty((n, 2))
        pos[:, 0] = (ids % sx + 0.5) * self.domain_size_x / sx
        pos[:, 1] = (ids // sx + 0.5) * self.domain_size_y / sy
        if initialization_cov_drifters is None:
            cov = np.zeros((2, 2))
        elif np.isscalar(initialization_cov_drifters):
            cov = np.eye(2) * initialization_cov_drifters
        else:
            cov = np.asarray(initialization_cov_drifters)
        assert cov.shape == (2, 2), 'initialization_cov_drifters has the wrong shape: ' + str(cov)
        if np.any(cov != 0):
            for d in range(n):
                pos[d, :] = np.random.multivariate_normal(pos[d, :], cov)
        self.setDrifterPositions(pos)

    def _getClosestPositions(self, obs=None):
        pos = np.array(self.getDrifterPositions(), dtype=np.float64, copy=True)
        bc = self.boundaryConditions
        if not (bc.isPeriodicNorthSouth() or bc.isPeriodicEastWest()):
            return pos
        ox, oy = self.getObservationPosition() if obs is None else obs[:2]
        for col, periodic, L, o in ((0, bc.isPeriodicEastWest(), self.domain_size_x, ox),
                                    (1, bc.isPeriodicNorthSouth(), self.domain_size_y, oy)):
            if periodic:
                cand = pos[:, col][:, None] + np.array([-L, 0.0, L])[None, :]
                pos[:, col] = cand[np.arange(len(pos)), np.argmin(np.abs(cand - o), axis=1)]
        return pos

    def getInnovations(self, obs=None):
        if obs is None:
            obs = self.getObservationPosition()
            closest = self._getClosestPositions()
        else:
            closest = self._getClosestPositions(obs)
        return np.asarray(obs[:2])[None, :] - closest

    def getDistances(self, obs=None):
        inn = self.getInnovations(obs)
        return np.sqrt(inn[:, 0] ** 2 + inn[:, 1] ** 2)

    def getGaussianWeight(self, distances=None, normalize=True):
        d = self.getDistances() if distances is None else distances
        var = self.getObservationVariance()
        w = (1.0 / np.sqrt(2 * np.pi * var)) * np.exp(-(d ** 2 / (2 * var)))
        return w / np.sum(w) if normalize else w

    def getCauchyWeight(self, distances=None, normalize=True):
        d = self.getDistances() if distances is None else distances
        var = self.getObservationVariance()
        w = 1.0 / (np.pi * np.sqrt(var) * (1 + (d ** 2 / var)))
        return w / np.sum(w) if normalize else w

    def _enforceBoundaryConditionsOnPosition(self, x, y):
        # the reference wraps y < 0 with the x size (BaseDrifterCollection.py:284) - kept
        if x < 0:
            x = self.domain_size_x + x
        if y < 0:
            y = self.domain_size_x + y
        if x > self.domain_size_x:
            x = x - self.domain_size_x
        if y > self.domain_size_y:
            y = y - self.domain_size_y
        return x, y

    def getCollectionMean(self, obs=None):
        mean_x, mean_y = np.mean(self._getClosestPositions(obs=obs), axis=0)
        return np.array(self._enforceBoundaryConditionsOnPosition(mean_x, mean_y))

    def resample(self, newSampleIndices, reinitialization_variance):
        old = np.array(self.getDrifterPositions(), dtype=np.float64, copy=True)
        n = len(newSampleIndices)
        if self.getNumDrifters() != n:
            raise RuntimeError("ERROR: The size of the new ensemble differs from the old size!")
        new = np.zeros((n, 2))
        if reinitialization_variance == 0:
            new[:, :] = old[newSampleIndices, :]
        else:
            once = np.zeros(n, dtype=bool)
            var = np.eye(2) * reinitialization_variance
            for i, idx in enumerate(newSampleIndices):
                if once[idx]:
                    new[i, :] = np.random.multivariate_normal(old[idx, :], var)
                else:
                    new[i, :] = old[idx, :]
                    once[idx] = True
        self.setDrifterPositions(new)
        self.enforceBoundaryConditions()

    def initializeUniform(self):
        positions = np.random.rand(self.getNumDrifters() + 1, 2)
        positions[-1, :] = positions[-1, :] * 0.5 + 0.25
        positions[:, 0] *= self.domain_size_x
        positions[:, 1] *= self.domain_size_y
        self.setDrifterPositions(positions[:-1, :])
        self.setObservationPosition(positions[-1, :])
