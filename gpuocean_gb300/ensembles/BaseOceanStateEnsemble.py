"""Common interface of the ensembles of ocean states (drop-in for
``ensembles/BaseOceanStateEnsemble.py:34-342``).

An ensemble holds particles (ocean states, each with drifters) and, for twin
experiments, a synthetic truth.  This base class carries what the data
assimilation layer reads from any ensemble - innovations, their norms,
Gaussian particle weights and the sizes of the problem - on top of an
``observeParticles`` that the concrete ensembles implement on the device.
"""
from __future__ import annotations

import abc

import numpy as np


class BaseOceanStateEnsemble(abc.ABC):
    """Ensemble of ocean states.  Concrete ensembles set ``particles``,
    ``numParticles``, ``particlesActive``, ``driftersPerOceanModel``, the grid
    (``nx, ny, dx, dy, dt``), ``observation_variance``, ``observation_cov``
    and ``observation_cov_inverse``, and implement the abstract methods."""

    # ------------------------------------------------------------------
    # what a concrete ensemble provides
    # ------------------------------------------------------------------
    @abc.abstractmethod
    def cleanUp(self):
        """Free the device memory of the ensemble."""

    @abc.abstractmethod
    def resample(self, newSampleIndices, reinitialization_variance):
        """Particle i becomes a copy of particle newSampleIndices[i]."""

    @abc.abstractmethod
    def step_truth(self, t, stochastic=True):
        """Advance the truth by t seconds."""

    @abc.abstractmethod
    def step_particles(self, t, stochastic=True):
        """Advance every particle by t seconds."""

    @abc.abstractmethod
    def observeParticles(self, gpu=False, innovation=False, observations=None):
        """(particles, drifters, 2): (hu, hv) of every particle at the observed
        positions, or the innovation y - H(psi) when ``innovation``."""

    @abc.abstractmethod
    def observeTrueDrifters(self):
        """Positions of the truth's drifters."""

    @abc.abstractmethod
    def observeTrueState(self):
        """(drifters, 4): [x, y, hu, hv] of the truth at its drifters."""

    @abc.abstractmethod
    def downloadTrueOceanState(self):
        """(eta, hu, hv) of the truth, interior cells."""

    def setTrueDrifterPositions(self, newPositions):
        raise NotImplementedError("This function must be implemented in child class")

    def __del__(self):
        try:
            self.cleanUp()
        except Exception:
            pass

    # ------------------------------------------------------------------
    # innovations and weights (E/BaseOceanStateEnsemble.py:222-290)
    # ------------------------------------------------------------------
    def getInnovations(self, observations=None):
        """y^m - H(psi_i^m) for every particle: (particles, drifters, 2)."""
        return self.observeParticles(innovation=True, observations=observations)

    def getInnovationNorms(self, observations=None):
        """Per particle the 2-norm over drifters of the per-drifter 2-norms
        of its innovation."""
        innovations = self.getInnovations(observations=observations)
        return np.linalg.norm(np.linalg.norm(innovations, axis=2), axis=1)

    def getGaussianWeight(self, innovations=None, normalize=True, R_scale=1.0):
        """Particle weights from a Gaussian observation error with covariance
        R = R_scale * observation_cov: log w_i = -1/2 sum_d d_id^T R^-1 d_id
        (inactive particles: weight 0).  ``normalize``: weights summing to 1,
        computed stably from the largest log-weight; otherwise the density
        with its normalising constant.  1-D innovations (one scalar per
        particle) use the variance R[0, 0]."""
        if innovations is None:
            innovations = self.getInnovations()
        innovations = np.asarray(innovations)
        R = self.getObservationCov() * R_scale
        Rinv = self.getObservationCovInverse() / R_scale
        if innovations.ndim == 1:
            var = R[0, 0]
            log_w = -(innovations ** 2 / (2 * var))
            norm = 1.0 / np.sqrt(2 * np.pi * var)
        else:
            assert R.shape == (2, 2), 'Observation covariance matrix must be 2x2'
            assert Rinv.shape == (2, 2), 'Inverse of the observation covariance matrix must be 2x2'
            n_part = int(self.getNumParticles())
            n_drift = innovations.shape[1]
            quad = np.einsum("pdi,ij,pdj->p", innovations[:n_part], Rinv, innovations[:n_part])
            active = np.asarray(self.particlesActive[:n_part], dtype=bool)
            log_w = np.where(active, -0.5 * quad, -np.inf)
            norm = 1.0 / ((2 * np.pi) ** n_drift * np.linalg.det(R) ** (n_drift / 2.0))
        if normalize:
            shifted = np.exp(log_w - log_w.max())
            return shifted / shifted.sum()
        return norm * np.exp(log_w)

    # ------------------------------------------------------------------
    # sizes and parameters
    # ------------------------------------------------------------------
    def getNx(self):
        return np.int32(self.nx)

    def getNy(self):
        return np.int32(self.ny)

    def getDx(self):
        return np.float32(self.dx)

    def getDy(self):
        return np.float32(self.dy)

    def getDt(self):
        return np.float32(self.dt)

    def getDomainSizeX(self):
        return self.getNx() * self.getDx()

    def getDomainSizeY(self):
        return self.getNy() * self.getDy()

    def getObservationVariance(self):
        return self.observation_variance

    def getNumParticles(self):
        return np.int32(self.numParticles)

    def getNumDrifters(self):
        return np.int32(self.driftersPerOceanModel)

    def getNumActiveParticles(self):
        return sum(self.particlesActive)

    def getBoundaryConditions(self):
        return self.particles[0].boundary_conditions

    def getObservationCov(self):
        return self.observation_cov

    def getObservationCovInverse(self):
        return self.observation_cov_inverse

    def downloadParticleOceanState(self, particleNo):
        """(eta, hu, hv) of one active particle, interior cells."""
        assert -1 < particleNo < self.getNumParticles(), "particle out of range"
        assert self.particlesActive[particleNo], "Trying to download state of deactivated particle"
        return self.particles[particleNo].download(interior_domain_only=True)
