"""Ensemble of perturbed copies of one simulator plus a synthetic truth
(drop-in for ``ensembles/OceanNoiseEnsemble.py:43-790``, drifter-position and
direct-flow observations).

The truth and all particles advance in one batched engine; the model error
is applied after every RK2 step, as ``CDKLM16.step`` does.
"""
from __future__ import annotations

import numpy as np

from ..drifters.GPUDrifterCollection import GPUDrifterCollection
from ..SWEsimulators import CDKLM16
from .BatchedEnsemble import BatchedEnsemble
from .MultiLevelOceanEnsemble import _device_statistic


def _desingularise(h, hu, eps):
    """U/OceanographicUtilities.py:413-414."""
    return hu / np.maximum(np.minimum(h * h / (2.0 * eps) + 0.5 * eps, eps), np.abs(h))


class ObservationType:
    DrifterPosition = 1
    UnderlyingFlow = 2
    DirectUnderlyingFlow = 3
    StaticBuoys = 4


class OceanNoiseEnsemble:
    def __init__(self, gpu_ctx, numParticles, sim, num_drifters=1, observation_type=ObservationType.DrifterPosition,
                 buoys_positions=None, observation_variance=None, observation_variance_factor=5.0,
                 initialization_variance_factor_drifter_position=0.0, initialization_variance_factor_ocean_field=0.0,
                 compensate_for_eta=True, ensemble_small_scale_perturbation=True, rng_seed=2024):
        self.gpu_ctx = gpu_ctx
        self.numParticles = numParticles
        self.particles = [None] * (numParticles + 1)
        self.particlesActive = [True] * numParticles
        self.obs_index = numParticles
        self.t = 0.0
        self.observation_type = observation_type
        self.observedDrifterPositions = []
        eta, hu, hv = sim.download()
        Hi = sim.downloadBathymetry()[0]
        self.nx, self.ny, self.dx, self.dy, self.dt = sim.nx, sim.ny, sim.dx, sim.dy, sim.dt
        self.boundaryConditions = sim.boundary_conditions
        self.g, self.f, self.beta, self.r = sim.g, sim.f, sim.coriolis_beta, sim.r
        self.observation_variance = (observation_variance_factor * self.dx) ** 2 if observation_variance is None \
            else observation_variance
        self.observation_cov = np.eye(2) * self.observation_variance
        self.observation_cov_inverse = np.eye(2) * (1.0 / self.observation_variance)
        self.initialization_cov_drifters = np.eye(2) * initialization_variance_factor_drifter_position * self.dx
        self.driftersPerOceanModel = np.int32(num_drifters)
        self.compensate_for_eta = compensate_for_eta
        self.base_H = np.asarray(Hi)
        # mean cell-centre depth (E/OceanNoiseEnsemble.py:152-155)
        Hm = sim.downloadBathymetry()[1][2:-2, 2:-2]
        self.mean_depth = np.mean(Hm)
        self.constant_depth = np.max(Hm) == np.min(Hm)
        me = sim.model_error
        # sim.f is already compensated for the first interior cell; pass it back uncompensated
        f_in = float(sim.f) + float(sim.coriolis_beta) * 2 * float(sim.dy)
        for i in range(numParticles + 1):
            p = CDKLM16.CDKLM16(gpu_ctx, eta, hu, hv, Hi, self.nx, self.ny, self.dx, self.dy, self.dt, self.g,
                                f_in, self.r, coriolis_beta=self.beta, boundary_conditions=self.boundaryConditions)
            if me is not None:
                p.setSOARModelError(small_scale_perturbation_amplitude=me.soar_q0,
                                    small_scale_perturbation_interpolation_factor=int(me.interpolation_factor))
            if initialization_variance_factor_ocean_field != 0.0:
                p.perturbState(perturbation_scale=initialization_variance_factor_ocean_field)
            d = GPUDrifterCollection(gpu_ctx, int(num_drifters), observation_variance=self.observation_variance,
                                     boundaryConditions=self.boundaryConditions,
                                     initialization_cov_drifters=self.initialization_cov_drifters,
                                     domain_size_x=self.nx * self.dx, domain_size_y=self.ny * self.dy)
            if buoys_positions is not None:
                d.setDrifterPositions(buoys_positions)
            else:
                d.uniformly_distribute_drifters(initialization_cov_drifters=self.initialization_cov_drifters)
            p.attachDrifters(d)
            self.particles[i] = p
        self.engine = BatchedEnsemble(self.particles)
        if me is not None:
            self.engine.set_noise([p.model_error for p in self.particles], rng_seed=rng_seed)
        self._addObservation(self.observeTrueDrifters())

    def cleanUp(self):
        self.engine.release()
        for p in self.particles:
            if p is not None:
                p.cleanUp(do_gc=False)

    def _addObservation(self, positions):
        self.observedDrifterPositions.append([self.t, positions])

    def step(self, t, stochastic_particles=True, stochastic_truth=True):
        """All particles and the truth advance by t (S/.../OceanNoiseEnsemble.py:517-532)."""
        if stochastic_particles != stochastic_truth:
            raise NotImplementedError("truth and particles share one batched step")
        self.engine.step(t, apply_stochastic_term=stochastic_particles, noise_cadence="step")
        self.t = self.particles[self.obs_index].t
        return self.t

    def observeDrifters(self):
        out = np.empty((self.numParticles, self.driftersPerOceanModel, 2))
        for p in range(self.numParticles):
            out[p] = self.particles[p].drifters.getDrifterPositions()
        return out

    def observeTrueDrifters(self):
        return self.particles[self.obs_index].drifters.getDrifterPositions()

    def observeTrueState(self):
        if self.observedDrifterPositions[-1][0] != self.t:
            self._addObservation(self.observeTrueDrifters())
        if self.observation_type == ObservationType.DrifterPosition:
            return self.observedDrifterPositions[-1][1]
        eta, hu, hv = self.downloadTrueOceanState()
        pos = self.observedDrifterPositions[-1][1]
        ix = np.floor(pos[:, 0] / self.dx).astype(int)
        iy = np.floor(pos[:, 1] / self.dy).astype(int)
        return np.stack([pos[:, 0], pos[:, 1], np.asarray(hu)[iy, ix], np.asarray(hv)[iy, ix]], axis=1)

    # ------------------------------------------------------------------
    # observation operator and statistics (E/BaseOceanStateEnsemble.py:79-176)
    # ------------------------------------------------------------------
    def getNumDrifters(self):
        return int(self.driftersPerOceanModel)

    def observeParticles(self, gpu=False, innovation=False, observations=None):
        """(hu, hv) of every particle at the observed cells, (particles,
        drifters, 2), or the innovation against the truth's observation
        (E/BaseOceanStateEnsemble.py:79-145).  All particles are observed in
        one launch.  gpu=True observes at the truth's drifters in device
        memory (the reference's GPU path); otherwise at the cells of
        observations[:, :2], found in float64 as the reference's CPU path
        does.  Innovation: obs * (mean_depth + eta) / mean_depth - particle
        when compensate_for_eta, else obs - particle."""
        if self.observation_type == ObservationType.DrifterPosition:
            raise ValueError('Observation type DataAssimilationUtils.ObservationType.DrifterPosition is not supported')
        n = self.getNumParticles()
        if gpu:
            assert not innovation, 'Innovation is not supported when the observations are made on the GPU'
            obs = self.engine.observe(first=0, count=n, drifters=self.particles[self.obs_index].drifters)
            out = obs[:, :, 1:].astype(np.float64)
        else:
            if observations is None:
                observations = self.observeTrueState()
            observations = np.asarray(observations)
            ix = np.floor(observations[:, 0] / self.dx).astype(np.int64)
            iy = np.floor(observations[:, 1] / self.dy).astype(np.int64)
            # the cell centres select exactly the cells found above
            centres = np.stack([(ix + 0.5) * self.dx, (iy + 0.5) * self.dy], axis=1)
            obs = self.engine.observe(centres, first=0, count=n)
            if innovation:
                md = np.float32(self.mean_depth)
                comp = ((md + obs[:, :, 0]) / md).astype(np.float64) if self.compensate_for_eta else 1.0
                out = np.stack([observations[:, 2] * comp - obs[:, :, 1].astype(np.float64),
                                observations[:, 3] * comp - obs[:, :, 2].astype(np.float64)], axis=2)
            else:
                out = obs[:, :, 1:].astype(np.float64)
        for p in range(n):
            if not self.particlesActive[p]:
                out[p] = np.nan
        return out

    def estimate(self, func, **kwargs):
        """func over the particles of (eta, hu, hv), shape (3, ny, nx)
        (E/BaseOceanStateEnsemble.py:147-158).  np.mean and np.var (with
        ddof) run on the device in one pass; other funcs on the downloads."""
        stat = _device_statistic(func, kwargs)
        if stat is not None:
            m, v = self.engine.moments(0, self.getNumParticles(), "state", ddof=stat[1], mean=stat[0] == "mean",
                                       var=stat[0] == "var")
            return m if stat[0] == "mean" else v
        st = np.moveaxis(np.array([np.array(self.downloadParticleOceanState(e))
                                   for e in range(self.getNumParticles())]), 0, -1)
        return func(st, axis=-1, **kwargs)

    def estimateVelocity(self, func, desingularise=0.00001, **kwargs):
        """func over the particles of the desingularised velocities (u, v),
        shape (2, ny, nx) (E/BaseOceanStateEnsemble.py:160-176)."""
        stat = _device_statistic(func, kwargs)
        if stat is not None:
            m, v = self.engine.moments(0, self.getNumParticles(), "velocity", desingularise=desingularise,
                                       ddof=stat[1], mean=stat[0] == "mean", var=stat[0] == "var")
            return m if stat[0] == "mean" else v
        _, Hm = self.particles[0].downloadBathymetry(interior_domain_only=True)
        vel = []
        for e in range(self.getNumParticles()):
            eta, hu, hv = self.downloadParticleOceanState(e)
            h = eta + Hm
            vel.append(np.array([_desingularise(h, hu, desingularise), _desingularise(h, hv, desingularise)]))
        return func(np.moveaxis(np.array(vel), 0, -1), axis=-1, **kwargs)

    def getDistances(self, obs=None):
        obs = self.observeTrueDrifters() if obs is None else obs
        return np.array([np.linalg.norm(self.particles[p].drifters.getDrifterPositions() - obs, axis=1).mean()
                         for p in range(self.numParticles)])

    def downloadParticleOceanState(self, particleNo):
        return self.particles[particleNo].download(interior_domain_only=True)

    def downloadTrueOceanState(self):
        return self.particles[self.obs_index].download(interior_domain_only=True)

    def getNumParticles(self):
        return self.numParticles

    def getNx(self):
        return self.nx

    def getNy(self):
        return self.ny
