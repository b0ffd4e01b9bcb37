"""Ensemble of perturbed copies of one simulator plus a synthetic truth
(drop-in for ``ensembles/OceanNoiseEnsemble.py:43-790``, drifter-position and
direct-flow observations).

The truth and all particles advance in one batched engine; the model error
is applied after every RK2 step, as ``CDKLM16.step`` does.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .. import _lib
from ..drifters.GPUDrifterCollection import GPUDrifterCollection
from ..SWEsimulators import CDKLM16
from ..utils import Common
from .BaseOceanStateEnsemble import BaseOceanStateEnsemble
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


class OceanNoiseEnsemble(BaseOceanStateEnsemble):
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
        if observation_type == ObservationType.StaticBuoys and buoys_positions is not None:
            assert len(buoys_positions) == num_drifters, \
                "number of given buoys positions does not match the specified num_drifters"
        self.buoys_positions = buoys_positions
        # statistics under the first drifter, one entry per
        # getEnsembleVarAndRMSEUnderDrifter call
        for q in ("eta", "hu", "hv"):
            for name in ("varianceUnderDrifter_", "rmseUnderDrifter_", "rmseMeanUnderDrifter_",
                         "rmseWeightedUnderDrifter_", "rUnderDrifter_"):
                setattr(self, name + q, [])
        self.tArray = []
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
        if observation_type == ObservationType.StaticBuoys:
            if self.buoys_positions is None:
                self.buoys_positions = self.particles[-1].drifters.getDrifterPositions()
            bp = np.asarray(self.buoys_positions, dtype=np.float64)
            self.buoys_ids = np.stack([np.floor(bp[:, 0] / self.dx), np.floor(bp[:, 1] / self.dy)],
                                      axis=1).astype(int)
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
        """All particles and the truth advance by t in one batched block, the
        model error after every step of the particles and of the truth as
        their flags say (E/OceanNoiseEnsemble.py:517-532)."""
        flags = [bool(stochastic_particles)] * self.numParticles + [bool(stochastic_truth)]
        self.engine.step(t, apply_stochastic_term=flags, noise_cadence="step")
        self.t = self.particles[self.obs_index].t
        return self.t

    def step_truth(self, t, stochastic=True):
        """Only the truth advances by t (E/OceanNoiseEnsemble.py:535-537)."""
        self.engine.step(t, apply_stochastic_term=bool(stochastic), noise_cadence="step", members=[self.obs_index])
        self.t = self.particles[self.obs_index].t
        return self.t

    def step_particles(self, t, stochastic=True):
        """Only the particles advance by t; returns the ensemble's time, which
        follows the truth (E/OceanNoiseEnsemble.py:539-543)."""
        self.engine.step(t, apply_stochastic_term=bool(stochastic), noise_cadence="step",
                         members=range(self.numParticles))
        return self.t

    def resample(self, newSampleIndices, reinitialization_variance):
        """Particle i becomes an exact copy of particle newSampleIndices[i]:
        state and previous state by device copies (every source read before
        any destination is written), drifters at the truth's positions for
        flow observations and at the source particle's positions otherwise
        (E/OceanNoiseEnsemble.py:364-406).  reinitialization_variance is
        ignored, as in the reference."""
        if self.observation_type == ObservationType.DrifterPosition:
            raise ValueError('Observation type DataAssimilationUtils.ObservationType.DrifterPosition is not supported')
        idx = [int(i) for i in newSampleIndices]
        assert len(idx) == self.numParticles
        flow = self.observation_type in (ObservationType.UnderlyingFlow, ObservationType.DirectUnderlyingFlow)
        true_pos = self.observeTrueDrifters() if flow else None
        new_pos = [true_pos if flow else self.particles[src].drifters.getDrifterPositions() for src in idx]
        eng = self.engine
        eng._after_members()
        st = eng.stream.handle
        planes = lambda p: (p.gpu_data.h0, p.gpu_data.hu0, p.gpu_data.hv0,
                            p.gpu_data.h1, p.gpu_data.hu1, p.gpu_data.hv1)
        sources = sorted({src for i, src in enumerate(idx) if src != i})
        stash = {}
        for src in sources:
            bufs = []
            for a in planes(self.particles[src]):
                nbytes = int(a.pitch) * (int(self.ny) + 4)
                b = Common.DevicePtr(nbytes)
                _lib.call("goc_memcpy_d2d_async", b.ptr, a.ptr, ctypes.c_size_t(nbytes), st)
                bufs.append(b)
            stash[src] = bufs
        for i, src in enumerate(idx):
            if src == i:
                continue
            for a, b in zip(planes(self.particles[i]), stash[src]):
                _lib.call("goc_memcpy_d2d_async", a.ptr, b.ptr, ctypes.c_size_t(int(a.pitch) * (int(self.ny) + 4)), st)
        eng._before_members()
        eng.synchronize()
        for bufs in stash.values():
            for b in bufs:
                b.free()
        for i in range(self.numParticles):
            self.particles[i].drifters.setDrifterPositions(np.asarray(new_pos[i]))

    def observeDrifters(self):
        out = np.empty((self.numParticles, self.driftersPerOceanModel, 2))
        for p in range(self.numParticles):
            out[p] = self.particles[p].drifters.getDrifterPositions()
        return out

    def observeTrueDrifters(self):
        return self.particles[self.obs_index].drifters.getDrifterPositions()

    def observeTrueState(self, apply_observation_error=True):
        """The truth observed at its drifters, [[x, y, hu, hv], ...] (or the
        positions for drifter-position observations), following
        E/OceanNoiseEnsemble.py:436-515: flow observations read hu, hv of the
        truth's cell (UnderlyingFlow: the drifter's displacement since the
        previous observation over the elapsed time, times the depth the
        reference reads there - at the cell index of the array that includes
        the ghost cells, a reference quirk kept for identical results;
        StaticBuoys: at the buoys' cells).  With apply_observation_error each
        hu, hv gets N(0, observation_variance) noise from numpy's global
        generator, drawn in the reference's order."""
        if self.observedDrifterPositions[-1][0] != self.t:
            self._addObservation(self.observeTrueDrifters())
        if self.observation_type == ObservationType.DrifterPosition:
            return self.observedDrifterPositions[-1][1]
        D = int(self.driftersPerOceanModel)
        out = np.empty((D, 4))
        sd = np.sqrt(self.observation_variance)
        if self.observation_type == ObservationType.UnderlyingFlow:
            (t1, p1), (t0, p0) = self.observedDrifterPositions[-1], self.observedDrifterPositions[-2]
            Hm = self.particles[self.obs_index].downloadBathymetry()[1]
            for d in range(D):
                x, y = p1[d, 0], p1[d, 1]
                depth = Hm[int(np.floor(y / self.dy)), int(np.floor(x / self.dx))]
                hu = (x - p0[d, 0]) / (t1 - t0) * depth
                hv = (y - p0[d, 1]) / (t1 - t0) * depth
                if apply_observation_error:
                    hu += np.random.normal(scale=sd)
                    hv += np.random.normal(scale=sd)
                out[d] = (x, y, hu, hv)
            return out
        eta, hu_f, hv_f = self.downloadTrueOceanState()
        hu_f, hv_f = np.asarray(hu_f), np.asarray(hv_f)
        for d in range(D):
            if self.observation_type == ObservationType.StaticBuoys:
                ix, iy = self.buoys_ids[d]
                x, y = self.buoys_positions[d][0], self.buoys_positions[d][1]
            else:
                x, y = self.observedDrifterPositions[-1][1][d]
                ix, iy = int(np.floor(x / self.dx)), int(np.floor(y / self.dy))
            hu, hv = hu_f[iy, ix], hv_f[iy, ix]
            if apply_observation_error:
                hu += np.random.normal(scale=sd)
                hv += np.random.normal(scale=sd)
            out[d] = (x, y, hu, hv)
        return out

    def setTrueDrifterPositions(self, newPositions):
        """Move the truth's drifters (E/OceanNoiseEnsemble.py:588-593)."""
        self.particles[self.obs_index].drifters.setDrifterPositions(newPositions)

    def getCauchyWeight(self, distances=None, normalize=True):
        """Particle weights from a Cauchy distribution of the drifter
        distances to the truth, scale sqrt(observation variance)
        (E/OceanNoiseEnsemble.py:571-586)."""
        if distances is None:
            distances = self.getDistances()
        var = self.getObservationVariance()
        w = 1.0 / (np.pi * np.sqrt(var) * (1 + (np.asarray(distances) ** 2 / var)))
        return w / np.sum(w) if normalize else w

    def findLargestPossibleTimeStep(self):
        """Largest stable dt over every particle and the truth:
        0.25 min(dx / max|u +- sqrt(g h)|, dy / max|v +- sqrt(g h)|), from
        the batched CFL reduction on the device (E/OceanNoiseEnsemble.py:
        595-619 downloads every state; it also scans the ghost cells, whose
        values behind walls are stale)."""
        return float(np.min(self.engine.max_dt()))

    def printMaxOceanStates(self):
        for no, sim in enumerate(self.particles):
            eta, hu, hv = sim.download()
            print("------- simNo: " + ("True state" if no == self.obs_index else str(no)) + " -------")
            print("t = " + str(sim.t))
            print("Max eta: ", np.max(eta))
            print("Max hu:  ", np.max(hu))
            print("Max hv:  ", np.max(hv))

    def downloadEnsembleStatisticalFields(self):
        """Ensemble mean of (eta, hu, hv), its distance from the truth
        |truth - mean| and the ratio of the spread
        sqrt(sum (x - mean)^2 / (N + 1)) to that distance, per interior cell
        (E/OceanNoiseEnsemble.py:723-775): one device pass over the particles
        for the mean and variance."""
        n = int(self.numParticles)
        mean, var = self.engine.moments(0, n, "state", ddof=0)
        truth = np.array(self.downloadTrueOceanState(), dtype=np.float64)
        mean = mean.astype(np.float64)
        rmse = np.sqrt((truth - mean) ** 2)
        with np.errstate(divide="ignore", invalid="ignore"):
            r = np.sqrt(var.astype(np.float64) * n / (1.0 + n)) / rmse
        m32, e32, r32 = (x.astype(np.float32) for x in (mean, rmse, r))
        return m32[0], m32[1], m32[2], e32[0], e32[1], e32[2], r32[0], r32[1], r32[2]

    def getEnsembleVarAndRMSEUnderDrifter(self, t, allDrifters=False):
        """Statistics of (eta, hu, hv) in the cell under the truth's first
        drifter, appended to the *UnderDrifter_* lists: the unbiased spread,
        the RMS distance of the particles from the truth, the distance of
        the mean from the truth, the RMS distance relative to |truth| and the
        ratio spread / RMS distance (E/OceanNoiseEnsemble.py:621-721).  All
        particles are read in one observation launch."""
        pos = self.observeTrueState()[0][0:2]
        ix, iy = int(np.floor(pos[0] / self.dx)), int(np.floor(pos[1] / self.dy))
        centre = np.array([[(ix + 0.5) * self.dx, (iy + 0.5) * self.dy]])
        vals = self.engine.observe(centre, first=0, count=self.numParticles + 1)[:, 0, :].astype(np.float64)
        truth, parts = vals[self.obs_index], vals[:self.numParticles]
        parts = parts[~np.isnan(parts[:, 0])]
        k = len(parts)
        mean = parts.mean(axis=0)
        rmse = np.sqrt(np.sum((truth - parts) ** 2, axis=0) / k)
        rmse_mean = np.sqrt((truth - mean) ** 2)
        rmse_w = rmse / np.abs(truth)
        sigma = np.sqrt(np.sum((parts - mean) ** 2, axis=0) / (k - 1.0))
        r = sigma / rmse
        for c, q in enumerate(("eta", "hu", "hv")):
            getattr(self, "varianceUnderDrifter_" + q).append(sigma[c])
            getattr(self, "rmseUnderDrifter_" + q).append(rmse[c])
            getattr(self, "rmseMeanUnderDrifter_" + q).append(rmse_mean[c])
            getattr(self, "rmseWeightedUnderDrifter_" + q).append(rmse_w[c])
            getattr(self, "rUnderDrifter_" + q).append(r[c])
        self.tArray.append(t)

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
        """(particles, drifters): distance of every particle's drifters from
        the truth's (E/OceanNoiseEnsemble.py:545-554; obs is not used there
        either)."""
        return np.linalg.norm(self.observeTrueDrifters() - self.observeDrifters(), axis=2)

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
