"""Ensemble of CDKLM16 models built from simulator arguments
(drop-in for ``ensembles/OceanModelEnsemble.py:34-218``).

All members advance together through the batched engine: one persistent
launch per RK2 step for the whole ensemble, SOAR model error for all members
in two launches, drifters advected inside the step launch.  Members that the
batched engine does not take (sponge boundaries, a north-angle texture) step
one by one through their own CUDA path, as the reference's ensemble does.
"""
from __future__ import annotations

import logging

import numpy as np

from ..drifters.GPUDrifterCollection import GPUDrifterCollection
from ..SWEsimulators import CDKLM16
from .BatchedEnsemble import BatchedEnsemble


class OceanModelEnsemble:
    def __init__(self, gpu_ctx, sim_args, data_args, model_error_args, numParticles,
                 observation_variance=0.01 ** 2, initialization_variance_factor_ocean_field=0.0,
                 super_dir_name=None, netcdf_filename=None, rank=0, rng_seed=None):
        self.logger = logging.getLogger(__name__)
        self.gpu_ctx = gpu_ctx
        self.sim_args, self.data_args = sim_args, data_args
        self.numParticles = numParticles
        self.observation_variance = observation_variance
        self.initialization_variance_factor_ocean_field = initialization_variance_factor_ocean_field
        if np.isscalar(observation_variance):
            self.observation_cov = np.eye(2) * observation_variance
            self.observation_cov_inverse = np.eye(2) * (1.0 / observation_variance)
        else:
            self.observation_cov = observation_variance
            self.observation_cov_inverse = np.linalg.inv(observation_variance)
        self.particles = [None] * numParticles
        self.drifterForecast = [None] * numParticles
        for i in range(numParticles):
            self.particles[i] = CDKLM16.CDKLM16(gpu_ctx, **sim_args, **data_args, local_particle_id=i)
            if 'small_scale_perturbation_amplitude' in model_error_args:
                self.particles[i].setSOARModelError(**model_error_args)
            elif 'kl_scaling' in model_error_args:
                self.particles[i].setKLModelError(**model_error_args)
            if initialization_variance_factor_ocean_field != 0.0:
                self.particles[i].perturbState(q0_scale=initialization_variance_factor_ocean_field)
        self.nx, self.ny = self.particles[0].nx, self.particles[0].ny
        self.dx, self.dy = self.particles[0].dx, self.particles[0].dy
        self.t = self.particles[0].t
        self.particlesActive = [True] * numParticles
        self.engine = None
        self.rng_seed = rng_seed if rng_seed is not None else 1234 + 7919 * rank

    def _engine(self):
        """The batched engine over all particles, or None when they step one
        by one (members the engine rejects)."""
        if self.engine is None:
            try:
                self.engine = BatchedEnsemble(self.particles)
            except NotImplementedError as e:
                self.logger.info("particles step one by one: %s", e)
                self.engine = False
                return None
            if all(p.model_error is not None for p in self.particles):
                self.engine.set_noise([p.model_error for p in self.particles], rng_seed=self.rng_seed)
        return self.engine or None

    def attachDrifters(self, drifter_positions):
        for i in range(self.numParticles):
            if len(drifter_positions) > 0:
                d = GPUDrifterCollection(self.gpu_ctx, len(drifter_positions),
                                         observation_variance=self.observation_variance,
                                         boundaryConditions=self.data_args['boundary_conditions'],
                                         domain_size_x=self.data_args['nx'] * self.data_args['dx'],
                                         domain_size_y=self.data_args['ny'] * self.data_args['dy'])
                d.setDrifterPositions(drifter_positions)
                self.particles[i].attachDrifters(d)
        if self.engine:
            self.engine._build(self.engine.max_substeps)

    def cleanUp(self):
        if self.engine:
            self.engine.release()
        for p in self.particles:
            if p is not None:
                p.cleanUp(do_gc=False)

    def stepToObservation(self, observation_time, write_now=False, courant_number=0.8):
        """Advance to observation_time in the blocks that
        CDKLM16.dataAssimilationStep takes for each member (S/CDKLM16.py:
        742-806; plan from ``ObservationSchedule.blocks_to_observation``),
        all members at once.  Full blocks with model error run as one graph
        with the model error inside; a shorter first block is stepped and
        then perturbed with its own scale."""
        from ..SWEsimulators.ObservationSchedule import blocks_to_observation, refresh_dt_after
        eng = self._engine()
        p0 = self.particles[0]
        if eng is None:
            for p in self.particles:
                p.dataAssimilationStep(observation_time, write_now=write_now, courant_number=courant_number)
            self.t = observation_time
            return
        plan = blocks_to_observation(observation_time - p0.t, p0.model_time_step)
        eng.updateDt(courant_number=courant_number)
        noisy = eng._noise is not None
        for blk in plan:
            scaled = noisy and blk.perturbation is not None and blk.perturbation != 1.0
            eng.step(blk.length, apply_stochastic_term=noisy and blk.perturbation == 1.0)
            if scaled:
                eng.perturb(perturbation_scale=blk.perturbation)
            for p in self.particles:
                p.total_time_steps += 1
            if refresh_dt_after(p0.total_time_steps):
                eng.updateDt(courant_number=courant_number)
        self.t = observation_time

    def modelStep(self, sub_t, rank="", update_dt=True):
        eng = self._engine()
        if eng is None:
            for p in self.particles:
                p.step(sub_t, apply_stochastic_term=p.model_error is not None)
                if update_dt:
                    p.updateDt()
            self.t = self.particles[0].t
            return self.t
        eng.step(sub_t, apply_stochastic_term=eng._noise is not None, noise_cadence="step")
        if update_dt:
            eng.updateDt()
        self.t = self.particles[0].t
        return self.t

    def updateDt(self):
        eng = self._engine()
        if eng is None:
            for p in self.particles:
                p.updateDt()
        else:
            eng.updateDt()

    def observeParticles(self, drifter_positions):
        """hu, hv of every particle at the cells of the given positions,
        (particles, drifters, 2), in one launch (E/OceanModelEnsemble.py:
        observeParticles; cells found in float64 on the host)."""
        pos = np.asarray(drifter_positions, dtype=np.float64)
        dx, dy = float(self.data_args['dx']), float(self.data_args['dy'])
        ix = np.floor(pos[:, 0] / dx)
        iy = np.floor(pos[:, 1] / dy)
        eng = self._engine()
        if eng is None:
            out = np.empty((len(self.particles), len(pos), 2))
            jx, jy = ix.astype(np.int64), iy.astype(np.int64)
            for k, p in enumerate(self.particles):
                _, hu, hv = p.download(interior_domain_only=True)
                out[k, :, 0] = np.asarray(hu)[jy, jx]
                out[k, :, 1] = np.asarray(hv)[jy, jx]
            return out
        centres = np.stack([(ix + 0.5) * dx, (iy + 0.5) * dy], axis=1)
        obs = eng.observe(centres, first=0, count=len(self.particles))
        return obs[:, :, 1:].astype(np.float64)

    def getNumParticles(self):
        return self.numParticles

    def syncGPU(self):
        if self.engine:
            self.engine.synchronize()
        for p in self.particles:
            p.gpu_stream.synchronize()
