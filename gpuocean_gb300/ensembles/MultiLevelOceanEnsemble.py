"""Multi-level ensemble (drop-in for ``ensembles/MultiLevelOceanEnsemble.py:32-518``).

Level 0 is a list of simulators; every higher level is a pair of equally
long lists (fine partner, coarse partner).  All simulators of all levels -
grids of different sizes - advance in one batched launch per RK2 step over
the member/tile work queue.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .. import _lib
from ..utils import Common
from .BatchedEnsemble import BatchedEnsemble


def _device_statistic(func, kwargs):
    """("mean" | "var", ddof) when func is a statistic the device computes
    (np.mean, or np.var with at most a ddof keyword), else None."""
    if func is np.mean and not kwargs:
        return "mean", 0
    if func is np.var and set(kwargs) <= {"ddof"}:
        return "var", int(kwargs.get("ddof", 0))
    return None


class MultiLevelOceanEnsemble:
    def __init__(self, ML_ensemble, rng_seed=4242):
        assert len(ML_ensemble) > 1, "Single level ensembles are not valid"
        for l_idx in range(1, len(ML_ensemble)):
            assert len(ML_ensemble[l_idx]) == 2, "All higher levels need an ensemble of fine and coarse simulations each"
        self.ML_ensemble = ML_ensemble
        self.Nes = np.zeros(len(ML_ensemble), dtype=np.int32)
        self.Nes[0] = len(ML_ensemble[0])
        for l_idx in range(1, len(ML_ensemble)):
            self.Nes[l_idx] = len(ML_ensemble[l_idx][0])
        self.numLevels = len(self.Nes)
        first = [ML_ensemble[0][0]] + [ML_ensemble[l][0][0] for l in range(1, self.numLevels)]
        self.nxs = np.array([s.nx for s in first], dtype=np.int32)
        self.nys = np.array([s.ny for s in first], dtype=np.int32)
        self.dxs = np.array([s.dx for s in first])
        self.dys = np.array([s.dy for s in first])
        self.boundary_conditions = ML_ensemble[0][0].boundary_conditions
        self.t = ML_ensemble[0][0].t
        self.members = self._flat()
        self.drifters = None
        self.drift_dt = None
        self.driftTrajectory = None
        self.drift_sensitivity = None
        self.engine = BatchedEnsemble(self.members)
        if all(s.model_error is not None for s in self.members):
            from ..SWEsimulators.ModelErrorKL import ModelErrorKL
            sources = None
            if all(isinstance(s.model_error, ModelErrorKL) for s in self.members):
                # a coarse partner is perturbed with its fine partner's normals
                # and rollers (perturbSimilarAs in dataAssimilationStep,
                # S/CDKLM16.py:782-790): the KL basis lives on the unit square,
                # so both see the same field at their own resolution
                sources = np.arange(len(self.members), dtype=np.int32)
                for l_idx, ((fa, n), (ca, _)) in enumerate(self._groups()[1:], start=1):
                    sources[ca:ca + n] = np.arange(fa, fa + n)
            self.engine.set_noise([s.model_error for s in self.members], rng_seed=rng_seed, sources=sources)

    def _flat(self):
        out = list(self.ML_ensemble[0])
        for l_idx in range(1, self.numLevels):
            out += list(self.ML_ensemble[l_idx][0]) + list(self.ML_ensemble[l_idx][1])
        return out

    def step(self, t, apply_stochastic_term=True, **kwargs):
        """Every simulator of every level advances by t."""
        self.engine.step(t, apply_stochastic_term=apply_stochastic_term, noise_cadence="step")
        self.t = self.ML_ensemble[0][0].t

    def _leaders(self):
        """Engine indices of the simulators whose own dataAssimilationStep
        the reference calls (level 0 and the fine partners); the coarse
        partners ride along as ``otherSim``."""
        groups = self._groups()
        first, n0 = groups[0]
        out = list(range(first, first + n0))
        for (fa, n), _ in groups[1:]:
            out += list(range(fa, fa + n))
        return out

    def _run_to(self, end_time, courant_number):
        """Every member to end_time in the blocks of
        CDKLM16.dataAssimilationStep (S/CDKLM16.py:742-806), the coarse
        partners perturbed like their fine partners after each block.  dt:
        all members at the start, the leaders again after every fifth block
        they have taken."""
        from ..SWEsimulators.ObservationSchedule import blocks_to_observation, refresh_dt_after
        eng = self.engine
        s0 = self.ML_ensemble[0][0]
        plan = blocks_to_observation(end_time - s0.t, s0.model_time_step)
        leaders = self._leaders()
        eng.updateDt(courant_number=courant_number)
        noisy = eng._noise is not None
        for blk in plan:
            eng.step(blk.length, apply_stochastic_term=noisy and blk.perturbation == 1.0)
            if noisy and blk.perturbation is not None and blk.perturbation != 1.0:
                eng.perturb(perturbation_scale=blk.perturbation)
            for m in leaders:
                self.members[m].total_time_steps += 1
            if refresh_dt_after(s0.total_time_steps):
                eng.updateDt(courant_number=courant_number, members=leaders)

    def stepToObservation(self, obs_time, courant_number=0.8):
        """Advance to obs_time as the reference does
        (E/MultiLevelOceanEnsemble.py:110-141): with drifters attached, in
        stretches of at most drift_dt, the drifters moving after each."""
        s0 = self.ML_ensemble[0][0]
        t = s0.t
        while t < obs_time:
            end = obs_time
            if getattr(self, "drifters", None) is not None:
                step = min(obs_time - t, self.drift_dt)
                end = t + step
            self._run_to(end, courant_number)
            if getattr(self, "drifters", None) is not None:
                self.drift(step)
            t = end
        self.t = s0.t

    # ------------------------------------------------------------------
    # state transfer (E/MultiLevelOceanEnsemble.py:143-239)
    # ------------------------------------------------------------------
    def _groups(self):
        """Member ranges of the flat engine order: level 0, then per higher
        level the fine partners followed by the coarse partners."""
        out = [(0, int(self.Nes[0]))]
        a = int(self.Nes[0])
        for l_idx in range(1, self.numLevels):
            n = int(self.Nes[l_idx])
            out.append(((a, n), (a + n, n)))
            a += 2 * n
        return out

    def download(self, interior_domain_only=True):
        """State per level, (3, ny, nx, Ne); higher levels a [fine, coarse]
        pair (E/MultiLevelOceanEnsemble.py:143-170)."""
        def states(sims):
            return np.moveaxis(np.array([np.array(s.download(interior_domain_only=interior_domain_only))
                                         for s in sims]), 0, -1)
        out = [states(self.ML_ensemble[0])]
        for l_idx in range(1, self.numLevels):
            out.append([states(self.ML_ensemble[l_idx][0]), states(self.ML_ensemble[l_idx][1])])
        return out

    def downloadVelocities(self, interior_domain_only=True):
        """(u, v) = (hu, hv) / (eta + Hm) per level, (2, ny, nx, Ne)
        (E/MultiLevelOceanEnsemble.py:187-224)."""
        def vel(sims):
            _, Hm = sims[0].downloadBathymetry(interior_domain_only=interior_domain_only)
            out = []
            for s in sims:
                eta, hu, hv = s.download(interior_domain_only=interior_domain_only)
                out.append(np.array([hu / (eta + Hm), hv / (eta + Hm)]))
            return np.moveaxis(np.array(out), 0, -1)
        out = [vel(self.ML_ensemble[0])]
        for l_idx in range(1, self.numLevels):
            out.append([vel(self.ML_ensemble[l_idx][0]), vel(self.ML_ensemble[l_idx][1])])
        return out

    def upload(self, ML_state):
        """Interior states back into every member (E/MultiLevelOceanEnsemble.py:227-239)."""
        def put(sims, st):
            for e, s in enumerate(sims):
                s.upload(*np.pad(st[:, :, :, e], ((0, 0), (2, 2), (2, 2))))
        put(self.ML_ensemble[0], ML_state[0])
        for l_idx in range(1, self.numLevels):
            put(self.ML_ensemble[l_idx][0], ML_state[l_idx][0])
            put(self.ML_ensemble[l_idx][1], ML_state[l_idx][1])

    # ------------------------------------------------------------------
    # estimators (E/MultiLevelOceanEnsemble.py:242-267)
    # ------------------------------------------------------------------
    def estimate(self, func, **kwargs):
        """ML estimator of a statistic of (eta, hu, hv).  np.mean and np.var
        (with ddof) run on the device: one pass over each level group's
        members plus one launch assembling the estimate on the finest grid;
        any other func runs on the downloaded states."""
        stat = _device_statistic(func, kwargs)
        if stat is not None:
            return self._device_estimate("state", *stat)
        return self._estimate_pure(self.download(), func, **kwargs)

    def estimateVelocity(self, func, **kwargs):
        """ML estimator of a statistic of (u, v) = (hu, hv) / (eta + Hm)."""
        stat = _device_statistic(func, kwargs)
        if stat is not None:
            return self._device_estimate("velocity", *stat)
        return self._estimate_pure(self.downloadVelocities(), func, **kwargs)

    def _estimate_pure(self, ML_state, func, **kwargs):
        """The estimator on downloaded states (E/MultiLevelOceanEnsemble.py:258-267):
        level-0 statistic plus the fine-coarse differences, on the finest grid."""
        L = self.numLevels
        est = np.zeros(ML_state[-1][0].shape[:-1])
        est += func(ML_state[0], axis=-1, **kwargs).repeat(2 ** (L - 1), 1).repeat(2 ** (L - 1), 2)
        for l_idx in range(1, L):
            d = func(ML_state[l_idx][0], axis=-1, **kwargs) - \
                func(ML_state[l_idx][1], axis=-1, **kwargs).repeat(2, 1).repeat(2, 2)
            est += d.repeat(2 ** (L - l_idx - 1), 1).repeat(2 ** (L - l_idx - 1), 2)
        return est

    def _device_estimate(self, quantity, which, ddof):
        eng = self.engine
        groups = self._groups()
        bufs = []
        try:
            def stat(first, n):
                m, v = eng.moments(first, n, quantity=quantity, ddof=ddof, mean=which == "mean",
                                   var=which == "var", download=False)
                b = m if which == "mean" else v
                bufs.append(b)
                return b.ptr
            L = self.numLevels
            fine = (ctypes.c_void_p * L)()
            coarse = (ctypes.c_void_p * L)()
            fine[0] = stat(*groups[0])
            for l_idx in range(1, L):
                fine[l_idx] = stat(*groups[l_idx][0])
                coarse[l_idx] = stat(*groups[l_idx][1])
            nx = np.ascontiguousarray(self.nxs, dtype=np.int32)
            ny = np.ascontiguousarray(self.nys, dtype=np.int32)
            planes = 3 if quantity == "state" else 2
            out_shape = (planes, int(ny[-1]), int(nx[-1]))
            out = Common.DevicePtr(8 * int(np.prod(out_shape)))
            bufs.append(out)
            _lib.call("goc_ml_combine", L, fine, coarse, nx.ctypes.data, ny.ctypes.data, planes, out.ptr,
                      eng.stream.handle)
            eng.kernels_launched += 1
            return eng._download(out, out_shape, np.float64)
        finally:
            for b in bufs:
                b.free()

    # ------------------------------------------------------------------
    # drifters (E/MultiLevelOceanEnsemble.py:450-489)
    # ------------------------------------------------------------------
    def attachDrifters(self, drifterEnsembleSize, numDrifters=None, drifterPositions=None, drift_dt=60,
                       drift_sensitivity=1.0):
        """Drifters that move with the multi-level estimates of the mean and
        variance of the velocity (MLDrifterCollection): `numDrifters` unique
        drifters (or one per row of drifterPositions), each with
        drifterEnsembleSize realisations, moved every drift_dt seconds of
        stepToObservation; their positions are recorded now."""
        from ..drifters.MLDrifterCollection import DriftTrajectory, MLDrifterCollection
        assert numDrifters is not None or drifterPositions is not None, \
            "Please provide either numDrifters or drifterPositions"
        assert numDrifters is None or drifterPositions is None, \
            "Both numDrifters and drifterPositions are given, please provide only one of them"
        if numDrifters is None:
            numDrifters = np.asarray(drifterPositions).shape[0]
        self.drifters = MLDrifterCollection(numDrifters, drifterEnsembleSize,
                                            boundaryConditions=self.ML_ensemble[0][0].boundary_conditions,
                                            domain_size_x=self.nxs[0] * self.dxs[0],
                                            domain_size_y=self.nys[0] * self.dys[0])
        if drifterPositions is not None:
            self.drifters.setDrifterPositions(np.asarray(drifterPositions))
        mts = self.ML_ensemble[0][0].model_time_step
        assert drift_dt >= mts, "We require that the drift_dt (" + str(drift_dt) + \
            ") is larger than the model time step (" + str(mts) + ")"
        self.drift_dt = drift_dt
        self.drift_sensitivity = drift_sensitivity
        self.drifterEnsembeSize = drifterEnsembleSize
        self.driftTrajectory = [DriftTrajectory() for _ in range(drifterEnsembleSize)]
        self.registerDrifterPositions()

    def drift(self, dt):
        """Move the drifters by dt with the multi-level mean velocity, the
        variance (ddof 1) scaling their random walk (both estimated on the
        device on the finest grid)."""
        assert self.drifters is not None, "No drifters found. Can't call drift() before attachDrifters(...)"
        mean = self.estimateVelocity(np.mean)
        var = self.estimateVelocity(np.var, ddof=1)
        self.drifters.drift(mean[0], mean[1], self.dxs[-1], self.dys[-1], dt=dt, sensitivity=self.drift_sensitivity,
                            u_var=var[0], v_var=var[1])

    def registerDrifterPositions(self):
        """Record the current positions of every realisation."""
        assert self.drifters is not None, "There are no drifters in this ensemble"
        assert self.driftTrajectory is not None, \
            "Something went wrong. The ensemble has drifters but no observation objects..."
        for e in range(self.drifterEnsembeSize):
            self.driftTrajectory[e].add_observation_from_mldrifters(self.t, self.drifters, e)

    def saveDriftTrajectoriesToFile(self, path, filename_prefix):
        import os
        for e in range(self.drifterEnsembeSize):
            self.driftTrajectory[e].to_pickle(os.path.join(path, filename_prefix + str(e).zfill(4) + ".pickle"))

    def cleanUp(self):
        self.engine.release()
        for s in self.members:
            s.cleanUp(do_gc=False)
