"""Multi-level ensemble (drop-in for ``ensembles/MultiLevelOceanEnsemble.py:32-518``).

Level 0 is a list of simulators; every higher level is a pair of equally
long lists (fine partner, coarse partner).  All simulators of all levels -
grids of different sizes - advance in one batched launch per RK2 step over
the member/tile work queue.
"""
from __future__ import annotations

import numpy as np

from .BatchedEnsemble import BatchedEnsemble


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
        self.engine = BatchedEnsemble(self.members)
        if all(s.model_error is not None for s in self.members):
            self.engine.set_noise([s.model_error for s in self.members], rng_seed=rng_seed)

    def _flat(self):
        out = list(self.ML_ensemble[0])
        for l_idx in range(1, self.numLevels):
            out += list(self.ML_ensemble[l_idx][0]) + list(self.ML_ensemble[l_idx][1])
        return out

    def step(self, t, apply_stochastic_term=True, **kwargs):
        """Every simulator of every level advances by t."""
        self.engine.step(t, apply_stochastic_term=apply_stochastic_term, noise_cadence="step")
        self.t = self.ML_ensemble[0][0].t

    def stepToObservation(self, obs_time, courant_number=0.8):
        """Advance to obs_time with model error every model_time_step."""
        s0 = self.ML_ensemble[0][0]
        mts = s0.model_time_step
        self.engine.updateDt(courant_number=courant_number)
        n_blocks = int(round((obs_time - s0.t) / mts))
        for b in range(n_blocks):
            self.engine.step(mts, apply_stochastic_term=self.engine._noise is not None)
            if (b + 1) % 5 == 0:
                self.engine.updateDt(courant_number=courant_number)
        self.t = s0.t

    def download(self, interior_domain_only=True):
        """State per level: level 0 (Ne, 3, ny, nx); higher levels a pair."""
        def states(sims):
            return np.array([np.array(s.download(interior_domain_only=interior_domain_only)) for s in sims])
        out = [states(self.ML_ensemble[0])]
        for l_idx in range(1, self.numLevels):
            out.append([states(self.ML_ensemble[l_idx][0]), states(self.ML_ensemble[l_idx][1])])
        return out

    def estimate(self, func, **kwargs):
        """Multi-level estimator: func over level 0 plus the fine-coarse
        differences of the higher levels, on the finest grid."""
        state = self.download()
        est = func(state[0], axis=0, **kwargs)
        for l_idx in range(1, self.numLevels):
            fine = func(state[l_idx][0], axis=0, **kwargs)
            coarse = func(state[l_idx][1], axis=0, **kwargs)
            ry = fine.shape[-2] // est.shape[-2]
            rx = fine.shape[-1] // est.shape[-1]
            est = np.repeat(np.repeat(est, ry, axis=-2), rx, axis=-1)
            ry = fine.shape[-2] // coarse.shape[-2]
            rx = fine.shape[-1] // coarse.shape[-1]
            est = est + fine - np.repeat(np.repeat(coarse, ry, axis=-2), rx, axis=-1)
        return est

    def cleanUp(self):
        self.engine.release()
        for s in self.members:
            s.cleanUp(do_gc=False)
