"""Golden vectors for the observation operator and the ensemble statistics,
produced by the reference's own Python code.

Calls, on seeded float32 member states held by stand-in simulators (objects
with the ``download`` / ``downloadBathymetry`` methods and grid attributes the
reference reads):

* ``BaseOceanStateEnsemble.estimate`` and ``estimateVelocity`` with np.mean
  and np.var, and ``observeParticles`` (CPU path, with and without
  innovation) - E/BaseOceanStateEnsemble.py:79-176;
* ``MultiLevelOceanEnsemble.estimate`` and ``estimateVelocity`` with np.mean
  and np.var(ddof=1) on three levels - E/MultiLevelOceanEnsemble.py:143-267.

PyCUDA, matplotlib and pandas are absent here and are replaced by inert
stubs; only NumPy code of the reference runs.  ``observeParticles`` calls
``np.int``, which NumPy 2 removed; it is aliased to ``int`` while the script
runs.  Writes ``ensemble_stats_reference.npz`` next to this file.

Usage:  python tests/golden/make_ensemble_stats_golden.py REFERENCE_ROOT (or $GPUOCEAN_REFERENCE)
"""
import os
import sys
from unittest import mock

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def import_reference(root):
    sys.dont_write_bytecode = True   # the checkout is read-only: no __pycache__ inside it
    for name in ["pycuda", "pycuda.driver", "pycuda.gpuarray", "pycuda.compiler", "pycuda.curandom",
                 "pycuda.autoinit", "matplotlib", "matplotlib.pyplot", "matplotlib.gridspec",
                 "matplotlib.animation", "matplotlib.colors", "netCDF4", "mpi4py", "pandas"]:
        sys.modules.setdefault(name, mock.MagicMock())
    sys.path.insert(0, os.path.join(root, "src"))
    from gpuocean.ensembles import BaseOceanStateEnsemble, MultiLevelOceanEnsemble
    from gpuocean.dataassimilation import DataAssimilationUtils
    return BaseOceanStateEnsemble.BaseOceanStateEnsemble, MultiLevelOceanEnsemble.MultiLevelOceanEnsemble, \
        DataAssimilationUtils


class StandInSim:
    """What the reference's ensembles read from a simulator."""

    def __init__(self, state, Hm, dx, dy):
        self.state = np.asarray(state, dtype=np.float32)
        self.Hm = np.asarray(Hm, dtype=np.float32)
        self.ny, self.nx = self.Hm.shape
        self.dx, self.dy = np.float32(dx), np.float32(dy)
        self.t = 0.0
        self.boundary_conditions = None

    def download(self, interior_domain_only=False):
        return self.state[0], self.state[1], self.state[2]

    def downloadBathymetry(self, interior_domain_only=False):
        return None, self.Hm

    def cleanUp(self, do_gc=True):
        pass


def member_states(rng, n, ny, nx, Hm, nearly_dry=False):
    eta = 0.1 * rng.standard_normal((n, ny, nx))
    if nearly_dry:   # two nearly dry cells, for the desingularised velocities
        eta[:, 0, :2] = -Hm[0, :2] + np.array([3e-6, -2e-6])
    hu = 4.0 * rng.standard_normal((n, ny, nx))
    hv = 4.0 * rng.standard_normal((n, ny, nx))
    return np.stack([eta, hu, hv], axis=1).astype(np.float32)


def base_case(Base, dautils):
    rng = np.random.default_rng(11)
    n, ny, nx, dx, dy = 7, 9, 11, 250.0, 300.0
    Hm = (60.0 + 5.0 * rng.standard_normal((ny, nx))).astype(np.float32)
    Hm[0, :2] = 1e-3
    states = member_states(rng, n, ny, nx, Hm, nearly_dry=True)
    D = 5
    pos = np.stack([rng.uniform(0, nx * dx, D), rng.uniform(0, ny * dy, D)], axis=1).astype(np.float32)
    truth = rng.standard_normal((2, D))
    observations = np.concatenate([pos, truth.T], axis=1)

    cls = type("StandInEnsemble", (Base,), {"cleanUp": lambda self: None})
    ens = object.__new__(cls)
    ens.particles = [StandInSim(s, Hm, dx, dy) for s in states]
    ens.particlesActive = [True] * n
    ens.numParticles = n
    ens.driftersPerOceanModel = D
    ens.observation_type = dautils.ObservationType.UnderlyingFlow
    ens.dx, ens.dy = np.float32(dx), np.float32(dy)
    ens.compensate_for_eta = True
    ens.mean_depth = 60.0
    ens.getNumParticles = lambda: n
    ens.getNumDrifters = lambda: D
    ens.downloadParticleOceanState = lambda p: ens.particles[p].download(interior_domain_only=True)

    out = dict(base_states=states, base_Hm=Hm, base_dx=dx, base_dy=dy, base_observations=observations)
    out["base_mean"] = ens.estimate(np.mean)
    out["base_var"] = ens.estimate(np.var)
    out["base_var_ddof1"] = ens.estimate(np.var, ddof=1)
    out["base_vel_mean"] = ens.estimateVelocity(np.mean)
    out["base_vel_var"] = ens.estimateVelocity(np.var)
    had = hasattr(np, "int")
    np.int = int
    try:
        out["base_observed"] = ens.observeParticles(observations=observations)
        out["base_innovation"] = ens.observeParticles(innovation=True, observations=observations)
    finally:
        if not had:
            del np.int
    return out


def ml_case(ML):
    rng = np.random.default_rng(12)
    Lx, Ly = 24 * 400.0, 16 * 500.0
    grids = [(4, 6), (8, 12), (16, 24)]
    Nes = [5, 4, 3]

    def level(ny, nx, n):
        Hm = (60.0 + 5.0 * rng.standard_normal((ny, nx))).astype(np.float32)
        st = member_states(rng, n, ny, nx, Hm)
        return st, Hm, [StandInSim(s, Hm, Lx / nx, Ly / ny) for s in st]

    out = {}
    s0, h0, sims0 = level(*grids[0], Nes[0])
    out["ml_l0_states"], out["ml_l0_Hm"] = s0, h0
    ML_ensemble = [sims0]
    for l in (1, 2):
        sf, hf, simsf = level(*grids[l], Nes[l])
        sc, hc, simsc = level(*grids[l - 1], Nes[l])
        out[f"ml_l{l}_fine_states"], out[f"ml_l{l}_fine_Hm"] = sf, hf
        out[f"ml_l{l}_coarse_states"], out[f"ml_l{l}_coarse_Hm"] = sc, hc
        ML_ensemble.append([simsf, simsc])
    ens = ML(ML_ensemble)
    out["ml_mean"] = ens.estimate(np.mean)
    out["ml_var_ddof1"] = ens.estimate(np.var, ddof=1)
    out["ml_vel_mean"] = ens.estimateVelocity(np.mean)
    out["ml_vel_var_ddof1"] = ens.estimateVelocity(np.var, ddof=1)
    return out


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GPUOCEAN_REFERENCE")
    if not root:
        sys.exit("usage: %s REFERENCE_ROOT (or set GPUOCEAN_REFERENCE)" % sys.argv[0])
    Base, ML, dautils = import_reference(root)
    out = {}
    out.update(base_case(Base, dautils))
    out.update(ml_case(ML))
    path = os.path.join(HERE, "ensemble_stats_reference.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, {k: np.shape(v) for k, v in out.items()})


if __name__ == "__main__":
    main()
