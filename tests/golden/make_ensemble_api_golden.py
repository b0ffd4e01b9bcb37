"""Golden vectors for the ensemble API that the data-assimilation layer
calls, produced by the reference's own Python code.

On seeded inputs held by stand-in objects, this calls the reference's
``BaseOceanStateEnsemble.getGaussianWeight`` (2-D and 1-D innovations,
normalised or not, one particle inactive) and ``getInnovationNorms``
(E/BaseOceanStateEnsemble.py:222-290), and ``OceanNoiseEnsemble``'s
``getCauchyWeight``, ``downloadEnsembleStatisticalFields``,
``getEnsembleVarAndRMSEUnderDrifter`` and ``findLargestPossibleTimeStep``
(E/OceanNoiseEnsemble.py:571-775).  Only NumPy code of the reference runs;
PyCUDA, matplotlib and the other absent modules are inert stubs, and the
NumPy aliases the reference uses (np.infty, np.int) are restored.  Writes
``ensemble_api_reference.npz`` next to this file.

Usage:  python tests/golden/make_ensemble_api_golden.py REFERENCE_ROOT (or $GPUOCEAN_REFERENCE)
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
    from gpuocean.ensembles import BaseOceanStateEnsemble, OceanNoiseEnsemble
    return BaseOceanStateEnsemble.BaseOceanStateEnsemble, OceanNoiseEnsemble.OceanNoiseEnsemble


class StandInSim:
    def __init__(self, state, Hi):
        self.state = np.asarray(state, dtype=np.float32)   # with 2 ghost cells
        self.Hi = np.asarray(Hi, dtype=np.float32)

    def download(self, interior_domain_only=False):
        s = self.state[:, 2:-2, 2:-2] if interior_domain_only else self.state
        return s[0].copy(), s[1].copy(), s[2].copy()

    def downloadBathymetry(self, interior_domain_only=False):
        return self.Hi.copy(), None


def stand_in(cls, n, **attrs):
    ens = object.__new__(type("StandIn" + cls.__name__, (cls,), {"cleanUp": lambda self: None,
                                                                  "__del__": lambda self: None}))
    ens.numParticles = n
    ens.particlesActive = [True] * n
    for k, v in attrs.items():
        setattr(ens, k, v)
    return ens


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GPUOCEAN_REFERENCE")
    if not root:
        sys.exit("usage: %s REFERENCE_ROOT (or set GPUOCEAN_REFERENCE)" % sys.argv[0])
    Base, Noise = import_reference(root)
    # NumPy 2 removed the aliases np.infty and np.int that the reference uses
    for alias, value in (("infty", np.inf), ("int", int)):
        if not hasattr(np, alias):
            setattr(np, alias, value)
    rng = np.random.default_rng(31)
    out = {}

    # weights and innovation norms
    n, D = 9, 4
    var = 0.37
    cov = np.array([[var, 0.05], [0.05, 1.3 * var]])
    inn = rng.standard_normal((n, D, 2)) * 0.8
    inn1 = rng.standard_normal(n)
    ens = stand_in(Base, n, observation_cov=cov, observation_cov_inverse=np.linalg.inv(cov),
                   driftersPerOceanModel=D)
    ens.particlesActive[3] = False
    ens.getInnovations = lambda observations=None: inn
    out.update(w_cov=cov, w_innovations=inn, w_innovations_1d=inn1, w_active=np.array(ens.particlesActive))
    out["w_gauss"] = ens.getGaussianWeight(innovations=inn)
    out["w_gauss_raw"] = ens.getGaussianWeight(innovations=inn, normalize=False)
    out["w_gauss_scaled"] = ens.getGaussianWeight(innovations=inn, R_scale=2.5)
    out["w_gauss_1d"] = ens.getGaussianWeight(innovations=inn1)
    out["w_gauss_1d_raw"] = ens.getGaussianWeight(innovations=inn1, normalize=False)
    out["w_innovation_norms"] = ens.getInnovationNorms()
    dist = np.abs(rng.standard_normal((n, D))) * 900.0
    noise = stand_in(Noise, n, observation_variance=(5 * 1000.0) ** 2)
    out.update(w_distances=dist, w_obs_var=np.float64(noise.observation_variance))
    out["w_cauchy"] = noise.getCauchyWeight(distances=dist)
    out["w_cauchy_raw"] = noise.getCauchyWeight(distances=dist, normalize=False)

    # statistics of an ensemble with a truth
    n, ny, nx, dx, dy, g = 6, 10, 12, 800.0, 700.0, 9.81
    Hi = (40.0 + 4.0 * rng.random((ny + 5, nx + 5))).astype(np.float32)

    def state():
        eta = 0.2 * rng.standard_normal((ny + 4, nx + 4))
        hu = 3.0 * rng.standard_normal((ny + 4, nx + 4))
        hv = 3.0 * rng.standard_normal((ny + 4, nx + 4))
        return np.stack([eta, hu, hv]).astype(np.float32)

    states = np.stack([state() for _ in range(n + 1)])
    sims = [StandInSim(s, Hi) for s in states]
    pos = np.array([[5.3 * dx, 6.6 * dy], [1.2 * dx, 2.5 * dy]])
    ens = stand_in(Noise, n, particles=sims, obs_index=n, dx=dx, dy=dy, g=g,
                   varianceUnderDrifter_eta=[], varianceUnderDrifter_hu=[], varianceUnderDrifter_hv=[],
                   rmseUnderDrifter_eta=[], rmseUnderDrifter_hu=[], rmseUnderDrifter_hv=[],
                   rmseMeanUnderDrifter_eta=[], rmseMeanUnderDrifter_hu=[], rmseMeanUnderDrifter_hv=[],
                   rmseWeightedUnderDrifter_eta=[], rmseWeightedUnderDrifter_hu=[],
                   rmseWeightedUnderDrifter_hv=[], rUnderDrifter_eta=[], rUnderDrifter_hu=[],
                   rUnderDrifter_hv=[], tArray=[])
    ens.observeTrueState = lambda: np.concatenate([pos, np.zeros((2, 2))], axis=1)
    out.update(s_states=states, s_Hi=Hi, s_dx=dx, s_dy=dy, s_g=g, s_pos=pos)
    fields = ens.downloadEnsembleStatisticalFields()
    out["s_fields"] = np.array(fields)
    ens.getEnsembleVarAndRMSEUnderDrifter(120.0)
    keys = []
    for name in ("varianceUnderDrifter_", "rmseUnderDrifter_", "rmseMeanUnderDrifter_", "rmseWeightedUnderDrifter_",
                 "rUnderDrifter_"):
        for q in ("eta", "hu", "hv"):
            keys.append(getattr(ens, name + q)[-1])
    out["s_under_drifter"] = np.array(keys, dtype=np.float64)
    out["s_largest_dt"] = np.float64(ens.findLargestPossibleTimeStep())
    path = os.path.join(HERE, "ensemble_api_reference.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, {k: np.shape(v) for k, v in out.items()})


if __name__ == "__main__":
    main()
