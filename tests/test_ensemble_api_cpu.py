"""The host-side ensemble API (weights, innovation norms, statistics): the
oracle's restatement against vectors from the reference's own methods, and
the product's host code against the same vectors."""
import os

import numpy as np
import pytest

from oracle import ensemble_api_oracle as oa

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "ensemble_api_reference.npz"))


def test_oracle_weights_match_reference():
    g = GOLD
    act = g["w_active"]
    np.testing.assert_allclose(oa.gaussian_weight(g["w_innovations"], g["w_cov"], act), g["w_gauss"], rtol=1e-12)
    np.testing.assert_allclose(oa.gaussian_weight(g["w_innovations"], g["w_cov"], act, normalize=False),
                               g["w_gauss_raw"], rtol=1e-12)
    np.testing.assert_allclose(oa.gaussian_weight(g["w_innovations"], g["w_cov"], act, R_scale=2.5),
                               g["w_gauss_scaled"], rtol=1e-12)
    np.testing.assert_allclose(oa.gaussian_weight(g["w_innovations_1d"], g["w_cov"], act), g["w_gauss_1d"],
                               rtol=1e-12)
    np.testing.assert_allclose(oa.gaussian_weight(g["w_innovations_1d"], g["w_cov"], act, normalize=False),
                               g["w_gauss_1d_raw"], rtol=1e-12)
    np.testing.assert_allclose(oa.innovation_norms(g["w_innovations"]), g["w_innovation_norms"], rtol=1e-12)
    np.testing.assert_allclose(oa.cauchy_weight(g["w_distances"], float(g["w_obs_var"])), g["w_cauchy"], rtol=1e-12)
    np.testing.assert_allclose(oa.cauchy_weight(g["w_distances"], float(g["w_obs_var"]), normalize=False),
                               g["w_cauchy_raw"], rtol=1e-12)


def test_oracle_statistics_match_reference():
    g = GOLD
    st = g["s_states"]                       # particles 0..n-1, truth last, with ghost cells
    inner = st[:, :, 2:-2, 2:-2]
    # the reference accumulates in float32: agreement to float32 rounding
    np.testing.assert_allclose(oa.statistical_fields(inner[-1], inner[:-1]), g["s_fields"], rtol=2e-5, atol=1e-6)
    dx, dy = float(g["s_dx"]), float(g["s_dy"])
    ix, iy = int(np.floor(g["s_pos"][0, 0] / dx)), int(np.floor(g["s_pos"][0, 1] / dy))
    vals = inner[:, :, iy, ix]
    np.testing.assert_allclose(oa.under_drifter(vals[-1], vals[:-1]), g["s_under_drifter"], rtol=1e-5)
    np.testing.assert_allclose(oa.largest_timestep(st, g["s_Hi"], float(g["s_g"]), dx, dy), g["s_largest_dt"],
                               rtol=1e-6)


class _Weights:
    """The product's base class on the golden inputs (host code only)."""

    def __new__(cls):
        from gpuocean_gb300.ensembles.BaseOceanStateEnsemble import BaseOceanStateEnsemble

        class StandIn(BaseOceanStateEnsemble):
            cleanUp = resample = step_truth = step_particles = observeTrueDrifters = lambda *a, **k: None
            observeTrueState = downloadTrueOceanState = lambda *a, **k: None

            def observeParticles(self, gpu=False, innovation=False, observations=None):
                return GOLD["w_innovations"]

        e = StandIn()
        e.numParticles = len(GOLD["w_active"])
        e.particlesActive = [bool(x) for x in GOLD["w_active"]]
        e.observation_cov = GOLD["w_cov"]
        e.observation_cov_inverse = np.linalg.inv(GOLD["w_cov"])
        e.driftersPerOceanModel = GOLD["w_innovations"].shape[1]
        return e


def test_product_weights_match_reference():
    g = GOLD
    e = _Weights()
    np.testing.assert_allclose(e.getGaussianWeight(), g["w_gauss"], rtol=1e-12)
    np.testing.assert_allclose(e.getGaussianWeight(normalize=False), g["w_gauss_raw"], rtol=1e-12)
    np.testing.assert_allclose(e.getGaussianWeight(R_scale=2.5), g["w_gauss_scaled"], rtol=1e-12)
    np.testing.assert_allclose(e.getGaussianWeight(innovations=g["w_innovations_1d"]), g["w_gauss_1d"], rtol=1e-12)
    np.testing.assert_allclose(e.getGaussianWeight(innovations=g["w_innovations_1d"], normalize=False),
                               g["w_gauss_1d_raw"], rtol=1e-12)
    np.testing.assert_allclose(e.getInnovationNorms(), g["w_innovation_norms"], rtol=1e-12)
    assert e.getGaussianWeight()[3] == 0.0


def test_product_cauchy_weight_matches_reference():
    from gpuocean_gb300.ensembles.OceanNoiseEnsemble import OceanNoiseEnsemble
    e = object.__new__(OceanNoiseEnsemble)
    e.observation_variance = float(GOLD["w_obs_var"])
    e.engine = None
    np.testing.assert_allclose(e.getCauchyWeight(distances=GOLD["w_distances"]), GOLD["w_cauchy"], rtol=1e-12)
    np.testing.assert_allclose(e.getCauchyWeight(distances=GOLD["w_distances"], normalize=False),
                               GOLD["w_cauchy_raw"], rtol=1e-12)
