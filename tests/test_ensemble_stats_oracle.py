"""The observation / ensemble-statistics oracle against vectors produced by the
reference's own Python code (tests/golden/make_ensemble_stats_golden.py), and
the host logic of the multi-level estimator.  CPU only."""
import os

import numpy as np
import pytest

from oracle import ensemble_stats_oracle as eso

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ensemble_stats_reference.npz")


@pytest.fixture(scope="module")
def g():
    return np.load(GOLDEN)


def rel_close(a, b, rtol):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = max(np.abs(b).max(), 1e-30)
    return np.abs(a - b).max() <= rtol * scale


def test_moments_match_reference_estimate(g):
    st = g["base_states"]
    mean, var = eso.moments(st)
    _, var1 = eso.moments(st, ddof=1)
    # the reference reduces float32 arrays in float32
    assert rel_close(mean, g["base_mean"], 1e-6)
    assert rel_close(var, g["base_var"], 1e-6)
    assert rel_close(var1, g["base_var_ddof1"], 1e-6)


def test_desingularised_velocity_moments(g):
    vel = eso.velocities(g["base_states"], g["base_Hm"], eps=1e-5)
    mean, var = eso.moments(vel)
    assert rel_close(mean, g["base_vel_mean"], 1e-6)
    assert rel_close(var, g["base_vel_var"], 1e-6)


def test_observe_particles_match_reference(g):
    obs = g["base_observations"]
    st = g["base_states"]
    dx, dy = float(g["base_dx"]), float(g["base_dy"])
    np.testing.assert_array_equal(eso.observe_particles(st, obs, dx, dy), g["base_observed"])
    inn = eso.observe_particles(st, obs, dx, dy, innovation=True, mean_depth=60.0)
    np.testing.assert_allclose(inn, g["base_innovation"], rtol=1e-12, atol=1e-12)


def test_kernel_restatement_agrees_with_cpu_path(g):
    """observeUnderlyingFlow on ghost-padded arrays (zero reference cell 2)
    selects the cells the CPU path selects for these positions."""
    obs = g["base_observations"]
    dx, dy = float(g["base_dx"]), float(g["base_dy"])
    for p, st in enumerate(g["base_states"]):
        pad = [np.pad(a, 2) for a in st]
        got = eso.observe_underlying_flow(pad[1], pad[2], obs[:, :2], dx, dy)
        np.testing.assert_array_equal(got, g["base_observed"][p])


def _ml_stats(g, fn):
    lv = [fn(g["ml_l0_states"], g["ml_l0_Hm"])]
    for l in (1, 2):
        lv.append((fn(g[f"ml_l{l}_fine_states"], g[f"ml_l{l}_fine_Hm"]),
                   fn(g[f"ml_l{l}_coarse_states"], g[f"ml_l{l}_coarse_Hm"])))
    return lv


@pytest.mark.parametrize("which", ["mean", "var1"])
@pytest.mark.parametrize("quantity", ["state", "velocity"])
def test_ml_estimate_matches_reference(g, which, quantity):
    def fn(st, Hm):
        v = st if quantity == "state" else eso.velocities(st, Hm)
        m, v1 = eso.moments(v, ddof=1)
        return m if which == "mean" else v1
    est = eso.ml_estimate(_ml_stats(g, fn))
    key = {("state", "mean"): "ml_mean", ("state", "var1"): "ml_var_ddof1",
           ("velocity", "mean"): "ml_vel_mean", ("velocity", "var1"): "ml_vel_var_ddof1"}[(quantity, which)]
    assert est.shape == g[key].shape
    assert rel_close(est, g[key], 2e-6)


def test_ml_estimate_float32_terms_reproduce_reference_bitwise(g):
    """With the same float32 level statistics (NumPy's), the estimator's
    float32 differences and float64 accumulation give the reference's
    result exactly - the arithmetic the device kernel uses."""
    def fn(st, Hm):
        return np.mean(np.moveaxis(st, 0, -1), axis=-1)
    est = eso.ml_estimate(_ml_stats(g, fn))
    np.testing.assert_array_equal(est, g["ml_mean"])
