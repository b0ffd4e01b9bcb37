"""The host drifter collections (CPUDrifterCollection, MLDrifterCollection)
against trajectories of the reference's own classes on the same inputs and
the same seeds of numpy's global generator
(``tests/golden/make_ml_drifters_golden.py``)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from ml_drifter_cases import CASE  # noqa: E402

GOLD = np.load(os.path.join(HERE, "golden", "ml_drifters_reference.npz"))


def _bc(*b):
    from gpuocean_gb300.utils import Common
    return Common.BoundaryConditions(*b)


def _close(a, b):
    # the reference steps drifters one at a time in scalar float arithmetic;
    # these collections step them together: agreement to float64 rounding of
    # positions of ~1e4 m
    np.testing.assert_allclose(a, b, rtol=0, atol=1e-7)


def test_cpu_collection_plain_drift():
    from gpuocean_gb300.drifters.CPUDrifterCollection import CPUDrifterCollection
    c = CASE()
    np.random.seed(c["seed"])
    d = CPUDrifterCollection(c["n"], boundaryConditions=_bc(1, 1, 1, 1), domain_size_x=c["Lx"], domain_size_y=c["Ly"])
    d.setDrifterPositions(c["pos"])
    d.setObservationPosition(c["obs"])
    for k in range(3):
        d.drift(c["eta"], c["hu"], c["hv"], c["Hm"], c["dx"], c["dy"], c["dt"], x_zero_ref=2, y_zero_ref=2)
        _close(d.positions, GOLD[f"plain_{k}"])


def test_cpu_collection_random_walk():
    from gpuocean_gb300.drifters.CPUDrifterCollection import CPUDrifterCollection
    c = CASE()
    for tag, uv, vv in (("scalar", 0.04, 0.09), ("field", c["u_var"], c["v_var"])):
        np.random.seed(c["seed"] + 1)
        d = CPUDrifterCollection(c["n"], boundaryConditions=_bc(2, 2, 2, 2), domain_size_x=c["Lx"],
                                 domain_size_y=c["Ly"])
        d.setDrifterPositions(c["pos"])
        d.setObservationPosition(c["obs"])
        for k in range(3):
            d.driftFromVelocities(c["u"], c["v"], c["dx"], c["dy"], c["dt"], u_var=uv, v_var=vv)
            _close(d.positions, GOLD[f"walk_{tag}_{k}"])


def test_ml_collection_biased_and_unbiased_walk():
    from gpuocean_gb300.drifters.MLDrifterCollection import MLDrifterCollection
    c = CASE()
    for biased in (True, False):
        np.random.seed(c["seed"] + 2)
        d = MLDrifterCollection(c["n_unique"], c["ens"], boundaryConditions=_bc(2, 2, 2, 2), domain_size_x=c["Lx"],
                                domain_size_y=c["Ly"], use_biased_walk=biased)
        d.setDrifterPositions(c["unique_pos"])
        for k in range(3):
            d.drift(c["u"], c["v"], c["dx"], c["dy"], c["dt"], u_var=c["u_var"], v_var=c["v_var"])
            _close(d.positions, GOLD[f"ml_{int(biased)}_{k}"])
        _close(d.getDrifterPositionsForEnsembleMember(1), GOLD[f"ml_{int(biased)}_member1"])
        _close(d.getDrifterPositionsForDrifter(2), GOLD[f"ml_{int(biased)}_drifter2"])


def test_drift_trajectory_records_and_splits_paths():
    from gpuocean_gb300.drifters.MLDrifterCollection import DriftTrajectory, MLDrifterCollection
    c = CASE()
    np.random.seed(1)
    d = MLDrifterCollection(c["n_unique"], c["ens"], boundaryConditions=_bc(2, 2, 2, 2), domain_size_x=c["Lx"],
                            domain_size_y=c["Ly"])
    d.setDrifterPositions(c["unique_pos"])
    tr = DriftTrajectory(jump_limit=0.5 * c["Lx"])
    for k in range(4):
        tr.add_observation_from_mldrifters(60.0 * k, d, 1)
        d.drift(c["u"], c["v"], c["dx"], c["dy"], c["dt"], u_var=c["u_var"], v_var=c["v_var"])
    assert tr.get_num_observations() == 4 and tr.get_num_drifters() == c["n_unique"]
    assert list(tr.get_observation_times()) == [60, 120, 180]
    np.testing.assert_array_equal(tr.get_drifter_position(120.0), tr.positions[2])
    paths = tr.get_drifter_path(1, 0, 180, in_km=False)
    assert sum(len(p) for p in paths) == 4
