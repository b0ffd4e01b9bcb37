"""The FP64 oracle against the reference's own CDKLM16 regression vectors.

The vectors (test/timestep50 of the reference, converted by
tests/golden/make_timestep50.py) are float32 GPU results of the reference
after 50 s (56 RK2 steps) on a 50 x 70 grid.  The reference's tolerance is
max relative difference < 5e-4 (assertAlmostEqual(places=3)); the oracle
agrees to 1e-4.
"""
import os

import numpy as np
import pytest

import cases
from oracle.cdklm16_oracle import BC, OracleCDKLM16, bathymetry_init, max_dt_f32

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "cdklm16_timestep50.npz"))


def run_oracle(name, t_end=cases.T_END, **kw):
    c = cases.make_case(name)
    sim = OracleCDKLM16(c["eta0"], c["hu0"], c["hv0"], c["H"], c["nx"], c["ny"], c["dx"], c["dy"], c["dt"],
                        c["g"], c["f"], c["r"], coriolis_beta=c["coriolis_beta"],
                        boundary_conditions=BC(*c["bc"]), **kw)
    sim.step(t_end)
    return c, sim


@pytest.mark.parametrize("name", list(cases.CASES))
def test_oracle_matches_reference_golden(name):
    c, sim = run_oracle(name)
    assert sim.num_iterations == 56
    eta, hu, hv = sim.download(interior_domain_only=True)
    k = c["golden"]
    for a, f in ((eta, "eta"), (hu, "u"), (hv, "v")):
        assert cases.rel_max_diff(a, GOLD[k + "/" + f]) < 1.5e-4, (name, f)


def test_golden_fixture_shapes():
    assert len(GOLD.files) == 36
    for k in GOLD.files:
        assert GOLD[k].shape == (70, 50) and GOLD[k].dtype == np.float32


def test_bathymetry_periodic_and_closed():
    rng = np.random.default_rng(0)
    nx, ny = 9, 7
    H = rng.uniform(5, 10, size=(ny + 5, nx + 5)).astype(np.float32)
    Hi, Hm = bathymetry_init(H, nx, ny, BC(2, 2, 2, 2))
    assert np.array_equal(Hi[0:2], Hi[ny:ny + 2]) and np.array_equal(Hi[:, nx + 2:], Hi[:, 2:5])
    Hi, Hm = bathymetry_init(H, nx, ny, BC(1, 1, 1, 1))
    assert np.array_equal(Hi[0], Hi[4]) and np.array_equal(Hi[:, nx + 4], Hi[:, nx])
    assert Hm.shape == (ny + 4, nx + 4) and Hm.dtype == np.float32


def test_bathymetry_land_cells():
    nx, ny = 6, 5
    H = np.full((ny + 5, nx + 5), 10.0, dtype=np.float32)
    H = np.ma.array(H, mask=np.zeros_like(H, dtype=bool))
    H.mask[3:5, 3:5] = True
    Hi, Hm = bathymetry_init(H, nx, ny, BC(1, 1, 1, 1))
    assert Hm[3, 3] == np.float32(1e20)          # all four corners land
    assert Hm[2, 2] == np.float32(((10 + 10) + 10 + 1e-30) / 3)  # three wet corners


def test_max_dt_known_answer():
    # lake at rest: dt = 0.25 dx / sqrt(g H)
    nx, ny = 8, 8
    e = np.zeros((ny + 4, nx + 4), np.float32)
    Hm = np.full_like(e, 60.0)
    dt = max_dt_f32(e, e, e, Hm, nx, ny, 200.0, 200.0, 9.81)
    assert dt == np.float32(np.float32(50.0) / np.sqrt(np.float32(9.81) * np.float32(60.0)))
