"""The KL model-error oracle against the reference's own CPU twin
(tests/golden/make_kl_golden.py).  CPU only.

The twin and the GPU kernels define the same field in the interior for
rollers of zero and equal basis ranges; the twin fills its ghost ring by a
boundary copy where the kernels evaluate the basis, so at walls the balanced
momentum of the boundary cells differs (periodic boundaries agree
everywhere: the basis is periodic on the unit square)."""
import os

import numpy as np
import pytest

from oracle import kl_oracle as ko

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "kl_reference.npz")


@pytest.fixture(scope="module")
def g():
    return np.load(GOLDEN)


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("name", ["walls", "periodic", "walls_sin_only"])
def test_kl_oracle_matches_reference_cpu_twin(g, name):
    nx, ny, dx, dy = int(g["nx"]), int(g["ny"]), float(g["dx"]), float(g["dy"])
    d = ko.kl_d_eta(nx, ny, g[f"{name}_rns"], include_cos=bool(int(g[f"{name}_include_cos"])),
                    kl_decay=np.float32(1.2), kl_scaling=np.float32(0.05))
    z = np.zeros((ny + 4, nx + 4))
    eta, hu, hv = ko.kl_perturb_state(z, z, z, g["Hi"], d, dx, dy, float(g["f"]), 0.0, float(g["g"]))
    ge, gu, gv = g[f"{name}_eta"], g[f"{name}_hu"], g[f"{name}_hv"]
    inner = (slice(2, -2), slice(2, -2))
    core = (slice(3, -3), slice(3, -3))
    assert _rel(eta[inner], ge[inner]) < 2e-6
    assert _rel(g[f"{name}_eta_only"][inner], ge[inner]) == 0.0
    region = inner if name == "periodic" else core
    assert _rel(hu[region], gu[region]) < 3e-6
    assert _rel(hv[region], gv[region]) < 3e-6
