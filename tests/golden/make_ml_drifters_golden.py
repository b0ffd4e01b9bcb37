"""Golden trajectories of the reference's host drifter collections.

Runs the reference's ``CPUDrifterCollection`` (D/CPUDrifterCollection.py:
29-232) and ``MLDrifterCollection`` (D/MLDrifterCollection.py:24-176) on
seeded velocity and variance fields - plain drift from (eta, hu, hv, Hm),
a random walk with scalar and with field variances, the multi-level biased
walk on a periodic domain and its unbiased variant - with numpy's global
generator seeded before each case, and writes the positions after every
step to ``ml_drifters_reference.npz`` next to this file.  Only NumPy code of
the reference runs (PyCUDA and the other absent modules are inert stubs).

Usage:  python tests/golden/make_ml_drifters_golden.py REFERENCE_ROOT (or $GPUOCEAN_REFERENCE)
"""
import os
import sys
from unittest import mock

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from ml_drifter_cases import CASE  # noqa: E402


def import_reference(root):
    sys.dont_write_bytecode = True   # the checkout is read-only: no __pycache__ inside it
    for name in ["pycuda", "pycuda.driver", "pycuda.gpuarray", "pycuda.compiler", "pycuda.curandom",
                 "pycuda.autoinit", "matplotlib", "matplotlib.pyplot", "matplotlib.gridspec",
                 "matplotlib.animation", "matplotlib.colors", "netCDF4", "mpi4py", "pandas"]:
        sys.modules.setdefault(name, mock.MagicMock())
    sys.path.insert(0, os.path.join(root, "src"))
    from gpuocean.drifters import CPUDrifterCollection, MLDrifterCollection
    from gpuocean.utils import Common
    return CPUDrifterCollection.CPUDrifterCollection, MLDrifterCollection.MLDrifterCollection, Common


def run(CPU, ML, Common):
    c = CASE()
    out = {}
    Lx, Ly = c["Lx"], c["Ly"]
    # plain drift from the state, walls
    np.random.seed(c["seed"])
    d = CPU(c["n"], boundaryConditions=Common.BoundaryConditions(1, 1, 1, 1), domain_size_x=Lx, domain_size_y=Ly)
    d.setDrifterPositions(c["pos"])
    d.setObservationPosition(c["obs"])
    for k in range(3):
        d.drift(c["eta"], c["hu"], c["hv"], c["Hm"], c["dx"], c["dy"], c["dt"], x_zero_ref=2, y_zero_ref=2)
        out[f"plain_{k}"] = d.positions.copy()
    # random walk with a scalar and with field variances, doubly periodic
    for tag, uv, vv in (("scalar", 0.04, 0.09), ("field", c["u_var"], c["v_var"])):
        np.random.seed(c["seed"] + 1)
        d = CPU(c["n"], boundaryConditions=Common.BoundaryConditions(2, 2, 2, 2), domain_size_x=Lx, domain_size_y=Ly)
        d.setDrifterPositions(c["pos"])
        d.setObservationPosition(c["obs"])
        for k in range(3):
            d.driftFromVelocities(c["u"], c["v"], c["dx"], c["dy"], c["dt"], u_var=uv, v_var=vv)
            out[f"walk_{tag}_{k}"] = d.positions.copy()
    # multi-level drifters on the periodic domain, biased and unbiased walk
    for biased in (True, False):
        np.random.seed(c["seed"] + 2)
        d = ML(c["n_unique"], c["ens"], boundaryConditions=Common.BoundaryConditions(2, 2, 2, 2), domain_size_x=Lx,
               domain_size_y=Ly, use_biased_walk=biased)
        d.setDrifterPositions(c["unique_pos"])
        for k in range(3):
            d.drift(c["u"], c["v"], c["dx"], c["dy"], c["dt"], u_var=c["u_var"], v_var=c["v_var"])
            out[f"ml_{int(biased)}_{k}"] = d.positions.copy()
        out[f"ml_{int(biased)}_member1"] = d.getDrifterPositionsForEnsembleMember(1)
        out[f"ml_{int(biased)}_drifter2"] = d.getDrifterPositionsForDrifter(2)
    return out


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GPUOCEAN_REFERENCE")
    if not root:
        sys.exit("usage: %s REFERENCE_ROOT (or set GPUOCEAN_REFERENCE)" % sys.argv[0])
    out = run(*import_reference(root))
    path = os.path.join(HERE, "ml_drifters_reference.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, len(out), "arrays")


if __name__ == "__main__":
    main()
