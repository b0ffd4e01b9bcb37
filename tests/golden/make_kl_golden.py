"""Golden vectors for the Karhunen-Loeve model error, produced by the
reference's own CPU twin (``ModelErrorKL.perturbOceanStateCPU`` and
``perturbEtaCPU``, S/ModelErrorKL.py:511-566).

The twin is imported from a reference checkout (PyCUDA and matplotlib are
absent here and are replaced by inert stubs; the GPU constructor is bypassed
and only NumPy code runs) and called with injected normals and rollers of
zero on a 40 x 30 grid (default basis 1..10 in both directions), for wall
and periodic boundaries, with and without the cosine basis.  Writes
``kl_reference.npz`` next to this file.

Usage:  python tests/golden/make_kl_golden.py REFERENCE_ROOT (or $GPUOCEAN_REFERENCE)
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
                 "matplotlib.animation", "matplotlib.colors", "netCDF4", "mpi4py"]:
        sys.modules.setdefault(name, mock.MagicMock())
    sys.path.insert(0, os.path.join(root, "src"))
    from gpuocean.SWEsimulators import ModelErrorKL
    return ModelErrorKL.ModelErrorKL


class BC:
    def __init__(self, north, east, south, west):
        self.north, self.east, self.south, self.west = north, east, south, west


class Uploadable:
    """Stands in for the device array the twin uploads its normals to."""

    def upload(self, *a, **k):
        pass

    def release(self):
        pass


def make(cls, nx, ny, dx, dy, bc, include_cos, kl_decay=1.2, kl_scaling=0.05):
    """A ModelErrorKL with the attributes its CPU functions read
    (S/ModelErrorKL.py:98-146)."""
    me = object.__new__(cls)
    me.nx, me.ny = np.int32(nx), np.int32(ny)
    me.dx, me.dy = np.float32(dx), np.float32(dy)
    me.boundary_conditions = bc
    me.kl_decay, me.kl_scaling = np.float32(kl_decay), np.float32(kl_scaling)
    me.include_cos, me.include_sin = np.int32(include_cos), np.int32(1)
    me.basis_x_start = me.basis_y_start = np.int32(1)
    me.basis_x_end = me.basis_y_end = np.int32(10)
    me.N_basis_x = me.N_basis_y = np.int32(10)
    me.rand_nx, me.rand_ny = np.int32(10), np.int32(20)
    me.KL_basis_fields_sin = None
    me.KL_basis_fields_cos = None
    me.random_numbers_host = np.zeros((20, 10), dtype=np.float32)
    me.random_numbers = Uploadable()
    me.gpu_stream = None
    me.np_rng = np.random.default_rng(0)
    me.use_lcg = False
    me.rng = None
    return me


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GPUOCEAN_REFERENCE")
    if not root:
        sys.exit("usage: %s REFERENCE_ROOT (or set GPUOCEAN_REFERENCE)" % sys.argv[0])
    cls = import_reference(root)
    nx, ny, dx, dy = 40, 30, 500.0, 400.0
    rng = np.random.default_rng(21)
    Hi = (60.0 + 8.0 * rng.standard_normal((ny + 5, nx + 5))).astype(np.float32)
    f, g = 1.2e-4, 9.81
    out = {"nx": nx, "ny": ny, "dx": dx, "dy": dy, "f": f, "g": g, "Hi": Hi}
    cases = {"walls": (BC(1, 1, 1, 1), 1), "periodic": (BC(2, 2, 2, 2), 1), "walls_sin_only": (BC(1, 1, 1, 1), 0)}
    for name, (bc, include_cos) in cases.items():
        rns = rng.standard_normal((20, 10)).astype(np.float32)
        me = make(cls, nx, ny, dx, dy, bc, include_cos)
        z = np.zeros((ny + 4, nx + 4))
        eta, hu, hv = z.copy(), z.copy(), z.copy()
        me.perturbOceanStateCPU(eta, hu, hv, Hi[2:-2, 2:-2], f, beta=0.0, g=g, random_numbers=rns,
                                roll_x_sin=0.0, roll_y_sin=0.0, roll_x_cos=0.0, roll_y_cos=0.0)
        eta_only = z.copy()
        me.perturbEtaCPU(eta_only, random_numbers=rns, roll_x_sin=0.0, roll_y_sin=0.0, roll_x_cos=0.0,
                         roll_y_cos=0.0)
        out.update({f"{name}_rns": rns, f"{name}_include_cos": include_cos, f"{name}_eta": eta,
                    f"{name}_hu": hu, f"{name}_hv": hv, f"{name}_eta_only": eta_only})
    path = os.path.join(HERE, "kl_reference.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


if __name__ == "__main__":
    main()
