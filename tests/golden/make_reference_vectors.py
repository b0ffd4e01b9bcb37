"""Golden vectors for the SOAR noise, the LCG and the drifters, produced by the
reference's own CPU code.

The reference keeps CPU twins of its GPU kernels for testing:
``OceanStateNoise._applyQ_CPU`` (SOAR), ``_obtainOceanPerturbations_CPU``
(geostrophic balance), ``_interpolate_CPU`` (bicubic up-sampling),
``_CPUUpdateRandom`` (LCG + Box-Muller) and ``CPUDrifterCollection.drift``.
This script imports them from a reference checkout (PyCUDA and matplotlib are
absent here and are replaced by inert stubs; only CPU functions are called)
and writes ``noise_drift_reference.npz`` next to this file.

Usage:  python tests/golden/make_reference_vectors.py REFERENCE_ROOT (or $GPUOCEAN_REFERENCE)
"""
import os
import sys
from unittest import mock

import numpy as np


def import_reference(root):
    sys.dont_write_bytecode = True   # the checkout is read-only: no __pycache__ inside it
    for name in ["pycuda", "pycuda.driver", "pycuda.gpuarray", "pycuda.compiler", "pycuda.curandom",
                 "pycuda.autoinit", "matplotlib", "matplotlib.pyplot", "matplotlib.gridspec",
                 "matplotlib.animation", "matplotlib.colors", "netCDF4", "mpi4py"]:
        sys.modules.setdefault(name, mock.MagicMock())
    sys.path.insert(0, os.path.join(root, "src"))
    from gpuocean.SWEsimulators import OceanStateNoise
    from gpuocean.drifters import CPUDrifterCollection
    from gpuocean.utils import Common
    return OceanStateNoise.OceanStateNoise, CPUDrifterCollection.CPUDrifterCollection, Common


def make_noise(cls, nx, ny, dx, dy, pns, pew, factor=1, q0=None, L=None):
    """An OceanStateNoise with the attributes its CPU functions read (the GPU
    constructor is bypassed); sizes follow S/OceanStateNoise.py:96-160."""
    n = object.__new__(cls)
    n.nx, n.ny = np.int32(nx), np.int32(ny)
    n.dx, n.dy = np.float32(dx), np.float32(dy)
    n.cutoff = np.int32(2)
    n.periodicNorthSouth, n.periodicEastWest = np.int32(pns), np.int32(pew)
    n.interpolation_factor = np.int32(factor)
    n.coarse_nx = np.int32(np.ceil(nx / factor))
    n.coarse_ny = np.int32(np.ceil(ny / factor))
    n.coarse_dx = np.float32(dx * factor)
    n.coarse_dy = np.float32(dy * factor)
    n.rand_ghost_cells_x = np.int32(0 if pew else 4)
    n.rand_ghost_cells_y = np.int32(0 if pns else 4)
    n.rand_nx = np.int32(n.coarse_nx + 2 * n.rand_ghost_cells_x)
    n.rand_ny = np.int32(n.coarse_ny + 2 * n.rand_ghost_cells_y)
    n.seed_ny = np.int32(n.rand_ny)
    n.seed_nx = np.int32(np.ceil(n.rand_nx / 2))
    n.soar_q0 = np.float32(dx / 100000 if q0 is None else q0)
    n.soar_L = np.float32(0.75 * n.coarse_dx if L is None else L)
    n.use_lcg = True
    n.rng = None
    n.random_numbers = None
    n.perpendicular_random_numbers = None
    n.reduction_buffer = None
    n.local_size = (16, 16, 1)
    n.global_size_random_numbers = (int(np.ceil(n.seed_nx / 16)), int(np.ceil(n.seed_ny / 16)))
    n.random_numbers_host = np.zeros((n.rand_ny, n.rand_nx), dtype=np.float32)
    return n


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GPUOCEAN_REFERENCE")
    if not root:
        sys.exit("usage: %s REFERENCE_ROOT (or set GPUOCEAN_REFERENCE)" % sys.argv[0])
    Noise, CPUDrifters, Common = import_reference(root)
    out = {}
    rng = np.random.default_rng(20240601)

    # SOAR + geostrophic balance, interpolation factor 1, four boundary cases
    # (the set-up of test/stochastic/OceanStateNoise_parent.py:37-80)
    nx, ny, dx, dy, f, g = 30, 40, 7.0, 7.0, 0.02, 9.81
    for pns, pew in ((1, 1), (0, 0), (1, 0), (0, 1)):
        key = f"soar_ns{pns}_ew{pew}"
        n = make_noise(Noise, nx, ny, dx, dy, pns, pew)
        xi = rng.standard_normal((n.rand_ny, n.rand_nx)).astype(np.float32)
        n.random_numbers_host = xi.copy()
        H = np.ones((ny + 5, nx + 5)) * 5.0
        d_eta, d_hu, d_hv = n._obtainOceanPerturbations_CPU(H, f, 0.0, g)
        out[key + "/xi"] = xi
        out[key + "/coarse"] = n._applyQ_CPU()
        out[key + "/d_eta"] = d_eta
        out[key + "/d_hu"] = d_hu
        out[key + "/d_hv"] = d_hv
        out[key + "/params"] = np.array([nx, ny, dx, dy, f, g, 5.0, n.soar_q0, n.soar_L, 1], dtype=np.float64)

    # bicubic up-sampling with odd factors 3, 5 (periodic, the alignment case
    # of test_interpolation_*_ocean)
    for factor in (3, 5):
        fnx, fny = 10 * factor, 12 * factor
        key = f"bicubic_f{factor}"
        n = make_noise(Noise, fnx, fny, dx, dy, 1, 1, factor=factor)
        xi = rng.standard_normal((n.rand_ny, n.rand_nx)).astype(np.float32)
        n.random_numbers_host = xi.copy()
        H = np.ones((fny + 5, fnx + 5)) * 5.0
        d_eta, d_hu, d_hv = n._obtainOceanPerturbations_CPU(H, f, 0.0, g)
        out[key + "/xi"] = xi
        out[key + "/coarse"] = n._applyQ_CPU()
        out[key + "/d_eta"] = d_eta
        out[key + "/d_hu"] = d_hu
        out[key + "/d_hv"] = d_hv
        out[key + "/params"] = np.array([fnx, fny, dx, dy, f, g, 5.0, n.soar_q0, n.soar_L, factor], dtype=np.float64)

    # LCG uniform and Box-Muller normal draws (uint64 seeds, 2 draws per seed)
    n = make_noise(Noise, 37, 9, dx, dy, 0, 1)   # odd random-field width
    seeds = (np.random.RandomState(7).rand(n.seed_ny, n.seed_nx) * 2147483648.0).astype(np.uint64)
    n.host_seed = seeds.copy()
    n._CPUUpdateRandom(False)
    out["lcg/seed_in"] = seeds
    out["lcg/uniform"] = n.random_numbers_host.copy()
    out["lcg/seed_after_uniform"] = n.host_seed.copy()
    n._CPUUpdateRandom(True)
    out["lcg/normal"] = n.random_numbers_host.copy()
    out["lcg/seed_after_normal"] = n.host_seed.copy()
    u, s1 = n._lcg(np.uint64(1871412062))
    out["lcg/special_seed"] = np.array([1871412062, int(s1)], dtype=np.uint64)
    out["lcg/special_u"] = np.array([u])

    # drifters: CPU collection on a periodic square domain, 5 Euler steps
    nx = ny = 24
    dxd = dyd = 100.0
    eta = (0.05 * rng.standard_normal((ny + 4, nx + 4))).astype(np.float32)
    hu = (0.5 * rng.standard_normal((ny + 4, nx + 4))).astype(np.float32)
    hv = (0.5 * rng.standard_normal((ny + 4, nx + 4))).astype(np.float32)
    Hm = np.full((ny + 4, nx + 4), 10.0, dtype=np.float32)
    bc = Common.BoundaryConditions(2, 2, 2, 2)
    coll = CPUDrifters(40, boundaryConditions=bc, domain_size_x=nx * dxd, domain_size_y=ny * dyd)
    pos0 = rng.uniform(0, nx * dxd, size=(41, 2))
    coll.positions[:, :] = pos0
    traj = [coll.positions.copy()]
    for _ in range(5):
        coll.drift(eta.astype(np.float64), hu.astype(np.float64), hv.astype(np.float64), Hm.astype(np.float64),
                   dxd, dyd, 20.0, x_zero_ref=2, y_zero_ref=2)
        traj.append(coll.positions.copy())
    out["drift/eta"], out["drift/hu"], out["drift/hv"], out["drift/Hm"] = eta, hu, hv, Hm
    out["drift/traj"] = np.array(traj)
    out["drift/params"] = np.array([nx, ny, dxd, dyd, 20.0], dtype=np.float64)

    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "noise_drift_reference.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, len(out), "arrays")


if __name__ == "__main__":
    main()
