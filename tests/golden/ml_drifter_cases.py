"""Inputs of the host drifter trajectories (shared by
``make_ml_drifters_golden.py`` and the CPU test)."""
import numpy as np


def CASE():
    rng = np.random.default_rng(41)
    nx, ny, dx, dy = 20, 14, 1000.0, 1200.0
    Lx, Ly = nx * dx, ny * dy
    Hm = (50.0 + 5.0 * rng.random((ny + 4, nx + 4))).astype(np.float32)
    eta = (0.2 * rng.standard_normal((ny + 4, nx + 4))).astype(np.float32)
    hu = (10.0 * rng.standard_normal((ny + 4, nx + 4))).astype(np.float32)
    hv = (10.0 * rng.standard_normal((ny + 4, nx + 4))).astype(np.float32)
    u = 0.3 * rng.standard_normal((ny, nx))
    v = 0.3 * rng.standard_normal((ny, nx))
    u_var = 0.02 * rng.random((ny, nx))
    v_var = 0.02 * rng.random((ny, nx))
    n = 9
    pos = np.stack([rng.uniform(0.05, 0.95, n) * Lx, rng.uniform(0.05, 0.95, n) * Ly], axis=1)
    obs = np.array([0.4 * Lx, 0.6 * Ly])
    # unique ML drifters, some close to the periodic boundaries
    unique_pos = np.array([[0.2 * dx, 0.3 * dy], [Lx - 0.2 * dx, 5.5 * dy], [7.4 * dx, Ly - 0.1 * dy],
                           [12.6 * dx, 8.2 * dy]])
    return dict(nx=nx, ny=ny, dx=dx, dy=dy, Lx=Lx, Ly=Ly, Hm=Hm, eta=eta, hu=hu, hv=hv, u=u, v=v, u_var=u_var,
                v_var=v_var, n=n, pos=pos, obs=obs, unique_pos=unique_pos, n_unique=len(unique_pos), ens=5,
                dt=120.0, seed=17)
