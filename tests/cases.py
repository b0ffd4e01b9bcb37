"""Initial conditions of the reference's CDKLM16 regression cases.

Restates ``test/testUtils.py:111-142`` (Gaussian bumps) and :99-107 (bottom
topography) and the set-up of ``test/schemes/CDKLM16_test.py:40-66,150-420``:
nx=50, ny=70, dx=dy=200, dt=0.9, T=50 s, H=60, f=r=0.
"""
import numpy as np

NX, NY = 50, 70
DX = DY = 200.0
DT = 0.9
G = 9.81
T_END = 50.0
DEPTH = 60.0


def _bump(eta, nx, ny, dx, dy, xc, yc):
    size = 500.0 * min(dx, dy)
    j = np.arange(-2, ny + 2)[:, None]
    i = np.arange(-2, nx + 2)[None, :]
    x = dx * i - xc
    y = dy * j - yc
    inside = np.sqrt(x ** 2 + y ** 2) < size
    eta += np.where(inside, np.exp(-(x ** 2 / size + y ** 2 / size)), 0.0).astype(np.float32)


def central_bump(eta, nx=NX, ny=NY, dx=DX, dy=DY):
    _bump(eta, nx, ny, dx, dy, dx * nx / 2.0, dy * ny / 2.0)


def corner_bump(eta, nx=NX, ny=NY, dx=DX, dy=DY):
    _bump(eta, nx, ny, dx, dy, 4 * dx, 4 * dy)


def upper_corner_bump(eta, nx=NX, ny=NY, dx=DX, dy=DY):
    _bump(eta, nx, ny, dx, dy, (nx - 4) * dx, (ny - 4) * dy)


def bottom_topography(Hi, nx=NX, ny=NY):
    j = np.arange(-2, ny + 3)[:, None].astype(np.float64)
    i = np.arange(-2, nx + 3)[None, :].astype(np.float64)
    Hi[:, :] = (6 + 2.0 * np.cos(0.3 * (i + i / (np.sin(0.5 * j) + 2.5)))
                + 2.0 * np.sin(2 * np.pi * (j + i) / (2.0 * ny))).astype(np.float32)


# name -> (bc (north, east, south, west), bump, f, beta, bathymetry, golden key)
CASES = {
    "wall_central": ((1, 1, 1, 1), central_bump, 0.0, 0.0, False, "wallBC_central"),
    "wall_corner": ((1, 1, 1, 1), corner_bump, 0.0, 0.0, False, "wallBC_corner"),
    "wall_upperCorner": ((1, 1, 1, 1), upper_corner_bump, 0.0, 0.0, False, "wallBC_upperCorner"),
    "periodic_central": ((2, 2, 2, 2), central_bump, 0.0, 0.0, False, "wallBC_central"),
    "periodic_corner": ((2, 2, 2, 2), corner_bump, 0.0, 0.0, False, "periodic_corner"),
    "periodic_upperCorner": ((2, 2, 2, 2), upper_corner_bump, 0.0, 0.0, False, "periodic_upperCorner"),
    "periodicNS_central": ((2, 1, 2, 1), central_bump, 0.0, 0.0, False, "wallBC_central"),
    "periodicNS_corner": ((2, 1, 2, 1), corner_bump, 0.0, 0.0, False, "periodicNS_corner"),
    "periodicNS_upperCorner": ((2, 1, 2, 1), upper_corner_bump, 0.0, 0.0, False, "periodicNS_upperCorner"),
    "periodicEW_central": ((1, 2, 1, 2), central_bump, 0.0, 0.0, False, "wallBC_central"),
    "periodicEW_corner": ((1, 2, 1, 2), corner_bump, 0.0, 0.0, False, "periodicEW_corner"),
    "periodicEW_upperCorner": ((1, 2, 1, 2), upper_corner_bump, 0.0, 0.0, False, "periodicEW_upperCorner"),
    "coriolis_central": ((1, 1, 1, 1), central_bump, 0.01, 0.0, False, "coriolis_central"),
    "betamodel_central": ((1, 1, 1, 1), central_bump, 0.01 + 2 * 1e-6 * DY, 1e-6, False, "betamodel_central"),
    "bathymetry_central": ((1, 1, 1, 1), central_bump, 0.0, 0.0, True, "wallBC_central_bathymetry"),
}


def make_case(name):
    bc, bump, f, beta, bathy, key = CASES[name]
    shape = (NY + 4, NX + 4)
    eta0 = np.zeros(shape, dtype=np.float32)
    hu0 = np.zeros(shape, dtype=np.float32)
    hv0 = np.zeros(shape, dtype=np.float32)
    Hi = np.ones((shape[0] + 1, shape[1] + 1), dtype=np.float32) * DEPTH
    bump(eta0)
    if bathy:
        bottom_topography(Hi)
    return dict(eta0=eta0, hu0=hu0, hv0=hv0, H=Hi, nx=NX, ny=NY, dx=DX, dy=DY, dt=DT,
                g=G, f=f, r=0.0, coriolis_beta=beta, bc=bc, golden=key)


def rel_max_diff(a, ref):
    """max |a - ref| / max |ref| over the interior (test/schemes/CDKLM16_test.py:113-143)."""
    return float(np.max(np.abs(np.asarray(a, np.float64) - ref)) / np.max(np.abs(ref)))
