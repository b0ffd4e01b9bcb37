"""Synthetic initial conditions for the benchmark and test configurations.

* ``gaussian_bump_case``  256x256 walls, constant depth, Gaussian eta bump
  (the plain deterministic CDKLM16 configuration).
* ``double_jet_case``     512x300, periodic in x, walls in y, beta plane,
  Gaussian-random bathymetry and two geostrophically balanced tanh jets.
* ``multilevel_grids``    level grids sharing one physical domain.

Every field is generated from a seeded ``numpy.random.default_rng`` so that
all runs see the same inputs.  Nothing here touches the GPU.
"""
from __future__ import annotations

import numpy as np


def gaussian_bump_case(nx=256, ny=256, dx=200.0, dy=200.0, depth=60.0, amplitude=0.1, sigma_cells=10.0,
                       g=9.81, f=1.2e-4):
    """Gaussian eta bump (amplitude, sigma in cells) at the interior centre over
    the full (ny+4, nx+4) array including ghost cells; hu = hv = 0."""
    x = (np.arange(nx + 4) - 2 + 0.5) * dx
    y = (np.arange(ny + 4) - 2 + 0.5) * dy
    xc, yc = nx * dx / 2.0, ny * dy / 2.0
    r2 = (x[None, :] - xc) ** 2 + (y[:, None] - yc) ** 2
    eta = (amplitude * np.exp(-r2 / (2.0 * (sigma_cells * dx) ** 2))).astype(np.float32)
    zeros = np.zeros_like(eta)
    H = np.full((ny + 5, nx + 5), depth, dtype=np.float32)
    return dict(eta0=eta, hu0=zeros.copy(), hv0=zeros.copy(), H=H, nx=nx, ny=ny, dx=dx, dy=dy, g=g, f=f, r=0.0,
                boundary=(1, 1, 1, 1))


def random_bathymetry(shape, mean=230.0, std=10.0, corr_cells=20.0, seed=2):
    """Gaussian random field: N(0,1) filtered with a Gaussian of `corr_cells`
    correlation length in Fourier space, normalised to `std`, plus `mean`."""
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal(shape)
    ky = np.fft.fftfreq(shape[0])[:, None]
    kx = np.fft.rfftfreq(shape[1])[None, :]
    filt = np.exp(-0.5 * (2 * np.pi * corr_cells) ** 2 * (kx ** 2 + ky ** 2))
    field = np.fft.irfft2(np.fft.rfft2(noise) * filt, s=shape)
    field = (field - field.mean()) / field.std() * std
    return (mean + field).astype(np.float32)


def double_jet_case(nx=512, ny=300, dx=5000.0, dy=5000.0, g=9.81, f0=1.2e-4, beta=2e-11, amplitude=0.2,
                    width_cells=20.0, seed=2):
    """Two tanh eta jets at Ly/3 and 2Ly/3 in discrete geostrophic balance on a
    beta plane f = f0 + beta (y - y_mid).  Periodic in x, walls in y.

    Returns constructor arguments of CDKLM16: ``f`` is passed so that the
    simulator's compensation for the first interior cell yields
    f(y) = f0 + beta (y - y_mid) at cell centres.
    """
    H = random_bathymetry((ny + 5, nx + 5), seed=seed)
    Ly = ny * dy
    y = (np.arange(ny + 4) - 2 + 0.5) * dy
    w = width_cells * dy
    prof = amplitude * (np.tanh((y - Ly / 3.0) / w) - np.tanh((y - 2.0 * Ly / 3.0) / w)) / 2.0
    eta = np.repeat(prof[:, None], nx + 4, axis=1).astype(np.float32)
    Hm = 0.25 * (H[:-1, :-1] + H[1:, :-1] + H[:-1, 1:] + H[1:, 1:])
    fy = f0 + beta * (y - 0.5 * Ly)
    deta_dy = np.zeros_like(eta, dtype=np.float64)
    deta_dy[1:-1, :] = (eta[2:, :] - eta[:-2, :]) / (2.0 * dy)
    hu = (-(g * (Hm + eta) / fy[:, None]) * deta_dy).astype(np.float32)
    hv = np.zeros_like(eta)
    f_arg = f0 - beta * 0.5 * Ly + 2.0 * beta * dy
    return dict(eta0=eta, hu0=hu, hv0=hv, H=H, nx=nx, ny=ny, dx=dx, dy=dy, g=g, f=f_arg, r=0.0,
                coriolis_beta=beta, boundary=(1, 2, 1, 2))


def multilevel_grids(levels=((128, 64, 512), (256, 128, 128), (512, 256, 32)), Lx=2560e3, Ly=1500e3):
    """(nx, ny, n_members, dx, dy) of level grids over one physical domain."""
    return [(nx, ny, n, Lx / nx, Ly / ny) for nx, ny, n in levels]


def resample_case(case, nx, ny):
    """The double-jet case re-gridded to (nx, ny) over the same physical domain."""
    Lx, Ly = case["nx"] * case["dx"], case["ny"] * case["dy"]
    out = double_jet_case(nx=nx, ny=ny, dx=Lx / nx, dy=Ly / ny)
    return out
