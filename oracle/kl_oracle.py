"""FP64 NumPy restatement of GPU Ocean's Karhunen-Loeve model error.

TEST INFRASTRUCTURE ONLY: the checker for the CUDA KL kernels.  No product
code imports it.

Follows the reference GPU kernels (K/ = src/gpuocean/gpu_kernels):

* ``kl_d_eta``            the basis sum of kl_sample_eta / kl_sample_ocean_state,
                          K/ocean_noise.cu:671-764 and :770-874, on the interior
                          plus one ghost ring (where the ocean-state kernel
                          evaluates it for the balance)
* ``kl_perturb_state``    the geostrophic balance and update of
                          kl_sample_ocean_state, K/ocean_noise.cu:876-947

The unit-square coordinates are formed in float32 as the kernels form them
(``(ti + 0.5 - 2) / nx`` in double, stored as float, plus the roller in
float, times 2n in float); sines, cosines, powers and sums are float64.

Pinned against vectors produced by the reference's own CPU twin
(``ModelErrorKL._CPUSampleKL`` / ``perturbOceanStateCPU``,
``tests/golden/kl_reference.npz`` made by
``tests/golden/make_kl_golden.py``).  The CPU twin agrees with the GPU kernels
only where both define the same field: rollers of zero (the twin shifts by
whole cells with np.roll, the kernels shift the argument), equal x and y
basis ranges (the twin pairs the y frequency with the x basis index), f
constant (the twin's Coriolis is f + beta j dy), and cells away from the
boundary ring (the twin fills its ghost ring by a boundary copy, the kernels
evaluate the basis there).
"""
from __future__ import annotations

import numpy as np


def _coords(n, roll):
    """float32 coordinates of full-array cells 1 .. n + 2 (K/ocean_noise.cu:826-834)."""
    t = np.arange(1, n + 3)
    x = ((t + 0.5 - 2) / n).astype(np.float32)
    return (x + np.float32(roll)).astype(np.float32)


def kl_d_eta(nx, ny, rns, basis_x_start=1, basis_x_end=10, basis_y_start=1, basis_y_end=10,
             include_cos=True, include_sin=True, kl_decay=1.2, kl_scaling=1.0, perturbation_scale=1.0,
             rollers=(0.0, 0.0, 0.0, 0.0)):
    """d_eta on full-array cells (tj, ti) in [1, ny + 2] x [1, nx + 2], shape
    (ny + 2, nx + 2).  rns: (2 Ny, Nx) normals, sine rows first.  rollers:
    (x_sin, y_sin, x_cos, y_cos)."""
    rns = np.asarray(rns, dtype=np.float64)
    NX, NY = basis_x_end - basis_x_start + 1, basis_y_end - basis_y_start + 1
    assert rns.shape == (2 * NY, NX)
    xs, ys = _coords(nx, rollers[0]), _coords(ny, rollers[1])
    xc, yc = _coords(nx, rollers[2]), _coords(ny, rollers[3])
    amp = float(np.float32(perturbation_scale * np.float32(kl_scaling)))
    d = np.zeros((ny + 2, nx + 2))
    for j in range(NY):
        m = basis_y_start + j
        am = float(m) ** (-float(kl_decay))
        sy = np.sin(np.pi * (np.float32(2 * m) * ys).astype(np.float64))
        cy = np.cos(np.pi * (np.float32(2 * m) * yc).astype(np.float64))
        for i in range(NX):
            n = basis_x_start + i
            an = float(n) ** (-float(kl_decay))
            if include_sin:
                sx = np.sin(np.pi * (np.float32(2 * n) * xs).astype(np.float64))
                d += amp * rns[j, i] * am * an * np.outer(sy, sx)
            if include_cos:
                cx = np.cos(np.pi * (np.float32(2 * n) * xc).astype(np.float64))
                d += amp * rns[NY + j, i] * am * an * np.outer(cy, cx)
    return d


def kl_perturb_state(eta, hu, hv, Hi, d_eta, dx, dy, f, beta=0.0, g=9.81, north=(0.0, 1.0)):
    """Adds d_eta and the balanced (hu, hv) to the interior of (ny+4, nx+4)
    copies of the state (K/ocean_noise.cu:876-947); Hi: (ny+5, nx+5) corner
    depths; d_eta from kl_d_eta.  Returns (eta, hu, hv) in float64."""
    eta, hu, hv = (np.array(a, dtype=np.float64) for a in (eta, hu, hv))
    Hi = np.asarray(Hi, dtype=np.float64)
    ny, nx = eta.shape[0] - 4, eta.shape[1] - 4
    tj, ti = np.meshgrid(np.arange(2, ny + 2), np.arange(2, nx + 2), indexing="ij")
    H_mid = 0.25 * (Hi[tj, ti] + Hi[tj, ti + 1] + Hi[tj + 1, ti] + Hi[tj + 1, ti + 1])
    cor = f + beta * ((ti + 0.5) * dx * north[0] + (tj + 0.5) * dy * north[1])
    d = d_eta[1:-1, 1:-1]
    ex = (d_eta[1:-1, 2:] - d_eta[1:-1, :-2]) / (2.0 * dx)
    ey = (d_eta[2:, 1:-1] - d_eta[:-2, 1:-1]) / (2.0 * dy)
    eta[2:-2, 2:-2] += d
    hu[2:-2, 2:-2] += -(g / cor) * (H_mid + d) * ey
    hv[2:-2, 2:-2] += (g / cor) * (H_mid + d) * ex
    return eta, hu, hv
