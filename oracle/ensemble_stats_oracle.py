"""FP64 NumPy restatement of GPU Ocean's observation operator and ensemble
statistics.

TEST INFRASTRUCTURE ONLY: the checker for the CUDA observation and moment
kernels.  No product code imports it.

Follows the reference (K/ = src/gpuocean/gpu_kernels, E/ = src/gpuocean/ensembles,
U/ = src/gpuocean/utils):

* ``observe_underlying_flow``  observeUnderlyingFlow, K/observationKernels.cu:29-83
* ``observe_particles``        BaseOceanStateEnsemble.observeParticles, CPU path
                               with and without innovation, E/BaseOceanStateEnsemble.py:79-145
* ``desingularise``            U/OceanographicUtilities.py:413-414
* ``moments``                  estimate / estimateVelocity with np.mean and np.var
                               (E/BaseOceanStateEnsemble.py:147-176), member axis first
* ``ml_estimate``              MultiLevelOceanEnsemble._estimate_pure,
                               E/MultiLevelOceanEnsemble.py:258-267

Pinned against vectors produced by the reference's own Python code
(``tests/golden/ensemble_stats_reference.npz``, made by
``tests/golden/make_ensemble_stats_golden.py``).  Cell indices of the
observation operator are computed in float32 (IEEE division), as the kernel
does; everything else in float64.
"""
from __future__ import annotations

import numpy as np


def observed_cells(positions, dx, dy, x_zero_ref=0, y_zero_ref=0):
    """(ix, iy) of the cells holding (x, y) positions, K/observationKernels.cu:67-68."""
    p = np.asarray(positions, dtype=np.float32)
    ix = np.floor(p[:, 0] / np.float32(dx)).astype(np.int64) + x_zero_ref
    iy = np.floor(p[:, 1] / np.float32(dy)).astype(np.int64) + y_zero_ref
    return ix, iy


def observe_underlying_flow(hu, hv, positions, dx, dy, x_zero_ref=2, y_zero_ref=2):
    """(hu, hv) at each position from arrays with ghost cells,
    K/observationKernels.cu:29-83; returns (num_drifters, 2)."""
    ix, iy = observed_cells(positions, dx, dy, x_zero_ref, y_zero_ref)
    return np.stack([np.asarray(hu)[iy, ix], np.asarray(hv)[iy, ix]], axis=1)


def observe_particles(states, observations, dx, dy, innovation=False, compensate_for_eta=True, mean_depth=None):
    """CPU path of observeParticles (E/BaseOceanStateEnsemble.py:79-145).

    states: (particles, 3, ny, nx) interior (eta, hu, hv); observations:
    (drifters, 4) rows (x, y, hu, hv) of the truth.  Returns (particles,
    drifters, 2): (hu, hv) of each particle at the observed cells, or the
    innovation obs * eta_compensation - particle with eta_compensation =
    (mean_depth + eta) / mean_depth (float32) when compensate_for_eta.
    """
    obs = np.asarray(observations, dtype=np.float64)
    ix = np.floor(obs[:, 0] / dx).astype(np.int64)
    iy = np.floor(obs[:, 1] / dy).astype(np.int64)
    out = np.empty((len(states), len(obs), 2))
    for p, st in enumerate(states):
        eta, hu, hv = (np.asarray(a, dtype=np.float64) for a in st)
        if innovation:
            # float32 states and a float32 (or weak Python) mean depth: the
            # compensation factor is a float32 quantity
            md = np.float32(mean_depth)
            e32 = np.asarray(st[0], dtype=np.float32)[iy, ix]
            comp = ((md + e32) / md).astype(np.float64) if compensate_for_eta else 1.0
            out[p, :, 0] = obs[:, 2] * comp - hu[iy, ix]
            out[p, :, 1] = obs[:, 3] * comp - hv[iy, ix]
        else:
            out[p, :, 0] = hu[iy, ix]
            out[p, :, 1] = hv[iy, ix]
    return out


def desingularise(h, hu, eps):
    """U/OceanographicUtilities.py:413-414."""
    return hu / np.maximum(np.minimum(h * h / (2.0 * eps) + 0.5 * eps, eps), np.abs(h))


def velocities(states, Hm, eps=None):
    """(members, 2, ny, nx) velocities of (members, 3, ny, nx) states:
    desingularised (estimateVelocity, E/BaseOceanStateEnsemble.py:163-176)
    when eps is given, plain hu / (eta + Hm) otherwise (downloadVelocities,
    E/MultiLevelOceanEnsemble.py:187-224)."""
    s = np.asarray(states, dtype=np.float64)
    h = s[:, 0] + np.asarray(Hm, dtype=np.float64)
    if eps is None:
        return np.stack([s[:, 1] / h, s[:, 2] / h], axis=1)
    return np.stack([desingularise(h, s[:, 1], eps), desingularise(h, s[:, 2], eps)], axis=1)


def moments(values, ddof=0):
    """Mean and variance over the member axis (axis 0) in float64: the
    statistics estimate(np.mean) / estimate(np.var, ddof=...) compute over
    the reference's last axis."""
    v = np.asarray(values, dtype=np.float64)
    return v.mean(axis=0), v.var(axis=0, ddof=ddof)


def ml_estimate(level_stats):
    """MultiLevelOceanEnsemble._estimate_pure (E/MultiLevelOceanEnsemble.py:258-267)
    from per-level statistics: level_stats[0] is the level-0 statistic
    (planes, ny0, nx0); level_stats[l] for l > 0 is the pair (fine, coarse)
    with fine on a grid twice as fine as coarse.  Returns the estimate on the
    finest grid in float64."""
    L = len(level_stats)
    top = level_stats[-1][0] if L > 1 else level_stats[0]
    est = np.zeros(np.shape(top))
    r = 2 ** (L - 1)
    est += np.asarray(level_stats[0]).repeat(r, 1).repeat(r, 2)
    for l in range(1, L):
        fine, coarse = level_stats[l]
        d = np.asarray(fine) - np.asarray(coarse).repeat(2, 1).repeat(2, 2)
        r = 2 ** (L - l - 1)
        est += d.repeat(r, 1).repeat(r, 2)
    return est
