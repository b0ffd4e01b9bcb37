"""NumPy restatement of the host-side ensemble API that data assimilation
reads: particle weights, innovation norms and ensemble statistics.

TEST INFRASTRUCTURE ONLY: the checker for the drop-in ensemble classes.  No
product code imports it.

Follows the reference (E/ = src/gpuocean/ensembles):

* ``gaussian_weight``      BaseOceanStateEnsemble.getGaussianWeight, E/BaseOceanStateEnsemble.py:235-290
* ``innovation_norms``     BaseOceanStateEnsemble.getInnovationNorms, :226-233
* ``cauchy_weight``        OceanNoiseEnsemble.getCauchyWeight, E/OceanNoiseEnsemble.py:571-586
* ``largest_timestep``     OceanNoiseEnsemble.findLargestPossibleTimeStep, :595-619
* ``under_drifter``        OceanNoiseEnsemble.getEnsembleVarAndRMSEUnderDrifter, :621-721
* ``statistical_fields``   OceanNoiseEnsemble.downloadEnsembleStatisticalFields, :723-775

Pinned against the reference's own methods run on the same inputs
(``tests/golden/ensemble_api_reference.npz``, made by
``tests/golden/make_ensemble_api_golden.py``).
"""
from __future__ import annotations

import numpy as np


def gaussian_weight(innovations, cov, active, normalize=True, R_scale=1.0):
    """log w_i = -1/2 sum over drifters of d^T (R_scale cov)^-1 d (one
    particle per row; inactive particles -inf); for 1-D innovations
    log w_i = -d_i^2 / (2 R[0,0]).  Normalised by the exp-normalise trick, or
    multiplied by the Gaussian density's constant."""
    innovations = np.asarray(innovations, dtype=np.float64)
    R = np.asarray(cov, dtype=np.float64) * R_scale
    Rinv = np.linalg.inv(np.asarray(cov, dtype=np.float64)) / R_scale
    n = innovations.shape[0]
    log_w = np.zeros(n)
    if innovations.ndim == 1:
        for i in range(n):
            log_w[i] = -(innovations[i] ** 2) / (2 * R[0, 0])
        const = 1.0 / np.sqrt(2 * np.pi * R[0, 0])
    else:
        D = innovations.shape[1]
        for i in range(n):
            if not active[i]:
                log_w[i] = -np.inf
                continue
            acc = 0.0
            for d in range(D):
                v = innovations[i, d]
                acc += v @ Rinv @ v
            log_w[i] = -0.5 * acc
        const = 1.0 / ((2 * np.pi) ** D * np.linalg.det(R) ** (D / 2.0))
    if normalize:
        e = np.exp(log_w - np.max(log_w))
        return e / e.sum()
    return const * np.exp(log_w)


def innovation_norms(innovations):
    """Per particle sqrt(sum over drifters of |d|^2)."""
    inn = np.asarray(innovations, dtype=np.float64)
    return np.sqrt(np.sum(np.sqrt(np.sum(inn ** 2, axis=2)) ** 2, axis=1))


def cauchy_weight(distances, variance, normalize=True):
    """1 / (pi sqrt(var) (1 + dist^2 / var)), optionally normalised over all
    entries."""
    d = np.asarray(distances, dtype=np.float64)
    w = 1.0 / (np.pi * np.sqrt(variance) * (1.0 + d ** 2 / variance))
    return w / w.sum() if normalize else w


def largest_timestep(states, Hi, g, dx, dy, interior=False):
    """0.25 min(dx / max|u +- sqrt(g w)|, dy / max|v +- sqrt(g w)|) over all
    states (arrays with 2 ghost cells), w = corner-mean depth + eta; with
    ``interior`` only interior cells count."""
    Hi = np.asarray(Hi, dtype=np.float64)
    depth = 0.25 * (Hi[1:, 1:] + Hi[1:, :-1] + Hi[:-1, 1:] + Hi[:-1, :-1])
    max_u = max_v = 0.0
    for st in states:
        eta, hu, hv = (np.asarray(a, dtype=np.float64) for a in st)
        w = depth + eta
        u, v, c = hu / w, hv / w, np.sqrt(g * w)
        if interior:
            u, v, c = u[2:-2, 2:-2], v[2:-2, 2:-2], c[2:-2, 2:-2]
        max_u = max(max_u, np.max(np.abs(u + c)), np.max(np.abs(u - c)))
        max_v = max(max_v, np.max(np.abs(v + c)), np.max(np.abs(v - c)))
    return 0.25 * min(dx / max_u, dy / max_v)


def under_drifter(truth, particles):
    """Statistics of one cell: truth (3,), particles (n, 3).  Returns the 15
    values spread (ddof 1), RMS distance from the truth, distance of the mean
    from the truth, RMS distance over |truth|, spread over RMS distance, each
    for (eta, hu, hv)."""
    truth = np.asarray(truth, dtype=np.float64)
    p = np.asarray(particles, dtype=np.float64)
    p = p[~np.isnan(p[:, 0])]
    n = len(p)
    mean = p.sum(axis=0) / n
    rmse = np.sqrt(((truth - p) ** 2).sum(axis=0) / n)
    rmse_mean = np.abs(truth - mean)
    rmse_w = rmse / np.abs(truth)
    sigma = np.sqrt(((p - mean) ** 2).sum(axis=0) / (n - 1.0))
    return np.concatenate([sigma, rmse, rmse_mean, rmse_w, sigma / rmse])


def statistical_fields(truth, particles):
    """Ensemble mean of (eta, hu, hv), |truth - mean| and
    sqrt(sum (x - mean)^2 / (n + 1)) / |truth - mean| per cell; truth
    (3, ny, nx), particles (n, 3, ny, nx).  Returns a (9, ny, nx) array in
    the reference's order (means, distances, ratios)."""
    truth = np.asarray(truth, dtype=np.float64)
    p = np.asarray(particles, dtype=np.float64)
    n = p.shape[0]
    mean = p.sum(axis=0) / n
    rmse = np.abs(truth - mean)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.sqrt(((p - mean) ** 2).sum(axis=0) / (1.0 + n)) / rmse
    return np.concatenate([mean, rmse, r])
