"""Observation operator and ensemble statistics on the device against the
oracle (tests/test_ensemble_stats_oracle.py pins it to the reference's own
Python code) and against the reference's observeUnderlyingFlow kernel.

Bars: the observation operator is bit-exact (it copies values); the member
moments agree with the FP64 oracle within 2e-6 of the field's magnitude
(mean) and 1e-5 of the variance's magnitude (float32 shifted sums over up
to 160 members); the multi-level assembly is bit-exact given the same level
statistics (float32 differences, float64 accumulation, in level order)."""
import ctypes

import numpy as np
import pytest

from oracle import ensemble_stats_oracle as eso
from oracle import ref_kernels as rk

pytestmark = pytest.mark.gpu


from test_ensemble_gpu import _member  # noqa: E402  (a double-jet member of the given grid)


def _states(sims):
    return np.stack([np.stack([np.asarray(a, np.float32) for a in s.download(interior_domain_only=True)])
                     for s in sims])


def _stepped(ctx, n, nx, ny, bc=(1, 2, 1, 2), seeds=None, steps=2):
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    seeds = seeds if seeds is not None else [3] * n
    sims = [_member(ctx, nx, ny, bc, sd) for sd in seeds]
    rng = np.random.default_rng(17)
    for s in sims:   # members differ: each gets its own small eta perturbation
        eta, hu, hv = (np.array(a, np.float32) for a in s.download())
        eta[2:-2, 2:-2] += (0.01 * rng.standard_normal((ny, nx))).astype(np.float32)
        s.upload(eta, hu, hv)
        s.updateDt()
    ens = BatchedEnsemble(sims, autotune=False)
    for _ in range(steps):
        ens.step(300.0)
    ens.synchronize()
    return ens, sims


def _close(a, b, rtol):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() <= rtol * max(np.abs(b).max(), 1e-30)


def test_observe_underlying_flow_matches_reference_kernel(gpu_ctx):
    """The drop-in entry against the reference's own kernel on the same
    arrays: identical (hu, hv) for every drifter."""
    if not rk.available():
        pytest.skip("reference kernels not built (no reference sources)")
    from gpuocean_gb300 import _lib
    from gpuocean_gb300.utils import Common
    nx, ny, dx, dy = 77, 45, 150.0, 170.0
    rng = np.random.default_rng(5)
    hu = rng.standard_normal((ny + 4, nx + 4)).astype(np.float32)
    hv = rng.standard_normal((ny + 4, nx + 4)).astype(np.float32)
    D = 300
    pos = np.stack([rng.uniform(0, nx * dx, D), rng.uniform(0, ny * dy, D)], axis=1).astype(np.float32)
    pos[:8, 0] = (np.arange(8) * 9 * dx).astype(np.float32)     # on cell faces
    ref = rk.ref_observe_underlying_flow(nx, ny, dx, dy, hu, hv, pos)
    stream = Common.Stream()
    arrs = [Common.CUDAArray2D(stream, nx, ny, 2, 2, a) for a in (hu, hv)]
    pbuf = Common.CUDAArray2D(stream, 2, D, 0, 0, pos)
    obuf = Common.CUDAArray2D(stream, 2, D, 0, 0, np.zeros((D, 2), np.float32))
    _lib.call("goc_observe_underlying_flow", nx, ny, ctypes.c_float(dx), ctypes.c_float(dy), 2, 2, None, 0,
              arrs[0].ptr, int(arrs[0].pitch), arrs[1].ptr, int(arrs[1].pitch), ctypes.c_float(60.0), D,
              pbuf.ptr, int(pbuf.pitch), obuf.ptr, int(obuf.pitch), stream.handle)
    got = obuf.download(stream)
    np.testing.assert_array_equal(got, ref)
    np.testing.assert_array_equal(got, eso.observe_underlying_flow(hu, hv, pos, dx, dy))
    for a in arrs + [pbuf, obuf]:
        a.release()


def test_ensemble_observe_all_members(gpu_ctx):
    ens, sims = _stepped(gpu_ctx, 6, 64, 40)
    rng = np.random.default_rng(8)
    pos = np.stack([rng.uniform(0, 64 * sims[0].dx, 40), rng.uniform(0, 40 * sims[0].dy, 40)], axis=1)
    got = ens.observe(pos, first=1, count=4)
    assert got.shape == (4, 40, 3)
    for i, s in enumerate(sims[1:5]):
        eta, hu, hv = (np.asarray(a, np.float32) for a in s.download())
        ix, iy = eso.observed_cells(pos, s.dx, s.dy, 2, 2)
        np.testing.assert_array_equal(got[i], np.stack([eta[iy, ix], hu[iy, ix], hv[iy, ix]], axis=1))
    ens.release()


@pytest.mark.parametrize("n,nx,ny", [(7, 64, 40), (160, 48, 24)])   # one slice; many slices + finish pass
@pytest.mark.parametrize("ddof", [0, 1])
def test_state_moments(gpu_ctx, n, nx, ny, ddof):
    ens, sims = _stepped(gpu_ctx, n, nx, ny, steps=1)
    mean, var = ens.moments(ddof=ddof)
    ref_m, ref_v = eso.moments(_states(sims), ddof=ddof)
    assert mean.shape == (3, ny, nx) and var.shape == (3, ny, nx)
    for q in range(3):
        assert _close(mean[q], ref_m[q], 2e-6), q
        assert _close(var[q], ref_v[q], 1e-5), q
    ens.release()


@pytest.mark.parametrize("eps", [None, 1e-5])
def test_velocity_moments(gpu_ctx, eps):
    ens, sims = _stepped(gpu_ctx, 9, 64, 40)
    Hm = np.asarray(sims[0].downloadBathymetry()[1], np.float32)[2:-2, 2:-2]
    mean, var = ens.moments(quantity="velocity", desingularise=eps, ddof=1)
    vel = eso.velocities(_states(sims), Hm, eps=eps)
    ref_m, ref_v = eso.moments(vel, ddof=1)
    for q in range(2):
        assert _close(mean[q], ref_m[q], 2e-6), q
        assert _close(var[q], ref_v[q], 1e-5), q
    ens.release()


def test_multilevel_estimators(gpu_ctx):
    """Device ML estimator: with the device's own level statistics, the
    assembly equals the reference formula bit for bit; against the FP64
    oracle within the moment bars."""
    from gpuocean_gb300.ensembles.MultiLevelOceanEnsemble import MultiLevelOceanEnsemble
    grids = [(32, 16), (64, 32), (128, 64)]
    Nes = [6, 4, 3]
    seeds = iter(range(100, 200))

    def level(nx, ny, n):
        out = []
        for _ in range(n):
            s = _member(gpu_ctx, nx, ny, (1, 2, 1, 2), 3)
            eta, hu, hv = (np.array(a, np.float32) for a in s.download())
            r = np.random.default_rng(next(seeds))
            eta[2:-2, 2:-2] += (0.01 * r.standard_normal((ny, nx))).astype(np.float32)
            hu[2:-2, 2:-2] += (0.5 * r.standard_normal((ny, nx))).astype(np.float32)
            s.upload(eta, hu, hv)
            out.append(s)
        return out

    ML = [level(*grids[0], Nes[0])]
    for l in (1, 2):
        ML.append([level(*grids[l], Nes[l]), level(*grids[l - 1], Nes[l])])
    mlens = MultiLevelOceanEnsemble(ML)
    state = mlens.download()
    vel = mlens.downloadVelocities()
    for quantity, ml_state, est_fn in (("state", state, mlens.estimate), ("velocity", vel, mlens.estimateVelocity)):
        for func, kw in ((np.mean, {}), (np.var, {"ddof": 1})):
            got = est_fn(func, **kw)
            assert got.dtype == np.float64 and got.shape == ml_state[-1][0].shape[:-1]
            # level statistics as the device computed them, assembled by the reference formula
            which = "mean" if func is np.mean else "var"
            lv = []
            for g_idx, grp in enumerate(mlens._groups()):
                def dev(first, n):
                    m, v = mlens.engine.moments(first, n, quantity=quantity, ddof=kw.get("ddof", 0))
                    return m if which == "mean" else v
                lv.append(dev(*grp) if g_idx == 0 else (dev(*grp[0]), dev(*grp[1])))
            np.testing.assert_array_equal(got, eso.ml_estimate(lv))
            # and the FP64 oracle on the downloaded states
            ref = mlens._estimate_pure(
                [np.asarray(ml_state[0], np.float64)] +
                [[np.asarray(a, np.float64) for a in ml_state[l]] for l in (1, 2)], func, **kw)
            assert _close(got, ref, 2e-5)
    mlens.cleanUp()


def test_noise_ensemble_observe_particles(gpu_ctx):
    """OceanNoiseEnsemble.observeParticles (both paths, with innovation)
    against the oracle's restatement of the reference's CPU path."""
    from gpuocean_gb300.ensembles.OceanNoiseEnsemble import OceanNoiseEnsemble, ObservationType
    sim = _member(gpu_ctx, 64, 40, (1, 2, 1, 2), 3)
    sim.updateDt()
    ens = OceanNoiseEnsemble(gpu_ctx, 5, sim, num_drifters=12, observation_type=ObservationType.UnderlyingFlow)
    ens.step(300.0, stochastic_particles=False, stochastic_truth=False)
    obs = ens.observeTrueState()
    states = np.stack([np.stack([np.asarray(a, np.float32) for a in ens.downloadParticleOceanState(p)])
                       for p in range(5)])
    dx, dy = float(ens.dx), float(ens.dy)
    np.testing.assert_array_equal(ens.observeParticles(observations=obs), eso.observe_particles(states, obs, dx, dy))
    np.testing.assert_allclose(ens.observeParticles(innovation=True, observations=obs),
                               eso.observe_particles(states, obs, dx, dy, innovation=True,
                                                     mean_depth=ens.mean_depth), rtol=0, atol=1e-12)
    truth_pos = ens.particles[ens.obs_index].drifters.getDrifterPositions()
    gpu = ens.observeParticles(gpu=True)
    for p in range(5):
        pad = [np.asarray(a, np.float32) for a in ens.particles[p].download()]
        np.testing.assert_array_equal(gpu[p], eso.observe_underlying_flow(pad[1], pad[2], truth_pos, dx, dy))
    m = ens.estimate(np.mean)
    assert _close(m, eso.moments(states)[0], 2e-6)
    ens.cleanUp()
