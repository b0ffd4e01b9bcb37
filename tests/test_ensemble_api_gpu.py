"""The ensemble API the data-assimilation layer calls, on the GPU: a truth
and particles stepped with different stochastic flags or on their own,
resampling, particle weights and ensemble statistics, against plain
simulators and the oracle's restatement of the reference's methods."""
import numpy as np
import pytest

from oracle import ensemble_api_oracle as oa

pytestmark = pytest.mark.gpu


def _base_sim(ctx, with_noise=True):
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils import BenchmarkCases, Common
    c = BenchmarkCases.double_jet_case(nx=64, ny=40, dx=20000.0, dy=20000.0, seed=4)
    sim = CDKLM16.CDKLM16(ctx, c["eta0"], c["hu0"], c["hv0"], c["H"], 64, 40, c["dx"], c["dy"], 0.0, c["g"],
                          c["f"], 0.0, coriolis_beta=c["coriolis_beta"],
                          boundary_conditions=Common.BoundaryConditions(1, 2, 1, 2))
    sim.updateDt()
    if with_noise:
        sim.setSOARModelError(small_scale_perturbation_amplitude=2e-4, small_scale_perturbation_interpolation_factor=1)
    return sim, c


def _ensemble(ctx, n=5, obs=None):
    from gpuocean_gb300.ensembles.OceanNoiseEnsemble import ObservationType, OceanNoiseEnsemble
    sim, c = _base_sim(ctx)
    np.random.seed(3)
    ens = OceanNoiseEnsemble(ctx, n, sim, num_drifters=3,
                             observation_type=ObservationType.DirectUnderlyingFlow if obs is None else obs)
    return ens, sim, c


def _interior(sim):
    return [np.asarray(a).copy() for a in sim.download(interior_domain_only=True)]


def _plain_like(ctx, ens, sim):
    """A simulator without model error built as the ensemble builds its
    members (the base simulator's state and corner depths, its f before the
    constructor's compensation)."""
    from gpuocean_gb300.SWEsimulators import CDKLM16
    eta, hu, hv = sim.download()
    Hi = sim.downloadBathymetry()[0]
    f_in = float(sim.f) + float(sim.coriolis_beta) * 2 * float(sim.dy)
    return CDKLM16.CDKLM16(ctx, eta, hu, hv, Hi, ens.nx, ens.ny, ens.dx, ens.dy, ens.dt, ens.g, f_in, ens.r,
                           coriolis_beta=ens.beta, boundary_conditions=ens.boundaryConditions)


@pytest.mark.parametrize("particles,truth", [(True, False), (False, True)])
def test_truth_and_particles_with_different_flags(gpu_ctx, particles, truth):
    """Deterministic members equal a plain simulator stepped on its own;
    stochastic ones do not."""
    ens, sim, _ = _ensemble(gpu_ctx)
    plain = _plain_like(gpu_ctx, ens, sim)
    ens.step(300.0, stochastic_particles=particles, stochastic_truth=truth)
    plain.step(300.0)
    ref = _interior(plain)
    truth_state = _interior(ens.particles[ens.obs_index])
    part_state = _interior(ens.particles[0])
    assert all(np.array_equal(a, b) for a, b in zip(truth_state if not truth else part_state, ref))
    assert not np.array_equal((part_state if particles else truth_state)[0], ref[0])
    assert ens.t == ens.particles[ens.obs_index].t == ens.particles[0].t == pytest.approx(300.0)
    ens.cleanUp()


def test_step_truth_and_particles_separately(gpu_ctx):
    ens, sim, _ = _ensemble(gpu_ctx)
    plain = _plain_like(gpu_ctx, ens, sim)
    t = ens.step_truth(120.0, stochastic=False)
    assert t == pytest.approx(120.0)
    assert ens.particles[0].t == 0.0
    plain.step(120.0)
    assert all(np.array_equal(a, b) for a, b in zip(_interior(ens.particles[ens.obs_index]), _interior(plain)))
    ens.step_particles(120.0, stochastic=True)
    assert all(p.t == pytest.approx(120.0) for p in ens.particles)
    assert not np.array_equal(_interior(ens.particles[0])[0], _interior(plain)[0])
    ens.cleanUp()


def test_resample_copies_states_and_places_drifters(gpu_ctx):
    ens, sim, _ = _ensemble(gpu_ctx, n=4)
    ens.step(180.0)
    before = [(np.array(p.download()), np.array(p.downloadPrevTimestep())) for p in ens.particles[:4]]
    truth_pos = ens.observeTrueDrifters()
    idx = [2, 2, 0, 1]
    ens.resample(idx, 0.0)
    for i, src in enumerate(idx):
        now, prev = np.array(ens.particles[i].download()), np.array(ens.particles[i].downloadPrevTimestep())
        assert np.array_equal(now, before[src][0]) and np.array_equal(prev, before[src][1])
        assert np.array_equal(ens.particles[i].drifters.getDrifterPositions(), truth_pos)
    # the ensemble keeps stepping from the copies
    ens.step(60.0)
    assert np.isfinite(_interior(ens.particles[0])[0]).all()
    ens.cleanUp()


def test_weights_and_statistics_against_oracle(gpu_ctx):
    ens, sim, c = _ensemble(gpu_ctx, n=6)
    ens.step(600.0)
    n = ens.getNumParticles()
    states = [np.array(ens.downloadParticleOceanState(p), dtype=np.float64) for p in range(n)]
    truth = np.array(ens.downloadTrueOceanState(), dtype=np.float64)

    # innovations, norms, Gaussian weights
    np.random.seed(5)
    obs = ens.observeTrueState()
    inn = ens.getInnovations(observations=obs)
    assert inn.shape == (n, 3, 2)
    np.testing.assert_allclose(ens.getInnovationNorms(observations=obs), oa.innovation_norms(inn), rtol=1e-12)
    ens.particlesActive[2] = False
    w = ens.getGaussianWeight(innovations=inn)
    np.testing.assert_allclose(w, oa.gaussian_weight(inn, ens.getObservationCov(), ens.particlesActive), rtol=1e-10)
    assert w[2] == 0.0 and w.sum() == pytest.approx(1.0)
    ens.particlesActive[2] = True
    d = ens.getDistances()
    np.testing.assert_allclose(ens.getCauchyWeight(), oa.cauchy_weight(d, ens.getObservationVariance()), rtol=1e-12)

    # mean, distance to the truth and spread ratio per cell
    fields = np.array(ens.downloadEnsembleStatisticalFields(), dtype=np.float64)
    want = oa.statistical_fields(truth, np.array(states))
    np.testing.assert_allclose(fields[:3], want[:3], rtol=1e-5, atol=1e-6 * np.abs(want[:3]).max())
    np.testing.assert_allclose(fields[3:6], want[3:6], rtol=1e-4, atol=1e-5 * np.abs(want[:3]).max())
    ok = want[3:6] > 1e-3 * np.abs(want[:3]).max()
    np.testing.assert_allclose(fields[6:][ok], want[6:][ok], rtol=1e-3)

    # statistics under the first true drifter
    np.random.seed(6)
    ens.getEnsembleVarAndRMSEUnderDrifter(600.0)
    np.random.seed(6)
    pos = ens.observeTrueState()[0][0:2]
    ix, iy = int(np.floor(pos[0] / ens.dx)), int(np.floor(pos[1] / ens.dy))
    vals = np.array([s[:, iy, ix] for s in states])
    want = oa.under_drifter(truth[:, iy, ix], vals)
    got = [getattr(ens, name + q)[-1] for name in ("varianceUnderDrifter_", "rmseUnderDrifter_",
                                                  "rmseMeanUnderDrifter_", "rmseWeightedUnderDrifter_",
                                                  "rUnderDrifter_") for q in ("eta", "hu", "hv")]
    np.testing.assert_allclose(got, want, rtol=1e-6)
    assert ens.tArray[-1] == 600.0

    # largest stable time step over all members (interior cells)
    full = [np.array(p.download(), dtype=np.float64) for p in ens.particles]
    Hi = np.asarray(ens.particles[0].downloadBathymetry()[0], dtype=np.float64)
    want_dt = oa.largest_timestep(full, Hi, float(ens.g), float(ens.dx), float(ens.dy), interior=True)
    assert ens.findLargestPossibleTimeStep() == pytest.approx(want_dt, rel=1e-5)
    ens.cleanUp()


def test_multilevel_step_to_observation_with_drifters(gpu_ctx):
    """The multi-level ensemble steps to an observation as the reference does
    (every member's dataAssimilationStep, coarse partners as otherSim, in
    stretches of drift_dt): the batched states equal member-by-member
    dataAssimilationStep calls bit for bit, and the multi-level drifters move
    with the device estimates after every stretch."""
    from gpuocean_gb300.ensembles.MultiLevelOceanEnsemble import MultiLevelOceanEnsemble
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils import BenchmarkCases, Common
    lv = [BenchmarkCases.double_jet_case(nx=32, ny=20, dx=40000.0, dy=40000.0),
          BenchmarkCases.double_jet_case(nx=64, ny=40, dx=20000.0, dy=20000.0)]

    def mk(cc):
        return CDKLM16.CDKLM16(gpu_ctx, cc["eta0"], cc["hu0"], cc["hv0"], cc["H"], cc["nx"], cc["ny"], cc["dx"],
                               cc["dy"], 0.0, cc["g"], cc["f"], 0.0, coriolis_beta=cc["coriolis_beta"],
                               boundary_conditions=Common.BoundaryConditions(2, 2, 2, 2), model_time_step=60.0)

    def levels():
        return [[mk(lv[0]) for _ in range(3)], [[mk(lv[1]) for _ in range(2)], [mk(lv[0]) for _ in range(2)]]]

    class Quiet:
        """Stands in for a model error that adds nothing: the reference's
        dataAssimilationStep with a coarse partner calls perturbSimilarAs,
        which needs one."""
        def perturbSim(self, sim, **kw):
            pass

        def perturbSimSimilarAs(self, sim, **kw):
            pass

    ml_sims, twin = levels(), levels()
    for s in twin[1][0] + twin[1][1]:
        s.model_error = Quiet()
    ml = MultiLevelOceanEnsemble(ml_sims)
    np.random.seed(9)
    start = np.array([[300e3, 400e3], [900e3, 200e3]])
    ml.attachDrifters(4, drifterPositions=start, drift_dt=120)
    ml.stepToObservation(600.0)
    for end in (120.0, 240.0, 360.0, 480.0, 600.0):
        for s in twin[0]:
            s.dataAssimilationStep(end)
        for f, c in zip(*twin[1]):
            f.dataAssimilationStep(end, otherSim=c)
    flat_twin = twin[0] + twin[1][0] + twin[1][1]
    for a, b in zip(ml.members, flat_twin):
        assert a.t == pytest.approx(600.0) and a.t == b.t and a.num_iterations == b.num_iterations
        assert all(np.array_equal(x, y) for x, y in zip(_interior(a), _interior(b)))
        assert a.dt == b.dt
    tr = ml.driftTrajectory[0]
    assert tr.get_num_observations() == 1
    pos = ml.drifters.getDrifterPositions()
    assert pos.shape == (2 * 4, 2) and np.all(np.isfinite(pos))
    # the realisations moved (by the slow double-jet currents: metres over
    # ten minutes, so no tolerance of allclose applies)
    assert not np.array_equal(ml.drifters.getDrifterPositionsForDrifter(0), np.repeat(start[:1], 4, axis=0))
    ml.registerDrifterPositions()
    assert ml.driftTrajectory[3].get_num_observations() == 2
    ml.cleanUp()
