"""The batched ensemble engine against member-by-member stepping."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _member(ctx, nx, ny, bc, seed, drifters=0):
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.drifters import GPUDrifterCollection
    from gpuocean_gb300.utils import BenchmarkCases, Common
    c = BenchmarkCases.double_jet_case(nx=nx, ny=ny, dx=5000.0, dy=5000.0, seed=seed)
    b = Common.BoundaryConditions(*bc)
    sim = CDKLM16.CDKLM16(ctx, c["eta0"], c["hu0"], c["hv0"], c["H"], nx, ny, c["dx"], c["dy"], 0.0, c["g"],
                          c["f"], 0.0, coriolis_beta=c["coriolis_beta"], boundary_conditions=b)
    if drifters:
        rng = np.random.default_rng(seed)
        d = GPUDrifterCollection.GPUDrifterCollection(ctx, drifters, boundaryConditions=b,
                                                      domain_size_x=nx * c["dx"], domain_size_y=ny * c["dy"],
                                                      gpu_stream=sim.gpu_stream)
        d.setDrifterPositions(np.stack([rng.uniform(0, nx * c["dx"], drifters),
                                        rng.uniform(0, ny * c["dy"], drifters)], axis=1))
        d.setObservationPosition(np.array([nx * c["dx"] / 3, ny * c["dy"] / 3]))
        sim.attachDrifters(d)
    return sim


SPECS = [(64, 40, (1, 2, 1, 2), 3), (33, 17, (1, 1, 1, 1), 4), (48, 48, (2, 2, 2, 2), 5), (128, 64, (2, 1, 2, 1), 6)]


@pytest.mark.parametrize("use_graph", [False, True])
def test_batched_equals_member_by_member(gpu_ctx, use_graph):
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    a = [_member(gpu_ctx, *s, drifters=50) for s in SPECS]
    b = [_member(gpu_ctx, *s, drifters=50) for s in SPECS]
    for s in a + b:
        s.updateDt()
    ens = BatchedEnsemble(a, use_graph=use_graph)
    for _ in range(4):
        ens.step(60.0)
        for s in b:
            s.step(60.0)
    ens.synchronize()
    for sa, sb in zip(a, b):
        assert sa.t == sb.t and sa.num_iterations == sb.num_iterations
        for x, y in zip(sa.download(), sb.download()):
            xi, yi = np.asarray(x)[2:-2, 2:-2], np.asarray(y)[2:-2, 2:-2]
            assert np.array_equal(xi, yi)
        assert np.array_equal(sa.drifters.getDrifterPositions(), sb.drifters.getDrifterPositions())
        assert np.array_equal(sa.drifters.getObservationPosition(), sb.drifters.getObservationPosition())


def test_tma_staging_status(gpu_ctx):
    """Members whose buffers and row pitch sit on 16-byte boundaries stage
    their interior tiles by TMA (33x17 has a 148-byte pitch: ordinary loads);
    no staging wait runs out.  Results are covered by the bit-identity test
    above, whose 128x64 member has interior tiles in runs of two."""
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    a = [_member(gpu_ctx, *s) for s in SPECS]
    ens = BatchedEnsemble(a, autotune=False)
    ens.set_tile_shape(0)  # 32x16
    assert ens.tile_shape == (32, 16)
    for _ in range(2):
        ens.step(60.0)
    ens.synchronize()
    staged, tiles, errors = ens.tma_status()
    assert staged == 3
    # interior 32x16 tiles: 2 x 2 of the 128x64 member per RK2 step (none
    # on the smaller grids), at least one step per 60 s block
    assert tiles >= 2 * 4
    assert errors == 0


def test_staging_wait_gives_up(gpu_ctx):
    """The wait that guards TMA staging is bounded by the GPU's clock: on a
    barrier phase that nothing completes it gives up after its limit and says
    so, and the context stays usable (a step runs afterwards)."""
    import ctypes
    from gpuocean_gb300 import _lib
    timed_out, waited = ctypes.c_int(), ctypes.c_double()
    _lib.call("goc_selftest_wait_timeout", ctypes.c_double(5.0), ctypes.byref(timed_out), ctypes.byref(waited))
    assert timed_out.value == 1
    assert 5.0 <= waited.value < 1000.0
    sim = _member(gpu_ctx, 64, 40, (1, 2, 1, 2), 3)
    sim.step(60.0)
    assert np.isfinite(np.asarray(sim.download()[0])).all()


def test_batched_dt_matches_single(gpu_ctx):
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    a = [_member(gpu_ctx, *s) for s in SPECS]
    ens = BatchedEnsemble(a)
    dts = ens.updateDt(courant_number=0.8)
    for s, v in zip(a, dts):
        assert np.float32(v) == np.float32(s.downloadMaxDt())


def test_member_counts_and_shared_bathymetry(gpu_ctx):
    """Identical corner depths and identical beta-plane Coriolis tables are
    read from one copy; the shared tables give the members' own results."""
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    spec = [(128, 64, (1, 2, 1, 2), 3)] * 3 + [(128, 64, (1, 2, 1, 2), 9)]
    a = [_member(gpu_ctx, *s) for s in spec]
    b = [_member(gpu_ctx, *s) for s in spec]
    ens = BatchedEnsemble(a)
    assert ens._bathy_owner == [0, 0, 0, 3]
    assert ens._coriolis_owner == [0, 0, 0, 0]
    tx, ty = ens.tile_shape
    assert ens.n_tiles == 4 * ((128 + tx - 1) // tx) * ((64 + ty - 1) // ty)
    for s in a + b:
        s.updateDt()
    for _ in range(2):
        ens.step(60.0)
        for s in b:
            s.step(60.0)
    ens.synchronize()
    for sa, sb in zip(a, b):
        for x, y in zip(sa.download(), sb.download()):
            assert np.array_equal(np.asarray(x)[2:-2, 2:-2], np.asarray(y)[2:-2, 2:-2])


def _with_noise(sims, factor, seed):
    rng = np.random.default_rng(seed)
    for s in sims:
        s.setSOARModelError(small_scale_perturbation_amplitude=1e-3, small_scale_perturbation_interpolation_factor=factor)
    xis = []
    for s in sims:
        n = s.model_error
        xi = rng.standard_normal((n.rand_ny, n.rand_nx)).astype(np.float32)
        n.setRandomNumbers(xi)
        xis.append(xi)
    return xis


@pytest.mark.parametrize("factor", [1, 3])
def test_batched_noise_block_cadence_equals_member_by_member(gpu_ctx, factor):
    """dataAssimilationStep cadence: block of steps, then one perturbation."""
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    specs = [(48, 30, (1, 2, 1, 2), 3), (24, 42, (1, 1, 1, 1), 4), (36, 36, (2, 2, 2, 2), 5)]
    a = [_member(gpu_ctx, *s, drifters=20) for s in specs]
    b = [_member(gpu_ctx, *s, drifters=20) for s in specs]
    xa, xb = _with_noise(a, factor, 1), _with_noise(b, factor, 1)
    for s in a + b:
        s.updateDt()
    ens = BatchedEnsemble(a)
    ens.set_noise([s.model_error for s in a])  # injected random fields, no device RNG
    for _ in range(3):
        ens.step(60.0, apply_stochastic_term=True)
        for s in b:
            s.step(60.0, apply_stochastic_term=False)
            s.perturbState(update_random_field=False)
    ens.synchronize()
    for sa, sb in zip(a, b):
        for x, y in zip(sa.download(), sb.download()):
            assert np.array_equal(np.asarray(x)[2:-2, 2:-2], np.asarray(y)[2:-2, 2:-2])
        assert np.array_equal(sa.drifters.getDrifterPositions(), sb.drifters.getDrifterPositions())


def test_batched_noise_step_cadence_equals_member_by_member(gpu_ctx, monkeypatch):
    """CDKLM16.step cadence: perturbation after every RK2 step, before drift."""
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    from gpuocean_gb300.SWEsimulators import CDKLM16
    specs = [(48, 30, (1, 2, 1, 2), 3), (24, 42, (1, 1, 1, 1), 4)]
    a = [_member(gpu_ctx, *s, drifters=20) for s in specs]
    b = [_member(gpu_ctx, *s, drifters=20) for s in specs]
    _with_noise(a, 1, 2), _with_noise(b, 1, 2)
    for s in a + b:
        s.updateDt()
    orig = CDKLM16.CDKLM16.perturbState
    monkeypatch.setattr(CDKLM16.CDKLM16, "perturbState",
                        lambda self, **kw: orig(self, update_random_field=False))
    ens = BatchedEnsemble(a)
    ens.set_noise([s.model_error for s in a])
    for _ in range(2):
        ens.step(60.0, apply_stochastic_term=True, noise_cadence="step")
        for s in b:
            s.step(60.0, apply_stochastic_term=True)
    ens.synchronize()
    for sa, sb in zip(a, b):
        for x, y in zip(sa.download(), sb.download()):
            assert np.array_equal(np.asarray(x)[2:-2, 2:-2], np.asarray(y)[2:-2, 2:-2])
        assert np.array_equal(sa.drifters.getDrifterPositions(), sb.drifters.getDrifterPositions())


def test_device_rng_noise_statistics(gpu_ctx):
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    a = [_member(gpu_ctx, 48, 30, (1, 2, 1, 2), 3) for _ in range(4)]
    _with_noise(a, 1, 3)
    ens = BatchedEnsemble(a)
    ens.set_noise([s.model_error for s in a], rng_seed=99)
    before = [np.asarray(s.download()[0]) for s in a]
    ens.perturb()
    ens.synchronize()
    xis = [s.model_error.getRandomNumbers() for s in a]
    assert all(abs(x.mean()) < 0.2 and abs(x.std() - 1) < 0.2 for x in xis)
    assert not np.array_equal(xis[0], xis[1])
    after = [np.asarray(s.download()[0]) for s in a]
    assert all(not np.array_equal(x, y) for x, y in zip(before, after))


def test_ensemble_classes_run(gpu_ctx):
    from gpuocean_gb300.ensembles.MultiLevelOceanEnsemble import MultiLevelOceanEnsemble
    from gpuocean_gb300.ensembles.OceanModelEnsemble import OceanModelEnsemble
    from gpuocean_gb300.utils import BenchmarkCases, Common
    c = BenchmarkCases.double_jet_case(nx=64, ny=40)
    sim_args = dict(dt=0.0, g=c["g"], f=c["f"], r=0.0, coriolis_beta=c["coriolis_beta"], model_time_step=60.0)
    data_args = dict(eta0=c["eta0"], hu0=c["hu0"], hv0=c["hv0"], H=c["H"], nx=64, ny=40, dx=c["dx"], dy=c["dy"],
                     boundary_conditions=Common.BoundaryConditions(1, 2, 1, 2))
    ens = OceanModelEnsemble(gpu_ctx, sim_args, data_args, dict(small_scale_perturbation_amplitude=1e-4), 4)
    ens.attachDrifters(np.array([[1e5, 1e5], [2e5, 1e5]]))
    ens.stepToObservation(600.0)
    assert abs(ens.particles[0].t - 600.0) < 1e-6
    obs = ens.observeParticles(np.array([[1e5, 1e5]]))
    assert obs.shape == (4, 1, 2) and np.all(np.isfinite(obs))
    # two-level ensemble with grids of different size in one launch
    lv = [BenchmarkCases.double_jet_case(nx=32, ny=20), BenchmarkCases.double_jet_case(nx=64, ny=40)]

    def mk(cc):
        from gpuocean_gb300.SWEsimulators import CDKLM16
        s = CDKLM16.CDKLM16(gpu_ctx, cc["eta0"], cc["hu0"], cc["hv0"], cc["H"], cc["nx"], cc["ny"], cc["dx"],
                            cc["dy"], 0.0, cc["g"], cc["f"], 0.0, coriolis_beta=cc["coriolis_beta"],
                            boundary_conditions=Common.BoundaryConditions(1, 2, 1, 2), model_time_step=60.0)
        return s
    ml = MultiLevelOceanEnsemble([[mk(lv[0]) for _ in range(3)], [[mk(lv[1]) for _ in range(2)],
                                                                  [mk(lv[0]) for _ in range(2)]]])
    for s in ml.members:
        s.updateDt()
    ml.step(120.0, apply_stochastic_term=False)
    assert all(abs(s.t - 120.0) < 1e-6 for s in ml.members)
    est = ml.estimate(np.mean)
    assert est.shape == (3, 40, 64) and np.all(np.isfinite(est))


def test_ocean_model_ensemble_kl_model_error(gpu_ctx):
    """KL model-error arguments (``kl_scaling`` present) give every particle a
    KL model error, as E/OceanModelEnsemble.py's constructor does; the batched
    engine perturbs all members in its block launches.  Two ensembles with
    the same seed step to identical states, members differ from one another
    and from the unperturbed run."""
    from gpuocean_gb300.ensembles.OceanModelEnsemble import OceanModelEnsemble
    from gpuocean_gb300.SWEsimulators.ModelErrorKL import ModelErrorKL
    from gpuocean_gb300.utils import BenchmarkCases, Common
    c = BenchmarkCases.double_jet_case(nx=64, ny=40)
    sim_args = dict(dt=0.0, g=c["g"], f=c["f"], r=0.0, coriolis_beta=c["coriolis_beta"], model_time_step=60.0)
    data_args = dict(eta0=c["eta0"], hu0=c["hu0"], hv0=c["hv0"], H=c["H"], nx=64, ny=40, dx=c["dx"], dy=c["dy"],
                     boundary_conditions=Common.BoundaryConditions(1, 2, 1, 2))
    kl = dict(kl_decay=1.25, kl_scaling=0.025, basis_x_start=2, basis_x_end=8, basis_y_start=1, basis_y_end=7)
    runs = []
    for args in (kl, kl, {}):
        ens = OceanModelEnsemble(gpu_ctx, sim_args, data_args, args, 3, rng_seed=5)
        if args:
            assert all(isinstance(p.model_error, ModelErrorKL) for p in ens.particles)
        ens.stepToObservation(300.0)
        ens.syncGPU()
        assert all(abs(p.t - 300.0) < 1e-6 for p in ens.particles)
        runs.append([np.asarray(p.download()[0]) for p in ens.particles])
        ens.cleanUp()
    assert all(np.array_equal(x, y) for x, y in zip(runs[0], runs[1]))
    assert all(np.all(np.isfinite(x)) for x in runs[0])
    assert not np.array_equal(runs[0][0], runs[0][1])
    assert all(not np.array_equal(x, y) for x, y in zip(runs[0], runs[2]))


def test_ocean_model_ensemble_sponge_members_step_one_by_one(gpu_ctx):
    """Particles with sponge boundaries (not taken by the batched engine)
    step one by one, each through its own dataAssimilationStep: the states
    equal a lone simulator's and the observation operator reads their hu, hv
    at the drifters' cells (E/OceanModelEnsemble.py:168-198)."""
    from gpuocean_gb300.ensembles.OceanModelEnsemble import OceanModelEnsemble
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils import Common
    nx, ny, dx, dy = 50, 70, 200.0, 200.0
    x = np.arange(nx + 4) - 2 + 0.5 - nx / 2.0
    y = np.arange(ny + 4) - 2 + 0.5 - ny / 2.0
    eta0 = (0.5 * np.exp(-(x[None, :] ** 2 + y[:, None] ** 2) / 50.0)).astype(np.float32)
    z = np.zeros_like(eta0)
    H = np.full((ny + 5, nx + 5), 10.0, np.float32)
    bc = Common.BoundaryConditions(4, 4, 4, 4, spongeCells=dict(north=6, east=6, south=6, west=6))
    sim_args = dict(dt=0.0, g=9.81, f=0.0, r=0.0, model_time_step=60.0)
    data_args = dict(eta0=eta0, hu0=z, hv0=z.copy(), H=H, nx=nx, ny=ny, dx=dx, dy=dy, boundary_conditions=bc)
    ens = OceanModelEnsemble(gpu_ctx, sim_args, data_args, {}, 2)
    ens.stepToObservation(300.0)
    assert ens.engine is False
    lone = CDKLM16.CDKLM16(gpu_ctx, **sim_args, **data_args)
    lone.dataAssimilationStep(300.0)
    want = [np.asarray(a) for a in lone.download()]
    for p in ens.particles:
        assert abs(p.t - 300.0) < 1e-6
        for a, b in zip(p.download(), want):
            assert np.array_equal(np.asarray(a), b)
    pos = np.array([[1234.0, 4321.0], [9000.0, 100.0]])
    obs = ens.observeParticles(pos)
    _, hu, hv = lone.download(interior_domain_only=True)
    jx, jy = (pos[:, 0] // dx).astype(int), (pos[:, 1] // dy).astype(int)
    assert obs.shape == (2, 2, 2)
    assert np.array_equal(obs[1, :, 0], np.asarray(hu)[jy, jx]) and np.array_equal(obs[1, :, 1], np.asarray(hv)[jy, jx])
    assert np.abs(obs).max() > 0
    ens.cleanUp()
    lone.cleanUp()


def test_every_tile_shape_gives_identical_states(gpu_ctx):
    """The autotuner may pick any tile shape: each computes bit-identical
    states (the per-cell arithmetic does not depend on the tiling)."""
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    shapes = BatchedEnsemble.tile_shapes()
    assert len(shapes) >= 3 and shapes[0] == (32, 16)
    results = []
    for idx in range(len(shapes)):
        a = [_member(gpu_ctx, *s, drifters=20) for s in SPECS]
        for s in a:
            s.updateDt()
        ens = BatchedEnsemble(a, autotune=False)
        ens.set_tile_shape(idx)
        assert ens.tile_shape == shapes[idx]
        for _ in range(2):
            ens.step(60.0)
        ens.synchronize()
        results.append([[np.asarray(x)[2:-2, 2:-2] for x in s.download()] for s in a])
        ens.release()
    for r in results[1:]:
        for sa, sb in zip(results[0], r):
            for x, y in zip(sa, sb):
                assert np.array_equal(x, y)


def test_autotune_keeps_the_state_and_picks_a_shape(gpu_ctx):
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble, _AUTOTUNE_CACHE
    a = [_member(gpu_ctx, *s) for s in SPECS]
    before = [[np.asarray(x)[2:-2, 2:-2].copy() for x in s.download()] for s in a]
    _AUTOTUNE_CACHE.clear()
    ens = BatchedEnsemble(a, autotune=True)
    assert ens.tile_shape in BatchedEnsemble.tile_shapes()
    assert set(ens.autotune_timings) == set(BatchedEnsemble.tile_shapes())
    after = [[np.asarray(x)[2:-2, 2:-2] for x in s.download()] for s in a]
    for sa, sb in zip(before, after):
        for x, y in zip(sa, sb):
            assert np.array_equal(x, y)


def test_packed_drifter_transfers(gpu_ctx):
    """download_drifters / upload_observation_positions move every member's
    drifter rows in one launch and one copy, equal to the per-collection
    accessors."""
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    sims = [_member(gpu_ctx, *s, drifters=30 + 7 * i) for i, s in enumerate(SPECS)]
    for s in sims:
        s.updateDt()
    ens = BatchedEnsemble(sims, autotune=False)
    ens.step(120.0)
    rows = ens.download_drifters()
    assert rows.shape == (ens.drifter_rows(), 2) == (sum(31 + 7 * i for i in range(len(SPECS))), 2)
    off = 0
    for s in sims:
        n = s.drifters.getNumDrifters()
        assert np.array_equal(rows[off:off + n], s.drifters.getDrifterPositions())
        assert np.array_equal(rows[off + n], s.drifters.getObservationPosition())
        off += n + 1
    obs = np.random.default_rng(3).uniform(0, 1e5, (len(sims), 2)).astype(np.float32)
    ens.upload_observation_positions(obs)
    ens.synchronize()
    for s, o in zip(sims, obs):
        assert np.array_equal(s.drifters.getObservationPosition(), o)
    ens.release()


def test_batched_wind_drift_equals_member_by_member(gpu_ctx):
    """Drifters with wind drift (3 x 4 wind textures at three time stamps,
    factor 0.02) in the batched engine - moved in launches of their own -
    equal the collections drifted by the plain simulators, bit for bit; the
    members without wind keep drifting inside the step.  Blocks may start or
    end on a wind time stamp (the fourth block starts on one); a block that
    crosses one is refused."""
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    from gpuocean_gb300.drifters import GPUDrifterCollection
    from gpuocean_gb300.utils import WindStress
    rng = np.random.default_rng(8)
    wu = [(5.0 * rng.standard_normal((4, 3))).astype(np.float32) for _ in range(3)]
    wv = [(5.0 * rng.standard_normal((4, 3))).astype(np.float32) for _ in range(3)]

    def members():
        out = []
        for i, spec in enumerate(SPECS[:3]):
            s = _member(gpu_ctx, *spec, drifters=40)
            if i != 1:
                old = s.drifters
                wind = WindStress.WindStress(t=[0.0, 1800.0, 3600.0], wind_u=wu, wind_v=wv)
                d = GPUDrifterCollection.GPUDrifterCollection(
                    gpu_ctx, 40, boundaryConditions=s.boundary_conditions, domain_size_x=old.domain_size_x,
                    domain_size_y=old.domain_size_y, gpu_stream=s.gpu_stream, wind=wind, wind_drift_factor=0.02)
                d.setDrifterPositions(old.getDrifterPositions())
                d.setObservationPosition(old.getObservationPosition())
                s.attachDrifters(d)
            s.updateDt()
            out.append(s)
        return out
    a, b = members(), members()
    ens = BatchedEnsemble(a)
    for _ in range(4):
        ens.step(600.0)
        for s in b:
            s.step(600.0)
    ens.synchronize()
    for sa, sb in zip(a, b):
        assert np.array_equal(sa.drifters.getDrifterPositions(), sb.drifters.getDrifterPositions())
        assert np.array_equal(sa.drifters.getObservationPosition(), sb.drifters.getObservationPosition())
        for x, y in zip(sa.download(), sb.download()):
            assert np.array_equal(np.asarray(x)[2:-2, 2:-2], np.asarray(y)[2:-2, 2:-2])
    with pytest.raises(NotImplementedError):
        ens.step(1800.0)   # 2400 s -> 4200 s would cross the wind's third time stamp
    ens.release()
