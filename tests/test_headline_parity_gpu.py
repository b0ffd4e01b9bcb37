"""Parity of the batched engine at the benchmark's own sizes.

The benchmark's number comes from the batched engine on 512 x 300 members
(periodic in x, walls in y, beta plane, shared random bathymetry, SOAR model
error at coarse factor 8 every 60 s, 1000 drifters per member) and on the
multi-level ensemble (64 x 128, 128 x 256, 256 x 512 members of one domain).
These tests step exactly those configurations - strips of 19 tile rows in
runs of up to 8 tiles handing over stage-1 rows, the partial last tile row
(300 = 18 x 16 + 12), TMA staging over long runs, shared bathymetry and
Coriolis tables, factor-8 noise, 1000 drifters - through the engine (CUDA
graph, autotuned tile shape) and member by member through the plain
simulators, and require bit-identical states and drifter positions; and one
such member against the reference's own kernels for 40 blocks.

Normals are injected (the same draws on both sides), so the comparison does
not depend on a random-number generator.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NOISE_FACTOR = 8
MODEL_TIME_STEP = 60.0


def _soar_q0(L_cells=8.0, std=0.003):
    oy, ox = np.mgrid[-2:3, -2:3]
    d = np.sqrt(ox ** 2 + oy ** 2) / L_cells
    return std / np.sqrt(np.sum(((1 + d) * np.exp(-d)) ** 2))


def _member(ctx, case, m, n_drifters):
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.SWEsimulators.OceanStateNoise import OceanStateNoise
    from gpuocean_gb300.drifters import GPUDrifterCollection
    from gpuocean_gb300.utils import Common
    bc = Common.BoundaryConditions(*case["boundary"])
    sim = CDKLM16.CDKLM16(ctx, case["eta0"], case["hu0"], case["hv0"], case["H"], case["nx"], case["ny"],
                          case["dx"], case["dy"], 0.0, case["g"], case["f"], 0.0,
                          coriolis_beta=case["coriolis_beta"], boundary_conditions=bc,
                          model_time_step=MODEL_TIME_STEP)
    if n_drifters:
        Lx, Ly = case["nx"] * case["dx"], case["ny"] * case["dy"]
        rng = np.random.default_rng(5000 + m)
        d = GPUDrifterCollection.GPUDrifterCollection(ctx, n_drifters, boundaryConditions=bc, domain_size_x=Lx,
                                                      domain_size_y=Ly, gpu_stream=sim.gpu_stream)
        d.setDrifterPositions(np.stack([rng.uniform(0, Lx, n_drifters), rng.uniform(0, Ly, n_drifters)], axis=1))
        d.setObservationPosition(np.array([0.5 * Lx, 0.5 * Ly]))
        sim.attachDrifters(d)
    cdx = case["dx"] * NOISE_FACTOR
    sim.model_error = OceanStateNoise.fromsim(sim, soar_q0=_soar_q0(), soar_L=8.0 * cdx,
                                              interpolation_factor=NOISE_FACTOR, strict_odd_factor=False)
    return sim


def _inject(pairs, block):
    """The same N(0, 1) random field into both copies of every member."""
    for m, (a, b) in enumerate(pairs):
        n = a.model_error
        xi = np.random.default_rng(1000 + m + 7919 * block).standard_normal(
            (int(n.rand_ny), int(n.rand_nx))).astype(np.float32)
        a.model_error.setRandomNumbers(xi)
        b.model_error.setRandomNumbers(xi)


def _assert_identical(a, b):
    for sa, sb in zip(a, b):
        assert sa.t == sb.t and sa.num_iterations == sb.num_iterations
        for x, y in zip(sa.download(), sb.download()):
            assert np.array_equal(np.asarray(x)[2:-2, 2:-2], np.asarray(y)[2:-2, 2:-2])
        if sa.hasDrifters:
            assert np.array_equal(sa.drifters.getDrifterPositions(), sb.drifters.getDrifterPositions())
            assert np.array_equal(sa.drifters.getObservationPosition(), sb.drifters.getObservationPosition())


def _run_pairs(ens, a, b, blocks, cadence="block"):
    """`blocks` 60 s blocks with model error on both sides; dt recomputed at
    the start and after every fifth block, as dataAssimilationStep does."""
    ens.updateDt(courant_number=0.8)
    for s in b:
        s.updateDt(courant_number=0.8)
    for blk in range(blocks):
        _inject(list(zip(a, b)), blk)
        ens.step(MODEL_TIME_STEP, apply_stochastic_term=True, noise_cadence=cadence)
        for s in b:
            if cadence == "block":
                s.step(MODEL_TIME_STEP, apply_stochastic_term=False)
                s.perturbState(update_random_field=False)
            else:
                s.step(MODEL_TIME_STEP, apply_stochastic_term=True)
        if (blk + 1) % 5 == 0:
            ens.updateDt(courant_number=0.8)
            for s in b:
                s.updateDt(courant_number=0.8)
    ens.synchronize()


def test_c3_members_batched_equal_member_by_member(gpu_ctx):
    """Eight benchmark members (512 x 300, 1000 drifters each, SOAR factor 8
    after every 60 s block) for 12 blocks: engine and plain simulators agree
    bit for bit on every interior cell and every drifter."""
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    from gpuocean_gb300.utils.BenchmarkCases import double_jet_case
    case = double_jet_case()
    a = [_member(gpu_ctx, case, m, 1000) for m in range(8)]
    b = [_member(gpu_ctx, case, m, 1000) for m in range(8)]
    ens = BatchedEnsemble(a)   # CUDA graph, autotuned tile shape
    ens.set_noise([s.model_error for s in a])
    assert ens._bathy_owner == [0] * 8 and ens._coriolis_owner == [0] * 8
    _run_pairs(ens, a, b, blocks=12)
    assert a[0].num_iterations >= 40
    _assert_identical(a, b)
    staged, tiles, errors = ens.tma_status()
    assert staged == 8 and tiles > 0 and errors == 0
    ens.release()


def test_c3_members_step_cadence(gpu_ctx, monkeypatch):
    """The CDKLM16.step cadence (model error after every RK2 step, before the
    drifters move; OceanNoiseEnsemble.step) on four benchmark members."""
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils.BenchmarkCases import double_jet_case
    case = double_jet_case()
    a = [_member(gpu_ctx, case, m, 1000) for m in range(4)]
    b = [_member(gpu_ctx, case, m, 1000) for m in range(4)]
    orig = CDKLM16.CDKLM16.perturbState
    monkeypatch.setattr(CDKLM16.CDKLM16, "perturbState", lambda self, **kw: orig(self, update_random_field=False))
    ens = BatchedEnsemble(a)
    ens.set_noise([s.model_error for s in a])
    _run_pairs(ens, a, b, blocks=3, cadence="step")
    _assert_identical(a, b)
    ens.release()


def test_c4_levels_batched_equal_member_by_member(gpu_ctx):
    """Two members of each multi-level grid (64 x 128, 128 x 256, 256 x 512
    cells of one 2560 km x 1500 km domain: different dt, so members take
    different numbers of steps per block) in one engine, 6 blocks with SOAR
    factor 8 and 200 drifters per member."""
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    from gpuocean_gb300.utils.BenchmarkCases import double_jet_case
    a, b = [], []
    m = 0
    for nx, ny in ((128, 64), (256, 128), (512, 256)):
        c = double_jet_case(nx=nx, ny=ny, dx=2560e3 / nx, dy=1500e3 / ny)
        for _ in range(2):
            a.append(_member(gpu_ctx, c, m, 200))
            b.append(_member(gpu_ctx, c, m, 200))
            m += 1
    ens = BatchedEnsemble(a)
    ens.set_noise([s.model_error for s in a])
    _run_pairs(ens, a, b, blocks=6)
    assert len({s.num_iterations for s in a}) > 1
    _assert_identical(a, b)
    ens.release()


def test_c3_member_40_blocks_against_reference_kernels(gpu_ctx):
    """One benchmark member through the batched engine for 40 blocks (160
    RK2 steps, 1000 drifters, SOAR factor 8 after every block on injected
    normals) against the reference's own kernels replaying
    dataAssimilationStep: step(60 s) with the drifters after every step,
    then perturbState.  The reference refreshes no ghost cells after that
    perturbation, so its next first stage would read pre-perturbation
    periodic images; the replay refreshes them (this package's step reads
    periodic neighbours from the interior and never sees stale images).

    The RK2 step is bit-identical to the reference's; the transfer of the
    SOAR field agrees to 2e-5 of each perturbation (fast-math there, no FMA
    contraction here).  40 such transfers bound the difference by 40 x 2e-5
    = 8e-4 of one perturbation; 40 independent perturbations spread the
    state by about sqrt(40) ~ 6 perturbations, so about 1.3e-4 of that
    spread (the reference with the same draws against the reference without
    model error); the test allows 2e-4 for the dynamics to carry the
    differences along."""
    from oracle import ref_kernels as rk
    if not rk.available():
        pytest.skip("reference kernels not built (no reference sources)")
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    from gpuocean_gb300.utils.BenchmarkCases import double_jet_case
    case = double_jet_case()
    sim = _member(gpu_ctx, case, 0, 1000)
    sim.updateDt(courant_number=0.8)
    dt = float(sim.dt)
    ref = rk.RefCDKLM16("cdklm_jet512", case["eta0"], case["hu0"], case["hv0"], case["H"], case["nx"], case["ny"],
                        case["dx"], case["dy"], dt, case["g"], sim.f, 0.0,
                        sim.coriolis_f_arr.download(sim.gpu_stream), sim.angle_arr.download(sim.gpu_stream),
                        bc=case["boundary"], beta=case["coriolis_beta"])
    q0, L = _soar_q0(), 8.0 * case["dx"] * NOISE_FACTOR
    rnoise = rk.RefNoise("noise_jet512", ref, q0, L, interpolation_factor=NOISE_FACTOR)
    pos = np.concatenate([sim.drifters.getDrifterPositions(), sim.drifters.getObservationPosition()[None, :]])
    Lx, Ly = case["nx"] * case["dx"], case["ny"] * case["dy"]
    rdrift = rk.RefDrifters(pos.astype(np.float32), Lx, Ly, 0, 1)
    quiet = rk.RefCDKLM16("cdklm_jet512", case["eta0"], case["hu0"], case["hv0"], case["H"], case["nx"],
                          case["ny"], case["dx"], case["dy"], dt, case["g"], sim.f, 0.0,
                          sim.coriolis_f_arr.download(sim.gpu_stream), sim.angle_arr.download(sim.gpu_stream),
                          bc=case["boundary"], beta=case["coriolis_beta"])
    ens = BatchedEnsemble([sim])
    ens.set_noise([sim.model_error])
    for blk in range(40):
        xi = np.random.default_rng(1000 + 7919 * blk).standard_normal(
            (rnoise.rand_ny, rnoise.rand_nx)).astype(np.float32)
        sim.model_error.setRandomNumbers(xi)
        ens.step(MODEL_TIME_STEP, apply_stochastic_term=True)
        ref.step(MODEL_TIME_STEP, drifters=rdrift)
        rnoise.set_random(xi)
        rnoise.perturb(ref)
        ref._boundary(ref.h0)
        quiet.step(MODEL_TIME_STEP)
    ens.synchronize()
    assert sim.num_iterations == ref.num_iterations >= 160
    mine = [np.asarray(x)[2:-2, 2:-2].astype(np.float64) for x in sim.download()]
    theirs = [np.asarray(x)[2:-2, 2:-2].astype(np.float64) for x in ref.download()]
    calm = [np.asarray(x)[2:-2, 2:-2].astype(np.float64) for x in quiet.download()]
    diff = [float(np.max(np.abs(x - y))) for x, y in zip(mine, theirs)]
    spread = [float(np.max(np.abs(x - y))) for x, y in zip(theirs, calm)]
    dpos = float(np.max(np.abs(np.asarray(sim.drifters.getDrifterPositions()) - rdrift.positions()[:-1])))
    print({"case": "C3 member, 40 blocks vs reference kernels", "max_abs_diff": diff,
           "perturbation_spread": spread, "max_abs_drifter_diff_m": dpos})
    for d, sp in zip(diff, spread):
        assert sp > 0 and d <= 2e-4 * sp, (diff, spread)
    assert dpos <= 1e-6 * max(Lx, Ly)
    ens.release()
    quiet.free()
    rdrift.free()
    rnoise.free()
    ref.free()
