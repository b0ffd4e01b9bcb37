"""Parity against the reference's own CUDA kernels (the second oracle).

The reference kernels are compiled from the reference sources into
``oracle/_ref/*.cubin`` (``oracle/build_ref.py``) and driven by
``oracle/ref_kernels.py``, which replays the reference host's launch sequence.
The product runs through its drop-in classes on the same inputs.

The RK2 step is compared bit for bit: the product evaluates the same
operations in the same order, compiled without FMA contraction as the
reference's step kernel is (--fmad=false), so after 1000 steps of the
256 x 256 Gaussian bump (CFL 0.45) and of the 512 x 300 double jet the states
are identical (the stated bound, max|d eta| <= 1e-5 m and max|d hu,hv| <=
1e-4 m^2/s, is met with zero difference).  The transfer of the SOAR field is
fast-math in the reference and built without FMA contraction here (it is
fused into the ensemble step, whose rounding it shares); it is compared
within 2e-5 of the perturbation on identical injected normal draws, and over
40 perturbed steps within 2e-4 of the spread the perturbations create;
drifter positions within 1e-6 of the domain size.  Both runs
get bit-identical inputs: the reference kernels read the Coriolis and angle
textures that the product's host built.
"""
import json
import time

import numpy as np
import pytest

from oracle import ref_kernels as rk

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not rk.available(), reason="reference kernels not built (no reference sources)")]


def _bump256():
    nx = ny = 256
    dx = dy = 200.0
    x = (np.arange(nx + 4) - 2 + 0.5 - nx / 2.0)
    y = (np.arange(ny + 4) - 2 + 0.5 - ny / 2.0)
    eta = (0.1 * np.exp(-(x[None, :] ** 2 + y[:, None] ** 2) / (2.0 * 10.0 ** 2))).astype(np.float32)
    z = np.zeros_like(eta)
    H = np.full((ny + 5, nx + 5), 60.0, np.float32)
    return dict(eta0=eta, hu0=z, hv0=z.copy(), H=H, nx=nx, ny=ny, dx=dx, dy=dy, g=9.81, f=1.2e-4, r=0.0,
                coriolis_beta=0.0, boundary=(1, 1, 1, 1))


def _textures(c, dt):
    from oracle.cdklm16_oracle import BC, OracleCDKLM16
    o = OracleCDKLM16(c["eta0"], c["hu0"], c["hv0"], c["H"], c["nx"], c["ny"], c["dx"], c["dy"], dt, c["g"],
                      c["f"], c["r"], coriolis_beta=c["coriolis_beta"], boundary_conditions=BC(*c["boundary"]))
    return o.ftex, o.angle_tex, o.f


def _product(ctx, c, dt):
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils import Common
    return CDKLM16.CDKLM16(ctx, c["eta0"], c["hu0"], c["hv0"], c["H"], c["nx"], c["ny"], c["dx"], c["dy"], dt,
                           c["g"], c["f"], c["r"], coriolis_beta=c["coriolis_beta"],
                           boundary_conditions=Common.BoundaryConditions(*c["boundary"]))


def _reference(config, c, dt, sim=None):
    """The reference kernels on the inputs of case `c`.  With `sim`, the
    Coriolis and angle textures and the compensated f are the ones the
    product's host computed (the same host arithmetic as S/CDKLM16.py:147-239),
    so that both runs see bit-identical inputs."""
    if sim is not None:
        ftex = sim.coriolis_f_arr.download(sim.gpu_stream)
        angle = sim.angle_arr.download(sim.gpu_stream)
        f = sim.f
    else:
        ftex, angle, f = _textures(c, dt)
    return rk.RefCDKLM16(config, c["eta0"], c["hu0"], c["hv0"], c["H"], c["nx"], c["ny"], c["dx"], c["dy"], dt,
                         c["g"], f, c["r"], ftex, angle, bc=c["boundary"], beta=c["coriolis_beta"])


def _interior(arrs, nx, ny):
    return [np.asarray(a)[2:ny + 2, 2:nx + 2] for a in arrs]


def _diffs(sim, ref, nx, ny):
    mine = _interior(sim.download(), nx, ny)
    theirs = _interior(ref.download(), nx, ny)
    return [float(np.max(np.abs(a.astype(np.float64) - b))) for a, b in zip(mine, theirs)], theirs


@pytest.fixture(scope="module")
def ctx():
    from gpuocean_gb300.utils import Common
    return Common.CUDAContext()


def test_bathymetry_matches_reference_kernels(ctx):
    from gpuocean_gb300.utils.BenchmarkCases import double_jet_case
    c = double_jet_case()
    sim = _product(ctx, c, 1.0)
    ref = _reference("cdklm_jet512", c, 1.0, sim)
    Bi, Bm = sim.downloadBathymetry()
    rBi, rBm = ref.bathymetry()
    np.testing.assert_array_equal(np.asarray(Bm), rBm)
    np.testing.assert_array_equal(np.asarray(Bi), rBi)
    ref.free()
    sim.cleanUp()


def test_bump256_1000_steps_within_stated_tolerance(ctx):
    c = _bump256()
    sim = _product(ctx, c, 0.0)
    sim.updateDt(courant_number=0.45)
    dt = float(sim.dt)
    ref = _reference("cdklm_bump256", c, dt, sim)
    ref_dt = float(np.float32(0.45 * ref.max_dt()))
    assert abs(ref_dt - dt) <= 1e-6 * dt, (ref_dt, dt)
    for _ in range(1000):
        sim.step(dt)
        ref.step(dt)
    (de, dhu, dhv), theirs = _diffs(sim, ref, c["nx"], c["ny"])
    print(json.dumps({"case": "bump256 1000 steps", "dt": dt, "max_abs_diff": [de, dhu, dhv],
                      "max_abs_ref": [float(np.max(np.abs(t))) for t in theirs]}))
    assert de <= 1e-5 and dhu <= 1e-4 and dhv <= 1e-4, (de, dhu, dhv)
    assert de == 0.0 and dhu == 0.0 and dhv == 0.0, "the RK2 step is expected to be bit-identical"
    ref.free()
    sim.cleanUp()


@pytest.mark.parametrize("boundary", [(1, 2, 1, 2), (1, 1, 1, 1)], ids=["periodic_x", "walls"])
def test_double_jet_1000_steps(ctx, boundary):
    from gpuocean_gb300.utils.BenchmarkCases import double_jet_case
    c = double_jet_case()
    c["boundary"] = boundary
    sim = _product(ctx, c, 0.0)
    sim.updateDt(courant_number=0.8)
    dt = float(sim.dt)
    ref = _reference("cdklm_jet512", c, dt, sim)
    for _ in range(1000):
        sim.step(dt)
        ref.step(dt)
    (de, dhu, dhv), theirs = _diffs(sim, ref, c["nx"], c["ny"])
    scale = [float(np.max(np.abs(t))) for t in theirs]
    print(json.dumps({"case": f"double jet 512x300 1000 steps, bc {boundary}", "dt": dt, "max_abs_diff": [de, dhu, dhv],
                      "max_abs_ref": scale}))
    assert de == 0.0 and dhu == 0.0 and dhv == 0.0, (de, dhu, dhv)
    ref.free()
    sim.cleanUp()


def test_friction_odd_grid_random_state(ctx):
    nx, ny = 77, 45
    rng = np.random.default_rng(11)
    H = (40.0 + 10.0 * rng.random((ny + 5, nx + 5))).astype(np.float32)
    eta = (0.3 * rng.standard_normal((ny + 4, nx + 4))).astype(np.float32)
    hu = (2.0 * rng.standard_normal((ny + 4, nx + 4))).astype(np.float32)
    hv = (2.0 * rng.standard_normal((ny + 4, nx + 4))).astype(np.float32)
    c = dict(eta0=eta, hu0=hu, hv0=hv, H=H, nx=nx, ny=ny, dx=150.0, dy=170.0, g=9.81, f=1.0e-4, r=2.4e-3,
             coriolis_beta=0.0, boundary=(1, 1, 1, 1))
    sim = _product(ctx, c, 0.0)
    sim.updateDt(courant_number=0.5)
    dt = float(sim.dt)
    ref = _reference("cdklm_fric77", c, dt, sim)
    for _ in range(200):
        sim.step(dt)
        ref.step(dt)
    (de, dhu, dhv), theirs = _diffs(sim, ref, nx, ny)
    scale = [float(np.max(np.abs(t))) for t in theirs]
    print(json.dumps({"case": "friction 77x45 random 200 steps", "max_abs_diff": [de, dhu, dhv],
                      "max_abs_ref": scale}))
    assert de == 0.0 and dhu == 0.0 and dhv == 0.0, (de, dhu, dhv)
    ref.free()
    sim.cleanUp()


def test_land_and_drying_beach_bit_identical(ctx):
    """An island of land cells (masked depths) and a beach that starts dry
    (eta = -H) and floods under a wave from the east: the land, dry-face and
    shallow-cell (desingularised) paths of the step against the reference
    kernel, bit for bit, with bottom friction."""
    nx, ny = 77, 45
    x = np.arange(nx + 5, dtype=np.float32)[None, :]
    H = (10.0 * (0.02 + np.clip((x - 8.0) / 25.0, 0.0, 1.0)) * np.ones((ny + 5, 1), np.float32)).astype(np.float32)
    H = np.ma.array(H, mask=np.zeros(H.shape, bool))
    H.mask[20:26, 40:46] = True
    xc = np.arange(nx + 4)[None, :] - 2 + 0.5
    yc = np.arange(ny + 4)[:, None] - 2 + 0.5
    eta = (0.6 * np.exp(-((xc - 30.0) ** 2 + (yc - 22.0) ** 2) / 40.0)).astype(np.float32)
    eta[:, :10] = -np.float32(0.2)   # the beach's cells (depth 0.2 m) start dry
    z = np.zeros_like(eta)
    c = dict(eta0=eta, hu0=z, hv0=z.copy(), H=H, nx=nx, ny=ny, dx=150.0, dy=170.0, g=9.81, f=1.0e-4, r=2.4e-3,
             coriolis_beta=0.0, boundary=(1, 1, 1, 1))
    sim = _product(ctx, c, 0.0)
    sim.updateDt(courant_number=0.5)
    dt = float(sim.dt)
    ref = _reference("cdklm_fric77", c, dt, sim)
    for _ in range(300):
        sim.step(dt)
        ref.step(dt)
    (de, dhu, dhv), theirs = _diffs(sim, ref, nx, ny)
    e = np.ma.getdata(theirs[0]).astype(np.float64)
    Hm = np.asarray(sim.downloadBathymetry()[1])[2:ny + 2, 2:nx + 2].astype(np.float64)
    land = Hm > 1e10
    h = np.where(land, np.nan, e + Hm)
    n_dry = int(np.sum(h <= 1e-5))
    n_shallow = int(np.sum((h > 1e-5) & (h < 0.1)))
    print(json.dumps({"case": "land + drying beach 77x45, 300 steps", "max_abs_diff": [de, dhu, dhv],
                      "land": int(land.sum()), "dry": n_dry, "shallow": n_shallow}))
    assert land.sum() > 0 and n_dry > 0 and n_shallow > 0
    assert de == 0.0 and dhu == 0.0 and dhv == 0.0, (de, dhu, dhv)
    ref.free()
    sim.cleanUp()


def _soar_q0(L_cells=8.0, std=0.003):
    oy, ox = np.mgrid[-2:3, -2:3]
    d = np.sqrt(ox ** 2 + oy ** 2) / L_cells
    return std / np.sqrt(np.sum(((1 + d) * np.exp(-d)) ** 2))


@pytest.mark.parametrize("factor,config,case", [(1, "noise_const", "bump"), (7, "noise_const", "bump"),
                                                (8, "noise_jet512", "jet"), (1, "noise_jet512", "jet")])
def test_soar_perturbation_on_injected_normals(ctx, factor, config, case):
    from gpuocean_gb300.SWEsimulators import OceanStateNoise
    from gpuocean_gb300.utils.BenchmarkCases import double_jet_case
    c = _bump256() if case == "bump" else double_jet_case()
    cdk = "cdklm_bump256" if case == "bump" else "cdklm_jet512"
    sim = _product(ctx, c, 1.0)
    ref = _reference(cdk, c, 1.0, sim)
    cdx = c["dx"] * factor
    q0, L = _soar_q0(), 8.0 * cdx
    noise = OceanStateNoise.OceanStateNoise.fromsim(sim, soar_q0=q0, soar_L=L, interpolation_factor=factor,
                                                    strict_odd_factor=False)
    rnoise = rk.RefNoise(config, ref, q0, L, interpolation_factor=factor)
    assert (int(noise.rand_ny), int(noise.rand_nx)) == (rnoise.rand_ny, rnoise.rand_nx)
    xi = np.random.default_rng(7).standard_normal((rnoise.rand_ny, rnoise.rand_nx)).astype(np.float32)
    before = _interior(sim.download(), c["nx"], c["ny"])
    noise.setRandomNumbers(xi)
    noise.perturbSim(sim, update_random_field=False)
    rnoise.set_random(xi)
    rnoise.perturb(ref)
    mine = _interior(sim.download(), c["nx"], c["ny"])
    theirs = _interior(ref.download(), c["nx"], c["ny"])
    rel = []
    for m, t, b in zip(mine, theirs, before):
        dp = (t.astype(np.float64) - b)             # the reference's perturbation
        err = np.max(np.abs(m.astype(np.float64) - t))
        rel.append(float(err / np.max(np.abs(dp))))
        print(json.dumps({"case": f"SOAR factor {factor} on {case}", "max_rel_diff_of_perturbation": rel[-1]}))
        assert np.max(np.abs(dp)) > 0
        assert err <= 2e-5 * np.max(np.abs(dp)) + 4 * np.spacing(np.float32(np.max(np.abs(t)))), \
            (factor, err, np.max(np.abs(dp)))
    rnoise.free()
    ref.free()
    sim.cleanUp()


def test_double_jet_with_model_error_and_drifters(ctx):
    """40 steps of the C3 member: SOAR model error after every step on the same
    injected draws, 200 drifters advected by both."""
    from gpuocean_gb300.SWEsimulators import OceanStateNoise
    from gpuocean_gb300.drifters import GPUDrifterCollection
    from gpuocean_gb300.utils import Common
    from gpuocean_gb300.utils.BenchmarkCases import double_jet_case
    c = double_jet_case()
    sim = _product(ctx, c, 0.0)
    sim.updateDt(courant_number=0.8)
    dt = float(sim.dt)
    ref = _reference("cdklm_jet512", c, dt, sim)
    factor = 8
    q0, L = _soar_q0(), 8.0 * c["dx"] * factor
    noise = OceanStateNoise.OceanStateNoise.fromsim(sim, soar_q0=q0, soar_L=L, interpolation_factor=factor,
                                                    strict_odd_factor=False)
    rnoise = rk.RefNoise("noise_jet512", ref, q0, L, interpolation_factor=factor)
    Lx, Ly = c["nx"] * c["dx"], c["ny"] * c["dy"]
    rng = np.random.default_rng(3)
    pos = np.stack([rng.random(201) * Lx, rng.random(201) * Ly], axis=1).astype(np.float32)
    drifters = GPUDrifterCollection.GPUDrifterCollection(
        ctx, 200, boundaryConditions=Common.BoundaryConditions(*c["boundary"]), domain_size_x=Lx, domain_size_y=Ly)
    drifters.setDrifterPositions(pos[:-1])
    drifters.setObservationPosition(pos[-1])
    rdrift = rk.RefDrifters(pos, Lx, Ly, 0, 1)
    # the reference without model error: the spread the 40 perturbations create
    quiet = _reference("cdklm_jet512", c, dt, sim)
    draws = np.random.default_rng(99).standard_normal((40, rnoise.rand_ny, rnoise.rand_nx)).astype(np.float32)
    for k in range(40):
        # the order of S/CDKLM16.py:519-575: RK2 step, model error on the k-th
        # injected draw, ghost fill, drift
        sim.step(dt, apply_stochastic_term=False)
        noise.setRandomNumbers(draws[k])
        noise.perturbSim(sim, update_random_field=False)
        sim.applyBoundaryConditions()
        drifters.driftFromSim(sim, dt)
        ref.step(dt)
        rnoise.set_random(draws[k])
        rnoise.perturb(ref)
        ref._boundary(ref.h0)
        rdrift.drift(ref, dt)
        quiet.step(dt)
    (de, dhu, dhv), theirs = _diffs(sim, ref, c["nx"], c["ny"])
    calm = _interior(quiet.download(), c["nx"], c["ny"])
    spread = [float(np.max(np.abs(t.astype(np.float64) - q))) for t, q in zip(theirs, calm)]
    mine_pos = np.asarray(drifters.getDrifterPositions())
    ref_pos = rdrift.positions()[:-1]
    dpos = float(np.max(np.abs(mine_pos - ref_pos)))
    print(json.dumps({"case": "double jet + SOAR + drifters, 40 steps", "max_abs_diff": [de, dhu, dhv],
                      "perturbation_spread": spread, "max_abs_drifter_diff_m": dpos}))
    # the step is bit-identical; what remains is the noise transfer's rounding
    # (fast-math there, no FMA contraction here: within 2e-5 of each
    # perturbation, test_soar_perturbation_on_injected_normals).  40 transfers
    # bound it by 40 x 2e-5 = 8e-4 of one perturbation; the 40 independent
    # perturbations spread the state by about sqrt(40) ~ 6 perturbations, so
    # about 1.3e-4 of that spread; 2e-4 leaves room for the dynamics.
    for d, sp in zip((de, dhu, dhv), spread):
        assert sp > 0 and d <= 2e-4 * sp, ((de, dhu, dhv), spread)
    assert dpos <= 1e-6 * max(Lx, Ly)
    quiet.free()
    rdrift.free()
    rnoise.free()
    ref.free()
    sim.cleanUp()


def test_reference_kernel_step_rate(ctx):
    """Throughput of the reference kernels launched per member (the way the
    reference's ensembles step), beside the product's plain per-member step,
    on the 512 x 300 double-jet member.  Printed as one JSON line."""
    from gpuocean_gb300.utils.BenchmarkCases import double_jet_case
    c = double_jet_case()
    sim = _product(ctx, c, 0.0)
    sim.updateDt(courant_number=0.8)
    dt = float(sim.dt)
    ref = _reference("cdklm_jet512", c, dt, sim)
    n = 300
    for _ in range(20):
        ref.step(dt)
        sim.step(dt)
    ref.synchronize()
    sim.gpu_stream.synchronize()
    t0 = time.perf_counter()
    for _ in range(n):
        ref.step(dt)
    ref.synchronize()
    t_ref = time.perf_counter() - t0
    t0 = time.perf_counter()
    for _ in range(n):
        sim.step(dt)
    sim.gpu_stream.synchronize()
    t_prod = time.perf_counter() - t0
    cells = c["nx"] * c["ny"] * n
    print(json.dumps({"case": "per-member step rate, double jet 512x300", "steps": n,
                      "reference_kernels_cell_steps_per_s": cells / t_ref,
                      "product_cell_steps_per_s": cells / t_prod}))
    ref.free()
    sim.cleanUp()


def _ref_block_rate(ctx, c, cdk, noise_cfg, n_drifters, members, blocks=3, block_s=60.0, factor=8):
    """Member-cell-steps/s of the reference kernels stepping `members`
    copies of case `c` one after the other, each block being
    step(block_s) + drifters after every step + one SOAR perturbation
    (injected normals), the member-by-member cadence of the reference's
    ensembles."""
    sim = _product(ctx, c, 0.0)
    sim.updateDt(courant_number=0.8)
    dt = float(sim.dt)
    refs = []
    rng = np.random.default_rng(1)
    for _ in range(members):
        ref = _reference(cdk, c, dt, sim)
        q0, L = _soar_q0(), 8.0 * c["dx"] * factor
        rn = rk.RefNoise(noise_cfg, ref, q0, L, interpolation_factor=factor)
        rn.set_random(rng.standard_normal((rn.rand_ny, rn.rand_nx)).astype(np.float32))
        rd = None
        if n_drifters:
            Lx, Ly = c["nx"] * c["dx"], c["ny"] * c["dy"]
            pos = np.stack([rng.random(n_drifters + 1) * Lx, rng.random(n_drifters + 1) * Ly], axis=1)
            rd = rk.RefDrifters(pos.astype(np.float32), Lx, Ly, 0, 1)
        refs.append((ref, rn, rd))

    def block(ref, rn, rd):
        ref.step(block_s, drifters=rd)
        rn.perturb(ref)
        ref._boundary(ref.h0)

    for r in refs:
        block(*r)
    refs[0][0].synchronize()
    steps0 = sum(r[0].num_iterations for r in refs)
    t0 = time.perf_counter()
    for _ in range(blocks):
        for r in refs:
            block(*r)
    refs[0][0].synchronize()
    wall = time.perf_counter() - t0
    steps = sum(r[0].num_iterations for r in refs) - steps0
    for ref, rn, rd in refs:
        rn.free()
        ref.free()
        if rd is not None:
            rd.free()
    sim.cleanUp()
    return steps * c["nx"] * c["ny"] / wall, wall / (blocks * members)


def test_reference_kernel_member_rates_c3_c4(ctx):
    """The reference's kernels stepped member by member (its ensembles'
    pattern) on the benchmark workloads: C3 (512 x 300 double jet, 1000
    drifters, SOAR every 60 s, coarse factor 8) and C4 (levels 128 x 64,
    256 x 128, 512 x 256 of one 2560 km x 1500 km domain, 512 / 128 / 32
    members, SOAR every 60 s).  Normals are injected, so the reference's
    random-number generation is not timed.  Printed as one JSON line."""
    from gpuocean_gb300.utils.BenchmarkCases import double_jet_case
    c3, _ = _ref_block_rate(ctx, double_jet_case(), "cdklm_jet512", "noise_jet512", 1000, members=4)
    levels = ((128, 64, 512), (256, 128, 128), (512, 256, 32))
    total_cells, total_time = 0.0, 0.0
    per_level = {}
    for nx, ny, n in levels:
        c = double_jet_case(nx=nx, ny=ny, dx=2560e3 / nx, dy=1500e3 / ny)
        rate, t_block = _ref_block_rate(ctx, c, f"cdklm_ml{nx}x{ny}", f"noise_ml{nx}x{ny}", 0, members=4)
        per_level[f"{nx}x{ny}"] = rate
        total_time += n * t_block
        total_cells += n * t_block * rate
    c4 = total_cells / total_time
    print(json.dumps({"case": "reference kernels member by member", "c3_member_cell_steps_per_s": c3,
                      "c4_member_cell_steps_per_s": c4, "c4_levels": per_level}))
    assert c3 > 0 and c4 > 0


def test_wind_drift_against_reference_kernel(ctx):
    """Drifters with wind drift (wind_drift_factor 0.02, 3 x 4 wind
    textures at two time stamps) against the reference's passiveDrifterKernel
    built for that texture size (K/driftKernels.cu:74-183): the reference
    reads both wind components with the x texture's size; with equal sizes
    (which this package requires) both read the same cells.  20 steps of the
    double jet, drift after every step at the simulator's time."""
    from gpuocean_gb300.drifters import GPUDrifterCollection
    from gpuocean_gb300.utils import Common, WindStress
    from gpuocean_gb300.utils.BenchmarkCases import double_jet_case
    c = double_jet_case()
    sim = _product(ctx, c, 0.0)
    sim.updateDt(courant_number=0.8)
    dt = float(sim.dt)
    ref = _reference("cdklm_jet512", c, dt, sim)
    rng = np.random.default_rng(21)
    wu = [(5.0 * rng.standard_normal((4, 3))).astype(np.float32) for _ in range(2)]
    wv = [(5.0 * rng.standard_normal((4, 3))).astype(np.float32) for _ in range(2)]
    wind = WindStress.WindStress(t=[0.0, 20 * dt], wind_u=wu, wind_v=wv)
    Lx, Ly = c["nx"] * c["dx"], c["ny"] * c["dy"]
    pos = np.stack([rng.random(301) * Lx, rng.random(301) * Ly], axis=1).astype(np.float32)
    drifters = GPUDrifterCollection.GPUDrifterCollection(
        ctx, 300, boundaryConditions=Common.BoundaryConditions(*c["boundary"]), domain_size_x=Lx, domain_size_y=Ly,
        wind=wind, wind_drift_factor=0.02)
    drifters.setDrifterPositions(pos[:-1])
    drifters.setObservationPosition(pos[-1])
    rdrift = rk.RefDrifters(pos, Lx, Ly, 0, 1, config="drift_wind3x4", wind=(wu[0], wu[1], wv[0], wv[1]),
                            wind_drift_factor=0.02)
    for k in range(20):
        sim.step(dt)
        drifters.driftFromSim(sim, dt)
        ref.step(dt)
        # wind_t of update_wind (D/GPUDrifterCollection.py:138-174) at the
        # simulator's time after the step
        rdrift.drift(ref, dt, wind_t=np.float32(min(1.0, max(0.0, ref.t / (20 * dt)))))
    mine = np.concatenate([np.asarray(drifters.getDrifterPositions()),
                           np.asarray(drifters.getObservationPosition())[None, :]])
    theirs = rdrift.positions()
    still = _reference("cdklm_jet512", c, dt, sim)
    calm = rk.RefDrifters(pos, Lx, Ly, 0, 1)
    for k in range(20):
        still.step(dt)
        calm.drift(still, dt)
    moved = float(np.max(np.abs(theirs - calm.positions())))
    dpos = float(np.max(np.abs(mine - theirs)))
    print(json.dumps({"case": "wind drift, 20 steps", "max_abs_drifter_diff_m": dpos,
                      "wind_displacement_m": moved}))
    # the wind moved the drifters: 0.02 x ~5 m/s over 20 steps of ~20 s is
    # tens of metres
    assert moved > 10.0
    assert dpos <= 1e-6 * max(Lx, Ly), dpos
    for o in (rdrift, calm, ref, still):
        o.free()
    sim.cleanUp()


@pytest.mark.parametrize("boundary", [(1, 1, 1, 1), (1, 2, 1, 2)], ids=["walls", "periodic_x"])
def test_rotated_grid_angle_texture(ctx, boundary):
    """A north-angle texture (6 x 5 values over a 64 x 48 grid): every cell
    uses its own north vector for its slopes, its four faces and its source
    terms (getNorth, K/CDKLM16_kernel.cu:70-79, 706-765), so each face is
    seen differently from its two sides.  200 RK2 steps stage by stage
    against the reference kernel built for that texture: bit-identical."""
    nx, ny = 64, 48
    x = (np.arange(nx + 4) - 2 + 0.5 - nx / 2.0)
    y = (np.arange(ny + 4) - 2 + 0.5 - ny / 2.0)
    eta = (0.2 * np.exp(-(x[None, :] ** 2 + y[:, None] ** 2) / (2.0 * 6.0 ** 2))).astype(np.float32)
    z = np.zeros_like(eta)
    H = np.full((ny + 5, nx + 5), 30.0, np.float32)
    ax, ay = np.meshgrid(np.arange(6), np.arange(5))
    angle = (0.4 + 0.15 * ax - 0.1 * ay).astype(np.float32)
    c = dict(eta0=eta, hu0=z, hv0=z.copy(), H=H, nx=nx, ny=ny, dx=500.0, dy=500.0, g=9.81, f=1.2e-4, r=0.0,
             coriolis_beta=0.0, boundary=boundary)
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils import Common
    sim = CDKLM16.CDKLM16(ctx, eta, z, z.copy(), H, nx, ny, 500.0, 500.0, 0.0, 9.81, 1.2e-4, 0.0, angle=angle,
                          boundary_conditions=Common.BoundaryConditions(*boundary))
    assert sim.angle_varies
    sim.updateDt(courant_number=0.6)
    dt = float(sim.dt)
    ref = _reference("cdklm_angle64", c, dt, sim)
    for _ in range(200):
        sim.step(dt)
        ref.step(dt)
    (de, dhu, dhv), theirs = _diffs(sim, ref, nx, ny)
    scale = [float(np.max(np.abs(t))) for t in theirs]
    print(json.dumps({"case": f"angle texture 64x48, 200 steps, bc {boundary}", "max_abs_diff": [de, dhu, dhv],
                      "max_abs_ref": scale}))
    assert scale[1] > 0 and scale[2] > 0
    assert de == 0.0 and dhu == 0.0 and dhv == 0.0, (de, dhu, dhv)
    ref.free()
    sim.cleanUp()
