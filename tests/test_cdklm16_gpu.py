"""CDKLM16 on the GPU against the reference goldens and the FP64 oracle."""
import os

import numpy as np
import pytest

import cases
from oracle.cdklm16_oracle import BC, OracleCDKLM16, bathymetry_init, max_dt_f32

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "cdklm16_timestep50.npz"))


def make_sims(gpu_ctx, name, **kw):
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils import Common
    c = cases.make_case(name)
    c.update({k: v for k, v in kw.items() if k in c})
    extra = {k: v for k, v in kw.items() if k not in c}
    sim = CDKLM16.CDKLM16(gpu_ctx, c["eta0"], c["hu0"], c["hv0"], c["H"], c["nx"], c["ny"], c["dx"], c["dy"],
                          c["dt"], c["g"], c["f"], c["r"], coriolis_beta=c["coriolis_beta"],
                          boundary_conditions=Common.BoundaryConditions(*c["bc"]), **extra)
    ref = OracleCDKLM16(c["eta0"], c["hu0"], c["hv0"], c["H"], c["nx"], c["ny"], c["dx"], c["dy"], c["dt"],
                        c["g"], c["f"], c["r"], coriolis_beta=c["coriolis_beta"],
                        boundary_conditions=BC(*c["bc"]), **extra)
    return c, sim, ref


@pytest.mark.parametrize("name", list(cases.CASES))
def test_cdklm16_matches_reference_golden_and_oracle(gpu_ctx, name):
    c, sim, ref = make_sims(gpu_ctx, name)
    sim.step(cases.T_END)
    ref.step(cases.T_END)
    assert sim.num_iterations == 56 and sim.t == ref.t
    got = sim.download(interior_domain_only=True)
    want = ref.download(interior_domain_only=True)
    k = c["golden"]
    for a, b, f in zip(got, want, ("eta", "u", "v")):
        # the reference's own tolerance against its golden vectors
        assert cases.rel_max_diff(a, GOLD[k + "/" + f]) < 5e-4, (name, f)
        # FP32 GPU vs FP64 oracle after 56 steps: max |diff| / max |ref| < 1e-4
        assert cases.rel_max_diff(a, b) < 1e-4, (name, f)
    # dt: GPU reduction == float32 host formula (bit-exact)
    sim.updateDt()
    dt_host = np.float32(0.8) * max_dt_f32(*[np.asarray(x) for x in sim.download()], np.asarray(sim.downloadBathymetry()[1]),
                                           c["nx"], c["ny"], c["dx"], c["dy"], c["g"])
    assert np.float32(sim.dt) == np.float32(dt_host)
    assert np.float32(sim.dt) == np.float32(sim._getMaxTimestepHost())
    sim.cleanUp()


@pytest.mark.parametrize("bc", [(1, 1, 1, 1), (2, 2, 2, 2), (2, 1, 2, 1), (1, 2, 1, 2)])
def test_bathymetry_init_bit_exact(gpu_ctx, bc):
    from gpuocean_gb300.utils import Common
    rng = np.random.default_rng(1)
    nx, ny = 37, 23
    H = rng.uniform(5, 100, size=(ny + 5, nx + 5)).astype(np.float32)
    H = np.ma.array(H, mask=rng.random(H.shape) < 0.1)
    s = Common.Stream()
    b = Common.Bathymetry(gpu_ctx, s, nx, ny, 2, 2, H, Common.BoundaryConditions(*bc))
    Bi, Bm = b.download(s)
    Hi, Hm = bathymetry_init(H, nx, ny, BC(*bc))
    assert np.array_equal(np.ma.getdata(Bi), Hi)
    assert np.array_equal(np.ma.getdata(Bm), Hm)
    b.release()


@pytest.mark.parametrize("nx,ny,bc", [(33, 17, (1, 1, 1, 1)), (45, 29, (2, 2, 2, 2)), (64, 20, (1, 2, 1, 2)),
                                      (13, 49, (2, 1, 2, 1)), (5, 3, (1, 1, 1, 1))])
def test_odd_sizes_vs_oracle(gpu_ctx, nx, ny, bc):
    """Partial tiles and tiny grids (the tile is 32 x 16)."""
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils import Common
    rng = np.random.default_rng(nx * 100 + ny)
    shape = (ny + 4, nx + 4)
    eta = (0.1 * rng.standard_normal(shape)).astype(np.float32)
    hu = (0.5 * rng.standard_normal(shape)).astype(np.float32)
    hv = (0.5 * rng.standard_normal(shape)).astype(np.float32)
    H = rng.uniform(20, 40, size=(ny + 5, nx + 5)).astype(np.float32)
    args = (eta, hu, hv, H, nx, ny, 100.0, 120.0, 0.5, 9.81, 1e-4, 0.0)
    sim = CDKLM16.CDKLM16(gpu_ctx, *args, boundary_conditions=Common.BoundaryConditions(*bc))
    ref = OracleCDKLM16(*args, boundary_conditions=BC(*bc))
    sim.step(10.0)
    ref.step(10.0)
    # rough random states: FP32 vs FP64 tolerance 2e-4 of the field maximum
    for a, b in zip(sim.download(interior_domain_only=True), ref.download(interior_domain_only=True)):
        assert cases.rel_max_diff(a, b) < 2e-4
    sim.cleanUp()


@pytest.mark.parametrize("rk", [1, 3])
def test_rk_orders_vs_oracle(gpu_ctx, rk):
    c, sim, ref = make_sims(gpu_ctx, "periodic_corner", rk_order=rk, dt=0.5)
    sim.step(10.0)
    ref.step(10.0)
    for a, b in zip(sim.download(interior_domain_only=True), ref.download(interior_domain_only=True)):
        assert cases.rel_max_diff(a, b) < 1e-4
    sim.cleanUp()


def test_friction_wind_and_dry_land(gpu_ctx):
    """Bottom friction, uniform wind stress and a land mask with dry cells."""
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils import Common, WindStress
    nx, ny = 40, 30
    shape = (ny + 4, nx + 4)
    x = np.arange(nx + 5)[None, :]
    H = np.ones((ny + 5, nx + 5), np.float32) * 10.0
    H = (H * (0.05 + np.clip((x - 5) / 20.0, 0, 1))).astype(np.float32)  # shelf to a beach at the west
    H = np.ma.array(H, mask=np.zeros(H.shape, bool))
    H.mask[10:14, 0:4] = True
    eta = np.zeros(shape, np.float32)
    cases.central_bump(eta, nx, ny, 100.0, 100.0)
    eta *= 0.5
    z = np.zeros(shape, np.float32)
    tau = [np.array([[2e-4]], np.float32)]
    wind = WindStress.WindStress(t=[0], stress_u=tau, stress_v=[np.array([[-1e-4]], np.float32)])
    args = (eta, z, z, H, nx, ny, 100.0, 100.0, 0.2, 9.81, 1e-4, 2.4e-3)
    sim = CDKLM16.CDKLM16(gpu_ctx, *args, wind=wind)
    ref = OracleCDKLM16(*args, wind_stress=(2e-4, -1e-4))
    sim.step(20.0)
    ref.step(20.0)
    for a, b in zip(sim.download(interior_domain_only=True), ref.download(interior_domain_only=True)):
        a = np.ma.getdata(a)
        assert np.all(np.isfinite(a))
        assert np.max(np.abs(a - b)) / np.max(np.abs(b)) < 1e-4
    sim.cleanUp()


def test_step_run_equals_step_by_step(gpu_ctx):
    """One long step() call (after its first step, the run of steps is a
    single library call) leaves the state, time and iteration count of the
    same dt sequence taken one step() call at a time."""
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils import BenchmarkCases, Common
    sims = []
    for _ in range(2):
        c = BenchmarkCases.double_jet_case(nx=96, ny=64, dx=5000.0, dy=5000.0, seed=7)
        s = CDKLM16.CDKLM16(gpu_ctx, c["eta0"], c["hu0"], c["hv0"], c["H"], 96, 64, c["dx"], c["dy"], 0.0, c["g"],
                            c["f"], c["r"], coriolis_beta=c["coriolis_beta"],
                            boundary_conditions=Common.BoundaryConditions(*c["boundary"]))
        s.updateDt(courant_number=0.8)
        sims.append(s)
    a, b = sims
    t_end = 25.5 * float(a.dt)
    a.step(t_end)
    dts, t_now = [], 0.0
    while t_now < t_end:
        dts.append(np.float32(min(b.dt, np.float32(t_end - t_now))))
        t_now += np.float64(dts[-1])
    for dt in dts:
        b.step(float(dt))
    assert a.num_iterations == b.num_iterations == 26
    assert a.t == b.t
    for x, y in zip(a.download(), b.download()):
        assert np.array_equal(np.asarray(x), np.asarray(y))
