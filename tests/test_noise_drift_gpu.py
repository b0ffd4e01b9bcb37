"""SOAR noise, random numbers and drifters on the GPU against the reference's
CPU twins (golden vectors) and the FP64 oracle."""
import os

import numpy as np
import pytest

from oracle import noise_oracle as N

pytestmark = pytest.mark.gpu

REF = np.load(os.path.join(os.path.dirname(__file__), "golden", "noise_drift_reference.npz"))


def _noise(ctx, stream, nx, ny, dx, dy, pns, pew, factor=1, q0=None, L=None, use_lcg=True):
    from gpuocean_gb300.SWEsimulators.OceanStateNoise import OceanStateNoise
    from gpuocean_gb300.utils import Common
    n, e = (2, 2) if pns else (1, 1), (2, 2) if pew else (1, 1)
    bc = Common.BoundaryConditions(n[0], e[0], n[1], e[1])
    return OceanStateNoise(ctx, stream, nx, ny, dx, dy, bc, False, soar_q0=q0, soar_L=L,
                           interpolation_factor=factor, use_lcg=use_lcg, np_seed=1)


def _ocean(stream, nx, ny, H):
    from gpuocean_gb300.utils import Common
    z = np.zeros((ny + 4, nx + 4), np.float32)
    return [Common.CUDAArray2D(stream, nx, ny, 2, 2, z) for _ in range(3)], \
        Common.CUDAArray2D(stream, nx + 1, ny + 1, 2, 2, np.full((ny + 5, nx + 5), H, np.float32))


@pytest.mark.parametrize("key", ["soar_ns1_ew1", "soar_ns0_ew0", "soar_ns1_ew0", "soar_ns0_ew1",
                                 "bicubic_f3", "bicubic_f5"])
def test_perturbation_matches_reference(gpu_ctx, key):
    from gpuocean_gb300.utils import Common
    nx, ny, dx, dy, f, g, H, q0, L, factor = REF[key + "/params"]
    nx, ny, factor = int(nx), int(ny), int(factor)
    pns, pew = (1, 1) if key.startswith("bicubic") else (int(key[7]), int(key[11]))
    s = Common.Stream()
    noise = _noise(gpu_ctx, s, nx, ny, dx, dy, pns, pew, factor=factor, q0=q0, L=L)
    noise.setRandomNumbers(REF[key + "/xi"])
    (eta, hu, hv), Hi = _ocean(s, nx, ny, H)
    noise.perturbOceanState(eta, hu, hv, Hi, f, 0.0, g, ghost_cells_x=2, ghost_cells_y=2, update_random_field=False)
    coarse = noise.getCoarseBuffer()
    # fast-math SOAR weights (as the reference builds this kernel): 1e-5 relative
    assert np.max(np.abs(coarse - REF[key + "/coarse"])) <= 1e-5 * np.abs(REF[key + "/coarse"]).max()
    e, u, v = (a.download(s)[2:-2, 2:-2] for a in (eta, hu, hv))
    for a, b in ((e, REF[key + "/d_eta"][2:-2, 2:-2]), (u, REF[key + "/d_hu"]), (v, REF[key + "/d_hv"])):
        assert np.max(np.abs(a - b)) <= 2e-5 * np.abs(b).max(), key
    # periodic ghost images of the perturbed state
    ef = eta.download(s)
    if pew:
        assert np.array_equal(ef[2:-2, 0:2], ef[2:-2, nx:nx + 2])
    if pns:
        assert np.array_equal(ef[0:2, 2:-2], ef[ny:ny + 2, 2:-2])


def test_geobalance_with_state_and_beta_vs_oracle(gpu_ctx):
    """Non-zero eta enters h in the factor-1 balance; beta-plane Coriolis."""
    from gpuocean_gb300.utils import Common
    nx, ny, dx, dy = 40, 30, 1000.0, 1000.0
    f, beta, g = 1e-4, 2e-11, 9.81
    rng = np.random.default_rng(3)
    s = Common.Stream()
    noise = _noise(gpu_ctx, s, nx, ny, dx, dy, 0, 1, q0=1e-3, L=3000.0)
    xi = rng.standard_normal((noise.rand_ny, noise.rand_nx)).astype(np.float32)
    noise.setRandomNumbers(xi)
    eta0 = (0.1 * rng.standard_normal((ny + 4, nx + 4))).astype(np.float32)
    H = rng.uniform(50, 60, (ny + 5, nx + 5)).astype(np.float32)
    eta = Common.CUDAArray2D(s, nx, ny, 2, 2, eta0)
    hu = Common.CUDAArray2D(s, nx, ny, 2, 2, np.zeros_like(eta0))
    hv = Common.CUDAArray2D(s, nx, ny, 2, 2, np.zeros_like(eta0))
    Hi = Common.CUDAArray2D(s, nx + 1, ny + 1, 2, 2, H)
    noise.perturbOceanState(eta, hu, hv, Hi, f, beta, g, ghost_cells_x=2, ghost_cells_y=2, update_random_field=False)
    coarse = N.soar_coarse(xi, nx, ny, dx, dy, np.float32(1e-3), np.float32(3000.0), 0, 1)
    re, ru, rv = eta0.astype(np.float64), np.zeros((ny + 4, nx + 4)), np.zeros((ny + 4, nx + 4))
    N.geostrophic_balance(re, ru, rv, coarse, H, nx, ny, dx, dy, f, beta, g)
    for a, b in ((eta, re), (hu, ru), (hv, rv)):
        got = a.download(s)[2:-2, 2:-2]
        assert np.max(np.abs(got - b[2:-2, 2:-2])) <= 2e-5 * np.abs(b[2:-2, 2:-2]).max()


def test_lcg_on_gpu_vs_oracle(gpu_ctx):
    from gpuocean_gb300.utils import Common
    from gpuocean_gb300.utils.RandomNumbers import RandomNumbers
    s = Common.Stream()
    rnx = REF["lcg/uniform"].shape[1]
    rny = REF["lcg/uniform"].shape[0]
    rn = RandomNumbers(gpu_ctx, s, rnx, rny, use_lcg=True, seed=0)
    rn.seed.upload(s, REF["lcg/seed_in"])
    buf = Common.CUDAArray2D(s, rnx, rny, 0, 0, np.zeros((rny, rnx), np.float32))
    rn.generateUniformDistribution(buf)
    u = buf.download(s)
    assert np.array_equal(rn.getSeed(), REF["lcg/seed_after_uniform"])
    uo, _ = N.lcg_uniform(REF["lcg/seed_in"], rnx)
    assert np.array_equal(u, uo.astype(np.float32))
    rn.generateNormalDistribution(buf)
    n = buf.download(s)
    no, so = N.lcg_normal(REF["lcg/seed_after_uniform"], rnx)
    assert np.array_equal(rn.getSeed(), so)
    # fast-math log/sqrt/cospi as in the reference build: 2e-5 absolute
    assert np.max(np.abs(n - no)) < 2e-5


def test_xorwow_statistics(gpu_ctx):
    from gpuocean_gb300.utils import Common
    from gpuocean_gb300.utils.RandomNumbers import RandomNumbers
    s = Common.Stream()
    rn = RandomNumbers(gpu_ctx, s, 200, 300, use_lcg=False, xorwow_seed=11)
    buf = Common.CUDAArray2D(s, 200, 300, 0, 0, np.zeros((300, 200), np.float32))
    rn.generateNormalDistribution(buf)
    a = buf.download(s)
    assert abs(a.mean()) < 0.02 and abs(a.var() - 1.0) < 0.03
    rn.generateNormalDistribution(buf)
    assert not np.array_equal(a, buf.download(s))


def test_drift_matches_reference_cpu_collection(gpu_ctx):
    from gpuocean_gb300.drifters.GPUDrifterCollection import GPUDrifterCollection
    from gpuocean_gb300.utils import Common
    nx, ny, dx, dy, dt = REF["drift/params"]
    nx, ny = int(nx), int(ny)
    s = Common.Stream()
    fields = [Common.CUDAArray2D(s, nx, ny, 2, 2, REF["drift/" + k]) for k in ("eta", "hu", "hv", "Hm")]
    traj = REF["drift/traj"]
    d = GPUDrifterCollection(gpu_ctx, traj.shape[1] - 1, boundaryConditions=Common.BoundaryConditions(2, 2, 2, 2),
                             domain_size_x=nx * dx, domain_size_y=ny * dy, gpu_stream=s)
    d.setDrifterPositions(traj[0][:-1])
    d.setObservationPosition(traj[0][-1])
    for k in range(1, traj.shape[0]):
        d.drift(*fields, nx, ny, 0.0, dx, dy, dt, 2, 2)
        pos = np.concatenate([d.getDrifterPositions(), d.getObservationPosition()[None, :]])
        assert np.max(np.abs(pos - traj[k])) < 2e-5 * nx * dx
