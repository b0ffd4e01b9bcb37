"""Open (sponge) boundaries and time-varying forcing against the reference's
own kernels (compiled from the reference sources, driven with the reference
host's launch sequence by oracle/ref_kernels.py).

* flow relaxation (flag 3) on every side, the reference's own sponge test
  (T/schemes/CombinedCDKLM16_test.py: 50 x 70, dx = dy = 200 m, H = 10 m,
  10 sponge cells, exterior eta of +1 along the north, 600 s);
* linear interpolation (flag 4) on every side with a Gaussian bump leaving
  the domain;
* flow relaxation north-south with per-cell exterior data at two time stamps
  and periodic east-west;
* textured wind stress (5 x 7) and atmospheric pressure (6 x 8) at three time
  stamps on a 77 x 45 walled grid.

The step kernels are bit-identical to the reference's (same operations, no FMA
contraction).  The boundary kernels are built with CUDA's default arithmetic on
both sides; the bar is bit-identity, reported as the largest difference."""
import json

import numpy as np
import pytest

from oracle import ref_kernels as rk

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not rk.available(), reason="reference kernels not built (no reference sources)")]


def _bcdata(t, sides, n_ns, n_ew):
    """Exterior data as both APIs take it: sides maps side -> list of (h, hu, hv)."""
    from gpuocean_gb300.utils import Common
    z = {"north": n_ns, "south": n_ns, "east": n_ew, "west": n_ew}
    full = {}
    for side, n in z.items():
        full[side] = sides.get(side) or [tuple(np.zeros(n, np.float32) for _ in range(3)) for _ in t]
    data = Common.BoundaryConditionsData(
        t=list(t), **{side: Common.SingleBoundaryConditionData(h=[a[0] for a in v], hu=[a[1] for a in v],
                                                                hv=[a[2] for a in v])
                      for side, v in full.items()})
    return data, dict(t=list(t), **full)


def _run(ctx, config, bc_config, nx, ny, dx, dy, H, eta0, bc, sponge, bc_data, T, dt=0.0, f=0.0, wind=None,
         pressure=None, direct=False):
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils import AtmosphericPressure, Common, WindStress
    z = np.zeros_like(eta0)
    kw = {}
    if wind is not None:
        kw["wind"] = WindStress.WindStress(t=list(wind[0]), stress_u=list(wind[1]), stress_v=list(wind[2]))
    if pressure is not None:
        kw["atmospheric_pressure"] = AtmosphericPressure.AtmosphericPressure(t=list(pressure[0]), P=list(pressure[1]),
                                                                            shiftValue=0)
    b = Common.BoundaryConditions(*bc, spongeCells=dict(zip(("north", "east", "south", "west"), sponge)))
    sim = CDKLM16.CDKLM16(ctx, eta0, z, z.copy(), H, nx, ny, dx, dy, dt, 9.81, f, 0.0, boundary_conditions=b,
                          boundary_conditions_data=bc_data[0] if bc_data else None, use_direct_lookup=direct, **kw)
    # the Coriolis and angle textures and the compensated f of the product's host
    ftex = sim.coriolis_f_arr.download(sim.gpu_stream)
    angle = sim.angle_arr.download(sim.gpu_stream)
    ref = rk.RefCDKLM16(config, eta0, z, z.copy(), H, nx, ny, dx, dy, float(sim.dt), 9.81, float(sim.f), 0.0,
                        ftex, angle, bc=bc,
                        sponge_cells=sponge, bc_data=bc_data[1] if bc_data else None, bc_config=bc_config,
                        wind=(wind[0], wind[1], wind[2]) if wind is not None else None,
                        pressure=(pressure[0], pressure[1]) if pressure is not None else None)
    sim.step(T)
    ref.step(T)
    got = [np.asarray(a, np.float64) for a in sim.download()]
    exp = [np.asarray(a, np.float64) for a in ref.download()]
    ref.free()
    sim.cleanUp()
    return got, exp


def _report(name, got, exp):
    diffs = {q: float(np.abs(g[2:-2, 2:-2] - e[2:-2, 2:-2]).max()) for q, g, e in zip(("eta", "hu", "hv"), got, exp)}
    scale = {q: float(np.abs(e[2:-2, 2:-2]).max()) for q, e in zip(("eta", "hu", "hv"), exp)}
    print(json.dumps({"case": name, "max_abs_diff": diffs, "max_abs": scale}))
    return diffs


def test_flow_relaxation_incoming_wave(gpu_ctx):
    nx, ny = 50, 70
    eta0 = np.zeros((ny + 4, nx + 4), np.float32)
    H = np.full((ny + 5, nx + 5), 10.0, np.float32)
    one = (np.array([1, 1], np.float32), np.zeros(2, np.float32), np.zeros(2, np.float32))
    data = _bcdata([0], {"north": [one]}, 2, 2)
    got, exp = _run(gpu_ctx, "cdklm_sponge50x70", "boundary", nx, ny, 200.0, 200.0, H, eta0, (3, 3, 3, 3),
                    (10, 10, 10, 10), data, 600.0)
    d = _report("flow relaxation, incoming wave (reference sponge test)", got, exp)
    assert np.abs(exp[0][2:-2, 2:-2]).max() > 0.1   # the wave entered
    assert max(d.values()) == 0.0


def test_linear_interpolation_outgoing_bump(gpu_ctx):
    nx, ny = 50, 70
    x = np.arange(nx + 4) - 2 + 0.5 - nx / 2.0
    y = np.arange(ny + 4) - 2 + 0.5 - ny / 2.0
    eta0 = (0.5 * np.exp(-(x[None, :] ** 2 + y[:, None] ** 2) / 50.0)).astype(np.float32)
    H = np.full((ny + 5, nx + 5), 10.0, np.float32)
    got, exp = _run(gpu_ctx, "cdklm_sponge50x70", "boundary", nx, ny, 200.0, 200.0, H, eta0, (4, 4, 4, 4),
                    (6, 6, 6, 6), None, 500.0)
    d = _report("linear interpolation, outgoing bump", got, exp)
    assert max(d.values()) == 0.0


def test_flow_relaxation_time_data_periodic_ew(gpu_ctx):
    nx, ny = 50, 70
    rng = np.random.default_rng(3)
    eta0 = (0.05 * rng.standard_normal((ny + 4, nx + 4))).astype(np.float32)
    H = np.full((ny + 5, nx + 5), 12.0, np.float32)
    xs = np.linspace(0, 1, nx + 4, dtype=np.float32)

    def side(a):
        return (a.astype(np.float32), (0.1 * a).astype(np.float32), np.zeros(nx + 4, np.float32))
    north = [side(0.3 * np.sin(2 * np.pi * xs)), side(-0.2 * np.cos(2 * np.pi * xs))]
    south = [side(0.1 * xs), side(0.2 * xs)]
    data = _bcdata([0.0, 400.0], {"north": north, "south": south}, nx + 4, ny + 4)
    got, exp = _run(gpu_ctx, "cdklm_sponge50x70", "boundary_data54x74", nx, ny, 200.0, 200.0, H, eta0, (3, 2, 3, 2),
                    (8, 0, 8, 0), data, 600.0, f=1e-4)
    d = _report("flow relaxation north-south, time-varying per-cell data, periodic east-west", got, exp)
    assert max(d.values()) == 0.0


def test_time_varying_textured_forcing(gpu_ctx):
    nx, ny = 77, 45
    rng = np.random.default_rng(11)
    x = np.arange(nx + 4) - 2 + 0.5 - nx / 2.0
    y = np.arange(ny + 4) - 2 + 0.5 - ny / 2.0
    eta0 = (0.1 * np.exp(-(x[None, :] ** 2 + y[:, None] ** 2) / 80.0)).astype(np.float32)
    H = (40.0 + 2.0 * rng.standard_normal((ny + 5, nx + 5))).astype(np.float32)
    tw = [0.0, 300.0, 900.0]
    us = [(1e-4 * rng.standard_normal((5, 7))).astype(np.float32) for _ in tw]
    vs = [(1e-4 * rng.standard_normal((5, 7))).astype(np.float32) for _ in tw]
    tp = [0.0, 450.0, 900.0]
    ps = [(50.0 * rng.standard_normal((6, 8))).astype(np.float32) for _ in tp]
    got, exp = _run(gpu_ctx, "cdklm_forcing77", "boundary", nx, ny, 150.0, 170.0, H, eta0, (1, 1, 1, 1),
                    (0, 0, 0, 0), None, 800.0, f=1.2e-4, wind=(tw, us, vs), pressure=(tp, ps))
    d = _report("time-varying textured wind stress and atmospheric pressure", got, exp)
    assert max(d.values()) == 0.0


def test_direct_lookup_pressure(gpu_ctx):
    """use_direct_lookup with a pressure array of the grid's own size, two
    time stamps, against the reference kernel built with the define its host
    writes (USE_DIRECT_LOOKUP True, which the preprocessor reads as 0: the
    reference interpolates the array, and so does this build)."""
    nx, ny = 77, 45
    rng = np.random.default_rng(12)
    x = np.arange(nx + 4) - 2 + 0.5 - nx / 2.0
    y = np.arange(ny + 4) - 2 + 0.5 - ny / 2.0
    eta0 = (0.1 * np.exp(-(x[None, :] ** 2 + y[:, None] ** 2) / 80.0)).astype(np.float32)
    H = (40.0 + 2.0 * rng.standard_normal((ny + 5, nx + 5))).astype(np.float32)
    tw = [0.0]
    us = [(1e-4 * rng.standard_normal((5, 7))).astype(np.float32)]
    vs = [(1e-4 * rng.standard_normal((5, 7))).astype(np.float32)]
    tp = [0.0, 600.0]
    ps = [(80.0 * rng.standard_normal((ny + 4, nx + 4))).astype(np.float32) for _ in tp]
    got, exp = _run(gpu_ctx, "cdklm_direct77", "boundary", nx, ny, 150.0, 170.0, H, eta0, (1, 1, 1, 1),
                    (0, 0, 0, 0), None, 800.0, f=1.2e-4, wind=(tw, us, vs), pressure=(tp, ps), direct=True)
    d = _report("atmospheric pressure by direct lookup", got, exp)
    assert max(d.values()) == 0.0
