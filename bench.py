"""Benchmark: member-cell-steps/s of the batched CDKLM16 ensemble on one GB300.

Workload (default ``c3``): 256 members on the double-jet domain
(nx=512, ny=300, dx=dy=5 km, periodic in x, walls in y, beta plane,
Gaussian-random bathymetry), 1000 drifters per member, stepped in blocks of
one model time step (60 s, ~3 RK2 steps per member at the CFL limit).  One
bench "step" is one such block for every member.  All inputs are synthetic
(seeded), as the reference's configurations are.

Output: one JSON line (rank 0).  ``--impl reference`` times the reference
algorithm on the host cores instead (the reference has no CPU step of its
own; the FP64 restatement under oracle/ stands in for it).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MODEL_TIME_STEP = 60.0
NOISE_FACTOR = 8          # coarse grid every 8 cells
NOISE_L_COARSE = 8.0      # SOAR length scale in coarse cells
NOISE_STD = 0.003         # target std of the SOAR eta perturbation [m]
# DRAM bytes (read + write) per member-cell-step of ensemble_rk2_kernel, from
# one ncu capture of a 96-member C3 launch (221.0 MB read + 148.7 MB written
# over 96 x 512 x 300 member-cell-steps, step built without FMA contraction);
# traffic of a bench launch is scaled by its member-cells.
NCU_DRAM_BYTES_PER_MEMBER_CELL = 369.7e6 / (96 * 512 * 300)
# Warp instructions per member-cell-step of the same capture
# (smsp__inst_executed.sum = 0.880e9): the step is bound by instruction issue,
# whose ceiling is 4 warp instructions per cycle per SM.
NCU_WARP_INST_PER_MEMBER_CELL = 0.880e9 / (96 * 512 * 300)
SM_COUNT = 152


def sample_extras(spec):
    """What the oracle's timed member block runs beside the step."""
    extras = [w for w, on in (("its SOAR model error", spec["noise"]),
                              (f"{spec['drifters']} drifters per member", spec["drifters"])) if on]
    return " with " + " and ".join(extras) if extras else ""


def model_error_text(spec):
    """The workload's model error as the bench lines describe it."""
    if not spec["noise"]:
        return None
    return (f"SOAR every {MODEL_TIME_STEP:.0f} s, coarse factor {NOISE_FACTOR}, L={NOISE_L_COARSE:g} coarse cells, "
            f"std {NOISE_STD} m")


def soar_q0(L_cells=NOISE_L_COARSE, std=NOISE_STD):
    """q0 such that the SOAR field sum_{5x5} Q xi has standard deviation `std`
    for unit normals: q0 = std / sqrt(sum s(d)^2), s(d) = (1 + d/L) exp(-d/L)."""
    oy, ox = np.mgrid[-2:3, -2:3]
    d = np.sqrt(ox ** 2 + oy ** 2) / L_cells
    return std / np.sqrt(np.sum(((1 + d) * np.exp(-d)) ** 2))


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------

def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# workload construction
# ---------------------------------------------------------------------------

def workload_spec(name, members):
    if name == "c3":
        return dict(name="c3", members=members, nx=512, ny=300, drifters=1000, noise=True)
    if name == "c1":
        return dict(name="c1", members=members, nx=256, ny=256, drifters=0, noise=False)
    raise SystemExit("unknown workload " + name)


def make_case(spec):
    from gpuocean_gb300.utils import BenchmarkCases
    if spec["name"] == "c3":
        return BenchmarkCases.double_jet_case(nx=spec["nx"], ny=spec["ny"])
    return BenchmarkCases.gaussian_bump_case(nx=spec["nx"], ny=spec["ny"])


def build_members(ctx, spec, case):
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.drifters import GPUDrifterCollection
    from gpuocean_gb300.utils import Common
    sims = []
    bc = Common.BoundaryConditions(*case["boundary"])
    for m in range(spec["members"]):
        sim = CDKLM16.CDKLM16(ctx, case["eta0"], case["hu0"], case["hv0"], case["H"], case["nx"], case["ny"],
                              case["dx"], case["dy"], 0.0, case["g"], case["f"], case["r"],
                              coriolis_beta=case.get("coriolis_beta", 0.0), boundary_conditions=bc,
                              model_time_step=MODEL_TIME_STEP)
        if spec["drifters"]:
            rng = np.random.default_rng(5000 + m)
            d = GPUDrifterCollection.GPUDrifterCollection(
                ctx, spec["drifters"], boundaryConditions=bc, domain_size_x=case["nx"] * case["dx"],
                domain_size_y=case["ny"] * case["dy"], gpu_stream=sim.gpu_stream)
            pos = np.stack([rng.uniform(0, case["nx"] * case["dx"], spec["drifters"]),
                            rng.uniform(0, case["ny"] * case["dy"], spec["drifters"])], axis=1)
            d.setDrifterPositions(pos)
            d.setObservationPosition(np.array([0.5 * case["nx"] * case["dx"], 0.5 * case["ny"] * case["dy"]]))
            sim.attachDrifters(d)
        if spec.get("noise"):
            from gpuocean_gb300.SWEsimulators.OceanStateNoise import OceanStateNoise
            cdx = case["dx"] * NOISE_FACTOR
            sim.model_error = OceanStateNoise.fromsim(sim, soar_q0=soar_q0(), soar_L=NOISE_L_COARSE * cdx,
                                                      interpolation_factor=NOISE_FACTOR, strict_odd_factor=False)
        sims.append(sim)
    return sims


def algorithmic_bytes_per_launch(sims, n_active, distinct_bathymetry):
    """24 B per member-cell-step (read + write eta, hu, hv), 4 B per corner of
    each distinct bathymetry, 16 B per drifter-step (read + write x, y)."""
    cells = sum(int(s.nx) * int(s.ny) for s in sims[:n_active])
    bathy = distinct_bathymetry * (int(sims[0].nx) + 5) * (int(sims[0].ny) + 5) * 4
    drift = sum((s.drifters.getNumDrifters() + 1) * 16 for s in sims[:n_active] if s.hasDrifters)
    return 24 * cells + bathy + drift


# ---------------------------------------------------------------------------
# the reference algorithm on the host (CPU baseline and the reference arm)
# ---------------------------------------------------------------------------

def _oracle_member_block(args):
    spec, m, n_blocks = args
    from oracle.cdklm16_oracle import BC, OracleCDKLM16
    from oracle.noise_oracle import bicubic_perturbation, drift, soar_coarse
    case = make_case(spec)
    nx, ny, dx, dy = case["nx"], case["ny"], case["dx"], case["dy"]
    bc = BC(*case["boundary"])
    sim = OracleCDKLM16(case["eta0"], case["hu0"], case["hv0"], case["H"], nx, ny, dx, dy, 0.0, case["g"], case["f"],
                        case["r"], coriolis_beta=case.get("coriolis_beta", 0.0), boundary_conditions=bc)
    rng = np.random.default_rng(1000 + m)
    pos = None
    if spec["drifters"]:
        pos = np.stack([rng.uniform(0, nx * dx, spec["drifters"] + 1), rng.uniform(0, ny * dy, spec["drifters"] + 1)],
                       axis=1)
    t0 = time.perf_counter()
    steps = 0
    for _ in range(n_blocks):
        before = sim.num_iterations
        sim.step(MODEL_TIME_STEP)
        taken = sim.num_iterations - before
        steps += taken
        if spec["noise"]:
            # the block's SOAR model error (normals from numpy: only the work
            # is timed here, the draws are not the engine's)
            cnx, cny = -(-nx // NOISE_FACTOR), -(-ny // NOISE_FACTOR)
            cdx, cdy = dx * NOISE_FACTOR, dy * NOISE_FACTOR
            pns, pew = bc.north == 2, bc.east == 2
            xi = rng.standard_normal((cny if pns else cny + 8, cnx if pew else cnx + 8))
            coarse = soar_coarse(xi, cnx, cny, cdx, cdy, soar_q0(), NOISE_L_COARSE * cdx, pns, pew)
            bicubic_perturbation(sim.Q0[0], sim.Q0[1], sim.Q0[2], coarse, sim.Hi, nx, ny, dx, dy, cnx, cny, cdx, cdy,
                                 float(sim.f), float(sim.coriolis_beta), case["g"])
        if pos is not None:
            # one drifter step per model step of the block
            for _ in range(taken):
                pos = drift(pos, sim.Q0[0], sim.Q0[1], sim.Q0[2], sim.Hm, nx, ny, dx, dy, sim.dt,
                            bc.north == 2, bc.east == 2)
    return steps * nx * ny, time.perf_counter() - t0


def cpu_reference_rate(spec, n_members, n_blocks, cores):
    """member-cell-steps/s of the FP64 oracle on `cores` processes."""
    jobs = [(spec, m, n_blocks) for m in range(n_members)]
    t0 = time.perf_counter()
    if cores <= 1:
        res = [_oracle_member_block(j) for j in jobs]
    else:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(cores) as pool:
            res = pool.map(_oracle_member_block, jobs)
    wall = time.perf_counter() - t0
    cells = sum(r[0] for r in res)
    return cells / wall, wall


def run_reference(args, spec, rank, world):
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    n_members = max(cores, 1)
    for _ in range(args.warmup):
        cpu_reference_rate(spec, n_members, 1, cores)
    # timed steps: at most K, and no more once 90 s of them have run
    rates, walls = [], []
    while len(rates) < max(1, args.steps) and sum(walls) < 90.0:
        r, w = cpu_reference_rate(spec, n_members, 1, cores)
        rates.append(r)
        walls.append(w)
    value = statistics.median(rates)
    wall = statistics.median(walls)
    sample = (f"{n_members} of the {spec['members']} members x 1 block of {MODEL_TIME_STEP:.0f} s of the "
              f"{spec['name']} workload per step{sample_extras(spec)}, FP64 NumPy restatement (the reference has no "
              f"CPU step), one member per process")
    line = {"metric": "member-cell-steps/s", "value": value, "unit": "member-cell-steps/s", "n_gpus": world,
            "steps": len(rates), "warmup": args.warmup, "ms_per_step": 1000.0 * wall, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": spec["name"], "members": spec["members"], "nx": spec["nx"], "ny": spec["ny"],
                       "drifters_per_member": spec["drifters"], "block_seconds": MODEL_TIME_STEP,
                       "model_error": model_error_text(spec)},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "member-cell-steps/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "member-cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# uneven multi-level ensemble (512 x 64x128, 128 x 128x256, 32 x 256x512)
# ---------------------------------------------------------------------------

def run_multilevel(ctx, args, levels=((128, 64, 512), (256, 128, 128), (512, 256, 32)), blocks=10, reps=3):
    """All levels share one physical domain (2560 km x 1500 km) and the
    double-jet physics with SOAR model error (independent per member).  The
    members of each grid advance in one persistent launch per RK2 step of
    their own engine, the three engines on their own streams (each engine's
    members share their scalar parameters, which its kernel then reads from
    the parameter space, and the levels' launches overlap); for comparison
    all 672 members also run as one engine.  Each configuration, and the
    member-by-member sample, is timed `reps` times (a repetition takes a few
    tens of milliseconds, so one host-side stall can dominate it) and reports
    the median.  Returns the batched and the member-by-member member-cell-steps/s."""
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.SWEsimulators.OceanStateNoise import OceanStateNoise
    from gpuocean_gb300.utils import BenchmarkCases, Common
    Lx, Ly = 2560e3, 1500e3
    bc = Common.BoundaryConditions(1, 2, 1, 2)

    def make():
        per_level = []
        for nx, ny, n in levels:
            c = BenchmarkCases.double_jet_case(nx=nx, ny=ny, dx=Lx / nx, dy=Ly / ny)
            lv = []
            for m in range(n):
                s = CDKLM16.CDKLM16(ctx, c["eta0"], c["hu0"], c["hv0"], c["H"], nx, ny, c["dx"], c["dy"], 0.0,
                                    c["g"], c["f"], 0.0, coriolis_beta=c["coriolis_beta"], boundary_conditions=bc,
                                    model_time_step=MODEL_TIME_STEP)
                s.model_error = OceanStateNoise.fromsim(s, soar_q0=soar_q0(),
                                                        soar_L=NOISE_L_COARSE * c["dx"] * NOISE_FACTOR,
                                                        interpolation_factor=NOISE_FACTOR, strict_odd_factor=False)
                lv.append(s)
            per_level.append(lv)
        return per_level

    def timed(engines):
        for e in engines:
            e.updateDt(courant_number=0.8)
        for _ in range(2):
            for e in engines:
                e.step(MODEL_TIME_STEP, apply_stochastic_term=True)
        for e in engines:
            e.synchronize()
        rates = []
        for _ in range(reps):
            t0 = time.perf_counter()
            cells = 0
            for _ in range(blocks):
                for e in engines:
                    cells += e.step(MODEL_TIME_STEP, apply_stochastic_term=True)
            for e in engines:
                e.synchronize()
            rates.append(cells / (time.perf_counter() - t0))
        return float(np.median(rates)), rates

    # all members as one engine
    per_level = make()
    sims = [s for lv in per_level for s in lv]
    one = BatchedEnsemble(sims)
    one.set_noise([s.model_error for s in sims], rng_seed=77)
    one_engine, one_engine_reps = timed([one])
    one.release()
    for s in sims:
        s.cleanUp(do_gc=False)
    # one engine per grid, each on its own stream
    per_level = make()
    sims = [s for lv in per_level for s in lv]
    engines = []
    for k, lv in enumerate(per_level):
        e = BatchedEnsemble(lv)
        e.set_noise([s.model_error for s in lv], rng_seed=77 + k)
        engines.append(e)
    batched, batched_reps = timed(engines)
    shape = [list(e.tile_shape) for e in engines]
    for e in engines:
        e.release()
    # member by member: a sample of every level, stepped from Python
    sample = [s for lv in range(len(levels)) for s in sims[sum(l[2] for l in levels[:lv]):][:8]]
    for s in sample:
        s.step(MODEL_TIME_STEP, apply_stochastic_term=False)
        s.perturbState()
    for s in sample:
        s.gpu_stream.synchronize()
    pm_rates = []
    for _ in range(reps):
        t0 = time.perf_counter()
        pm = 0
        for s in sample:
            before = s.num_iterations
            s.step(MODEL_TIME_STEP, apply_stochastic_term=False)
            s.perturbState()
            pm += (s.num_iterations - before) * int(s.nx) * int(s.ny)
        for s in sample:
            s.gpu_stream.synchronize()
        pm_rates.append(pm / (time.perf_counter() - t0))
    per_member = float(np.median(pm_rates))
    for s in sims:
        s.cleanUp(do_gc=False)
    return {"workload": "c4", "levels": [list(l) for l in levels], "members": len(sims),
            "value": batched, "unit": "member-cell-steps/s", "blocks": blocks, "repetitions": reps,
            "value_per_repetition": batched_reps, "engines": "one per grid, each on its own stream",
            "one_engine_value": one_engine, "one_engine_value_per_repetition": one_engine_reps,
            "per_member_baseline": per_member, "per_member_baseline_per_repetition": pm_rates,
            "batched_over_per_member": batched / per_member,
            "per_member_sample": len(sample), "tile_shape": shape}


def run_statistics(ens, sims, peak, peak_kind, n_positions=1000, repeats=10):
    """Observation operator and ensemble statistics on the C3 ensemble
    (every member at 512 x 300): one launch observing every member at
    n_positions shared positions, and mean + variance of (eta, hu, hv) and of
    the desingularised (u, v) over all members (E/BaseOceanStateEnsemble.py:
    79-176).  The member states (12 B per member-cell) exceed L2.  Algorithmic
    bytes: the member fields read once plus the two output fields.  The
    reference's path - download every member, reduce with NumPy - is timed
    once on the same members."""
    from gpuocean_gb300 import _lib
    n = len(sims)
    nx, ny = int(sims[0].nx), int(sims[0].ny)
    cells = nx * ny
    stream = ens.stream.handle
    ev = [ctypes.c_void_p(), ctypes.c_void_p()]
    for e in ev:
        _lib.call("goc_event_create", ctypes.byref(e))

    def timed(fn):
        fn()
        ens.synchronize()
        _lib.call("goc_event_record", ev[0], stream)
        for _ in range(repeats):
            fn()
        _lib.call("goc_event_record", ev[1], stream)
        ens.synchronize()
        ms = ctypes.c_float()
        _lib.call("goc_event_elapsed_ms", ev[0], ev[1], ctypes.byref(ms))
        return ms.value / repeats

    out = {"members": n, "nx": nx, "ny": ny}
    m, v = ens.moments(download=False)
    mu, vu = ens.moments(quantity="velocity", desingularise=1e-5, download=False)
    ens._ensure_table()
    for key, q, planes, eps, bm, bv in (("state", 0, 3, 0.0, m, v), ("velocity", 1, 2, 1e-5, mu, vu)):
        ms = timed(lambda: _lib.call("goc_ensemble_moments", ens._handle, 0, n, q, ctypes.c_float(eps), 0, bm.ptr,
                                     bv.ptr, stream))
        alg = n * cells * (12 if q == 0 else 16) + 2 * planes * cells * 4
        out[f"moments_{key}_ms"] = ms
        out[f"moments_{key}_gbs"] = alg / (ms * 1e-3) / 1e9
        out[f"moments_{key}_frac"] = out[f"moments_{key}_gbs"] / peak
    for b in (m, v, mu, vu):
        b.free()
    out["peak_gbs"], out["peak_kind"] = peak, peak_kind
    out["bytes_per_member_cell"] = {"state": 12, "velocity": "16 (eta, hu, hv, Hm)"}
    rng = np.random.default_rng(3)
    pos = np.stack([rng.uniform(0, nx * float(sims[0].dx), n_positions),
                    rng.uniform(0, ny * float(sims[0].dy), n_positions)], axis=1).astype(np.float32)
    ens.observe(pos)
    out_buf = ens._obs_out
    pbuf = ens._obs_pos
    out["observe_ms"] = timed(lambda: _lib.call("goc_ensemble_observe", ens._handle, 0, n, pbuf.ptr, 8,
                                                ctypes.c_longlong(0), n_positions, out_buf.ptr, stream))
    out["observe_positions"] = n_positions
    for e in ev:
        _lib.load().goc_event_destroy(e)
    # the reference's path: download every member's interior, reduce with NumPy
    t0 = time.perf_counter()
    st = np.moveaxis(np.array([np.array(s.download(interior_domain_only=True)) for s in sims]), 0, -1)
    np.mean(st, axis=-1)
    np.var(st, axis=-1)
    out["host_download_numpy_ms"] = 1000.0 * (time.perf_counter() - t0)
    out["device_over_host"] = out["host_download_numpy_ms"] / (out["moments_state_ms"])
    return out


def issue_roofline(member_cells, seconds, clk):
    """The fused step against its actual bound, instruction issue: warp
    instructions per launch (ncu count per member-cell-step x member-cells)
    per second, against 4 per cycle on each of the 152 SMs at the SM clock
    sampled during the timed region."""
    mhz = (clk or {}).get("sm_mhz") or 2070.0
    achieved = NCU_WARP_INST_PER_MEMBER_CELL * member_cells / seconds / 1e9
    peak = 4 * SM_COUNT * mhz * 1e6 / 1e9
    return {"achieved": achieved, "peak": peak, "unit": "G warp-instructions/s", "frac": achieved / peak,
            "source": "ncu smsp__inst_executed.sum of a 96-member launch, scaled per member-cell"}


def run_c2(ctx, days=10.0):
    """The double jet of one simulator for `days` of simulated time (512 x 300,
    dx = dy = 5 km, periodic x, walls y, beta plane, 230 m + 10 m random
    bathymetry): dt from updateDt at Courant 0.8, kept fixed; the model is
    stepped through the public API (CDKLM16.step, one fused RK2 launch per
    step), one hour per call; wall time on the host around the whole run."""
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils import BenchmarkCases, Common
    c = BenchmarkCases.double_jet_case(nx=512, ny=300)
    sim = CDKLM16.CDKLM16(ctx, c["eta0"], c["hu0"], c["hv0"], c["H"], 512, 300, c["dx"], c["dy"], 0.0, c["g"], c["f"],
                          c["r"], coriolis_beta=c["coriolis_beta"],
                          boundary_conditions=Common.BoundaryConditions(*c["boundary"]))
    sim.updateDt(courant_number=0.8)
    sim.step(3600.0)
    sim.gpu_stream.synchronize()
    t_end = days * 86400.0
    t0 = time.perf_counter()
    steps0 = sim.num_iterations
    while sim.t < t_end - 1e-6:
        sim.step(min(3600.0, t_end - sim.t))
    sim.gpu_stream.synchronize()
    wall = time.perf_counter() - t0
    steps = sim.num_iterations - steps0
    eta = np.asarray(sim.download(interior_domain_only=True)[0])
    out = {"config": f"double jet 512x300, {days:g} days, dt {float(sim.dt):.3f} s fixed", "steps": int(steps),
           "wall_s": wall, "cell_steps_per_s": steps * 512 * 300 / wall, "finite": bool(np.isfinite(eta).all())}
    sim.cleanUp()
    return out


def run_open_boundaries(ctx, hours=1.0):
    """Open boundaries and time-varying forcing on one 512 x 300 simulator:
    flow relaxation on every side (10 cells) toward exterior data at two time
    stamps, and a 9 x 7 wind-stress texture at three time stamps; a Gaussian
    bump on 200 m depth, beta plane.  Host wall time around `hours` of model
    time through CDKLM16.step (each RK2 step: two stage launches with the
    sponge between them and the time interpolation of both)."""
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils import Common, WindStress
    nx, ny, dx, dy = 512, 300, 5000.0, 5000.0
    rng = np.random.default_rng(17)
    yy, xx = np.mgrid[0:ny + 4, 0:nx + 4].astype(np.float64)
    eta0 = (0.5 * np.exp(-((xx - nx / 2) ** 2 + (yy - ny / 2) ** 2) / 40.0 ** 2)).astype(np.float32)
    z = np.zeros_like(eta0)
    H = np.full((ny + 5, nx + 5), 200.0, np.float32)
    t = [0.0, 7200.0]
    sides = {}
    for side, n in (("north", nx + 4), ("south", nx + 4), ("east", ny + 4), ("west", ny + 4)):
        sides[side] = Common.SingleBoundaryConditionData(
            h=[rng.uniform(-0.05, 0.05, n).astype(np.float32) for _ in t],
            hu=[np.zeros(n, np.float32) for _ in t], hv=[np.zeros(n, np.float32) for _ in t])
    data = Common.BoundaryConditionsData(t=t, **sides)
    bc = Common.BoundaryConditions(3, 3, 3, 3, spongeCells={"north": 10, "south": 10, "east": 10, "west": 10})
    wt = [0.0, 3600.0, 7200.0]
    wind = WindStress.WindStress(t=wt, stress_u=[rng.uniform(-1e-4, 1e-4, (7, 9)).astype(np.float32) for _ in wt],
                                 stress_v=[rng.uniform(-1e-4, 1e-4, (7, 9)).astype(np.float32) for _ in wt])
    sim = CDKLM16.CDKLM16(ctx, eta0, z, z.copy(), H, nx, ny, dx, dy, 0.0, 9.81, 1.2e-4, 0.0, coriolis_beta=2e-11,
                          boundary_conditions=bc, boundary_conditions_data=data, wind=wind)
    sim.updateDt(courant_number=0.8)
    sim.step(600.0)
    sim.gpu_stream.synchronize()
    steps0 = sim.num_iterations
    t0 = time.perf_counter()
    sim.step(hours * 3600.0)
    sim.gpu_stream.synchronize()
    wall = time.perf_counter() - t0
    steps = sim.num_iterations - steps0
    eta = np.asarray(sim.download(interior_domain_only=True)[0])
    sim.cleanUp()
    return {"config": "512x300, flow relaxation on all sides (10 cells, data at 2 times), 9x7 wind at 3 times",
            "steps": int(steps), "wall_s": wall, "cell_steps_per_s": steps * nx * ny / wall,
            "finite": bool(np.isfinite(eta).all())}


def run_netcdf(ctx, timesteps=10):
    """NetCDF output and hot start of the 512 x 300 double jet: host wall time
    per written time step (download of eta, hu, hv + the file write, the file
    closed at the end) and for CDKLM16.fromfilename of the last one.  The file
    lives in a temporary directory under the repository."""
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils import BenchmarkCases, Common
    c = BenchmarkCases.double_jet_case(nx=512, ny=300)
    with tempfile.TemporaryDirectory(dir=ROOT) as d:
        fn = os.path.join(d, "double_jet")
        sim = CDKLM16.CDKLM16(ctx, c["eta0"], c["hu0"], c["hv0"], c["H"], 512, 300, c["dx"], c["dy"], 0.0, c["g"],
                              c["f"], c["r"], coriolis_beta=c["coriolis_beta"],
                              boundary_conditions=Common.BoundaryConditions(*c["boundary"]),
                              write_netcdf=True, netcdf_filename=fn)
        sim.updateDt(courant_number=0.8)
        sim.step(600.0, write_now=False)
        sim.gpu_stream.synchronize()
        t0 = time.perf_counter()
        for _ in range(timesteps):
            sim.writeState()
        sim.closeNetCDF()
        write_s = time.perf_counter() - t0
        size = os.path.getsize(fn + ".nc")
        t0 = time.perf_counter()
        hot = CDKLM16.CDKLM16.fromfilename(ctx, fn + ".nc", cont_write_netcdf=False)
        hot.gpu_stream.synchronize()
        hot_s = time.perf_counter() - t0
        same = all(np.array_equal(np.asarray(a), np.asarray(b)) for a, b in zip(sim.download(), hot.download()))
        hot.cleanUp()
        sim.cleanUp()
    mb = 3 * 516 * 304 * 4 / 1e6
    return {"config": "double jet 512x300, classic NetCDF (64-bit offset)", "timesteps": timesteps + 1,
            "write_ms_per_timestep": 1000.0 * write_s / timesteps, "mb_per_timestep": mb,
            "write_mb_per_s": mb * timesteps / write_s, "file_mb": size / 1e6,
            "hot_start_ms": 1000.0 * hot_s, "hot_start_state_identical": bool(same)}


def run_kl(ens, sims, peak, peak_kind, repeats=10):
    """Karhunen-Loeve model error on the C3 ensemble (every member at
    512 x 300) with the double-jet case's KL parameters (basis 2..8 x 1..7,
    decay 1.25, scaling 0.025; S/ModelErrorKL.py, the reference's
    DoubleJetCase model_error=2): one batched perturbation of all members -
    the basis tables, then the balanced update of every member-cell - timed
    with CUDA events, normals drawn on the device.  Algorithmic bytes of the
    update: read and write eta, hu, hv (24 B per member-cell) plus the shared
    corner depths once."""
    from gpuocean_gb300 import _lib
    from gpuocean_gb300.SWEsimulators.ModelErrorKL import ModelErrorKL
    kls = [ModelErrorKL.fromsim(s, kl_decay=1.25, kl_scaling=0.025, basis_x_start=2, basis_x_end=8,
                                basis_y_start=1, basis_y_end=7, np_seed=9000 + m) for m, s in enumerate(sims)]
    ens.set_noise(kls, rng_seed=31)
    for _ in range(3):
        ens.perturb(perturbation_scale=1e-3)
    ens.synchronize()
    stream = ens.stream.handle
    ev = [ctypes.c_void_p(), ctypes.c_void_p()]
    for e in ev:
        _lib.call("goc_event_create", ctypes.byref(e))
    _lib.call("goc_event_record", ev[0], stream)
    for _ in range(repeats):
        ens.perturb(perturbation_scale=1e-3)
    _lib.call("goc_event_record", ev[1], stream)
    ens.synchronize()
    ms = ctypes.c_float()
    _lib.call("goc_event_elapsed_ms", ev[0], ev[1], ctypes.byref(ms))
    for e in ev:
        _lib.load().goc_event_destroy(e)
    per = ms.value / repeats
    nx, ny = int(sims[0].nx), int(sims[0].ny)
    cells = len(sims) * nx * ny
    alg = 24 * cells + 4 * (nx + 5) * (ny + 5)
    ens.release_noise()
    for k in kls:
        k.cleanUp()
    return {"members": len(sims), "nx": nx, "ny": ny, "perturbation_ms": per,
            "member_cells_per_s": cells / (per * 1e-3), "gbs": alg / (per * 1e-3) / 1e9,
            "frac": alg / (per * 1e-3) / 1e9 / peak, "peak_kind": peak_kind,
            "launches": "RNG + tables + update (3)"}


def run_adjoint(ctx, n=256, n_steps=400, every=10, n_points=64):
    """Adjoint of the CDKLM16 rollout: the Gaussian bump (n x n, dx = dy =
    200 m, H = 60 m, f = 1.2e-4, walls, 0.1 m amplitude, sigma 10 cells) with
    uniform wind stress (1e-4, 0) m^2/s^2, CFL 0.45, n_steps RK2 steps; loss =
    squared (u, v) misfit at n_points seeded cells every `every` steps against
    a truth run from half the bump without wind.  Times forward and backward
    of the autograd rollout with CUDA events on torch's stream, with the whole
    trajectory kept and with sqrt(N) checkpointing, and the kernels alone
    (one step VJP against one fused step)."""
    import torch
    from gpuocean_gb300.adjoint import CDKLM16Rollout, StepAdjoint
    from gpuocean_gb300.SWEsimulators import CDKLM16
    x = (np.arange(n + 4) - 2 + 0.5 - n / 2.0)
    eta = (0.1 * np.exp(-(x[None, :] ** 2 + x[:, None] ** 2) / 200.0)).astype(np.float32)
    z = np.zeros_like(eta)
    H = np.full((n + 5, n + 5), 60.0, np.float32)
    sim = CDKLM16.CDKLM16(ctx, eta, z, z.copy(), H, n, n, 200.0, 200.0, 0.0, 9.81, 1.2e-4, 0.0)
    sim.updateDt(courant_number=0.45)
    rng = np.random.default_rng(3)
    idx = rng.choice(n * n, size=n_points, replace=False)
    rows, cols = idx // n, idx % n
    out = {"config": f"bump {n}x{n}, wind (1e-4, 0), {n_steps} steps, (u, v) misfit at {n_points} cells every "
                     f"{every} steps", "dt": float(sim.dt)}
    ev = lambda: torch.cuda.Event(enable_timing=True)
    for label, frac in (("stored", 0.5), ("checkpointed", 0.0)):
        adj = StepAdjoint(sim, memory_fraction=frac)
        dev = adj.device
        Hm = torch.as_tensor(np.asarray(sim.downloadBathymetry()[1], np.float32)[2:-2, 2:-2], device=dev)
        q0 = adj.state(*sim.download())
        with torch.no_grad():
            t0 = [a.clone() for a in q0]
            t0[0] *= 0.5
            ts = CDKLM16Rollout.apply(adj, n_steps, every, *t0, torch.zeros(2, device=dev))
            hh = ts[:, 0] + Hm
            u_obs = ts[:, 1, rows, cols] / hh[:, rows, cols]
            v_obs = ts[:, 2, rows, cols] / hh[:, rows, cols]
        times = []
        for _ in range(3):
            xs = [a.clone().requires_grad_(True) for a in q0]
            w = torch.tensor([1.0e-4, 0.0], device=dev, requires_grad=True)
            e0, e1, e2 = ev(), ev(), ev()
            torch.cuda.synchronize()
            e0.record()
            st = CDKLM16Rollout.apply(adj, n_steps, every, *xs, w)
            hh = st[:, 0] + Hm
            loss = ((st[:, 1, rows, cols] / hh[:, rows, cols] - u_obs) ** 2).sum() + \
                   ((st[:, 2, rows, cols] / hh[:, rows, cols] - v_obs) ** 2).sum()
            e1.record()
            loss.backward()
            e2.record()
            torch.cuda.synchronize()
            times.append((e0.elapsed_time(e1), e1.elapsed_time(e2)))
        fwd, bwd = times[-1]
        out[label] = {"segment_steps": adj.segment_length(n_steps), "forward_ms": fwd, "backward_ms": bwd,
                      "adjoint_over_forward": bwd / fwd}
    # kernels alone: one step VJP (two stage-VJP launches) against one fused step
    qa, qb, qs = adj.zeros(), adj.zeros(), adj.zeros()
    la, ls, ln = adj.zeros(), adj.zeros(), adj.zeros()
    for a, b in zip(qa, q0):
        a.copy_(b)
    adj.step_with_stage(qa, qb, qs)
    for a in la:            # a dense adjoint: every reverse pass does its full work
        a.normal_()

    def timeit(fn, reps=200):
        for _ in range(10):
            fn()
        a, b = ev(), ev()
        torch.cuda.synchronize()
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    t_step = timeit(lambda: adj.step(qa, qb))
    t_vjp = timeit(lambda: adj.step_vjp(qa, qs, la, ls, ln, qb))   # qb: Q^{n+1} of qa
    out["kernels"] = {"step_ms": t_step, "step_vjp_ms": t_vjp, "vjp_over_step": t_vjp / t_step}
    sim.cleanUp()
    out["batched"] = run_adjoint_batched(ctx, ev, timeit)
    return out


def run_adjoint_batched(ctx, ev, timeit, n=128, members=128, n_steps=400, every=10, n_points=64):
    """The adjoint over `members` members of the n x n bump at once (states
    perturbed per member, one uniform wind each): one launch per forward step
    and two per step VJP for all members."""
    import torch
    from gpuocean_gb300.adjoint import CDKLM16EnsembleRollout, EnsembleStepAdjoint
    from gpuocean_gb300.SWEsimulators import CDKLM16
    x = (np.arange(n + 4) - 2 + 0.5 - n / 2.0)
    eta = (0.1 * np.exp(-(x[None, :] ** 2 + x[:, None] ** 2) / 200.0)).astype(np.float32)
    z = np.zeros_like(eta)
    sim = CDKLM16.CDKLM16(ctx, eta, z, z.copy(), np.full((n + 5, n + 5), 60.0, np.float32), n, n, 200.0, 200.0, 0.0,
                          9.81, 1.2e-4, 0.0)
    sim.updateDt(courant_number=0.45)
    adj = EnsembleStepAdjoint(sim, members)
    dev = adj.device
    rng = np.random.default_rng(5)
    base = torch.as_tensor(np.stack([np.asarray(a, np.float32) for a in sim.download()]), device=dev)
    scale = torch.as_tensor(rng.uniform(0.8, 1.2, members), dtype=torch.float32, device=dev)
    q0 = base.unsqueeze(0).repeat(members, 1, 1, 1)
    q0[:, 0] *= scale[:, None, None]
    winds = torch.as_tensor(rng.normal(0.0, 1.0e-4, (members, 2)), dtype=torch.float32, device=dev)
    idx = rng.choice(n * n, size=n_points, replace=False)
    rows, cols = idx // n, idx % n
    with torch.no_grad():
        t0 = q0.clone()
        t0[:, 0] *= 0.5
        ts = CDKLM16EnsembleRollout.apply(adj, n_steps, every, t0, torch.zeros_like(winds))
    times = []
    for _ in range(2):
        q = q0.clone().requires_grad_(True)
        w = winds.clone().requires_grad_(True)
        e0, e1, e2 = ev(), ev(), ev()
        torch.cuda.synchronize()
        e0.record()
        st = CDKLM16EnsembleRollout.apply(adj, n_steps, every, q, w)
        loss = ((st[..., 1:, rows, cols] - ts[..., 1:, rows, cols]) ** 2).sum()
        e1.record()
        loss.backward()
        e2.record()
        torch.cuda.synchronize()
        times.append((e0.elapsed_time(e1), e1.elapsed_time(e2)))
    fwd, bwd = times[-1]
    qa, qb, qs = adj.zeros(), adj.zeros(), adj.zeros()
    qa.copy_(q0)
    adj.step(qa, qb, qs)
    la, ls, ln = adj.zeros(), adj.zeros(), adj.zeros()
    la.normal_()
    t_step = timeit(lambda: adj.step(qa, qb))
    t_vjp = timeit(lambda: adj.step_vjp(qa, qs, la, ls, ln, qb))   # qb: Q^{n+1} of qa
    sim.cleanUp()
    cells = members * n * n
    return {"config": f"{members} members x {n}x{n} bump, per-member wind, {n_steps} steps, (hu, hv) misfit at "
                      f"{n_points} cells every {every} steps", "segment_steps": adj.segment_length(n_steps),
            "forward_ms": fwd, "backward_ms": bwd, "adjoint_over_forward": bwd / fwd,
            "kernels": {"step_ms": t_step, "step_vjp_ms": t_vjp, "vjp_over_step": t_vjp / t_step,
                        "forward_member_cell_steps_per_s": cells / (t_step * 1e-3),
                        "adjoint_member_cell_steps_per_s": cells / (t_vjp * 1e-3)}}


# ---------------------------------------------------------------------------
# main arm
# ---------------------------------------------------------------------------

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c3", choices=["c3", "c1"])
    ap.add_argument("--members", type=int, default=256)
    ap.add_argument("--per-member-sample", type=int, default=16)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-multilevel", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-statistics", action="store_true")
    ap.add_argument("--no-c2", action="store_true")
    args = ap.parse_args()
    rank, world, local = dist_env()
    spec = workload_spec(args.workload, args.members if args.workload == "c3" else 1)
    if args.impl == "reference":
        run_reference(args, spec, rank, world)
        return

    from gpuocean_gb300 import _lib
    from gpuocean_gb300.ensembles.BatchedEnsemble import BatchedEnsemble
    from gpuocean_gb300.utils import Common
    from gpuocean_gb300.utils.replicas import ReplicaGroup
    dist = ReplicaGroup(world, "nccl" if world > 1 else "gloo", rank=rank)
    ctx = Common.CUDAContext(device=local)
    case = make_case(spec)
    sims = build_members(ctx, spec, case)
    ens = BatchedEnsemble(sims)
    distinct_bathy = len(set(ens._bathy_owner))
    noise = bool(spec.get("noise"))
    if noise:
        # model error drawn on the device (XORWOW) for every member, every block
        ens.set_noise([s.model_error for s in sims], rng_seed=1000)
    ens.updateDt(courant_number=0.8)
    lib = _lib.load()
    stream = ens.stream.handle

    for _ in range(args.warmup):
        ens.step(MODEL_TIME_STEP, apply_stochastic_term=noise)
    ens.synchronize()

    ev = [ctypes.c_void_p() for _ in range(2)]
    for e in ev:
        _lib.call("goc_event_create", ctypes.byref(e))
    launches0 = ens.kernels_launched
    cells = 0
    clocks = ClockSampler(local)
    dist.barrier()
    ens.synchronize()
    clocks.start()
    wall0 = time.perf_counter()
    _lib.call("goc_event_record", ev[0], stream)
    for _ in range(args.steps):
        cells += ens.step(MODEL_TIME_STEP, apply_stochastic_term=noise)
    _lib.call("goc_event_record", ev[1], stream)
    ens.synchronize()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    dist.barrier()
    ms = ctypes.c_float()
    _lib.call("goc_event_elapsed_ms", ev[0], ev[1], ctypes.byref(ms))
    elapsed = dist.max(ms.value / 1000.0)
    launches = ens.kernels_launched - launches0
    # replicas: every rank runs the whole workload on its own GPU
    value = dist.throughput(cells, ms.value / 1000.0)

    # dominant kernel: per-launch CUDA-event times of the RK2 ensemble kernel
    # on the launching stream, over a few eager blocks
    sched = ens._schedule(MODEL_TIME_STEP)
    n_active = [int((sched[2] > k).sum()) for k in range(sched[3])]
    kev = [ctypes.c_void_p() for _ in range(2 * sched[3])]
    for e in kev:
        _lib.call("goc_event_create", ctypes.byref(e))
    ens._sched_key = None
    durations, bytes_k, cells_k = [], [], []
    for _ in range(3):
        scheds, table, n, nsub = ens._schedule(MODEL_TIME_STEP)
        _lib.call("goc_ensemble_set_schedule", ens._handle, table.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                  n.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), stream)
        for k in range(nsub):
            _lib.call("goc_event_record", kev[2 * k], stream)
            _lib.call("goc_ensemble_rk2_substep", ens._handle, k, stream)
            _lib.call("goc_event_record", kev[2 * k + 1], stream)
        _lib.call("goc_ensemble_end_block", ens._handle, int(nsub), stream)
        ens.synchronize()
        for k in range(nsub):
            t = ctypes.c_float()
            _lib.call("goc_event_elapsed_ms", kev[2 * k], kev[2 * k + 1], ctypes.byref(t))
            durations.append(t.value / 1000.0)
            bytes_k.append(algorithmic_bytes_per_launch(sims, n_active[k], distinct_bathy))
            cells_k.append(sum(int(s.nx) * int(s.ny) for s in sims[:n_active[k]]))
        for m, s in enumerate(sims):
            for x in scheds[m]:
                s.t += np.float64(x)
            if len(scheds[m]) % 2:
                s.gpu_data.swap()
        ens._ptrs = ens._current_ptrs()
    ens._sched_key = None
    avg_bytes = float(np.mean(bytes_k))
    traffic = NCU_DRAM_BYTES_PER_MEMBER_CELL * float(np.mean(cells_k))
    avg_dur = float(np.mean(durations))
    achieved = avg_bytes / avg_dur / 1e9
    peak, peak_kind = measured_peaks()

    # end to end through the public API: per block, upload from pinned host
    # memory every member's observation position and (with model error) the
    # block's N(0,1) draws, step, read back every member's drifter positions
    n_d = spec["drifters"]
    e2e = None
    if n_d:
        e2e_steps = max(2, args.steps // 2)
        in_obs = 8 * len(sims)
        rand_sizes = [int(s.model_error.rand_ny) * int(s.model_error.random_numbers.pitch) for s in sims] if noise else []
        in_rand = sum(rand_sizes)
        out_bytes = 8 * (n_d + 1) * len(sims)
        host_in = ctypes.c_void_p()
        host_out = ctypes.c_void_p()
        _lib.call("goc_host_alloc", ctypes.byref(host_in), in_obs + e2e_steps * in_rand)
        _lib.call("goc_host_alloc", ctypes.byref(host_out), out_bytes)
        obs = np.ctypeslib.as_array(ctypes.cast(host_in, ctypes.POINTER(ctypes.c_float)), shape=(len(sims), 2))
        obs[:, 0] = 0.5 * case["nx"] * case["dx"]
        obs[:, 1] = 0.5 * case["ny"] * case["dy"]
        pool = None
        if noise:
            draws = np.ctypeslib.as_array(ctypes.cast(host_in.value + in_obs, ctypes.POINTER(ctypes.c_float)),
                                          shape=(e2e_steps * in_rand // 4,))
            for m in range(len(sims)):
                # member m's normals for every block: default_rng(1000 + m)
                rng = np.random.default_rng(1000 + m)
                off = sum(rand_sizes[:m]) // 4
                for b in range(e2e_steps):
                    draws[b * in_rand // 4 + off: b * in_rand // 4 + off + rand_sizes[m] // 4] = \
                        rng.standard_normal(rand_sizes[m] // 4)
            pool = Common.DevicePtr(in_rand)
            ens.set_noise([s.model_error for s in sims], random_pool=pool)
        ens.synchronize()
        e2e_cells = 0
        t0 = time.perf_counter()
        for b in range(e2e_steps):
            # one copy of all observation positions, scattered on the device
            ens.upload_observation_positions(host_in.value)
            if noise:
                _lib.call("goc_memcpy_h2d_async", pool.ptr, host_in.value + in_obs + b * in_rand, in_rand, stream)
            e2e_cells += ens.step(MODEL_TIME_STEP, apply_stochastic_term=noise)
            # every member's drifters gathered on the device, one copy back
            ens.download_drifters(host_out.value)
        ens.synchronize()
        e2e_wall = time.perf_counter() - t0
        e2e = {"value": dist.throughput(e2e_cells, e2e_wall), "unit": "member-cell-steps/s",
               "h2d_bytes_per_step": in_obs + in_rand, "d2h_bytes_per_step": out_bytes}
        _lib.call("goc_host_free", host_in)
        _lib.call("goc_host_free", host_out)

    # per-member baseline: the plain simulator stepped member by member from
    # Python, as the reference's ensembles do
    pm_sims = sims[:max(1, min(args.per_member_sample, len(sims)))]
    ens.synchronize()

    def member_block(s):
        # CDKLM16.dataAssimilationStep cadence: a block of steps, then the model error
        s.step(MODEL_TIME_STEP, apply_stochastic_term=False)
        if noise:
            s.perturbState()

    for s in pm_sims:
        member_block(s)
    for s in pm_sims:
        s.gpu_stream.synchronize()
    # three wall-clock repetitions (each a few tens of milliseconds), median
    pm_rates = []
    for _ in range(3):
        t0 = time.perf_counter()
        pm_cells = 0
        for s in pm_sims:
            before = s.num_iterations
            member_block(s)
            pm_cells += (s.num_iterations - before) * int(s.nx) * int(s.ny)
        for s in pm_sims:
            s.gpu_stream.synchronize()
        pm_rates.append(pm_cells / (time.perf_counter() - t0))
    per_member_rate = float(np.median(pm_rates))

    ens_stats = None if args.no_statistics else run_statistics(ens, sims, *measured_peaks())
    kl = None if args.no_statistics else run_kl(ens, sims, *measured_peaks())
    c2 = None if args.no_c2 else run_c2(ctx)
    netcdf = None if args.no_c2 else run_netcdf(ctx)
    open_bc = None if args.no_c2 else run_open_boundaries(ctx)
    multilevel = None if args.no_multilevel else run_multilevel(ctx, args)
    adjoint = None if args.no_adjoint else run_adjoint(ctx)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        n_cpu_members = 2
        rate, wall_cpu = cpu_reference_rate(spec, n_cpu_members, 1, 1)
        cpu = {"value": rate, "unit": "member-cell-steps/s", "cores": 1, "kind": "port",
               "sample": f"{n_cpu_members} members x 1 block of {MODEL_TIME_STEP:.0f} s{sample_extras(spec)} "
                         f"({wall_cpu:.1f} s), FP64 NumPy restatement of the reference step on one core"}

    if rank == 0:
        line = {
            "metric": "member-cell-steps/s", "value": value, "unit": "member-cell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * elapsed / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": spec["name"], "members": len(sims), "nx": spec["nx"], "ny": spec["ny"],
                       "drifters_per_member": n_d, "block_seconds": MODEL_TIME_STEP,
                       "model_error": model_error_text(spec),
                       "substeps_per_block": int(sched[3]), "l2": "inputs larger than L2"
                       if 24 * sum(int(s.nx) * int(s.ny) for s in sims) > 129e6 else "inputs smaller than L2",
                       "parallelism": f"replicas x{world}",
                       "tile_shape": list(ens.tile_shape),
                       "autotune_ms_per_launch": {f"{a}x{b}": t for (a, b), t in
                                                  getattr(ens, "autotune_timings", {}).items()}},
            "per_member_baseline": {"value": per_member_rate, "unit": "member-cell-steps/s",
                                    "members_sampled": len(pm_sims), "value_per_repetition": pm_rates,
                                    "batched_over_per_member": value / world / per_member_rate},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of a 96-member "
                                           "launch, scaled per member-cell", "kernel": "ensemble_rk2_kernel",
                         "peak_kind": peak_kind, "avg_launch_ms": 1000.0 * avg_dur,
                         "algorithmic_bytes_per_launch": avg_bytes,
                         "issue": issue_roofline(float(np.mean(cells_k)), avg_dur, clk)},
            "e2e": e2e, "gpu_launches": launches, "clocks": clk, "cpu_baseline": cpu,
            "multilevel": multilevel, "adjoint": adjoint, "statistics": ens_stats, "kl_model_error": kl, "c2_ten_days": c2, "netcdf": netcdf, "open_boundaries": open_bc,
            "wall_s": wall,
        }
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
