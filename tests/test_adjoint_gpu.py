"""The hand-written CUDA adjoint of the RK2 step against autograd of the FP64
torch restatement (oracle/cdklm16_torch.py), and the rollout gradient against
central finite differences of the FP64 oracle.

Tolerances: one step's vector-Jacobian product agrees with FP64 autograd to
1e-4 of the largest gradient entry per field (the CUDA adjoint runs in FP32
on the FP32 forward state); the wind-stress gradient to 1e-4 relative.
"""
import json

import numpy as np
import pytest
import torch

from oracle.cdklm16_oracle import BC, OracleCDKLM16
from oracle.cdklm16_torch import TorchCDKLM16

pytestmark = pytest.mark.gpu


def _smooth(rng, shape, scale, width=4.0):
    a = rng.standard_normal(shape)
    k = np.exp(-0.5 * (np.arange(-8, 9) / width) ** 2)
    k /= k.sum()
    for ax in (0, 1):
        a = np.apply_along_axis(lambda r: np.convolve(r, k, mode="same"), ax, a)
    return (scale * a / np.max(np.abs(a))).astype(np.float32)


CASES = {
    "walls_f": dict(nx=64, ny=48, bc=(1, 1, 1, 1), f=1.0e-4, beta=0.0, r=0.0),
    "periodic_x_beta_friction": dict(nx=80, ny=40, bc=(1, 2, 1, 2), f=1.0e-4, beta=2.0e-9, r=3.0e-3),
    "periodic_xy": dict(nx=64, ny=32, bc=(2, 2, 2, 2), f=1.2e-4, beta=0.0, r=0.0),
}


def _case(name, seed=0):
    c = dict(CASES[name])
    rng = np.random.default_rng(seed)
    nx, ny = c["nx"], c["ny"]
    # depth constant within 5 cells of a wall: the wall-mirrored ghost cells
    # then have exactly the interior cell's depth.  Otherwise the flux
    # balancer's switch at a wall face (u_m > -u_p, K/CDKLM16_kernel.cu:137)
    # compares two numbers that are equal up to rounding, and FP32 and FP64
    # take different branches of a discontinuous flux there.
    taper = np.ones((ny + 5, nx + 5))
    if c["bc"][1] == 1:
        taper[:, :7] = 0.0
        taper[:, -7:] = 0.0
    if c["bc"][0] == 1:
        taper[:7, :] = 0.0
        taper[-7:, :] = 0.0
    c["H"] = (35.0 + taper * _smooth(rng, (ny + 5, nx + 5), 5.0)).astype(np.float32)
    c["eta"] = _smooth(rng, (ny + 4, nx + 4), 0.3)
    c["hu"] = _smooth(rng, (ny + 4, nx + 4), 8.0)
    c["hv"] = _smooth(rng, (ny + 4, nx + 4), 8.0)
    c["dx"], c["dy"], c["g"] = 200.0, 180.0, 9.81
    c["wind"] = (1.0e-4, -6.0e-5)
    return c


@pytest.fixture(scope="module")
def ctx():
    from gpuocean_gb300.utils import Common
    return Common.CUDAContext()


def _sim(ctx, c, dt):
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils import Common
    return CDKLM16.CDKLM16(ctx, c["eta"], c["hu"], c["hv"], c["H"], c["nx"], c["ny"], c["dx"], c["dy"], dt,
                           c["g"], c["f"], c["r"], coriolis_beta=c["beta"],
                           boundary_conditions=Common.BoundaryConditions(*c["bc"]))


def _torch_ref(c, dt, q0):
    o = OracleCDKLM16(c["eta"], c["hu"], c["hv"], c["H"], c["nx"], c["ny"], c["dx"], c["dy"], dt, c["g"], c["f"],
                      c["r"], coriolis_beta=c["beta"], boundary_conditions=BC(*c["bc"]))
    return TorchCDKLM16(o)


@pytest.mark.parametrize("name", list(CASES))
def test_step_vjp_matches_fp64_autograd(ctx, name):
    """One RK2 step's VJP at a random smooth state."""
    from gpuocean_gb300.adjoint import StepAdjoint
    c = _case(name)
    dt = 2.0
    sim = _sim(ctx, c, dt)
    adj = StepAdjoint(sim)
    adj.set_wind(c["wind"])
    q = adj.state(*sim.download())
    rng = np.random.default_rng(5)
    lam_next = adj.zeros()
    lam_host = [rng.standard_normal((c["ny"], c["nx"])) for _ in range(3)]
    for a, b in zip(lam_next, lam_host):
        a[2:-2, 2:-2] = torch.as_tensor(b, dtype=torch.float32)
    q_s, lam_s, lam_n = adj.zeros(), adj.zeros(), adj.zeros()
    adj.stage1(q, q_s)
    adj.reset_wind_grad()
    adj.step_vjp(q, q_s, lam_next, lam_s, lam_n)
    wind_bar = adj.wind_grad().cpu().numpy()
    torch.cuda.synchronize()
    ours = [a.cpu().numpy().astype(np.float64)[2:-2, 2:-2] for a in lam_n]

    tq = _torch_ref(c, dt, q)
    qt = [torch.tensor(a.cpu().numpy().astype(np.float64), requires_grad=True) for a in q]
    X = torch.tensor(float(np.float32(c["wind"][0])), dtype=torch.float64, requires_grad=True)
    Y = torch.tensor(float(np.float32(c["wind"][1])), dtype=torch.float64, requires_grad=True)
    out = tq.rk2_step(qt, X, Y, dt)
    loss = sum((o[2:-2, 2:-2] * torch.as_tensor(b)).sum() for o, b in zip(out, lam_host))
    loss.backward()
    ref = [a.grad.numpy()[2:-2, 2:-2] for a in qt]
    errs = [float(np.max(np.abs(a - b)) / np.max(np.abs(b))) for a, b in zip(ours, ref)]
    werr = [float(abs(wind_bar[0] - X.grad.item()) / abs(X.grad.item())),
            float(abs(wind_bar[1] - Y.grad.item()) / abs(Y.grad.item()))]
    print(json.dumps({"case": name, "rel_err_eta_hu_hv": errs, "rel_err_wind": werr}))
    assert max(errs) <= 1e-4, errs
    assert max(werr) <= 1e-4, werr
    sim.cleanUp()


def _stage_vjps(adj, q, q_s, lam):
    """Both stage VJPs of the CUDA adjoint: (x-bar of stage 2 w.r.t. Q*,
    a-bar of stage 2 w.r.t. Q^n, x-bar of stage 1 w.r.t. Q^n for y-bar = lam)."""
    import ctypes
    from gpuocean_gb300 import _lib
    from gpuocean_gb300.adjoint import _ptr
    s = adj._stream()
    common = (adj.pitch, adj.Hi.ptr, int(adj.Hi.pitch), adj.Hm.ptr, int(adj.Hm.pitch))
    xs, an, x0 = adj.zeros(), adj.zeros(), adj.zeros()
    _lib.call("goc_cdklm_stage_vjp", ctypes.byref(adj.params), ctypes.c_float(adj.dt), 1, *[_ptr(a) for a in q_s],
              *[_ptr(a) for a in q], *[_ptr(a) for a in lam], None, None, None, *[_ptr(a) for a in xs],
              *[_ptr(a) for a in an], *common, None, s)
    _lib.call("goc_cdklm_stage_vjp", ctypes.byref(adj.params), ctypes.c_float(adj.dt), 0, *[_ptr(a) for a in q],
              None, None, None, *[_ptr(a) for a in lam], None, None, None, *[_ptr(a) for a in x0], None, None, None,
              *common, None, s)
    torch.cuda.synchronize()
    return [[a.cpu().numpy().astype(np.float64)[2:-2, 2:-2] for a in v] for v in (xs, an, x0)]


def test_stage_vjps_of_moving_bump_match_autograd_at_the_same_point(ctx):
    """The Gaussian bump with a smooth current: each stage VJP against FP64
    autograd of the same stage evaluated at the same FP32 points (Q^n and the
    CUDA first stage Q*).

    Exact comparisons need states without FP32 ties: at rest, h = 60 m + eta
    with eta ~ 1e-5 m is quantised in FP32 (one ulp of 60 is 3.8e-6), so
    neighbouring depths, wave speeds and limiter arguments tie exactly in
    FP32 but not in FP64, and the two precisions take different subgradients
    (the CUDA adjoint differentiates the FP32 computation)."""
    from gpuocean_gb300.adjoint import StepAdjoint
    from oracle.cdklm16_torch import periodic_ghosts
    c = dict(_bump_case(64, moving=True), wind=(1.0e-4, -6.0e-5))
    dt = 2.0
    sim = _sim(ctx, c, dt)
    adj = StepAdjoint(sim)
    adj.set_wind(c["wind"])
    q = adj.state(*sim.download())
    q_s = adj.zeros()
    adj.stage1(q, q_s)
    rng = np.random.default_rng(4)
    lam = adj.zeros()
    lam_host = [rng.standard_normal((c["ny"], c["nx"])) for _ in range(3)]
    for a, b in zip(lam, lam_host):
        a[2:-2, 2:-2] = torch.as_tensor(b, dtype=torch.float32)
    xs, an, x0 = _stage_vjps(adj, q, q_s, lam)
    tq = _torch_ref(c, dt, q)
    X = torch.tensor(float(np.float32(c["wind"][0])), dtype=torch.float64)
    Y = torch.tensor(float(np.float32(c["wind"][1])), dtype=torch.float64)
    f64 = lambda v: [torch.tensor(a.cpu().numpy().astype(np.float64), requires_grad=True) for a in v]
    qn, qs = f64(q), f64(q_s)
    out = tq.stage(periodic_ghosts(qs, c["nx"], c["ny"], tq.bc),
                   periodic_ghosts(qn, c["nx"], c["ny"], tq.bc), X, Y, dt, 1)
    sum((o * torch.as_tensor(b)).sum() for o, b in zip(out, lam_host)).backward()
    ref_xs = [a.grad.numpy()[2:-2, 2:-2] for a in qs]
    ref_an = [a.grad.numpy()[2:-2, 2:-2] for a in qn]
    qn0 = f64(q)
    out = tq.stage(periodic_ghosts(qn0, c["nx"], c["ny"], tq.bc), None, X, Y, dt, 0)
    sum((o * torch.as_tensor(b)).sum() for o, b in zip(out, lam_host)).backward()
    ref_x0 = [a.grad.numpy()[2:-2, 2:-2] for a in qn0]
    errs = {k: [float(np.max(np.abs(a - b)) / np.max(np.abs(b))) for a, b in zip(o, r)]
            for k, o, r in (("stage2_qstar", xs, ref_xs), ("stage2_qn", an, ref_an), ("stage1", x0, ref_x0))}
    print(json.dumps({"case": "moving bump, stage VJPs", "rel_err": errs}))
    assert max(max(v) for v in errs.values()) <= 1e-5, errs
    sim.cleanUp()


def _bump_case(n=64, amplitude=0.1, moving=False):
    """The Gaussian-bump configuration (dx = dy = 200 m, H = 60 m, f = 1.2e-4,
    walls) on an n x n grid, sigma = 10 cells; at rest, or with a smooth
    random current of up to 0.1 m/s (hu, hv up to 6 m^2/s)."""
    x = (np.arange(n + 4) - 2 + 0.5 - n / 2.0)
    eta = (amplitude * np.exp(-(x[None, :] ** 2 + x[:, None] ** 2) / (2.0 * 10.0 ** 2))).astype(np.float32)
    hu = np.zeros_like(eta)
    hv = np.zeros_like(eta)
    if moving:
        rng = np.random.default_rng(21)
        hu = _smooth(rng, eta.shape, 6.0)
        hv = _smooth(rng, eta.shape, 6.0)
    return dict(nx=n, ny=n, bc=(1, 1, 1, 1), f=1.2e-4, beta=0.0, r=0.0, dx=200.0, dy=200.0, g=9.81,
                H=np.full((n + 5, n + 5), 60.0, np.float32), eta=eta, hu=hu, hv=hv)


def _misfit_setup(c, n_obs_points, seed):
    rng = np.random.default_rng(seed)
    idx = rng.choice(c["nx"] * c["ny"], size=n_obs_points, replace=False)
    return idx // c["nx"], idx % c["nx"]


def test_rollout_gradient_matches_fp64_finite_differences(ctx):
    """400 RK2 steps of the Gaussian bump (64 x 64) with uniform wind stress
    (1e-4, 0); loss = squared misfit of (u, v) at 64 seeded cells every 10
    steps against a truth run from a bump of half the amplitude without wind
    (FP64 oracle).
    Directional derivatives of the adjoint gradient are compared with central
    finite differences (eps = 1e-3) of the FP64 oracle rollout: along the
    gradient itself (relative error), along two random smooth directions
    (error relative to |grad| |direction|) and for the two wind components
    (error relative to |wind gradient|)."""
    from gpuocean_gb300.adjoint import CDKLM16Rollout, StepAdjoint
    c = _bump_case(64)
    n_steps, every = 400, 10
    sim = _sim(ctx, c, 0.0)
    sim.updateDt(courant_number=0.45)
    dt = float(sim.dt)
    adj = StepAdjoint(sim)
    dev = adj.device
    tau = np.array([1.0e-4, 0.0], dtype=np.float32)
    rows, cols = _misfit_setup(c, 64, 3)
    Hm = torch.as_tensor(np.asarray(sim.downloadBathymetry()[1], dtype=np.float32)[2:-2, 2:-2], device=dev)

    def uv(states):
        h = states[:, 0] + Hm
        return states[:, 1, rows, cols] / h[:, rows, cols], states[:, 2, rows, cols] / h[:, rows, cols]

    q0 = adj.state(*sim.download())
    o_base = OracleCDKLM16(c["eta"], c["hu"], c["hv"], c["H"], c["nx"], c["ny"], c["dx"], c["dy"], dt, c["g"],
                           c["f"], c["r"], boundary_conditions=BC(*c["bc"]))
    Hm64 = np.asarray(o_base.Hm, dtype=np.float64)[2:-2, 2:-2]
    base = [np.asarray(a.detach().cpu().numpy(), dtype=np.float64) for a in q0]

    def rollout64(q, tx, ty):
        o = OracleCDKLM16(c["eta"], c["hu"], c["hv"], c["H"], c["nx"], c["ny"], c["dx"], c["dy"], dt, c["g"],
                          c["f"], c["r"], boundary_conditions=BC(*c["bc"]))
        o.Q0 = [a.copy() for a in q]
        o.Q1 = [a.copy() for a in q]
        sh = (c["ny"] + 4, c["nx"] + 4)
        o.wind = (np.full(sh, tx), np.full(sh, ty))
        for k in range(n_steps // every):
            for _ in range(every):
                o.step(dt)
            e, hu, hv = (a[2:-2, 2:-2] for a in o.Q0)
            h = e[rows, cols] + Hm64[rows, cols]
            yield hu[rows, cols] / h, hv[rows, cols] / h

    # the truth (half the bump, no wind) in FP64, used by both sides
    truth0 = [b.copy() for b in base]
    truth0[0] = truth0[0] * 0.5
    obs = list(rollout64(truth0, 0.0, 0.0))
    u_obs_h = np.stack([a for a, _ in obs])
    v_obs_h = np.stack([b for _, b in obs])
    u_obs = torch.as_tensor(u_obs_h, dtype=torch.float32, device=dev)
    v_obs = torch.as_tensor(v_obs_h, dtype=torch.float32, device=dev)

    x = [a.clone().requires_grad_(True) for a in q0]
    w = torch.tensor(tau, device=dev, requires_grad=True)
    states = CDKLM16Rollout.apply(adj, n_steps, every, *x, w)
    u, v = uv(states)
    loss = ((u - u_obs) ** 2).sum() + ((v - v_obs) ** 2).sum()
    loss.backward()
    grads = [a.grad.double().cpu().numpy() for a in x]
    gw = w.grad.double().cpu().numpy()

    def loss64(q, tx, ty):
        return sum(np.sum((a - u_obs_h[k]) ** 2) + np.sum((b - v_obs_h[k]) ** 2)
                   for k, (a, b) in enumerate(rollout64(q, tx, ty)))

    def fd_state(delta, eps=1.0e-3):
        return (loss64([b + eps * dd for b, dd in zip(base, delta)], float(tau[0]), float(tau[1])) -
                loss64([b - eps * dd for b, dd in zip(base, delta)], float(tau[0]), float(tau[1]))) / (2 * eps)

    gnorm = np.sqrt(sum(float(np.sum(g * g)) for g in grads))
    results = {}
    # along the gradient (scaled to a 1e-2 m eta change at most)
    scale = 1.0e-2 / max(float(np.max(np.abs(g))) for g in grads)
    delta = [scale * g for g in grads]
    ad = sum(float(np.sum(g * dd)) for g, dd in zip(grads, delta))
    fd = fd_state(delta)
    results["gradient_direction"] = (ad, fd, abs(ad - fd) / abs(fd))
    rng = np.random.default_rng(9)
    for d in range(2):
        delta = [_smooth(rng, base[0].shape, s).astype(np.float64) for s in (0.01, 0.1, 0.1)]
        for a in delta:
            a[:2, :] = 0; a[-2:, :] = 0; a[:, :2] = 0; a[:, -2:] = 0
        dnorm = np.sqrt(sum(float(np.sum(dd * dd)) for dd in delta))
        ad = sum(float(np.sum(g * dd)) for g, dd in zip(grads, delta))
        fd = fd_state(delta)
        results[f"random_{d}"] = (ad, fd, abs(ad - fd) / (gnorm * dnorm))
    wnorm = float(np.sqrt(np.sum(gw * gw)))
    for comp in range(2):
        h = 1.0e-3 * 1.0e-4
        tp, tm = [float(tau[0]), float(tau[1])], [float(tau[0]), float(tau[1])]
        tp[comp] += h
        tm[comp] -= h
        fd = (loss64(base, *tp) - loss64(base, *tm)) / (2 * h)
        results[f"wind_{'xy'[comp]}"] = (float(gw[comp]), fd, abs(float(gw[comp]) - fd) / wnorm)
    loss_fd = loss64(base, float(tau[0]), float(tau[1]))
    print(json.dumps({"case": "rollout 400 steps 64x64 bump, FD of FP64 oracle", "results": results,
                      "loss_fp32": float(loss.item()), "loss_fp64": loss_fd}))
    # random directions: the adjoint of the FP32 forward against FP64 finite
    # differences, error relative to |grad| |direction|
    assert max(results["random_0"][2], results["random_1"][2]) <= 1e-4, results
    # along the gradient and for the wind the comparison is limited by the
    # FP32 forward itself: with H = 60 m and eta ~ 0.1 m an FP32 rollout of
    # 400 steps differs from the FP64 one by ~1e-3 of eta (h = H + eta loses
    # the low bits of eta), so the two losses have different minimisers by
    # that much; the adjoint itself is checked exactly against the FP64 VJP
    # chain on the FP32 trajectory (test below)
    assert results["gradient_direction"][2] <= 2e-3, results
    assert max(results["wind_x"][2], results["wind_y"][2]) <= 2e-3, results
    sim.cleanUp()


def _fd_study(ctx, moving, steps, with_fd32):
    """The 400-step rollout and loss of the FP64 finite-difference test on the
    64 x 64 bump (at rest, or with a smooth current everywhere), its adjoint
    gradient, and central differences along the gradient and two random
    smooth directions with the given steps: of the FP64 oracle rollout and,
    with with_fd32, of the FP32 forward that the adjoint differentiates (the
    product's own step).  Each directional derivative is taken along the
    difference that the two FP32-rounded inputs actually have.  Errors are
    relative to the directional derivative along the gradient and to
    |grad| |direction| along random directions."""
    from gpuocean_gb300.adjoint import CDKLM16Rollout, StepAdjoint
    c = _bump_case(64, moving=moving)
    n_steps, every = 400, 10
    sim = _sim(ctx, c, 0.0)
    sim.updateDt(courant_number=0.45)
    dt = float(sim.dt)
    adj = StepAdjoint(sim)
    dev = adj.device
    tau = np.array([1.0e-4, 0.0], dtype=np.float32)
    rows, cols = _misfit_setup(c, 64, 3)
    Hm = torch.as_tensor(np.asarray(sim.downloadBathymetry()[1], dtype=np.float32)[2:-2, 2:-2], device=dev)
    base32 = [a.detach().clone() for a in adj.state(*sim.download())]

    def rollout64(q):
        o = OracleCDKLM16(c["eta"], c["hu"], c["hv"], c["H"], c["nx"], c["ny"], c["dx"], c["dy"], dt, c["g"],
                          c["f"], c["r"], boundary_conditions=BC(*c["bc"]))
        Hm64 = np.asarray(o.Hm, dtype=np.float64)[2:-2, 2:-2]
        o.Q0 = [np.asarray(a, dtype=np.float64).copy() for a in q]
        o.Q1 = [a.copy() for a in o.Q0]
        sh = (c["ny"] + 4, c["nx"] + 4)
        o.wind = (np.full(sh, float(tau[0])), np.full(sh, float(tau[1])))
        for _ in range(n_steps // every):
            for _ in range(every):
                o.step(dt)
            e, hu, hv = (a[2:-2, 2:-2] for a in o.Q0)
            h = e[rows, cols] + Hm64[rows, cols]
            yield hu[rows, cols] / h, hv[rows, cols] / h

    base64 = [a.double().cpu().numpy() for a in base32]
    # the truth: half the bump (FP64), the same for both losses
    truth0 = [b.copy() for b in base64]
    truth0[0] = truth0[0] * 0.5
    obs = list(rollout64(truth0))
    u_obs_h = np.stack([a for a, _ in obs])
    v_obs_h = np.stack([b for _, b in obs])
    u_obs = torch.as_tensor(u_obs_h, device=dev)
    v_obs = torch.as_tensor(v_obs_h, device=dev)

    def loss_of(states):
        h = (states[:, 0] + Hm).double()
        u = states[:, 1, rows, cols].double() / h[:, rows, cols]
        v = states[:, 2, rows, cols].double() / h[:, rows, cols]
        return ((u - u_obs) ** 2).sum() + ((v - v_obs) ** 2).sum()

    x = [a.clone().requires_grad_(True) for a in base32]
    w = torch.tensor(tau, device=dev, requires_grad=True)
    loss_of(CDKLM16Rollout.apply(adj, n_steps, every, *x, w)).backward()
    grads = [a.grad.double() for a in x]

    def loss32(q):
        with torch.no_grad():
            return float(loss_of(CDKLM16Rollout.apply(adj, n_steps, every, *q, torch.tensor(tau, device=dev))))

    def loss64(q):
        return sum(float(np.sum((a - u_obs_h[k]) ** 2) + np.sum((b - v_obs_h[k]) ** 2))
                   for k, (a, b) in enumerate(rollout64(q)))

    gmax = max(float(g.abs().max()) for g in grads)
    gnorm = float(torch.sqrt(sum((g * g).sum() for g in grads)))
    rng = np.random.default_rng(9)
    directions = {"gradient": [g / gmax for g in grads]}
    for d in range(2):
        dd = [torch.as_tensor(_smooth(rng, base64[0].shape, s), dtype=torch.float64, device=dev)
              for s in (1.0, 10.0, 10.0)]
        for a in dd:
            a[:2, :] = 0; a[-2:, :] = 0; a[:, :2] = 0; a[:, -2:] = 0
        directions[f"random_{d}"] = dd
    results = {}
    for name, dd in directions.items():
        for step in steps:
            qp = [(b.double() + step * a).float() for b, a in zip(base32, dd)]
            qm = [(b.double() - step * a).float() for b, a in zip(base32, dd)]
            diff = [p.double() - m.double() for p, m in zip(qp, qm)]
            dnorm = float(torch.sqrt(sum((a * a).sum() for a in diff)))
            ad = float(sum((g * a).sum() for g, a in zip(grads, diff)))
            den = abs(ad) if name == "gradient" else gnorm * dnorm
            fd64 = loss64([p.double().cpu().numpy() for p in qp]) - loss64([m.double().cpu().numpy() for m in qm])
            r = dict(ad=ad, fd64=fd64, err64=abs(ad - fd64) / den)
            if with_fd32:
                fd32 = loss32(qp) - loss32(qm)
                r.update(fd32=fd32, err32=abs(ad - fd32) / den, fd32_vs_fd64=abs(fd32 - fd64) / den)
            results[f"{name}@{step:g}"] = r
    sim.cleanUp()
    return results


def test_rollout_fd_of_fp32_forward_matches_fp64_forward(ctx):
    """The bump at rest: finite differences of the FP32 forward (the
    product's step) agree with those of the FP64 oracle to ~1e-5, so the
    rounding of the FP32 trajectory is not what separates the adjoint from
    the FP64 finite differences.  That gap (~6e-4 along the gradient here)
    comes from the point itself: at rest, h = 60 m + eta is quantised in FP32
    (one ulp of 60 is 3.8e-6 m), so depths, wave speeds and limiter arguments
    of neighbouring cells tie in FP32 where they differ in FP64, and the
    adjoint - the derivative of the FP32 computation - takes the
    subgradients of those ties.  The moving bump below has no ties, and
    there the adjoint matches FP64 finite differences closely."""
    results = _fd_study(ctx, False, (1.0e-3,), True)
    print(json.dumps({"case": "rollout 400 steps 64x64 bump at rest, FD of FP32 and FP64 forwards",
                      "results": results}))
    assert max(r["fd32_vs_fd64"] for r in results.values()) <= 1e-4, results


def test_rollout_gradient_of_moving_bump_matches_fp64_fd(ctx):
    """The bump with a smooth current everywhere (no FP32 ties): the adjoint
    gradient of the 400-step rollout against FP64 central differences."""
    results = _fd_study(ctx, True, (1.0e-4, 1.0e-3), False)
    print(json.dumps({"case": "rollout 400 steps 64x64 moving bump, FD of FP64 forward", "results": results}))
    best = {}
    for key, r in results.items():
        name = key.split("@")[0]
        best[name] = min(best.get(name, np.inf), r["err64"])
    assert max(best.values()) <= 1e-4, results


def test_step_vjp_from_stage_outputs_equals_recompute(ctx):
    """The stage VJPs given the stage outputs (Q* and Q^{n+1} as the forward
    wrote them) skip the recompute of the stages' fluxes; without dry cells
    their results agree with the recomputing VJPs to rounding, for one
    simulator and for a batch of members.  The adjoint translation unit
    contracts multiply-adds and the two kernel variants recompute the
    forward slopes on different boxes, so the compiler may contract them
    differently: measured differences are a few ulps (2.9e-6 at values up
    to 27)."""

    def close(a, b):
        torch.testing.assert_close(a, b, rtol=2e-6, atol=2e-6 * float(b.abs().max()))

    from gpuocean_gb300.adjoint import EnsembleStepAdjoint, StepAdjoint
    c = dict(_bump_case(64, moving=True), wind=(1.0e-4, -6.0e-5))
    sim = _sim(ctx, c, 2.0)
    adj = StepAdjoint(sim)
    adj.set_wind(c["wind"])
    q = adj.state(*sim.download())
    q1, qs = adj.zeros(), adj.zeros()
    adj.step_with_stage(q, q1, qs)
    rng = np.random.default_rng(6)
    lam = adj.zeros()
    for a in lam:
        a[2:-2, 2:-2] = torch.as_tensor(rng.standard_normal((c["ny"], c["nx"])), dtype=torch.float32)
    out = []
    for q_next in (None, q1):
        ls, ln = adj.zeros(), adj.zeros()
        adj.reset_wind_grad()
        adj.step_vjp(q, qs, lam, ls, ln, q_next)
        out.append([a.clone() for a in ln] + [adj.wind_grad().clone()])
    for a, b in zip(*out):
        close(a, b)
    n = 3
    eadj = EnsembleStepAdjoint(sim, n)
    base = torch.stack([a for a in q]).unsqueeze(0).repeat(n, 1, 1, 1).contiguous()
    base[:, 1] += torch.as_tensor(np.stack([_smooth(rng, base.shape[2:], 0.5) for _ in range(n)]),
                                  device=base.device)
    e1, es = eadj.zeros(), eadj.zeros()
    eadj.step(base, e1, es)
    elam = eadj.zeros()
    elam.normal_()
    out = []
    for q_next in (None, e1):
        ls, ln = eadj.zeros(), eadj.zeros()
        eadj.reset_wind_grad()
        eadj.step_vjp(base, es, elam, ls, ln, q_next)
        out.append((ln[..., 2:-2, 2:-2].clone(), eadj.wind_grad().clone()))
    close(out[0][0], out[1][0])
    close(out[0][1], out[1][1])
    sim.cleanUp()


def test_rollout_adjoint_matches_fp64_vjp_chain(ctx):
    """100 steps of the moving bump with wind: the CUDA adjoint of the whole
    rollout (sqrt(N) checkpointing) against the chain of FP64 autograd stage
    VJPs evaluated at the same FP32 trajectory points (Q^n and Q* of every
    step)."""
    from gpuocean_gb300.adjoint import CDKLM16Rollout, StepAdjoint
    from oracle.cdklm16_torch import periodic_ghosts
    c = _bump_case(64, moving=True)
    n_steps, every = 100, 10
    sim = _sim(ctx, c, 0.0)
    sim.updateDt(courant_number=0.45)
    dt = float(sim.dt)
    adj = StepAdjoint(sim)
    dev = adj.device
    tau = np.array([1.0e-4, 2.0e-5], dtype=np.float32)
    rows, cols = _misfit_setup(c, 64, 3)
    Hm32 = np.asarray(sim.downloadBathymetry()[1], dtype=np.float32)[2:-2, 2:-2]
    Hm = torch.as_tensor(Hm32, device=dev)
    q0 = adj.state(*sim.download())
    rng = np.random.default_rng(12)
    n_obs = n_steps // every
    u_obs = torch.as_tensor(0.01 * rng.standard_normal((n_obs, 64)), dtype=torch.float32, device=dev)
    v_obs = torch.as_tensor(0.01 * rng.standard_normal((n_obs, 64)), dtype=torch.float32, device=dev)
    x = [a.clone().requires_grad_(True) for a in q0]
    w = torch.tensor(tau, device=dev, requires_grad=True)
    st = CDKLM16Rollout.apply(adj, n_steps, every, *x, w)
    h = st[:, 0] + Hm
    loss = ((st[:, 1, rows, cols] / h[:, rows, cols] - u_obs) ** 2).sum() + \
           ((st[:, 2, rows, cols] / h[:, rows, cols] - v_obs) ** 2).sum()
    loss.backward()
    ours = [a.grad.double().cpu().numpy()[2:-2, 2:-2] for a in x]
    ours_w = w.grad.double().cpu().numpy()

    # the FP32 trajectory with its first stages
    adj.set_wind(tau)
    traj, stars = [[a.clone() for a in q0]], []
    for _ in range(n_steps):
        qs = adj.zeros()
        adj.stage1(traj[-1], qs)
        nxt = [torch.empty_like(a) for a in q0]
        adj.step(traj[-1], nxt)
        stars.append(qs)
        traj.append(nxt)
    to64 = lambda v: [torch.tensor(a.cpu().numpy().astype(np.float64)) for a in v]
    traj = [to64(v) for v in traj]
    stars = [to64(v) for v in stars]
    tq = _torch_ref(c, dt, None)
    X = torch.tensor(float(tau[0]), dtype=torch.float64, requires_grad=True)
    Y = torch.tensor(float(tau[1]), dtype=torch.float64, requires_grad=True)
    Hm64 = torch.as_tensor(Hm32.astype(np.float64))
    uo, vo = u_obs.double().cpu(), v_obs.double().cpu()
    nx, ny = c["nx"], c["ny"]
    lam = [torch.zeros(ny, nx, dtype=torch.float64) for _ in range(3)]

    def interior_grad(q):
        g = [a.grad[2:-2, 2:-2].clone() for a in q]
        return g

    for n in range(n_steps - 1, -1, -1):
        if (n + 1) % every == 0:
            k = (n + 1) // every - 1
            s = [a.clone().requires_grad_(True) for a in traj[n + 1]]
            e, hu, hv = (a[2:-2, 2:-2] for a in s)
            hh = e[rows, cols] + Hm64[rows, cols]
            (((hu[rows, cols] / hh - uo[k]) ** 2).sum() + ((hv[rows, cols] / hh - vo[k]) ** 2).sum()).backward()
            lam = [a + b for a, b in zip(lam, interior_grad(s))]
        qn = [a.clone().requires_grad_(True) for a in traj[n]]
        qs = [a.clone().requires_grad_(True) for a in stars[n]]
        out = tq.stage(periodic_ghosts(qs, nx, ny, tq.bc), periodic_ghosts(qn, nx, ny, tq.bc), X, Y, dt, 1)
        sum((o * l).sum() for o, l in zip(out, lam)).backward()
        lam_s = interior_grad(qs)
        lam_direct = interior_grad(qn)
        qn2 = [a.clone().requires_grad_(True) for a in traj[n]]
        out = tq.stage(periodic_ghosts(qn2, nx, ny, tq.bc), None, X, Y, dt, 0)
        sum((o * l).sum() for o, l in zip(out, lam_s)).backward()
        lam = [a + b for a, b in zip(lam_direct, interior_grad(qn2))]
    ref = [a.numpy() for a in lam]
    ref_w = np.array([X.grad.item(), Y.grad.item()])
    errs = [float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(ours, ref)]
    werr = float(np.linalg.norm(ours_w - ref_w) / np.linalg.norm(ref_w))
    print(json.dumps({"case": "rollout 100 steps, CUDA adjoint vs FP64 VJP chain", "rel_l2_err": errs,
                      "wind_rel_err": werr}))
    assert max(errs) <= 1e-4 and werr <= 1e-4, (errs, werr)
    sim.cleanUp()


def test_checkpointed_rollout_equals_stored_rollout(ctx):
    """sqrt(N) checkpointing recomputes segments with the same kernels: the
    gradient is bit-identical to the one from the fully stored trajectory,
    and the fused step that keeps Q* matches the step and the first-stage
    kernels bit for bit."""
    from gpuocean_gb300.adjoint import CDKLM16Rollout, StepAdjoint
    c = _bump_case(64, moving=True)
    sim = _sim(ctx, c, 0.0)
    sim.updateDt(courant_number=0.45)
    q0 = None
    grads = []
    for frac in (0.5, 0.0):
        adj = StepAdjoint(sim, memory_fraction=frac)
        assert (adj.segment_length(37) == 37) == (frac > 0)
        q0 = adj.state(*sim.download())
        x = [a.clone().requires_grad_(True) for a in q0]
        w = torch.tensor([1.0e-4, -3.0e-5], device=adj.device, requires_grad=True)
        st = CDKLM16Rollout.apply(adj, 37, 5, *x, w)
        (st[:, 1] ** 2).sum().backward()
        grads.append([a.grad.clone() for a in x] + [w.grad.clone()])
    for a, b in zip(*grads):
        assert torch.equal(a, b)
    # the fused step with Q* against the plain step and the first stage
    q1, q1b, qs, qs_ref = adj.zeros(), adj.zeros(), adj.zeros(), adj.zeros()
    adj.step_with_stage(q0, q1, qs)
    adj.step(q0, q1b)
    adj.stage1(q0, qs_ref)
    torch.cuda.synchronize()
    for a, b in zip(q1, q1b):
        assert torch.equal(a[2:-2, 2:-2], b[2:-2, 2:-2])
    for a, b in zip(qs, qs_ref):
        assert torch.equal(a[2:-2, 2:-2], b[2:-2, 2:-2])
    sim.cleanUp()


@pytest.mark.parametrize("name", ["walls_f", "periodic_xy"])
def test_drift_vjp_matches_fp64_autograd(ctx, name):
    """One drift step's VJP (position and state adjoints) against FP64
    autograd of the torch restatement of the drift."""
    from gpuocean_gb300.adjoint import StepAdjoint
    from oracle.cdklm16_torch import drift as drift64, periodic_ghosts
    c = _case(name)
    sim = _sim(ctx, c, 5.0)
    adj = StepAdjoint(sim)
    q = adj.state(*sim.download())
    # ghost cells as the step leaves them: periodic images (walls: untouched)
    q1 = adj.zeros()
    adj.step(q, q1)
    rng = np.random.default_rng(8)
    Lx, Ly = c["nx"] * c["dx"], c["ny"] * c["dy"]
    n = 300
    pos = torch.as_tensor(np.stack([rng.uniform(0, Lx, n), rng.uniform(0, Ly, n)], axis=1), dtype=torch.float32,
                          device=adj.device)
    pbar_after = rng.standard_normal((n, 2))
    pbar = torch.as_tensor(pbar_after, dtype=torch.float32, device=adj.device).contiguous()
    lam = adj.zeros()
    adj.drift_vjp(q1, pos.clone(), pbar, lam)
    torch.cuda.synchronize()
    ours_p = pbar.double().cpu().numpy()
    ours_l = [a.double().cpu().numpy()[2:-2, 2:-2] for a in lam]
    Hm = torch.as_tensor(np.asarray(sim.downloadBathymetry()[1], dtype=np.float64))
    interior = [torch.tensor(a.cpu().numpy().astype(np.float64)[2:-2, 2:-2], requires_grad=True) for a in q1]
    full = [torch.as_tensor(a.cpu().numpy().astype(np.float64)) for a in q1]
    full = [torch.cat([a[:2], torch.cat([a[2:-2, :2], b, a[2:-2, -2:]], dim=1), a[-2:]], dim=0)
            for a, b in zip(full, interior)]
    bc = BC(*c["bc"])
    if bc.periodic_ew() or bc.periodic_ns():
        full = periodic_ghosts(full, c["nx"], c["ny"], bc)
    p0 = torch.tensor(pos.cpu().numpy().astype(np.float64), requires_grad=True)
    p1 = drift64(p0, *full, Hm, c["nx"], c["ny"], c["dx"], c["dy"], adj.dt, bc.periodic_ns(), bc.periodic_ew())
    (p1 * torch.as_tensor(pbar_after)).sum().backward()
    ref_p = p0.grad.numpy()
    ref_l = [a.grad.numpy() for a in interior]
    ep = float(np.max(np.abs(ours_p - ref_p)) / np.max(np.abs(ref_p)))
    el = [float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30)) for a, b in zip(ours_l, ref_l)]
    print(json.dumps({"case": f"drift VJP {name}", "rel_err_positions": ep, "rel_err_state": el}))
    assert ep <= 1e-5 and max(el) <= 1e-5, (ep, el)
    sim.cleanUp()


def test_drifter_rollout_matches_fp64_chain_and_fd(ctx):
    """100 steps of the moving bump with 64 drifters; loss = squared distance
    of the drifters to target positions every 10 steps plus a (u, v) misfit.
    The CUDA gradient against (a) the chain of FP64 autograd VJPs (stages and
    drift) on the same FP32 trajectory and (b) central finite differences of
    the FP64 oracle along a random initial-state direction."""
    from gpuocean_gb300.adjoint import CDKLM16DrifterRollout, StepAdjoint
    from oracle.cdklm16_torch import drift as drift64, periodic_ghosts
    from oracle.noise_oracle import drift as drift_np
    c = _bump_case(64, moving=True)
    n_steps, every = 100, 10
    sim = _sim(ctx, c, 0.0)
    sim.updateDt(courant_number=0.45)
    dt = float(sim.dt)
    adj = StepAdjoint(sim)
    dev = adj.device
    tau = np.array([1.0e-4, 0.0], dtype=np.float32)
    rng = np.random.default_rng(31)
    L = c["nx"] * c["dx"]
    nd = 64
    p0 = np.stack([rng.uniform(0.2 * L, 0.8 * L, nd), rng.uniform(0.2 * L, 0.8 * L, nd)], axis=1).astype(np.float32)
    target = torch.as_tensor(p0 + rng.normal(0.0, 50.0, p0.shape).astype(np.float32), device=dev)
    q0 = adj.state(*sim.download())
    x = [a.clone().requires_grad_(True) for a in q0]
    w = torch.tensor(tau, device=dev, requires_grad=True)
    pt = torch.as_tensor(p0, device=dev).requires_grad_(True)
    st, ps = CDKLM16DrifterRollout.apply(adj, n_steps, every, *x, w, pt)
    loss = ((ps - target) ** 2).sum() * 1.0e-4 + (st[:, 1, 10:20, 10:20] ** 2).sum()
    loss.backward()
    ours = [a.grad.double().cpu().numpy()[2:-2, 2:-2] for a in x]
    ours_p = pt.grad.double().cpu().numpy()
    ours_w = w.grad.double().cpu().numpy()

    # (a) FP64 VJP chain on the FP32 trajectory
    adj.set_wind(tau)
    traj, stars, track = [[a.clone() for a in q0]], [], [torch.as_tensor(p0, device=dev)]
    pos = track[0].clone()
    for _ in range(n_steps):
        qs, nxt = adj.zeros(), [torch.empty_like(a) for a in q0]
        adj.step_with_stage(traj[-1], nxt, qs)
        adj.drift(nxt, pos)
        traj.append(nxt)
        stars.append(qs)
        track.append(pos.clone())
    to64 = lambda v: [torch.tensor(a.cpu().numpy().astype(np.float64)) for a in v]
    traj, stars = [to64(v) for v in traj], [to64(v) for v in stars]
    track = [torch.tensor(a.cpu().numpy().astype(np.float64)) for a in track]
    tq = _torch_ref(c, dt, None)
    X = torch.tensor(float(tau[0]), dtype=torch.float64, requires_grad=True)
    Y = torch.tensor(float(tau[1]), dtype=torch.float64, requires_grad=True)
    Hm64 = torch.as_tensor(np.asarray(sim.downloadBathymetry()[1], dtype=np.float64))
    tg = target.double().cpu()
    nx, ny = c["nx"], c["ny"]
    bc = tq.bc
    lam = [torch.zeros(ny, nx, dtype=torch.float64) for _ in range(3)]
    pbar = torch.zeros(nd, 2, dtype=torch.float64)

    def with_interior(v):
        inner = [a[2:-2, 2:-2].clone().requires_grad_(True) for a in v]
        full = [torch.cat([a[:2], torch.cat([a[2:-2, :2], b, a[2:-2, -2:]], dim=1), a[-2:]], dim=0)
                for a, b in zip(v, inner)]
        return inner, full

    for n in range(n_steps - 1, -1, -1):
        if (n + 1) % every == 0:
            k = (n + 1) // every - 1
            pbar = pbar + 2.0e-4 * (track[n + 1] - tg)
            s = traj[n + 1]
            lam[1] = lam[1] + torch.zeros(ny, nx, dtype=torch.float64).index_put_(
                (torch.arange(10, 20)[:, None], torch.arange(10, 20)[None, :]), 2.0 * s[1][12:22, 12:22])
        # drift after step n (reads the state after it)
        inner, full = with_interior(traj[n + 1])
        pp = track[n].clone().requires_grad_(True)
        p1 = drift64(pp, *full, Hm64, nx, ny, c["dx"], c["dy"], dt, bc.periodic_ns(), bc.periodic_ew())
        (p1 * pbar).sum().backward()
        pbar = pp.grad.clone()
        lam = [a + b.grad for a, b in zip(lam, inner)]
        # the step
        qn = [a.clone().requires_grad_(True) for a in traj[n]]
        qs = [a.clone().requires_grad_(True) for a in stars[n]]
        out = tq.stage(periodic_ghosts(qs, nx, ny, bc), periodic_ghosts(qn, nx, ny, bc), X, Y, dt, 1)
        sum((o * l).sum() for o, l in zip(out, lam)).backward()
        lam_s = [a.grad[2:-2, 2:-2].clone() for a in qs]
        lam_d = [a.grad[2:-2, 2:-2].clone() for a in qn]
        qn2 = [a.clone().requires_grad_(True) for a in traj[n]]
        out = tq.stage(periodic_ghosts(qn2, nx, ny, bc), None, X, Y, dt, 0)
        sum((o * l).sum() for o, l in zip(out, lam_s)).backward()
        lam = [a + b.grad[2:-2, 2:-2] for a, b in zip(lam_d, qn2)]
    ref = [a.numpy() for a in lam]
    errs = [float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(ours, ref)]
    perr = float(np.linalg.norm(ours_p - pbar.numpy()) / np.linalg.norm(pbar.numpy()))
    ref_w = np.array([X.grad.item(), Y.grad.item()])
    werr = float(np.linalg.norm(ours_w - ref_w) / np.linalg.norm(ref_w))

    # (b) FD of the FP64 oracle with drifters along a random state direction
    o0 = OracleCDKLM16(c["eta"], c["hu"], c["hv"], c["H"], nx, ny, c["dx"], c["dy"], dt, c["g"], c["f"], c["r"],
                       boundary_conditions=BC(*c["bc"]))
    Hm_np = np.asarray(o0.Hm, dtype=np.float64)
    base = [np.asarray(a.cpu().numpy(), dtype=np.float64) for a in q0]
    tgt = target.double().cpu().numpy()

    def loss64(q):
        o = OracleCDKLM16(c["eta"], c["hu"], c["hv"], c["H"], nx, ny, c["dx"], c["dy"], dt, c["g"], c["f"], c["r"],
                          boundary_conditions=BC(*c["bc"]))
        o.Q0 = [a.copy() for a in q]
        o.Q1 = [a.copy() for a in q]
        sh = (ny + 4, nx + 4)
        o.wind = (np.full(sh, float(tau[0])), np.full(sh, float(tau[1])))
        p = p0.astype(np.float64)
        total = 0.0
        for k in range(n_steps):
            o.step(dt)
            p = drift_np(p, *o.Q0, Hm_np, nx, ny, c["dx"], c["dy"], dt, False, False)
            if (k + 1) % every == 0:
                total += 1.0e-4 * np.sum((p - tgt) ** 2) + np.sum(o.Q0[1][12:22, 12:22] ** 2)
        return total
    delta = [_smooth(rng, base[0].shape, s).astype(np.float64) for s in (0.01, 0.1, 0.1)]
    for a in delta:
        a[:2, :] = 0; a[-2:, :] = 0; a[:, :2] = 0; a[:, -2:] = 0
    eps = 1.0e-3
    fd = (loss64([b + eps * d for b, d in zip(base, delta)]) - loss64([b - eps * d for b, d in zip(base, delta)])) / (2 * eps)
    ad = sum(float(np.sum(g * d[2:-2, 2:-2])) for g, d in zip(ours, delta))
    gnorm = np.sqrt(sum(float(np.sum(g * g)) for g in ours))
    dnorm = np.sqrt(sum(float(np.sum(d * d)) for d in delta))
    fd_err = abs(ad - fd) / (gnorm * dnorm)
    print(json.dumps({"case": "drifter rollout 100 steps", "chain_rel_l2": errs, "positions_rel": perr,
                      "wind_rel": werr, "fd": [ad, fd, fd_err]}))
    assert max(errs) <= 1e-4 and perr <= 1e-4 and werr <= 1e-4, (errs, perr, werr)
    assert fd_err <= 1e-4, (ad, fd, fd_err)
    sim.cleanUp()


def test_member_batched_rollout_equals_single_rollouts(ctx):
    """Config-5 style batching: members sharing the configuration run in one
    launch per step (forward) and two per step VJP; each member's gradient is
    bit-identical to its own single rollout, the wind gradients agree to
    1e-6 (a different summation order of the per-tile partials)."""
    from gpuocean_gb300.adjoint import (CDKLM16EnsembleRollout, CDKLM16Rollout, EnsembleStepAdjoint,
                                        StepAdjoint)
    c = _case("walls_f")
    sim = _sim(ctx, c, 2.0)
    n_members, n_steps, every = 4, 30, 5
    rng = np.random.default_rng(17)
    base = np.stack([np.asarray(a, dtype=np.float32) for a in sim.download()])
    q0 = np.stack([base + np.stack([_smooth(rng, base[0].shape, s) for s in (0.05, 1.0, 1.0)])
                   for _ in range(n_members)]).astype(np.float32)
    winds = rng.normal(0.0, 1.0e-4, (n_members, 2)).astype(np.float32)
    for frac in (0.5, 0.0):
        eadj = EnsembleStepAdjoint(sim, n_members, memory_fraction=frac)
        q = torch.as_tensor(q0, device=eadj.device).requires_grad_(True)
        w = torch.as_tensor(winds, device=eadj.device).requires_grad_(True)
        st = CDKLM16EnsembleRollout.apply(eadj, n_steps, every, q, w)
        (st[:, :, 1] ** 2 + 0.1 * st[:, :, 0]).sum().backward()
        gq, gw = q.grad.cpu().numpy(), w.grad.cpu().numpy()
        adj = StepAdjoint(sim, memory_fraction=frac)
        for m in range(n_members):
            x = [torch.as_tensor(q0[m, k], device=adj.device).requires_grad_(True) for k in range(3)]
            wm = torch.as_tensor(winds[m], device=adj.device).requires_grad_(True)
            sm = CDKLM16Rollout.apply(adj, n_steps, every, *x, wm)
            assert torch.equal(sm, st[:, m])
            (sm[:, 1] ** 2 + 0.1 * sm[:, 0]).sum().backward()
            for k in range(3):
                assert np.array_equal(x[k].grad.cpu().numpy()[2:-2, 2:-2], gq[m, k, 2:-2, 2:-2])
            np.testing.assert_allclose(wm.grad.cpu().numpy(), gw[m], rtol=1e-6)
    sim.cleanUp()
