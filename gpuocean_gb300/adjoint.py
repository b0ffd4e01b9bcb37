"""Adjoint of the CDKLM16 RK2 step behind ``torch.autograd.Function``.

The reverse sweep is hand-written CUDA (``goc_cdklm_stage_vjp``); torch only
holds the buffers and routes gradients.  ``CDKLM16Rollout`` runs ``n_steps``
RK2 steps of a simulator's configuration from a given state and uniform wind
stress, returns the interior state every ``obs_every`` steps, and in backward
returns the gradients of any loss of those states with respect to the
initial (eta, hu, hv) and the wind stress.  Long rollouts keep only every
K-th state (K = ceil(sqrt(n_steps))) and recompute each segment of K steps in
the backward sweep, so memory grows as sqrt(n_steps).

Data-assimilation use (variational, 4D-Var style)::

    adj = StepAdjoint(sim)                        # a CDKLM16 with rk_order 2
    eta0 = torch.tensor(..., device="cuda", requires_grad=True)
    states = CDKLM16Rollout.apply(adj, 400, 10, eta0, hu0, hv0, wind)
    loss = misfit(states, observations)           # any torch expression
    loss.backward()                               # eta0.grad, ..., wind.grad

The reference has no adjoint; this covers its RK2 step (S/CDKLM16.py:519-530
with K/CDKLM16_kernel.cu:475-1090, S/ = src/gpuocean/SWEsimulators,
K/ = src/gpuocean/gpu_kernels) with uniform wind and no pressure field.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class StepAdjoint:
    """The RK2 step of ``sim`` (its parameters, bathymetry and Coriolis data)
    with a fixed dt and a uniform wind stress held in a device tensor."""

    def __init__(self, sim, dt=None, memory_fraction=0.5):
        if int(sim.rk_order) != 2:
            raise ValueError("the adjoint covers the RK2 step only")
        self.sim = sim
        self.memory_fraction = float(memory_fraction)
        self.nx, self.ny = int(sim.nx), int(sim.ny)
        self.dt = float(np.float32(sim.dt if dt is None else dt))
        self.device = torch.device("cuda", torch.cuda.current_device())
        self.pitch = 4 * (self.nx + 4)
        self.Hi = sim.bathymetry.Bi
        self.Hm = sim.bathymetry.Bm
        self.wsf = float(sim.wind_stress_factor)
        self.wind = torch.zeros(2, dtype=torch.float32, device=self.device)
        p = _lib.GocCdklmParams.from_buffer_copy(sim._params)
        p.wind_x_cur = p.wind_x_next = self.wind.data_ptr()
        p.wind_y_cur = p.wind_y_next = self.wind.data_ptr() + 4
        p.wind_x_nx = p.wind_x_ny = p.wind_y_nx = p.wind_y_ny = 1
        p.wind_t = 0.0
        self.params = p
        n = _lib.load().goc_cdklm_vjp_partials(self.nx, self.ny)
        self.partials = torch.zeros((2, n), dtype=torch.float32, device=self.device)
        sim.gpu_stream.synchronize()

    @property
    def shape(self):
        return (self.ny + 4, self.nx + 4)

    def zeros(self):
        return [torch.zeros(self.shape, dtype=torch.float32, device=self.device) for _ in range(3)]

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def set_wind(self, tau):
        """Uniform wind stress (x, y) before the simulator's wind_stress_factor."""
        self.wind.copy_(torch.as_tensor(tau, dtype=torch.float32, device=self.device))

    def state(self, eta, hu, hv):
        return [torch.as_tensor(np.asarray(a, dtype=np.float32), device=self.device).contiguous()
                for a in (eta, hu, hv)]

    def step(self, q_in, q_out):
        _lib.call("goc_cdklm_rk2_step", ctypes.byref(self.params), ctypes.c_float(self.dt),
                  *[_ptr(a) for a in q_in], *[_ptr(a) for a in q_out], self.pitch,
                  self.Hi.ptr, int(self.Hi.pitch), self.Hm.ptr, int(self.Hm.pitch), self._stream())

    def step_with_stage(self, q_in, q_out, q_star):
        """One RK2 step that also keeps the first-stage state Q*."""
        _lib.call("goc_cdklm_rk2_step_stage", ctypes.byref(self.params), ctypes.c_float(self.dt),
                  *[_ptr(a) for a in q_in], *[_ptr(a) for a in q_out], *[_ptr(a) for a in q_star], self.pitch,
                  self.Hi.ptr, int(self.Hi.pitch), self.Hm.ptr, int(self.Hm.pitch), self._stream())

    def segment_length(self, n_steps):
        """Steps per checkpoint segment: all of them when the trajectory and
        its first stages fit in ``memory_fraction`` of the free device
        memory (no recompute), else ceil(sqrt(n_steps))."""
        need = 2 * n_steps * 3 * 4 * (self.nx + 4) * (self.ny + 4)
        free, _ = torch.cuda.mem_get_info(self.device)
        if self.memory_fraction > 0 and need <= self.memory_fraction * free:
            return n_steps
        return max(1, int(math.ceil(math.sqrt(n_steps))))

    def stage1(self, q_in, q_star):
        _lib.call("goc_cdklm_stage", ctypes.byref(self.params), ctypes.c_float(self.dt), 0,
                  *[_ptr(a) for a in q_in], *[_ptr(a) for a in q_star], None, None, None, self.pitch,
                  self.Hi.ptr, int(self.Hi.pitch), self.Hm.ptr, int(self.Hm.pitch), self._stream())

    def drift(self, q, positions):
        """Advect (N, 2) positions in place by one forward-Euler step with the
        state q (the state after the step, as CDKLM16.drifterStep does)."""
        n = positions.shape[0]
        b = self.sim.boundary_conditions
        z = ctypes.c_void_p(self.wind.data_ptr())
        _lib.call("goc_drift", self.nx, self.ny, ctypes.c_float(self.sim.dx), ctypes.c_float(self.sim.dy),
                  ctypes.c_float(self.dt), 2, 2, *[_ptr(a) for a in q], self.pitch, self.Hm.ptr, int(self.Hm.pitch),
                  int(b.isPeriodicNorthSouth()), int(b.isPeriodicEastWest()), n - 1, _ptr(positions), 8,
                  ctypes.c_float(1.0), z, z, z, z, 1, 1, ctypes.c_float(0.0), ctypes.c_float(0.0), self._stream())

    def drift_vjp(self, q, positions, pos_bar, lam):
        """pos_bar (N, 2): adjoint of the positions after the drift on entry,
        of those before on return; the state adjoint is added to lam."""
        b = self.sim.boundary_conditions
        _lib.call("goc_drift_vjp", self.nx, self.ny, ctypes.c_float(self.sim.dx), ctypes.c_float(self.sim.dy),
                  ctypes.c_float(self.dt), 2, 2, *[_ptr(a) for a in q], self.pitch, self.Hm.ptr, int(self.Hm.pitch),
                  int(b.isPeriodicNorthSouth()), int(b.isPeriodicEastWest()), positions.shape[0], _ptr(positions), 8,
                  _ptr(pos_bar), 8, ctypes.c_float(1.0), *[_ptr(a) for a in lam], self._stream())

    def step_vjp(self, q_n, q_star, lam_next, lam_star, lam_n, q_next=None):
        """lam_n = (dQ^{n+1}/dQ^n)^T lam_next on interior cells; the wind-stress
        gradient accumulates on the device (``wind_grad``).  With q_next
        (Q^{n+1} as the forward step wrote it) the stage VJPs take the stage
        outputs instead of recomputing the stages' fluxes."""
        s = self._stream()
        common = (self.pitch, self.Hi.ptr, int(self.Hi.pitch), self.Hm.ptr, int(self.Hm.pitch))
        p = [_ptr(a) for a in q_n]
        ps = [_ptr(a) for a in q_star]
        if q_next is None:
            _lib.call("goc_cdklm_stage_vjp", ctypes.byref(self.params), ctypes.c_float(self.dt), 1,
                      *ps, *p, *[_ptr(a) for a in lam_next],
                      None, None, None, *[_ptr(a) for a in lam_star], *[_ptr(a) for a in lam_n],
                      *common, _ptr(self.partials[0]), s)
            _lib.call("goc_cdklm_stage_vjp", ctypes.byref(self.params), ctypes.c_float(self.dt), 0,
                      *p, None, None, None, *[_ptr(a) for a in lam_star],
                      *[_ptr(a) for a in lam_n], *[_ptr(a) for a in lam_n], None, None, None,
                      *common, _ptr(self.partials[1]), s)
            return None
        _lib.call("goc_cdklm_stage_vjp_out", ctypes.byref(self.params), ctypes.c_float(self.dt), 1,
                  *ps, *p, *[_ptr(a) for a in q_next], *[_ptr(a) for a in lam_next],
                  None, None, None, *[_ptr(a) for a in lam_star], *[_ptr(a) for a in lam_n],
                  *common, _ptr(self.partials[0]), s)
        _lib.call("goc_cdklm_stage_vjp_out", ctypes.byref(self.params), ctypes.c_float(self.dt), 0,
                  *p, None, None, None, *ps, *[_ptr(a) for a in lam_star],
                  *[_ptr(a) for a in lam_n], *[_ptr(a) for a in lam_n], None, None, None,
                  *common, _ptr(self.partials[1]), s)
        return None

    # -- address-level calls of the rollout loops: states live in stacked
    # (N, 3, ny+4, nx+4) buffers and are passed as three device addresses
    # (see _triple), which keeps the host's work per step to a few ctypes
    # calls --
    def _bound(self):
        b = getattr(self, "_bound_args", None)
        if b is None:
            lib = _lib.load()
            b = self._bound_args = {
                "step": lib.goc_cdklm_rk2_step, "stage": lib.goc_cdklm_rk2_step_stage,
                "vjp": lib.goc_cdklm_stage_vjp_out,
                "pre": (ctypes.byref(self.params), ctypes.c_float(self.dt)),
                "common": (self.pitch, self.Hi.ptr, int(self.Hi.pitch), self.Hm.ptr, int(self.Hm.pitch)),
                "part": (self.partials[0].data_ptr(), self.partials[1].data_ptr()),
                "plane": 4 * (self.nx + 4) * (self.ny + 4)}
        return b

    def _step_p(self, src, dst, stream):
        b = self._bound()
        _lib.check(b["step"](*b["pre"], *src, *dst, *b["common"], stream), "goc_cdklm_rk2_step")

    def _stage_p(self, src, dst, star, stream):
        b = self._bound()
        _lib.check(b["stage"](*b["pre"], *src, *dst, *star, *b["common"], stream), "goc_cdklm_rk2_step_stage")

    def _vjp_p(self, qn, qs, qnext, lam_next, lam_star, lam_n, stream):
        """step_vjp on addresses (q_next given)."""
        b = self._bound()
        f, pre, com = b["vjp"], b["pre"], b["common"]
        p0, p1 = b["part"]
        _lib.check(f(*pre, 1, *qs, *qn, *qnext, *lam_next, None, None, None, *lam_star, *lam_n, *com, p0, stream),
                   "goc_cdklm_stage_vjp_out")
        _lib.check(f(*pre, 0, *qn, None, None, None, *qs, *lam_star, *lam_n, *lam_n, None, None, None, *com, p1,
                     stream), "goc_cdklm_stage_vjp_out")

    def reset_wind_grad(self):
        self.partials.zero_()

    def wind_grad(self):
        """Wind-stress gradient accumulated by step_vjp since the last reset."""
        return self.wsf * self.partials.view(2, -1, 2).sum(dim=(0, 1))


def _triple(base, index, plane):
    """Device addresses of (eta, hu, hv) of state `index` of a stacked
    (N, 3, ny+4, nx+4) float32 buffer at address `base` (plane: bytes of one
    field)."""
    o = base + 3 * index * plane
    return (o, o + plane, o + 2 * plane)


def _rollout_forward(ctx, adj, n_steps, obs_every, init, wind, positions0):
    n_steps, obs_every = int(n_steps), int(obs_every)
    if n_steps < 1 or obs_every < 1:
        raise ValueError("n_steps and obs_every must be >= 1")
    if n_steps < obs_every:
        raise ValueError("n_steps must be at least obs_every")
    adj.set_wind(wind.detach())
    K = adj.segment_length(n_steps)
    dev, (H, W) = adj.device, adj.shape
    plane = adj._bound()["plane"]
    sh = torch.cuda.current_stream(dev).cuda_stream
    q0 = torch.stack([a.detach().to(torch.float32) for a in init])
    n_obs = n_steps // obs_every
    pos, track = None, None
    if positions0 is not None:
        pos = positions0.detach().to(torch.float32).contiguous().clone()
        track = torch.empty((n_steps + 1,) + tuple(pos.shape), dtype=torch.float32, device=dev)
        track[0].copy_(pos)
    if K >= n_steps:
        # the whole trajectory and its first stages
        states = torch.empty((n_steps + 1, 3, H, W), dtype=torch.float32, device=dev)
        stars = torch.empty((n_steps, 3, H, W), dtype=torch.float32, device=dev)
        states[0].copy_(q0)
        bs, bt = states.data_ptr(), stars.data_ptr()
        for n in range(n_steps):
            adj._stage_p(_triple(bs, n, plane), _triple(bs, n + 1, plane), _triple(bt, n, plane), sh)
            if pos is not None:
                adj.drift(states[n + 1], pos)
                track[n + 1].copy_(pos)
        outs = states[obs_every::obs_every, :, 2:-2, 2:-2][:n_obs].clone()
        ctx.stored, ctx.ckpt = (states, stars), None
    else:
        # every K-th state; the backward sweep recomputes the segments
        n_seg = (n_steps + K - 1) // K
        ckpt = torch.empty((n_seg, 3, H, W), dtype=torch.float32, device=dev)
        buf = torch.empty((2, 3, H, W), dtype=torch.float32, device=dev)
        ckpt[0].copy_(q0)
        buf[0].copy_(q0)
        outs = torch.empty((n_obs, 3, H - 4, W - 4), dtype=torch.float32, device=dev)
        bb, cur = buf.data_ptr(), 0
        for n in range(n_steps):
            adj._step_p(_triple(bb, cur, plane), _triple(bb, 1 - cur, plane), sh)
            cur = 1 - cur
            if pos is not None:
                adj.drift(buf[cur], pos)
                track[n + 1].copy_(pos)
            if (n + 1) % K == 0 and n + 1 < n_steps:
                ckpt[(n + 1) // K].copy_(buf[cur])
            if (n + 1) % obs_every == 0:
                outs[(n + 1) // obs_every - 1].copy_(buf[cur, :, 2:-2, 2:-2])
        ctx.stored, ctx.ckpt = None, ckpt
    ctx.adj, ctx.K, ctx.n_steps, ctx.obs_every, ctx.track = adj, K, n_steps, obs_every, track
    pouts = track[obs_every::obs_every][:n_obs].clone() if track is not None else None
    return outs, pouts


def _rollout_backward(ctx, grad, grad_pos):
    """The reverse sweep.  With checkpoints, segment s - 1 is recomputed on a
    second stream while the sweep runs over segment s (two segment buffers
    in turn): at grid sizes that leave SMs idle the two overlap."""
    adj, K, n_steps, every = ctx.adj, ctx.K, ctx.n_steps, ctx.obs_every
    dev, (H, W) = adj.device, adj.shape
    plane = adj._bound()["plane"]
    main = torch.cuda.current_stream(dev)
    mh = main.cuda_stream
    grad = grad.contiguous() if grad is not None else None
    lam, lam_n, lam_s = (torch.zeros((3, H, W), dtype=torch.float32, device=dev) for _ in range(3))
    adj.reset_wind_grad()
    track = ctx.track
    pos_bar = torch.zeros_like(track[0]) if track is not None else None

    def sweep(start, end, states, stars):
        nonlocal lam, lam_n, pos_bar
        bs, bt = states.data_ptr(), stars.data_ptr()
        ls = _triple(lam_s.data_ptr(), 0, plane)
        for n in range(end - 1, start - 1, -1):
            i = n - start
            if (n + 1) % every == 0:
                k = (n + 1) // every - 1
                if grad is not None:
                    lam[:, 2:-2, 2:-2] += grad[k]
                if pos_bar is not None and grad_pos is not None:
                    pos_bar += grad_pos[k]
            if pos_bar is not None:
                # the drift after step n read the state after it
                adj.drift_vjp(states[i + 1], track[n], pos_bar, lam)
            adj._vjp_p(_triple(bs, i, plane), _triple(bt, i, plane), _triple(bs, i + 1, plane),
                       _triple(lam.data_ptr(), 0, plane), ls, _triple(lam_n.data_ptr(), 0, plane), mh)
            lam, lam_n = lam_n, lam

    if ctx.ckpt is None:
        states, stars = ctx.stored
        sweep(0, n_steps, states, stars)
    else:
        ckpt = ctx.ckpt
        order = sorted(range(0, n_steps, K), reverse=True)
        bufs = [(torch.empty((K + 1, 3, H, W), dtype=torch.float32, device=dev),
                 torch.empty((K, 3, H, W), dtype=torch.float32, device=dev)) for _ in range(min(2, len(order)))]
        side = torch.cuda.Stream(dev)
        sh = side.cuda_stream
        ready = [torch.cuda.Event() for _ in bufs]
        free = [torch.cuda.Event() for _ in bufs]
        side.wait_stream(main)

        def recompute(start, b):
            st, sr = bufs[b]
            side.wait_event(free[b])
            with torch.cuda.stream(side):
                st[0].copy_(ckpt[start // K])
            bs, bt = st.data_ptr(), sr.data_ptr()
            for i in range(min(start + K, n_steps) - start):
                adj._stage_p(_triple(bs, i, plane), _triple(bs, i + 1, plane), _triple(bt, i, plane), sh)
            ready[b].record(side)

        recompute(order[0], 0)
        for idx, start in enumerate(order):
            b = idx % 2
            if idx + 1 < len(order):
                recompute(order[idx + 1], 1 - b)
            main.wait_event(ready[b])
            sweep(start, min(start + K, n_steps), *bufs[b])
            free[b].record(main)
        main.wait_stream(side)
    ctx.stored = ctx.ckpt = ctx.track = None
    return lam, adj.wind_grad(), pos_bar


class CDKLM16Rollout(torch.autograd.Function):
    """``apply(adj, n_steps, obs_every, eta0, hu0, hv0, wind)`` ->
    interior states (n_steps // obs_every, 3, ny, nx) after steps
    obs_every, 2 obs_every, ...  eta0/hu0/hv0: (ny+4, nx+4) float32 CUDA
    tensors (ghost cells are ignored); wind: (2,) stress.

    The forward keeps every K-th state (K from ``adj.segment_length``); the
    backward sweep recomputes each segment once, keeping its states and
    first stages, and runs the step VJPs over it in reverse.  With K =
    n_steps (the whole trajectory fits) nothing is recomputed."""

    @staticmethod
    def forward(ctx, adj, n_steps, obs_every, eta0, hu0, hv0, wind):
        states, _ = _rollout_forward(ctx, adj, n_steps, obs_every, (eta0, hu0, hv0), wind, None)
        return states

    @staticmethod
    def backward(ctx, grad):
        lam, wind_bar, _ = _rollout_backward(ctx, grad, None)
        return None, None, None, lam[0], lam[1], lam[2], wind_bar


class CDKLM16DrifterRollout(torch.autograd.Function):
    """``apply(adj, n_steps, obs_every, eta0, hu0, hv0, wind, positions0)``
    -> (states, positions): the rollout of ``CDKLM16Rollout`` with passive
    drifters (N, 2) advected after every step by the state after it
    (``CDKLM16.drifterStep``, S/CDKLM16.py:575 and
    D/GPUDrifterCollection.py:198-233, D/ = src/gpuocean/drifters); positions
    (n_obs, N, 2) at the observation steps.  Gradients of a loss of either
    output flow to the initial state, the wind stress and the initial
    positions.  No wind drift."""

    @staticmethod
    def forward(ctx, adj, n_steps, obs_every, eta0, hu0, hv0, wind, positions0):
        return _rollout_forward(ctx, adj, n_steps, obs_every, (eta0, hu0, hv0), wind, positions0)

    @staticmethod
    def backward(ctx, grad, grad_pos):
        lam, wind_bar, pos_bar = _rollout_backward(ctx, grad, grad_pos)
        return None, None, None, lam[0], lam[1], lam[2], wind_bar, pos_bar


class EnsembleStepAdjoint:
    """The RK2 step and its adjoint for ``n_members`` members that share the
    configuration of ``sim`` (parameters, bathymetry, Coriolis data) but not
    their state or their uniform wind stress.  States are stacked tensors
    (n_members, 3, ny+4, nx+4); one launch covers all members."""

    def __init__(self, sim, n_members, dt=None, memory_fraction=0.5):
        self.one = StepAdjoint(sim, dt=dt, memory_fraction=memory_fraction)
        self.n = int(n_members)
        self.nx, self.ny, self.dt, self.device = self.one.nx, self.one.ny, self.one.dt, self.one.device
        self.plane = (self.ny + 4) * (self.nx + 4)
        self.wind = torch.zeros((self.n, 2), dtype=torch.float32, device=self.device)
        p = _lib.GocCdklmParams.from_buffer_copy(self.one.params)
        p.wind_x_cur = p.wind_x_next = self.wind.data_ptr()
        p.wind_y_cur = p.wind_y_next = self.wind.data_ptr() + 4
        self.params = p
        per = _lib.load().goc_cdklm_vjp_partials(self.nx, self.ny)
        self.partials = torch.zeros((2, self.n, per), dtype=torch.float32, device=self.device)
        self.memory_fraction = float(memory_fraction)

    def zeros(self):
        return torch.zeros((self.n, 3, self.ny + 4, self.nx + 4), dtype=torch.float32, device=self.device)

    def set_wind(self, tau):
        """(n_members, 2) or (2,) uniform stress before wind_stress_factor."""
        tau = torch.as_tensor(tau, dtype=torch.float32, device=self.device)
        self.wind.copy_(tau.expand(self.n, 2))

    def _p3(self, q):
        if q is None:
            return (None, None, None)
        assert q.is_contiguous() and q.shape == (self.n, 3, self.ny + 4, self.nx + 4)
        b = q.data_ptr()
        return tuple(ctypes.c_void_p(b + 4 * c * self.plane) for c in range(3))

    def segment_length(self, n_steps):
        need = 2 * n_steps * self.n * 3 * 4 * self.plane
        free, _ = torch.cuda.mem_get_info(self.device)
        if self.memory_fraction > 0 and need <= self.memory_fraction * free:
            return n_steps
        return max(1, int(math.ceil(math.sqrt(n_steps))))

    def step(self, q_in, q_out, q_star=None):
        o = self.one
        _lib.call("goc_cdklm_rk2_step_members", ctypes.byref(self.params), ctypes.c_float(self.dt),
                  *self._p3(q_in), *self._p3(q_out), *self._p3(q_star), o.pitch, 3 * self.plane, self.n, 2,
                  o.Hi.ptr, int(o.Hi.pitch), o.Hm.ptr, int(o.Hm.pitch), o._stream())

    def step_vjp(self, q_n, q_star, lam_next, lam_star, lam_n, q_next=None):
        """lam_n = VJP of every member's step; the (n_members, 2) wind-stress
        gradient accumulates on the device (``wind_grad``).  q_next: as in
        ``StepAdjoint.step_vjp``."""
        o = self.one
        s = o._stream()
        common = (o.pitch, 3 * self.plane, self.n, 2, o.Hi.ptr, int(o.Hi.pitch), o.Hm.ptr, int(o.Hm.pitch))
        w0, w1 = ctypes.c_void_p(self.partials[0].data_ptr()), ctypes.c_void_p(self.partials[1].data_ptr())
        if q_next is None:
            _lib.call("goc_cdklm_stage_vjp_members", ctypes.byref(self.params), ctypes.c_float(self.dt), 1,
                      *self._p3(q_star), *self._p3(q_n), *self._p3(lam_next), None, None, None,
                      *self._p3(lam_star), *self._p3(lam_n), *common, w0, s)
            _lib.call("goc_cdklm_stage_vjp_members", ctypes.byref(self.params), ctypes.c_float(self.dt), 0,
                      *self._p3(q_n), None, None, None, *self._p3(lam_star), *self._p3(lam_n), *self._p3(lam_n),
                      None, None, None, *common, w1, s)
            return None
        _lib.call("goc_cdklm_stage_vjp_members_out", ctypes.byref(self.params), ctypes.c_float(self.dt), 1,
                  *self._p3(q_star), *self._p3(q_n), *self._p3(q_next), *self._p3(lam_next), None, None, None,
                  *self._p3(lam_star), *self._p3(lam_n), *common, w0, s)
        _lib.call("goc_cdklm_stage_vjp_members_out", ctypes.byref(self.params), ctypes.c_float(self.dt), 0,
                  *self._p3(q_n), None, None, None, *self._p3(q_star), *self._p3(lam_star), *self._p3(lam_n),
                  *self._p3(lam_n), None, None, None, *common, w1, s)
        return None

    def reset_wind_grad(self):
        self.partials.zero_()

    def wind_grad(self):
        return self.one.wsf * self.partials.view(2, self.n, -1, 2).sum(dim=(0, 2))


class CDKLM16EnsembleRollout(torch.autograd.Function):
    """``apply(adj, n_steps, obs_every, q0, wind)`` with an
    ``EnsembleStepAdjoint``: q0 (n_members, 3, ny+4, nx+4), wind
    (n_members, 2) -> interior states (n_obs, n_members, 3, ny, nx).  The
    batched form of ``CDKLM16Rollout`` (same storage and checkpointing)."""

    @staticmethod
    def forward(ctx, adj, n_steps, obs_every, q0, wind):
        n_steps, obs_every = int(n_steps), int(obs_every)
        if n_steps < obs_every or obs_every < 1:
            raise ValueError("need n_steps >= obs_every >= 1")
        adj.set_wind(wind.detach())
        K = adj.segment_length(n_steps)
        q = q0.detach().to(torch.float32).contiguous().clone()
        outs = []
        if K >= n_steps:
            states, stars = [q], []
            for n in range(n_steps):
                nxt, qs = torch.empty_like(q), torch.empty_like(q)
                adj.step(states[-1], nxt, qs)
                states.append(nxt)
                stars.append(qs)
                if (n + 1) % obs_every == 0:
                    outs.append(nxt[:, :, 2:-2, 2:-2].clone())
            ctx.segments = {0: (states, stars)}
        else:
            buf = torch.empty_like(q)
            ctx.segments = {0: (q.clone(), None)}
            for n in range(n_steps):
                adj.step(q, buf)
                q, buf = buf, q
                if (n + 1) % K == 0 and n + 1 < n_steps:
                    ctx.segments[n + 1] = (q.clone(), None)
                if (n + 1) % obs_every == 0:
                    outs.append(q[:, :, 2:-2, 2:-2].clone())
        ctx.adj, ctx.K, ctx.n_steps, ctx.obs_every = adj, K, n_steps, obs_every
        return torch.stack(outs)

    @staticmethod
    def backward(ctx, grad):
        adj, K, n_steps, every = ctx.adj, ctx.K, ctx.n_steps, ctx.obs_every
        grad = grad.contiguous()
        lam, lam_n, lam_s = adj.zeros(), adj.zeros(), adj.zeros()
        adj.reset_wind_grad()
        for start in sorted(ctx.segments, reverse=True):
            end = min(start + K, n_steps)
            states, stars = ctx.segments[start]
            if stars is None:
                states, stars = [states], []
                for _ in range(start, end):
                    nxt, qs = torch.empty_like(states[-1]), torch.empty_like(states[-1])
                    adj.step(states[-1], nxt, qs)
                    states.append(nxt)
                    stars.append(qs)
            for n in range(end - 1, start - 1, -1):
                if (n + 1) % every == 0:
                    lam[:, :, 2:-2, 2:-2] += grad[(n + 1) // every - 1]
                adj.step_vjp(states[n - start], stars[n - start], lam, lam_s, lam_n, states[n + 1 - start])
                lam, lam_n = lam_n, lam
            del states, stars
            ctx.segments[start] = None
        ctx.segments = None
        return None, None, None, lam, adj.wind_grad()


def _main(argv=None):
    """``python -m gpuocean_gb300.adjoint [--members M] [--n N] [--calls C]``:
    C step VJPs of M members of the N x N Gaussian bump (H = 60 m, walls)
    with a dense random adjoint, after 20 forward steps; prints the mean
    time of one step VJP and of one forward step.  A small, self-contained
    workload for timing and profiling the adjoint kernels."""
    import argparse
    import json
    from .SWEsimulators import CDKLM16
    from .utils import Common
    ap = argparse.ArgumentParser()
    ap.add_argument("--members", type=int, default=32)
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--calls", type=int, default=4)
    a = ap.parse_args(argv)
    ctx = Common.CUDAContext()
    n = a.n
    x = (np.arange(n + 4) - 2 + 0.5 - n / 2.0)
    eta = (0.1 * np.exp(-(x[None, :] ** 2 + x[:, None] ** 2) / 200.0)).astype(np.float32)
    z = np.zeros_like(eta)
    sim = CDKLM16.CDKLM16(ctx, eta, z, z.copy(), np.full((n + 5, n + 5), 60.0, np.float32), n, n, 200.0, 200.0,
                          0.0, 9.81, 1.2e-4, 0.0)
    sim.updateDt(courant_number=0.45)
    adj = EnsembleStepAdjoint(sim, a.members)
    base = torch.as_tensor(np.stack([np.asarray(v, np.float32) for v in sim.download()]), device=adj.device)
    q0 = base.unsqueeze(0).repeat(a.members, 1, 1, 1).contiguous()
    q1, qs = adj.zeros(), adj.zeros()
    for _ in range(20):
        adj.step(q0, q1, qs)
        q0, q1 = q1, q0
    adj.step(q0, q1, qs)      # q1 = Q^{n+1}, qs = Q* of q0
    lam, ls, ln = adj.zeros(), adj.zeros(), adj.zeros()
    lam.normal_()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    torch.cuda.synchronize()
    ev[0].record()
    for _ in range(a.calls):
        adj.step_vjp(q0, qs, lam, ls, ln, q1)
    ev[1].record()
    for _ in range(a.calls):
        adj.step(q0, q1, qs)
    ev[2].record()
    torch.cuda.synchronize()
    vjp, step = ev[0].elapsed_time(ev[1]) / a.calls, ev[1].elapsed_time(ev[2]) / a.calls
    print(json.dumps({"members": a.members, "n": n, "step_vjp_ms": vjp, "step_ms": step, "ratio": vjp / step}))
    sim.cleanUp()


if __name__ == "__main__":
    _main()
