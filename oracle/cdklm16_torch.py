"""FP64 torch restatement of one CDKLM16 RK2 step, for autograd.

TEST INFRASTRUCTURE ONLY: the reference gradients that the hand-written CUDA
adjoint is checked against.  It restates, on torch tensors, exactly the
arithmetic of ``oracle.cdklm16_oracle.cdklm_stage`` (which follows
K/CDKLM16_kernel.cu:475-1090 of GPU Ocean) for the configurations the
adjoint supports: RK2, a constant north angle, uniform wind stress (X, Y,
differentiable), no atmospheric pressure, walls or periodic boundaries.
Branches (minmod, desingularisation, dry-cell clamps) are taken with
``torch.where`` so that autograd follows the branch of the evaluated state;
masked-out branches use safe operands so that they carry no NaN gradients.
"""
from __future__ import annotations

import numpy as np
import torch

from .cdklm16_oracle import BC, DRY_EPS, DRY_FLAG, LAND_VALUE, Params


def _minmod_raw(b, c, f):
    one = torch.ones_like(b)
    sb, sc, sf = torch.copysign(one, b), torch.copysign(one, c), torch.copysign(one, f)
    return 0.25 * sb * (sb + sc) * (sc + sf) * torch.minimum(torch.minimum(b.abs(), c.abs()), f.abs())


def _minmod_slope(left, center, right, theta):
    return _minmod_raw((center - left) * theta, (right - left) * 0.5, (right - center) * theta)


def _desing(h, hu, eps):
    return hu / torch.maximum(torch.minimum(h * h / (2.0 * eps) + 0.5 * eps, torch.full_like(h, eps)), h.abs())


def _flux(Qm, Qp, H, P):
    g, cutoff = P.g, P.depth_cutoff
    hp = Qp[0] + H
    hm = Qm[0] + H
    wp = hp > cutoff
    wm = hm > cutoff
    cp = torch.where(wp, torch.sqrt(torch.where(wp, g * hp, torch.ones_like(hp))), torch.zeros_like(hp))
    cm = torch.where(wm, torch.sqrt(torch.where(wm, g * hm, torch.ones_like(hm))), torch.zeros_like(hm))
    z = torch.zeros_like(hp)
    up = torch.where(wp, Qp[1], z)
    um = torch.where(wm, Qm[1], z)
    Fp = [torch.where(wp, hp * Qp[1], z),
          torch.where(wp, hp * Qp[1] * Qp[1] + 0.5 * g * hp * hp, z),
          torch.where(wp, hp * Qp[1] * Qp[2], z)]
    Fm = [torch.where(wm, hm * Qm[1], z),
          torch.where(wm, hm * Qm[1] * Qm[1] + 0.5 * g * hm * hm, z),
          torch.where(wm, hm * Qm[1] * Qm[2], z)]
    am = torch.minimum(torch.minimum(um - cm, up - cp), z)
    ap = torch.maximum(torch.maximum(um + cm, up + cp), z)
    zero = (ap - am).abs() < P.flux_slope_eps
    den = torch.where(zero, torch.ones_like(ap), ap - am)
    F0 = ((ap * Fm[0] - am * Fp[0]) + ap * am * (Qp[0] - Qm[0])) / den
    F1 = ((ap * Fm[1] - am * Fp[1]) + ap * am * (Fp[0] - Fm[0])) / den
    fb = P.flux_balancer
    F2 = torch.where(Qm[1] > -Qp[1], fb * Fm[2], fb * Fp[2])
    F2 = F2 + (1.0 - fb) * (((ap * Fm[2] - am * Fp[2]) + ap * am * (hp * Qp[2] - hm * Qm[2])) / den)
    return [torch.where(zero, z, F0), torch.where(zero, z, F1), torch.where(zero, z, F2)]


def _wall_mirror(R, nx, ny, bc: BC):
    R0, R1, R2 = (a.clone() for a in R)
    ci = slice(2, nx + 2)
    ri = slice(2, ny + 2)
    if bc.north == 1:
        R0[ny + 2, ci], R1[ny + 2, ci], R2[ny + 2, ci] = R0[ny + 1, ci], R1[ny + 1, ci], -R2[ny + 1, ci]
        R0[ny + 3, ci], R1[ny + 3, ci], R2[ny + 3, ci] = R0[ny, ci], R1[ny, ci], -R2[ny, ci]
    if bc.south == 1:
        R0[1, ci], R1[1, ci], R2[1, ci] = R0[2, ci], R1[2, ci], -R2[2, ci]
        R0[0, ci], R1[0, ci], R2[0, ci] = R0[3, ci], R1[3, ci], -R2[3, ci]
    if bc.east == 1:
        R0[ri, nx + 2], R1[ri, nx + 2], R2[ri, nx + 2] = R0[ri, nx + 1], -R1[ri, nx + 1], R2[ri, nx + 1]
        R0[ri, nx + 3], R1[ri, nx + 3], R2[ri, nx + 3] = R0[ri, nx], -R1[ri, nx], R2[ri, nx]
    if bc.west == 1:
        R0[ri, 1], R1[ri, 1], R2[ri, 1] = R0[ri, 2], -R1[ri, 2], R2[ri, 2]
        R0[ri, 0], R1[ri, 0], R2[ri, 0] = R0[ri, 3], -R1[ri, 3], R2[ri, 3]
    return R0, R1, R2


def periodic_ghosts(Q, nx, ny, bc: BC):
    """K/boundary_kernels.cu:36-110 (north-south first), out of place."""
    out = []
    for a in Q:
        a = a.clone()
        if bc.north == 2:
            a[0:2, :] = a[ny:ny + 2, :].clone()
            a[ny + 2:ny + 4, :] = a[2:4, :].clone()
        if bc.east == 2:
            a[:, 0:2] = a[:, nx:nx + 2].clone()
            a[:, nx + 2:nx + 4] = a[:, 2:4].clone()
        out.append(a)
    return out


class TorchCDKLM16:
    """Static inputs of one simulator (from the FP64 numpy oracle) and a
    differentiable RK2 step.  ``oracle`` is an ``OracleCDKLM16``."""

    def __init__(self, oracle, wind=(0.0, 0.0)):
        o = oracle
        assert o.P.rk_order == 2
        self.P: Params = o.P
        self.bc: BC = o.bc
        self.nx, self.ny = o.nx, o.ny
        t = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64))
        Hk = np.array(o.Hi, dtype=np.float64)
        Hk[np.abs(Hk - LAND_VALUE) < DRY_EPS] = DRY_FLAG
        self.Hk = t(Hk)
        self.Hm_k = 0.25 * (self.Hk[:-1, :-1] + self.Hk[1:, :-1] + self.Hk[:-1, 1:] + self.Hk[1:, 1:])
        self.Hmb = t(o.Hm)
        self.F = t(o.F)
        self.north = (t(o.north[0]), t(o.north[1]))
        self.wsf = float(o.P.wind_stress_factor)

    def stage(self, Qin, Qn, X, Y, dt, rk_step):
        P, bc, nx, ny = self.P, self.bc, self.nx, self.ny
        g, dx, dy, th = P.g, P.dx, P.dy, P.theta
        cutoff, eps_d = P.depth_cutoff, P.desing_eps
        R0, R1, R2 = _wall_mirror(Qin, nx, ny, bc)
        Hk, Hm_k, Hmb, F = self.Hk, self.Hm_k, self.Hmb, self.F
        h = R0 + Hmb
        land = (Hmb - LAND_VALUE).abs() <= DRY_EPS
        nearly = (~land) & (h < eps_d)
        cut = nearly & (h <= cutoff)
        soft = nearly & (~cut)
        zero = torch.zeros_like(h)
        h_safe = torch.where(nearly | land, torch.ones_like(h), h)
        h_soft = torch.where(soft, h, torch.full_like(h, eps_d))
        eta = torch.where(land, torch.full_like(h, DRY_FLAG), torch.where(cut, -Hmb + cutoff, R0))
        u = torch.where(land | cut, zero, torch.where(soft, _desing(h_soft, R1, eps_d), R1 / h_safe))
        v = torch.where(land | cut, zero, torch.where(soft, _desing(h_soft, R2, eps_d), R2 / h_safe))
        nxn, nyn = self.north
        ex, ey = nyn, -nxn

        # x slopes at centre columns c = 1..nx+2
        L, C, Rr = slice(0, nx + 2), slice(1, nx + 3), slice(2, nx + 4)
        cidx = torch.arange(1, nx + 3)[None, :]
        ux = _minmod_slope(u[:, L], u[:, C], u[:, Rr], th)
        vx = _minmod_slope(v[:, L], v[:, C], v[:, Rr], th)
        lv, cv, rv = v[:, L], v[:, C], v[:, Rr]
        if bc.west == 1:
            lv = torch.where(cidx < 3, -lv, lv)
            cv = torch.where(cidx < 2, -cv, cv)
        if bc.east == 1:
            rv = torch.where(cidx > nx, -rv, rv)
            cv = torch.where(cidx > nx + 1, -cv, cv)
        nxc, nyc = nxn[:, C], nyn[:, C]
        lfv = (nxc * u[:, L] + nyc * lv) * F[:, L]
        cfv = (nxc * u[:, C] + nyc * cv) * F[:, C]
        rfv = (nxc * u[:, Rr] + nyc * rv) * F[:, Rr]
        Vc = dx / (2.0 * g)
        back = th * g * (eta[:, C] - eta[:, L] - Vc * (cfv + lfv))
        cent = 0.5 * g * (eta[:, Rr] - eta[:, L] - Vc * (rfv + 2.0 * cfv + lfv))
        fwd = th * g * (eta[:, Rr] - eta[:, C] - Vc * (cfv + rfv))
        Kx = _minmod_raw(back, cent, fwd)
        va = v[:, C]
        if bc.west == 1:
            va = torch.where(cidx < 2, -va, va)
        if bc.east == 1:
            va = torch.where(cidx > nx + 2, -va, va)
        dxfv = dx * F[:, C] * va
        H_w = 0.5 * (Hk[:-1, C] + Hk[1:, C])
        H_e = 0.5 * (Hk[:-1, 2:nx + 4] + Hk[1:, 2:nx + 4])
        e_c = eta[:, C]
        h_w = e_c + H_w - (Kx + dxfv) / (2.0 * g)
        h_e = e_c + H_e + (Kx + dxfv) / (2.0 * g)
        Kx = torch.where(h_w > 0, Kx, -dxfv + 2.0 * g * (e_c + H_w))
        Kx = torch.where(h_e > 0, Kx, -dxfv - 2.0 * g * (e_c + H_e))

        # x faces between c and c+1
        cm = torch.arange(1, nx + 2)[None, :]
        mC, pC = slice(1, nx + 2), slice(2, nx + 3)
        mS, pS = slice(0, nx + 1), slice(1, nx + 2)
        eb_m, eb_p = eta[:, mC], eta[:, pC]
        um_, up_ = u[:, mC], u[:, pC]
        vm_, vp_ = v[:, mC], v[:, pC]
        Rp = (up_ - 0.5 * ux[:, pS], vp_ - 0.5 * vx[:, pS])
        Rm = (um_ + 0.5 * ux[:, mS], vm_ + 0.5 * vx[:, mS])
        Hf = 0.5 * (Hk[:-1, pC] + Hk[1:, pC])
        if bc.west == 1:
            vm_ = torch.where(cm + 1 == 2, -vm_, vm_)
        if bc.east == 1:
            vp_ = torch.where(cm + 1 == nx + 2, -vp_, vp_)
        vpn = up_ * nxn[:, pC] + vp_ * nyn[:, pC]
        vmn = um_ * nxn[:, mC] + vm_ * nyn[:, mC]
        etap = torch.maximum(-Hf, eb_p - (Kx[:, pS] + dx * F[:, pC] * vpn) / (2.0 * g))
        etam = torch.maximum(-Hf, eb_m + (Kx[:, mS] + dx * F[:, mC] * vmn) / (2.0 * g))
        Fx = _flux([etam, Rm[0], Rm[1]], [etap, Rp[0], Rp[1]], Hf, P)
        dm, dp = eb_m == DRY_FLAG, eb_p == DRY_FLAG
        pe = 0.5 * g * (etap + Hf) * (etap + Hf)
        me = 0.5 * g * (etam + Hf) * (etam + Hf)
        zf = torch.zeros_like(Fx[0])
        Fx[1] = torch.where(dm & ~dp, pe, torch.where(~dm & dp, me, Fx[1]))
        for k in (0, 2):
            Fx[k] = torch.where(dm ^ dp, zf, Fx[k])
        for k in range(3):
            Fx[k] = torch.where(dm & dp, zf, Fx[k])

        # y slopes at centre rows r = 1..ny+2
        Lo, Ce, Up = slice(0, ny + 2), slice(1, ny + 3), slice(2, ny + 4)
        ridx = torch.arange(1, ny + 3)[:, None]
        uy = _minmod_slope(u[Lo], u[Ce], u[Up], th)
        vy = _minmod_slope(v[Lo], v[Ce], v[Up], th)
        lu, cu_, uu = u[Lo], u[Ce], u[Up]
        if bc.south == 1:
            lu = torch.where(ridx < 3, -lu, lu)
            cu_ = torch.where(ridx < 2, -cu_, cu_)
        if bc.north == 1:
            uu = torch.where(ridx > ny, -uu, uu)
            cu_ = torch.where(ridx > ny + 1, -cu_, cu_)
        exc, eyc = ex[Ce], ey[Ce]
        lfu = (exc * lu + eyc * v[Lo]) * F[Lo]
        cfu = (exc * cu_ + eyc * v[Ce]) * F[Ce]
        ufu = (exc * uu + eyc * v[Up]) * F[Up]
        Uc = dy / (2.0 * g)
        back = th * g * (eta[Ce] - eta[Lo] + Uc * (cfu + lfu))
        cent = 0.5 * g * (eta[Up] - eta[Lo] + Uc * (ufu + 2.0 * cfu + lfu))
        fwd = th * g * (eta[Up] - eta[Ce] + Uc * (cfu + ufu))
        Ly = _minmod_raw(back, cent, fwd)
        ua = u[Ce]
        if bc.south == 1:
            ua = torch.where(ridx < 2, -ua, ua)
        if bc.north == 1:
            ua = torch.where(ridx > ny + 2, -ua, ua)
        dyfu = dy * F[Ce] * ua
        H_s = 0.5 * (Hk[Ce, :-1] + Hk[Ce, 1:])
        H_n = 0.5 * (Hk[2:ny + 4, :-1] + Hk[2:ny + 4, 1:])
        e_c = eta[Ce]
        h_s = e_c + H_s - (Ly - dyfu) / (2.0 * g)
        h_n = e_c + H_n + (Ly - dyfu) / (2.0 * g)
        Ly = torch.where(h_s > 0, Ly, dyfu + 2.0 * g * (e_c + H_s))
        Ly = torch.where(h_n > 0, Ly, dyfu - 2.0 * g * (e_c + H_n))

        # y faces between r and r+1
        rm = torch.arange(1, ny + 2)[:, None]
        mR, pR = slice(1, ny + 2), slice(2, ny + 3)
        mS, pS = slice(0, ny + 1), slice(1, ny + 2)
        eb_m, eb_p = eta[mR], eta[pR]
        um_, up_ = u[mR], u[pR]
        vm_, vp_ = v[mR], v[pR]
        Rp = (up_ - 0.5 * uy[pS], vp_ - 0.5 * vy[pS])
        Rm = (um_ + 0.5 * uy[mS], vm_ + 0.5 * vy[mS])
        Hf = 0.5 * (Hk[pR, :-1] + Hk[pR, 1:])
        if bc.south == 1:
            um_ = torch.where(rm + 1 == 2, -um_, um_)
        if bc.north == 1:
            up_ = torch.where(rm + 1 == ny + 2, -up_, up_)
        upe = up_ * ex[pR] + vp_ * ey[pR]
        ume = um_ * ex[mR] + vm_ * ey[mR]
        etap = torch.maximum(-Hf, eb_p - (Ly[pS] - dy * F[pR] * upe) / (2.0 * g))
        etam = torch.maximum(-Hf, eb_m + (Ly[mS] - dy * F[mR] * ume) / (2.0 * g))
        Gf = _flux([etam, Rm[1], Rm[0]], [etap, Rp[1], Rp[0]], Hf, P)
        Gy = [Gf[0], Gf[2], Gf[1]]
        dm, dp = eb_m == DRY_FLAG, eb_p == DRY_FLAG
        pe = 0.5 * g * (etap + Hf) * (etap + Hf)
        me = 0.5 * g * (etam + Hf) * (etam + Hf)
        zg = torch.zeros_like(Gy[0])
        Gy[2] = torch.where(dm & ~dp, pe, torch.where(~dm & dp, me, Gy[2]))
        for k in (0, 1):
            Gy[k] = torch.where(dm ^ dp, zg, Gy[k])
        for k in range(3):
            Gy[k] = torch.where(dm & dp, zg, Gy[k])

        # interior update
        I, J = slice(2, nx + 2), slice(2, ny + 2)
        fd = [(Fx[k][J, 1:nx + 1] - Fx[k][J, 0:nx]) / dx for k in range(3)]
        if not P.one_dimensional:
            fd = [fd[k] + (Gy[k][1:ny + 1, I] - Gy[k][0:ny, I]) / dy for k in range(3)]
        ec, uc, vc = eta[J, I], u[J, I], v[J, I]
        Hm = Hm_k[J, I]
        fc = F[J, I]
        hsum = ec + Hm
        zc = torch.zeros_like(hsum)
        hu = torch.where(hsum > cutoff, uc * hsum, zc)
        hv = torch.where(hsum > cutoff, vc * hsum, zc)
        Kxc = Kx[J, 1:nx + 1]
        Lyc = Ly[1:ny + 1, I]
        eta_w = ec - (Kxc + dx * fc * vc) / (2.0 * g)
        eta_e = ec + (Kxc + dx * fc * vc) / (2.0 * g)
        eta_s = ec - (Lyc - dy * fc * uc) / (2.0 * g)
        eta_n = ec + (Lyc - dy * fc * uc) / (2.0 * g)
        nxc, nyc = nxn[J, I], nyn[J, I]
        exc, eyc = nyc, -nxc
        hu_e = hu * exc + hv * eyc
        hv_n = hu * nxc + hv * nyc
        hu_ec = fc * hv_n
        hv_nc = -fc * hu_e
        upx, upy = -nxc, nyc
        rtx, rty = upy, -upx
        hu_cor = rtx * hu_ec + rty * hv_nc
        hv_cor = upx * hu_ec + upy * hv_nc
        RHxp = 0.5 * (Hk[J, 3:nx + 3] + Hk[3:ny + 3, 3:nx + 3])
        RHxm = 0.5 * (Hk[J, I] + Hk[3:ny + 3, I])
        RHyp = 0.5 * (Hk[3:ny + 3, I] + Hk[3:ny + 3, 3:nx + 3])
        RHym = 0.5 * (Hk[J, I] + Hk[J, 3:nx + 3])
        bath1 = g * (0.5 * (eta_w + eta_e) + Hm) * (RHxp - RHxm)
        bath2 = g * (0.5 * (eta_n + eta_s) + Hm) * (RHyp - RHym)
        wet = (hsum >= cutoff) & (ec != DRY_FLAG)
        st1 = torch.where(wet, self.wsf * X + hu_cor + bath1 / dx, zc)
        st2 = torch.where(wet, self.wsf * Y + hv_cor + bath2 / dy, zc)
        L1 = -fd[0]
        L2 = -fd[1] + st1
        L3 = -fd[2] + st2

        Cf = zc
        if P.r > 0.0:
            small = hsum < eps_d
            hs_small = torch.where(small, hsum, torch.full_like(hsum, eps_d))
            hs_big = torch.where(small, torch.ones_like(hsum), hsum)
            us = _desing(hs_small, hu, eps_d)
            vs = _desing(hs_small, hv, eps_d)
            Cs = dt * P.r * _desing(hs_small, torch.sqrt(us * us + vs * vs + 1e-300), eps_d)
            ub, vb = hu / hs_big, hv / hs_big
            Cb = dt * P.r * torch.sqrt(ub * ub + vb * vb + 1e-300) / hs_big
            Cf = torch.where(small, Cs, Cb)

        if rk_step == 0:
            ne = ec + dt * L1
            nhu = (hu + dt * L2) / (1.0 + Cf)
            nhv = (hv + dt * L3) / (1.0 + Cf)
        else:
            eo, huo, hvo = (a[J, I] for a in Qn)
            ne = 0.5 * (eo + (ec + dt * L1))
            nhu = 0.5 * (huo + (hu + dt * L2)) / (1.0 + 0.5 * Cf)
            nhv = 0.5 * (hvo + (hv + dt * L3)) / (1.0 + 0.5 * Cf)
        dry = (ne + Hm) <= cutoff
        ne = torch.where(dry, -Hm + cutoff, ne)
        nhu = torch.where(dry, zc, nhu)
        nhv = torch.where(dry, zc, nhv)
        return torch.maximum(-Hm + cutoff, ne), nhu, nhv

    def _assemble(self, full, interior):
        nx, ny = self.nx, self.ny
        out = []
        for a, b in zip(full, interior):
            a = a.clone()
            a[2:ny + 2, 2:nx + 2] = b
            out.append(a)
        return periodic_ghosts(out, nx, ny, self.bc)

    def rk2_step(self, Q, X, Y, dt):
        """One RK2 step of full (ny+4, nx+4) arrays; ghost cells of the result
        are periodic images (periodic) or carried over (walls)."""
        Q = periodic_ghosts(Q, self.nx, self.ny, self.bc)
        Qs = self._assemble(Q, self.stage(Q, None, X, Y, dt, 0))
        return self._assemble(Q, self.stage(Qs, Q, X, Y, dt, 1))


def drift(positions, eta, hu, hv, Hm, nx, ny, dx, dy, dt, periodic_ns, periodic_ew, x0ref=2, y0ref=2):
    """One forward-Euler drifter step on torch tensors: the restatement of
    ``oracle.noise_oracle.drift`` (K/driftKernels.cu:74-183) for autograd.
    positions (N, 2); eta, hu, hv, Hm full (ny+4, nx+4) arrays."""
    u_f = hu / (Hm + eta)
    v_f = hv / (Hm + eta)
    x, y = positions[:, 0], positions[:, 1]
    fx, fy = torch.floor(x / dx), torch.floor(y / dy)
    cx = (fx + x0ref).long()
    cy = (fy + y0ref).long()
    frx, fry = x / dx - fx, y / dy - fy
    x0 = torch.where(frx < 0.5, cx - 1, cx)
    xf = torch.where(frx < 0.5, frx + 0.5, frx - 0.5)
    y0 = torch.where(fry < 0.5, cy - 1, cy)
    yf = torch.where(fry < 0.5, fry + 0.5, fry - 0.5)
    x0c, x1c = x0.clamp(0, nx + 3), (x0 + 1).clamp(0, nx + 3)
    y0c, y1c = y0.clamp(0, ny + 3), (y0 + 1).clamp(0, ny + 3)

    def interp(fld):
        a = (1 - xf) * fld[y0c, x0c] + xf * fld[y0c, x1c]
        b = (1 - xf) * fld[y1c, x0c] + xf * fld[y1c, x1c]
        return (1 - yf) * a + yf * b
    x = x + interp(u_f) * dt
    y = y + interp(v_f) * dt
    Lx, Ly = nx * dx, ny * dy
    if periodic_ew:
        x = torch.where(x < 0, x + Lx, x)
        x = torch.where(x > Lx, x - Lx, x)
    if periodic_ns:
        y = torch.where(y < 0, y + Ly, y)
        y = torch.where(y > Ly, y - Ly, y)
    return torch.stack([x, y], dim=1)
