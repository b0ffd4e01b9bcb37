"""FP64 NumPy restatement of GPU Ocean's CDKLM16 step, bathymetry set-up and CFL dt.

TEST INFRASTRUCTURE ONLY.  This module is the checker the parity tests, the
smoke test and the CPU leg of the benchmark compare the CUDA path against.  No
product code imports it.

It follows the reference kernels cell by cell (citations are relative to the
reference project, ``K/`` = ``src/gpuocean/gpu_kernels``, ``S/`` =
``src/gpuocean/SWEsimulators``, ``U/`` = ``src/gpuocean/utils``) but works on
the whole grid with vectorised float64 arithmetic.  Constants are first rounded
to float32, exactly as the reference formats them into its kernels, and then
promoted to float64.

Parity is pinned against the reference's own regression vectors
(``test/timestep50/CDKLM16_*.dat``, converted to ``tests/golden``).

Deliberate differences from the reference (each one is a reference defect):

* Wall ghost cells are always mirrored.  The reference mirrors them from the
  thread that owns the last interior row/column of a 12x32 block, so when
  ``nx % 12 == 1`` or ``ny % 32 == 1`` the cells next to the east/north wall
  read stale global ghost cells (``K/CDKLM16_kernel.cu:420-470``).
* The CFL reduction takes the minimum over every interior cell.  The
  reference's shared-memory tree for 384-thread blocks drops thread ids
  256..383 (``K/max_dt.cu:103-121``).
* RK3 writes its second stage after all reads; the reference writes it in place
  into the buffer other blocks are still reading (``K/CDKLM16_kernel.cu:1076``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

DRY_FLAG = float(np.float32(1.0e-30))        # K/CDKLM16_kernel.cu:34
DRY_EPS = 1.0e-3                              # K/CDKLM16_kernel.cu:35
LAND_VALUE = float(np.float32(1.0e20))        # U/Common.py:1430
FLT_MAX_DT = 100000.0                         # K/max_dt.cu:30


def f32(x) -> float:
    """Round a Python/NumPy scalar to float32 and return it as float64."""
    return float(np.float32(x))


@dataclass
class BC:
    """Boundary flags, 1 = wall, 2 = periodic (U/Common.py:920-960)."""
    north: int = 1
    east: int = 1
    south: int = 1
    west: int = 1

    def periodic_ns(self) -> bool:
        return self.north == 2 and self.south == 2

    def periodic_ew(self) -> bool:
        return self.east == 2 and self.west == 2


# ---------------------------------------------------------------------------
# helpers: limiter, desingularisation, texture lookup
# ---------------------------------------------------------------------------

def minmod_raw(b, c, f):
    """K/common.cu:538-545 (0.25*sgn(b)*(sgn(b)+sgn(c))*(sgn(c)+sgn(f))*min|.|)."""
    sb, sc, sf = np.copysign(1.0, b), np.copysign(1.0, c), np.copysign(1.0, f)
    return 0.25 * sb * (sb + sc) * (sc + sf) * np.minimum(np.minimum(np.abs(b), np.abs(c)), np.abs(f))


def minmod_slope(left, center, right, theta):
    """K/common.cu:524-536."""
    return minmod_raw((center - left) * theta, (right - left) * 0.5, (right - center) * theta)


def desingularize(h, hu, eps):
    """K/common.cu:664-666: hu / max(min(h^2/(2 eps) + eps/2, eps), |h|)."""
    return hu / np.maximum(np.minimum(h * h / (2.0 * eps) + 0.5 * eps, eps), np.abs(h))


def bilinear(tex, s, t):
    """Clamped, texel-centred bilinear lookup in normalised coordinates.

    K/interpolation.cu:137-190 (emulates tex2D with normalised coordinates).
    """
    tex = np.asarray(tex, dtype=np.float64)
    dny, dnx = tex.shape
    s = np.clip(np.asarray(s, dtype=np.float64) - 0.5 / dnx, 0.0, 1.0)
    t = np.clip(np.asarray(t, dtype=np.float64) - 0.5 / dny, 0.0, 1.0)
    x = s * dnx
    y = t * dny
    x0 = np.minimum(np.floor(x).astype(np.int64), dnx - 1)
    y0 = np.minimum(np.floor(y).astype(np.int64), dny - 1)
    ddx = x - x0
    ddy = y - y0
    x1 = np.minimum(x0 + 1, dnx - 1)
    y1 = np.minimum(y0 + 1, dny - 1)
    d00 = tex[y0, x0]
    d01 = tex[y0, x1]
    d10 = tex[y1, x0]
    d11 = tex[y1, x1]
    return d00 + ddx * (d01 - d00) + ddy * (d10 - d00) + ddx * ddy * (d00 + d11 - d01 - d10)


def cell_texture(tex, nx, ny):
    """Texture value at every cell centre of the (ny+4, nx+4) grid.

    K/CDKLM16_kernel.cu:49-57 (coriolisF) and :70-79 (getNorth) use
    s=(i+0.5)/(NX+4), t=(j+0.5)/(NY+4).
    """
    c = (np.arange(nx + 4) + 0.5) / (nx + 4.0)
    r = (np.arange(ny + 4) + 0.5) / (ny + 4.0)
    return bilinear(tex, c[None, :], r[:, None])


def subsample_texture(data, factor):
    """Bilinear spline re-sampling of a texture (S/CDKLM16.py:181-192).

    The reference returns the spline evaluated on an (x, y) grid, i.e. an array
    indexed [x, y], and uploads it as if it were [y, x].  Its own
    ``betamodel_central`` golden was produced with a correctly oriented
    texture, so the result is transposed back to [y, x] here.
    """
    from scipy.interpolate import RectBivariateSpline
    ny, nx = data.shape
    dx, dy = 1.0 / nx, 1.0 / ny
    spline = RectBivariateSpline(np.linspace(0.5 * dx, 1 - 0.5 * dx, nx),
                                 np.linspace(0.5 * dy, 1 - 0.5 * dy, ny),
                                 data.T, kx=1, ky=1)
    new_nx, new_ny = max(2, nx // factor), max(2, ny // factor)
    ndx, ndy = 1.0 / new_nx, 1.0 / new_ny
    return spline(np.linspace(0.5 * ndx, 1 - 0.5 * ndx, new_nx),
                  np.linspace(0.5 * ndy, 1 - 0.5 * ndy, new_ny)).T


# ---------------------------------------------------------------------------
# bathymetry: intersections BC + cell means
# ---------------------------------------------------------------------------

def bathymetry_init(Hi_host, nx, ny, bc: BC):
    """Return (Hi, Hm) exactly as ``Common.Bathymetry`` builds them.

    U/Common.py:1414-1491 (+ _boundaryConditions :1538-1561),
    K/boundary_kernels.cu:122-247, K/initHm_kernel.cu:38-106.
    """
    if np.ma.is_masked(Hi_host):
        Hi = Hi_host.copy().filled(np.float32(1e20)).astype(np.float32)
    else:
        Hi = np.array(Hi_host, dtype=np.float32, copy=True)
    assert Hi.shape == (ny + 5, nx + 5)
    # north-south
    if bc.north == 2 and bc.south == 2:
        for r in list(range(0, 2)) + list(range(ny + 2, ny + 5)):
            src = r + ny if r < 2 else r - ny
            Hi[r, :] = Hi[src, :]
    elif bc.north == 1 and bc.south == 1:
        Hi[0, :] = Hi[4, :]
        Hi[1, :] = Hi[3, :]
        Hi[ny + 4, :] = Hi[ny, :]
        Hi[ny + 3, :] = Hi[ny + 1, :]
    # east-west; the reference tests the north/south flags in the closed branch
    # (U/Common.py:1557) - reproduced.
    if bc.east == 2 and bc.west == 2:
        for c in list(range(0, 2)) + list(range(nx + 2, nx + 5)):
            src = c + nx if c < 2 else c - nx
            Hi[:, c] = Hi[:, src]
    elif bc.north == 1 and bc.south == 1:
        Hi[:, 0] = Hi[:, 4]
        Hi[:, 1] = Hi[:, 3]
        Hi[:, nx + 4] = Hi[:, nx]
        Hi[:, nx + 3] = Hi[:, nx + 1]
    # initBm in float32 arithmetic (its result is a stored float32 buffer)
    Hd = Hi.copy()
    dry = np.abs(Hd - np.float32(1e20)) <= np.float32(DRY_EPS)
    Hd[dry] = np.float32(1e-30)
    a, b, c, d = Hd[:-1, :-1], Hd[1:, :-1], Hd[:-1, 1:], Hd[1:, 1:]
    wet = (np.float32(4.0) - (a == np.float32(1e-30)) - (b == np.float32(1e-30))
           - (c == np.float32(1e-30)) - (d == np.float32(1e-30))).astype(np.float32)
    s = ((a + b) + c) + d
    with np.errstate(divide="ignore", invalid="ignore"):
        Hm = np.where(wet == 0, np.float32(1e20), s / wet).astype(np.float32)
    return Hi, Hm


# ---------------------------------------------------------------------------
# boundary ghost cells for the state
# ---------------------------------------------------------------------------

def periodic_ghosts(Q, nx, ny, bc: BC):
    """K/boundary_kernels.cu:36-110, north-south before east-west (U/Common.py:1310-1330)."""
    for a in Q:
        if bc.north == 2:
            a[0:2, :] = a[ny:ny + 2, :]
            a[ny + 2:ny + 4, :] = a[2:4, :]
        if bc.east == 2:
            a[:, 0:2] = a[:, nx:nx + 2]
            a[:, nx + 2:nx + 4] = a[:, 2:4]


def _wall_mirror(R0, R1, R2, nx, ny, bc: BC):
    """In-tile wall ghosts (K/CDKLM16_kernel.cu:420-470), straight edges only."""
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


# ---------------------------------------------------------------------------
# central-upwind flux (K/CDKLM16_kernel.cu:82-151)
# ---------------------------------------------------------------------------

def _flux(Qm, Qp, H, P):
    """CDKLM16_flux on arrays; Q = (eta, u, v) with u the face-normal velocity."""
    g, cutoff = P.g, P.depth_cutoff
    hp = Qp[0] + H
    hm = Qm[0] + H
    wp = hp > cutoff
    wm = hm > cutoff
    with np.errstate(invalid="ignore"):
        cp = np.where(wp, np.sqrt(np.where(wp, g * hp, 0.0)), 0.0)
        cm = np.where(wm, np.sqrt(np.where(wm, g * hm, 0.0)), 0.0)
    up = np.where(wp, Qp[1], 0.0)
    um = np.where(wm, Qm[1], 0.0)
    Fp = [np.where(wp, hp * Qp[1], 0.0),
          np.where(wp, hp * Qp[1] * Qp[1] + 0.5 * g * hp * hp, 0.0),
          np.where(wp, hp * Qp[1] * Qp[2], 0.0)]
    Fm = [np.where(wm, hm * Qm[1], 0.0),
          np.where(wm, hm * Qm[1] * Qm[1] + 0.5 * g * hm * hm, 0.0),
          np.where(wm, hm * Qm[1] * Qm[2], 0.0)]
    am = np.minimum(np.minimum(um - cm, up - cp), 0.0)
    ap = np.maximum(np.maximum(um + cm, up + cp), 0.0)
    zero = np.abs(ap - am) < P.flux_slope_eps
    den = np.where(zero, 1.0, ap - am)
    F0 = ((ap * Fm[0] - am * Fp[0]) + ap * am * (Qp[0] - Qm[0])) / den
    F1 = ((ap * Fm[1] - am * Fp[1]) + ap * am * (Fp[0] - Fm[0])) / den
    fb = P.flux_balancer
    F2 = np.where(Qm[1] > -Qp[1], fb * Fm[2], fb * Fp[2])
    F2 = F2 + (1.0 - fb) * (((ap * Fm[2] - am * Fp[2]) + ap * am * (hp * Qp[2] - hm * Qm[2])) / den)
    return [np.where(zero, 0.0, F0), np.where(zero, 0.0, F1), np.where(zero, 0.0, F2)]


# ---------------------------------------------------------------------------
# one Runge-Kutta stage of CDKLM16 (K/CDKLM16_kernel.cu:475-1090)
# ---------------------------------------------------------------------------

@dataclass
class Params:
    nx: int
    ny: int
    dx: float
    dy: float
    g: float
    r: float = 0.0
    theta: float = 1.8
    rk_order: int = 2
    desing_eps: float = 0.1
    flux_slope_eps: float = 0.1
    depth_cutoff: float = 1.0e-5
    flux_balancer: float = 0.8
    rho_o: float = 1025.0
    wind_stress_factor: float = 1.0
    one_dimensional: bool = False

    def rounded(self) -> "Params":
        p = Params(**self.__dict__)
        for k in ("dx", "dy", "g", "r", "theta", "desing_eps", "flux_slope_eps",
                  "depth_cutoff", "flux_balancer", "rho_o", "wind_stress_factor"):
            setattr(p, k, f32(getattr(self, k)))
        return p


def cdklm_stage(P: Params, bc: BC, Qin, Qout, Hi, Hm_buf, F, north, wind, pressure,
                dt, rk_step):
    """Evaluate one RK stage and write the interior of ``Qout`` (in place).

    Qin, Qout: lists [eta, hu, hv] of (ny+4, nx+4) float64 arrays.  For RK2
    stage 1 ``Qout`` holds Q^n on entry (K/CDKLM16_kernel.cu:996-1011).
    Hi: corner depths after the intersection BC (float32 values).
    Hm_buf: the initBm cell means.  F: Coriolis f per cell.  north: (2, ny+4, nx+4).
    wind: (X, Y) per cell wind stress (already time interpolated and scaled).
    pressure: (dPx, dPy) per cell central differences of atmospheric pressure.
    """
    nx, ny = P.nx, P.ny
    g, dx, dy, th = P.g, P.dx, P.dy, P.theta
    cutoff, eps_d = P.depth_cutoff, P.desing_eps
    R0, R1, R2 = (np.array(a, dtype=np.float64, copy=True) for a in Qin)
    _wall_mirror(R0, R1, R2, nx, ny, bc)

    Hk = np.array(Hi, dtype=np.float64)
    Hk[np.abs(Hk - LAND_VALUE) < DRY_EPS] = DRY_FLAG
    Hm_k = 0.25 * (Hk[:-1, :-1] + Hk[1:, :-1] + Hk[:-1, 1:] + Hk[1:, 1:])
    Hmb = np.array(Hm_buf, dtype=np.float64)

    # desingularise (:614-656)
    with np.errstate(divide="ignore", invalid="ignore"):
        h = R0 + Hmb
        land = np.abs(Hmb - LAND_VALUE) <= DRY_EPS
        nearly = (~land) & (h < eps_d)
        cut = nearly & (h <= cutoff)
        soft = nearly & (~cut)
        eta = np.where(land, DRY_FLAG, np.where(cut, -Hmb + cutoff, R0))
        u = np.where(land | cut, 0.0, np.where(soft, desingularize(h, R1, eps_d), R1 / h))
        v = np.where(land | cut, 0.0, np.where(soft, desingularize(h, R2, eps_d), R2 / h))
    nxn, nyn = north[0], north[1]
    ex, ey = nyn, -nxn                      # east vector (:745)

    # ---- x direction: slopes at centre columns c = 1..nx+2 (:673-737) ----
    L, C, Rr = slice(0, nx + 2), slice(1, nx + 3), slice(2, nx + 4)
    cidx = np.arange(1, nx + 3)[None, :]
    ux = minmod_slope(u[:, L], u[:, C], u[:, Rr], th)
    vx = minmod_slope(v[:, L], v[:, C], v[:, Rr], th)
    lv, cv, rv = v[:, L].copy(), v[:, C].copy(), v[:, Rr].copy()
    if bc.west == 1:
        lv = np.where(cidx < 3, -lv, lv)
        cv = np.where(cidx < 2, -cv, cv)
    if bc.east == 1:
        rv = np.where(cidx > nx, -rv, rv)
        cv = np.where(cidx > nx + 1, -cv, cv)
    nxc, nyc = nxn[:, C], nyn[:, C]
    lfv = (nxc * u[:, L] + nyc * lv) * F[:, L]
    cfv = (nxc * u[:, C] + nyc * cv) * F[:, C]
    rfv = (nxc * u[:, Rr] + nyc * rv) * F[:, Rr]
    Vc = dx / (2.0 * g)
    back = th * g * (eta[:, C] - eta[:, L] - Vc * (cfv + lfv))
    cent = 0.5 * g * (eta[:, Rr] - eta[:, L] - Vc * (rfv + 2.0 * cfv + lfv))
    fwd = th * g * (eta[:, Rr] - eta[:, C] - Vc * (cfv + rfv))
    Kx = minmod_raw(back, cent, fwd)
    # adjustSlopes_x (:160-203); note the east test is c > NX+2 here
    va = v[:, C].copy()
    if bc.west == 1:
        va = np.where(cidx < 2, -va, va)
    if bc.east == 1:
        va = np.where(cidx > nx + 2, -va, va)
    dxfv = dx * F[:, C] * va
    H_w = 0.5 * (Hk[:-1, C] + Hk[1:, C])
    H_e = 0.5 * (Hk[:-1, 2:nx + 4] + Hk[1:, 2:nx + 4])
    e_c = eta[:, C]
    h_w = e_c + H_w - (Kx + dxfv) / (2.0 * g)
    h_e = e_c + H_e + (Kx + dxfv) / (2.0 * g)
    Kx = np.where(h_w > 0, Kx, -dxfv + 2.0 * g * (e_c + H_w))
    Kx = np.where(h_e > 0, Kx, -dxfv - 2.0 * g * (e_c + H_e))

    # ---- x faces between c and c+1, c = 1..nx+1 (computeFFaceFlux :260-340) ----
    # slope arrays are indexed by centre c at [:, c-1]
    cm = np.arange(1, nx + 2)[None, :]
    mC, pC = slice(1, nx + 2), slice(2, nx + 3)           # cell columns
    mS, pS = slice(0, nx + 1), slice(1, nx + 2)           # slope columns
    eb_m, eb_p = eta[:, mC], eta[:, pC]
    um_, up_ = u[:, mC], u[:, pC]
    vm_, vp_ = v[:, mC].copy(), v[:, pC].copy()
    Rp = (up_ - 0.5 * ux[:, pS], vp_ - 0.5 * vx[:, pS])
    Rm = (um_ + 0.5 * ux[:, mS], vm_ + 0.5 * vx[:, mS])
    Hf = 0.5 * (Hk[:-1, pC] + Hk[1:, pC])
    if bc.west == 1:
        vm_ = np.where(cm + 1 == 2, -vm_, vm_)
    if bc.east == 1:
        vp_ = np.where(cm + 1 == nx + 2, -vp_, vp_)
    # the reference uses the north vector of the updated cell; the angle
    # texture is constant in every configuration handled here
    vpn = up_ * nxn[:, pC] + vp_ * nyn[:, pC]
    vmn = um_ * nxn[:, mC] + vm_ * nyn[:, mC]
    etap = np.maximum(-Hf, eb_p - (Kx[:, pS] + dx * F[:, pC] * vpn) / (2.0 * g))
    etam = np.maximum(-Hf, eb_m + (Kx[:, mS] + dx * F[:, mC] * vmn) / (2.0 * g))
    Fx = _flux([etam, Rm[0], Rm[1]], [etap, Rp[0], Rp[1]], Hf, P)
    dm, dp = eb_m == DRY_FLAG, eb_p == DRY_FLAG
    pe = 0.5 * g * (etap + Hf) * (etap + Hf)
    me = 0.5 * g * (etam + Hf) * (etam + Hf)
    Fx[1] = np.where(dm & ~dp, pe, np.where(~dm & dp, me, Fx[1]))
    for k in (0, 2):
        Fx[k] = np.where(dm ^ dp, 0.0, Fx[k])
    for k in range(3):
        Fx[k] = np.where(dm & dp, 0.0, Fx[k])

    # ---- y direction: slopes at centre rows r = 1..ny+2 (:779-842) ----
    Lo, Ce, Up = slice(0, ny + 2), slice(1, ny + 3), slice(2, ny + 4)
    ridx = np.arange(1, ny + 3)[:, None]
    uy = minmod_slope(u[Lo], u[Ce], u[Up], th)
    vy = minmod_slope(v[Lo], v[Ce], v[Up], th)
    lu, cu_, uu = u[Lo].copy(), u[Ce].copy(), u[Up].copy()
    if bc.south == 1:
        lu = np.where(ridx < 3, -lu, lu)
        cu_ = np.where(ridx < 2, -cu_, cu_)
    if bc.north == 1:
        uu = np.where(ridx > ny, -uu, uu)
        cu_ = np.where(ridx > ny + 1, -cu_, cu_)
    exc, eyc = ex[Ce], ey[Ce]
    lfu = (exc * lu + eyc * v[Lo]) * F[Lo]
    cfu = (exc * cu_ + eyc * v[Ce]) * F[Ce]
    ufu = (exc * uu + eyc * v[Up]) * F[Up]
    Uc = dy / (2.0 * g)
    back = th * g * (eta[Ce] - eta[Lo] + Uc * (cfu + lfu))
    cent = 0.5 * g * (eta[Up] - eta[Lo] + Uc * (ufu + 2.0 * cfu + lfu))
    fwd = th * g * (eta[Up] - eta[Ce] + Uc * (cfu + ufu))
    Ly = minmod_raw(back, cent, fwd)
    ua = u[Ce].copy()
    if bc.south == 1:
        ua = np.where(ridx < 2, -ua, ua)
    if bc.north == 1:
        ua = np.where(ridx > ny + 2, -ua, ua)
    dyfu = dy * F[Ce] * ua
    H_s = 0.5 * (Hk[Ce, :-1] + Hk[Ce, 1:])
    H_n = 0.5 * (Hk[2:ny + 4, :-1] + Hk[2:ny + 4, 1:])
    e_c = eta[Ce]
    h_s = e_c + H_s - (Ly - dyfu) / (2.0 * g)
    h_n = e_c + H_n + (Ly - dyfu) / (2.0 * g)
    Ly = np.where(h_s > 0, Ly, dyfu + 2.0 * g * (e_c + H_s))
    Ly = np.where(h_n > 0, Ly, dyfu - 2.0 * g * (e_c + H_n))

    # ---- y faces between r and r+1, r = 1..ny+1 (computeGFaceFlux :346-416) ----
    rm = np.arange(1, ny + 2)[:, None]
    mR, pR = slice(1, ny + 2), slice(2, ny + 3)
    mS, pS = slice(0, ny + 1), slice(1, ny + 2)
    eb_m, eb_p = eta[mR], eta[pR]
    um_, up_ = u[mR].copy(), u[pR].copy()
    vm_, vp_ = v[mR], v[pR]
    Rp = (up_ - 0.5 * uy[pS], vp_ - 0.5 * vy[pS])
    Rm = (um_ + 0.5 * uy[mS], vm_ + 0.5 * vy[mS])
    Hf = 0.5 * (Hk[pR, :-1] + Hk[pR, 1:])
    if bc.south == 1:
        um_ = np.where(rm + 1 == 2, -um_, um_)
    if bc.north == 1:
        up_ = np.where(rm + 1 == ny + 2, -up_, up_)
    upe = up_ * ex[pR] + vp_ * ey[pR]
    ume = um_ * ex[mR] + vm_ * ey[mR]
    etap = np.maximum(-Hf, eb_p - (Ly[pS] - dy * F[pR] * upe) / (2.0 * g))
    etam = np.maximum(-Hf, eb_m + (Ly[mS] - dy * F[mR] * ume) / (2.0 * g))
    Gf = _flux([etam, Rm[1], Rm[0]], [etap, Rp[1], Rp[0]], Hf, P)
    Gy = [Gf[0], Gf[2], Gf[1]]
    dm, dp = eb_m == DRY_FLAG, eb_p == DRY_FLAG
    pe = 0.5 * g * (etap + Hf) * (etap + Hf)
    me = 0.5 * g * (etam + Hf) * (etam + Hf)
    Gy[2] = np.where(dm & ~dp, pe, np.where(~dm & dp, me, Gy[2]))
    for k in (0, 1):
        Gy[k] = np.where(dm ^ dp, 0.0, Gy[k])
    for k in range(3):
        Gy[k] = np.where(dm & dp, 0.0, Gy[k])

    # ---- update interior cells (:874-1089) ----
    I, J = slice(2, nx + 2), slice(2, ny + 2)
    fd = [(Fx[k][J, 1:nx + 1] - Fx[k][J, 0:nx]) / dx for k in range(3)]
    if not P.one_dimensional:
        fd = [fd[k] + (Gy[k][1:ny + 1, I] - Gy[k][0:ny, I]) / dy for k in range(3)]
    ec, uc, vc = eta[J, I], u[J, I], v[J, I]
    Hm = Hm_k[J, I]
    fc = F[J, I]
    hsum = ec + Hm
    hu = np.where(hsum > cutoff, uc * hsum, 0.0)
    hv = np.where(hsum > cutoff, vc * hsum, 0.0)
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
    X, Y = wind[0][J, I], wind[1][J, I]
    atm_x = -pressure[0][J, I] * hsum / (2.0 * dx * P.rho_o)
    atm_y = -pressure[1][J, I] * hsum / (2.0 * dy * P.rho_o)
    bath1 = g * (0.5 * (eta_w + eta_e) + Hm) * (RHxp - RHxm)
    bath2 = g * (0.5 * (eta_n + eta_s) + Hm) * (RHyp - RHym)
    wet = (hsum >= cutoff) & (ec != DRY_FLAG)
    st1 = np.where(wet, X + hu_cor + atm_x + bath1 / dx, 0.0)
    st2 = np.where(wet, Y + hv_cor + atm_y + bath2 / dy, 0.0)
    L1 = -fd[0]
    L2 = -fd[1] + st1
    L3 = -fd[2] + st2

    C = np.zeros_like(hsum)
    if P.rk_order < 3 and P.r > 0.0:
        with np.errstate(divide="ignore", invalid="ignore"):
            small = hsum < eps_d
            us = desingularize(hsum, hu, eps_d)
            vs = desingularize(hsum, hv, eps_d)
            Cs = dt * P.r * desingularize(hsum, np.sqrt(us * us + vs * vs), eps_d)
            ub, vb = hu / hsum, hv / hsum
            Cb = dt * P.r * np.sqrt(ub * ub + vb * vb) / hsum
            C = np.where(small, Cs, Cb)

    eo, huo, hvo = Qout
    if P.rk_order < 3:
        if rk_step == 0:
            ne = ec + dt * L1
            nhu = (hu + dt * L2) / (1.0 + C)
            nhv = (hv + dt * L3) / (1.0 + C)
        else:
            ne = 0.5 * (eo[J, I] + (ec + dt * L1))
            nhu = 0.5 * (huo[J, I] + (hu + dt * L2)) / (1.0 + 0.5 * C)
            nhv = 0.5 * (hvo[J, I] + (hv + dt * L3)) / (1.0 + 0.5 * C)
    else:
        if rk_step == 0:
            ne, nhu, nhv = ec + dt * L1, hu + dt * L2, hv + dt * L3
        elif rk_step == 1:
            ne = 0.75 * eo[J, I] + 0.25 * (ec + dt * L1)
            nhu = 0.75 * huo[J, I] + 0.25 * (hu + dt * L2)
            nhv = 0.75 * hvo[J, I] + 0.25 * (hv + dt * L3)
        else:
            ne = (eo[J, I] + 2.0 * (ec + dt * L1)) / 3.0
            nhu = (huo[J, I] + 2.0 * (hu + dt * L2)) / 3.0
            nhv = (hvo[J, I] + 2.0 * (hv + dt * L3)) / 3.0
    dry = (ne + Hm) <= cutoff
    ne = np.where(dry, -Hm + cutoff, ne)
    nhu = np.where(dry, 0.0, nhu)
    nhv = np.where(dry, 0.0, nhv)
    return np.maximum(-Hm + cutoff, ne), nhu, nhv


# ---------------------------------------------------------------------------
# CFL time step (K/max_dt.cu:42-141, S/CDKLM16.py:814-861)
# ---------------------------------------------------------------------------

def max_dt_f32(eta, hu, hv, Hm, nx, ny, dx, dy, g):
    """Largest stable dt before the Courant factor, in float32 arithmetic.

    Each cell gives min(0.25 dx/|u +- c|, 0.25 dy/|v +- c|); dry and land cells
    give 1e5.  IEEE float32 divide and square root, as the reference's
    max_dt.cu is built with default (precise) flags.
    """
    e = np.asarray(eta, dtype=np.float32)[2:ny + 2, 2:nx + 2]
    H = np.asarray(Hm, dtype=np.float32)[2:ny + 2, 2:nx + 2]
    hu_ = np.asarray(hu, dtype=np.float32)[2:ny + 2, 2:nx + 2]
    hv_ = np.asarray(hv, dtype=np.float32)[2:ny + 2, 2:nx + 2]
    dx, dy, g = np.float32(dx), np.float32(dy), np.float32(g)
    h = e + H
    skip = (h <= 0) | (np.abs(H - np.float32(1e20)) < np.float32(DRY_EPS))
    with np.errstate(divide="ignore", invalid="ignore"):
        hs = np.where(skip, np.float32(1.0), h)
        u = hu_ / hs
        v = hv_ / hs
        c = np.sqrt(g * hs)
        q = np.float32(0.25)
        d = np.minimum(np.minimum(q * dx / np.abs(u + c), q * dx / np.abs(u - c)),
                       np.minimum(q * dy / np.abs(v + c), q * dy / np.abs(v - c)))
    d = np.where(skip, np.float32(FLT_MAX_DT), d).astype(np.float32)
    return np.float32(min(np.float32(FLT_MAX_DT), d.min()))


# ---------------------------------------------------------------------------
# the simulator (S/CDKLM16.py:48-584)
# ---------------------------------------------------------------------------

class OracleCDKLM16:
    """FP64 restatement of ``CDKLM16`` construction and ``step``.

    Only what the step reads is reproduced: f compensation and Coriolis/angle
    textures (S/CDKLM16.py:147-239), bathymetry (U/Common.py:1408-1491), the
    dry-state clamp of eta0 (:320-321), double buffering (U/Common.py:774-785),
    the RK driver with periodic ghost fills (:477-584) and updateDt (:814-841).
    Wind stress and atmospheric pressure are constant in time here.
    """

    def __init__(self, eta0, hu0, hv0, H, nx, ny, dx, dy, dt, g, f, r,
                 subsample_f=10, angle=None, t=0.0, theta=1.8, rk_order=2,
                 coriolis_beta=0.0, wind_stress=(0.0, 0.0), wind_stress_factor=1.0,
                 boundary_conditions=None, courant_number=0.8,
                 flux_slope_eps=1.0e-1, desingularization_eps=1.0e-1,
                 depth_cutoff=1.0e-5, one_dimensional=False, flux_balancer=0.8,
                 rho_o=1025.0):
        self.nx, self.ny = int(nx), int(ny)
        bc = boundary_conditions if boundary_conditions is not None else BC()
        self.bc = BC(int(bc.north), int(bc.east), int(bc.south), int(bc.west))
        angle = np.array([[0.0]], dtype=np.float32) if angle is None else np.asarray(angle)
        self.P = Params(self.nx, self.ny, dx, dy, g, r, theta, rk_order,
                        desingularization_eps, flux_slope_eps, depth_cutoff,
                        flux_balancer, rho_o, wind_stress_factor, one_dimensional).rounded()
        north0 = (math.sin(float(angle.flat[0])), math.cos(float(angle.flat[0])))
        beta = np.float32(coriolis_beta)
        # S/CDKLM16.py:148-149 compensates in double precision; Simulator
        # stores the result as float32 (S/Simulator.py:90)
        f_comp = np.float32(float(f) - float(coriolis_beta) * (2 * float(dx) * north0[0] + 2 * float(dy) * north0[1]))
        self.f = f_comp
        self.coriolis_beta = beta
        if beta != 0.0:
            gx, gy = 2, 2
            x = np.linspace((-gx + 0.5) * np.float32(dx), (self.nx + gx - 0.5) * np.float32(dx), self.nx + 2 * gx)
            y = np.linspace((-gy + 0.5) * np.float32(dy), (self.ny + gy - 0.5) * np.float32(dy), self.ny + 2 * gx)
            xx, yy = np.meshgrid(x, y)
            n = xx * np.sin(angle.flat[0]) + yy * np.cos(angle.flat[0])
            ftex = (f_comp + beta * n)
        else:
            ftex = np.array([[f_comp]], dtype=np.float32)
        if subsample_f and ftex.size >= np.asarray(eta0).size:
            ftex = subsample_texture(ftex, subsample_f)
        self.ftex = np.asarray(ftex, dtype=np.float32)
        self.angle_tex = np.asarray(angle, dtype=np.float32)
        self.F = cell_texture(self.ftex, self.nx, self.ny)
        ang = cell_texture(self.angle_tex, self.nx, self.ny)
        self.north = np.stack([np.sin(ang), np.cos(ang)])
        sh = (self.ny + 4, self.nx + 4)
        wsf = self.P.wind_stress_factor
        self.wind = (np.full(sh, wsf * f32(wind_stress[0])), np.full(sh, wsf * f32(wind_stress[1])))
        self.pressure = (np.zeros(sh), np.zeros(sh))
        self.Hi, self.Hm = bathymetry_init(H, self.nx, self.ny, self.bc)
        eta0 = np.maximum(np.asarray(eta0, dtype=np.float32), -self.Hm)
        q = [np.array(eta0, dtype=np.float64), np.array(hu0, dtype=np.float32).astype(np.float64),
             np.array(hv0, dtype=np.float32).astype(np.float64)]
        self.Q0 = [a.copy() for a in q]
        self.Q1 = [a.copy() for a in q]
        self.t = float(t)
        self.dt = dt
        self.courant_number = courant_number
        self.num_iterations = 0
        if self.dt <= 0:
            self.updateDt()

    def _stage(self, Qin, Qout, dt, k):
        e, u, v = cdklm_stage(self.P, self.bc, Qin, Qout, self.Hi, self.Hm, self.F,
                              self.north, self.wind, self.pressure, dt, k)
        nx, ny = self.nx, self.ny
        Qout[0][2:ny + 2, 2:nx + 2] = e
        Qout[1][2:ny + 2, 2:nx + 2] = u
        Qout[2][2:ny + 2, 2:nx + 2] = v

    def _bc(self, Q):
        periodic_ghosts(Q, self.nx, self.ny, self.bc)

    def step(self, t_end=0.0):
        if self.t == 0:
            self._bc(self.Q0)
        t_now = 0.0
        while t_now < t_end:
            local_dt = float(np.float32(min(self.dt, np.float32(t_end - t_now))))
            if self.P.rk_order == 2:
                self._stage(self.Q0, self.Q1, local_dt, 0)
                self._bc(self.Q1)
                self._stage(self.Q1, self.Q0, local_dt, 1)
            elif self.P.rk_order == 1:
                self._stage(self.Q0, self.Q1, local_dt, 0)
                self.Q0, self.Q1 = self.Q1, self.Q0
            else:
                self._stage(self.Q0, self.Q1, local_dt, 0)
                self._bc(self.Q1)
                # second stage: reads Q^n from Q0, result goes back into Q1
                nx, ny = self.nx, self.ny
                I, J = slice(2, nx + 2), slice(2, ny + 2)
                tmp = [a.copy() for a in self.Q0]
                e, u, v = cdklm_stage(self.P, self.bc, self.Q1, tmp, self.Hi, self.Hm, self.F,
                                      self.north, self.wind, self.pressure, local_dt, 1)
                for a, b in zip(self.Q1, (e, u, v)):
                    a[J, I] = b
                self._bc(self.Q1)
                self._stage(self.Q1, self.Q0, local_dt, 2)
            self._bc(self.Q0)
            self.t += float(np.float32(local_dt))
            t_now += float(np.float32(local_dt))
            self.num_iterations += 1
        return self.t

    def download(self, interior_domain_only=False):
        out = [a.copy() for a in self.Q0]
        if interior_domain_only:
            return [a[2:-2, 2:-2] for a in out]
        return out

    def max_dt(self):
        return max_dt_f32(self.Q0[0], self.Q0[1], self.Q0[2], self.Hm,
                          self.nx, self.ny, self.P.dx, self.P.dy, self.P.g)

    def updateDt(self, courant_number=None):
        cn = self.courant_number if courant_number is None else courant_number
        self.dt = cn * self.max_dt()
        return self.dt
