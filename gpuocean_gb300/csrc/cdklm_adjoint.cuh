// Hand-written reverse mode (vector-Jacobian products) of one CDKLM16
// Runge-Kutta stage, for sm_103a.
//
// A stage maps the stage input x (interior cells; ghost cells are periodic
// images or wall mirrors of interior cells) to the stage output
//   rk 0:  y = finish(x + dt R(x))                        (friction implicit)
//   rk 1:  y = finish(0.5 (a + x + dt R(x)))               (a = Q^n)
// The VJP kernel owns an output tile of x-bar.  It recomputes the forward
// stage on the tile + 2 cells from x staged on the tile + 4 cells (the same
// code as the forward kernel), then runs the reverse sweep in shared memory:
//   cell pass   y-bar -> L-bar (flux part kept per cell), source terms,
//               friction, RK combination, direct terms
//   face passes flux-bar -> (D-bar, slope-bar) of the two cells of a face
//   slope passes slope-bar -> D-bar of the three cells of a slope
//   cell pass   desingularisation: D-bar -> x-bar, folded onto the interior
//               cell each staged position stands for (wall mirrors)
// Scatter passes are coloured (two colours for faces, three for slopes) so
// that no two threads add to the same cell: the result is deterministic.
// Branches (limiter choice, dry clamps, desingularisation regime, flux
// switches) are those of the recomputed forward state.
#pragma once

#include "cdklm_tile.cuh"

namespace goc {

// Shared memory of the VJP tile.  The forward recompute uses D, Sx, Sy, Fx,
// Gy, Hi (and Fc with a Coriolis texture); after the cell pass the flux
// planes are reused: Fx holds the slope adjoints (x slopes, then y slopes)
// and Gy the flux-divergence adjoint of each cell, later the x-bar of each
// staged position.  18 planes with a constant f: three CTAs per SM.
template <int W, int H, bool HAS_FC>
struct AdjSmem {
    float D[3][H][W];
    float Sx[3][H][W];
    float Sy[3][H][W];
    float Fx[3][H][W];
    float Gy[3][H][W];
    float Db[3][H][W];      // adjoint of the desingularised (eta, u, v)
    float Hi[H][W];         // south-west corner depth of each cell (the passes read corners < (H, W))
    float Fc[HAS_FC ? H : 1][HAS_FC ? W : 1];
};

// ---------------------------------------------------------------------------
// scalar reverse functions
// ---------------------------------------------------------------------------

// Subgradient conventions at kinks and ties: a minimum or maximum of equal
// arguments passes half of the adjoint to each, and |x| has slope 0 at x = 0
// (the conventions of torch's autograd, against which the adjoint is tested).
// minmod_raw(b, c, f) = sgn * min(|b|, |c|, |f|) when all three share a
// sign, else 0.
__device__ __forceinline__ void minmod_raw_vjp(float b, float c, float f, float gb, float& bb, float& cb,
                                               float& fb) {
    const float sb = copysignf(1.0f, b), sc = copysignf(1.0f, c), sf = copysignf(1.0f, f);
    // no adjoint where the signs differ (branch-free: selects)
    const float g = (sb == sc && sc == sf) ? gb : 0.0f;
    const float ab = fabsf(b), ac = fabsf(c), af = fabsf(f);
    // inner min(|b|, |c|), outer min(., |f|)
    const float wb1 = ab < ac ? 1.0f : (ab == ac ? 0.5f : 0.0f);
    const float m1 = fminf(ab, ac);
    const float wm = m1 < af ? 1.0f : (m1 == af ? 0.5f : 0.0f);
    bb = b != 0.0f ? g * wb1 * wm : 0.0f;
    cb = c != 0.0f ? g * (1.0f - wb1) * wm : 0.0f;
    fb = f != 0.0f ? g * (1.0f - wm) : 0.0f;
}

__device__ __forceinline__ void minmod_slope_vjp(float l, float c, float r, float theta, float gs, float& lb,
                                                 float& cb, float& rb) {
    float b1, b2, b3;
    minmod_raw_vjp((c - l) * theta, (r - l) * 0.5f, (r - c) * theta, gs, b1, b2, b3);
    lb = -theta * b1 - 0.5f * b2;
    cb = theta * b1 - theta * b3;
    rb = 0.5f * b2 + theta * b3;
}

// desing(h, q, eps) = q / max(min(h^2/(2 eps) + eps/2, eps), |h|)
__device__ __forceinline__ void desing_vjp(float h, float q, float eps, float rbar, float& hb, float& qb) {
    const float a = (float)((double)(h * h / (2.0f * eps)) + 0.5 * (double)eps);
    const float m = fminf(a, eps);
    const float ah = fabsf(h);
    const float den = fmaxf(m, ah);
    const float r = q / den;
    qb = rbar / den;
    const float denb = -rbar * r / den;
    // den = max(m, |h|), m = min(a, eps)
    const float wh = ah > m ? 1.0f : (ah == m ? 0.5f : 0.0f);
    const float wa = a < eps ? 1.0f : (a == eps ? 0.5f : 0.0f);
    hb = (h != 0.0f ? denb * wh * copysignf(1.0f, h) : 0.0f) + denb * (1.0f - wh) * wa * h / eps;
}

// Reverse of desingularize_cell: (oe, ou, ov)-bar -> (eta, hu, hv)-bar.
__device__ __forceinline__ void desingularize_cell_vjp(const GocCdklmParams& p, float eta, float hu, float hv,
                                                       float Hm, float oeb, float oub, float ovb, float& eb,
                                                       float& hub, float& hvb) {
    const float h = eta + Hm;
    // the wet cell on every lane; land and shallow cells (rare) are redone
    // under a branch that a warp takes only when one of its lanes has one
    const float ih = 1.0f / h;
    hub = oub * ih;
    hvb = ovb * ih;
    eb = oeb - (oub * hu + ovb * hv) * ih * ih;
    const bool land = fabsf(Hm - p.land_value) <= kDryEps;
    const bool shallow = h < p.desing_eps;
    if (__any_sync(__activemask(), land || shallow)) {
        if (land || (shallow && h <= p.depth_cutoff)) {
            eb = 0.0f; hub = 0.0f; hvb = 0.0f;
        } else if (shallow) {
            float hb1, hb2;
            desing_vjp(h, hu, p.desing_eps, oub, hb1, hub);
            desing_vjp(h, hv, p.desing_eps, ovb, hb2, hvb);
            eb = oeb + hb1 + hb2;
        }
    }
}

// Reverse of cdklm_flux (H constant).  Branch-free: a dry side's terms and
// the case of vanishing wave speeds are evaluated on every lane and replaced
// by selects (the adjoint is checked against FP64 autograd, not for bits).
__device__ __forceinline__ void cdklm_flux_vjp(const GocCdklmParams& p, const StepConst& k, float em, float um_,
                                               float vm_, float ep, float up_, float vp_, float H, float F0b,
                                               float F1b, float F2b, float& emb, float& umb, float& vmb,
                                               float& epb, float& upb, float& vpb) {
    const float hp = ep + H;
    const float hm = em + H;
    const bool wp = hp > p.depth_cutoff, wm = hm > p.depth_cutoff;
    const float Fp0 = wp ? hp * up_ : 0.f;
    const float Fp1 = wp ? hp * up_ * up_ + k.half_g * hp * hp : 0.f;
    const float Fp2 = wp ? hp * up_ * vp_ : 0.f;
    const float up = wp ? up_ : 0.f, cp = wp ? sqrtf(p.g * hp) : 0.f;
    const float Fm0 = wm ? hm * um_ : 0.f;
    const float Fm1 = wm ? hm * um_ * um_ + k.half_g * hm * hm : 0.f;
    const float Fm2 = wm ? hm * um_ * vm_ : 0.f;
    const float um = wm ? um_ : 0.f, cm = wm ? sqrtf(p.g * hm) : 0.f;
    const float A = um + cm, B = up + cp, C = um - cm, D = up - cp;
    const float am = fminf(fminf(C, D), 0.0f);
    const float ap = fmaxf(fmaxf(A, B), 0.0f);
    const bool still = fabsf(ap - am) < p.flux_slope_eps;
    const float inv = 1.0f / (ap - am);
    const float apam = ap * am;
    const float fb = p.flux_balancer;
    const float N0 = (ap * Fm0 - am * Fp0) + apam * (ep - em);
    const float N1 = (ap * Fm1 - am * Fp1) + apam * (Fp0 - Fm0);
    const float dv = hp * vp_ - hm * vm_;
    const float N2 = (ap * Fm2 - am * Fp2) + apam * dv;
    const float N0b = F0b * inv, N1b = F1b * inv, N2b = F2b * (1.0f - fb) * inv;
    const float invb = F0b * N0 + F1b * N1 + F2b * (1.0f - fb) * N2;
    const bool upwind_m = um_ > -up_;
    float Fm2b = upwind_m ? F2b * fb : 0.f, Fp2b = upwind_m ? 0.f : F2b * fb;
    float apb = N0b * Fm0 + N1b * Fm1 + N2b * Fm2;
    float amb = -(N0b * Fp0 + N1b * Fp1 + N2b * Fp2);
    const float apamb = N0b * (ep - em) + N1b * (Fp0 - Fm0) + N2b * dv;
    const float Fm0b = N0b * ap - N1b * apam, Fp0b = -N0b * am + N1b * apam;
    const float Fm1b = N1b * ap, Fp1b = -N1b * am;
    Fm2b += N2b * ap;
    Fp2b += -N2b * am;
    float ep_b = N0b * apam;
    float em_b = -N0b * apam;
    float hpb = N2b * apam * vp_, hmb = -N2b * apam * vm_;
    float vp_b = N2b * apam * hp;
    float vm_b = -N2b * apam * hm;
    apb += apamb * am;
    amb += apamb * ap;
    apb -= invb * inv * inv;
    amb += invb * inv * inv;
    // ap = max(max(A, B), 0), am = min(min(C, D), 0)
    const float tA = fmaxf(A, B), tC = fminf(C, D);
    const float wt = tA > 0.0f ? 1.0f : (tA == 0.0f ? 0.5f : 0.0f);
    const float wA = A > B ? 1.0f : (A == B ? 0.5f : 0.0f);
    const float ws = tC < 0.0f ? 1.0f : (tC == 0.0f ? 0.5f : 0.0f);
    const float wC = C < D ? 1.0f : (C == D ? 0.5f : 0.0f);
    const float Ab = apb * wt * wA, Bb = apb * wt * (1.0f - wA);
    const float Cb = amb * ws * wC, Db = amb * ws * (1.0f - wC);
    const float umb_m = Ab + Cb, cmb = Ab - Cb;
    const float upb_m = Bb + Db, cpb = Bb - Db;
    // the wet sides' terms (a dry side has none)
    float um_b = 0.f, up_b = 0.f;
    {
        const float hmb_w = (cm > 0.0f ? cmb * 0.5f * p.g / cm : 0.0f) + Fm0b * um_ +
                            Fm1b * (um_ * um_ + p.g * hm) + Fm2b * um_ * vm_;
        const float umb_w = umb_m + Fm0b * hm + Fm1b * 2.0f * hm * um_ + Fm2b * hm * vm_;
        const float vmb_w = Fm2b * hm * um_;
        if (wm) { hmb += hmb_w; um_b += umb_w; vm_b += vmb_w; }
        const float hpb_w = (cp > 0.0f ? cpb * 0.5f * p.g / cp : 0.0f) + Fp0b * up_ +
                            Fp1b * (up_ * up_ + p.g * hp) + Fp2b * up_ * vp_;
        const float upb_w = upb_m + Fp0b * hp + Fp1b * 2.0f * hp * up_ + Fp2b * hp * vp_;
        const float vpb_w = Fp2b * hp * up_;
        if (wp) { hpb += hpb_w; up_b += upb_w; vp_b += vpb_w; }
    }
    ep_b += hpb;
    em_b += hmb;
    emb = still ? 0.f : em_b;
    umb = still ? 0.f : um_b;
    vmb = still ? 0.f : vm_b;
    epb = still ? 0.f : ep_b;
    upb = still ? 0.f : up_b;
    vpb = still ? 0.f : vp_b;
}

// Reverse of Tile::friction: C-bar -> (hsum, hu, hv)-bar (adds).
__device__ __forceinline__ void friction_vjp(const GocCdklmParams& p, float dt, float hsum, float hu, float hv,
                                             float Cb, float& hsb, float& hub, float& hvb) {
    if (!(p.r > 0.0f) || p.rk_order >= 3 || Cb == 0.0f) return;
    const float eps = p.desing_eps;
    if (hsum < eps) {
        const float u = desing(hsum, hu, eps), v = desing(hsum, hv, eps);
        const float s = sqrtf(u * u + v * v);
        float hb0, sb;
        desing_vjp(hsum, s, eps, Cb * dt * p.r, hb0, sb);
        hsb += hb0;
        if (s > 0.0f) {
            const float ub = sb * u / s, vb = sb * v / s;
            float hb1, q1, hb2, q2;
            desing_vjp(hsum, hu, eps, ub, hb1, q1);
            desing_vjp(hsum, hv, eps, vb, hb2, q2);
            hsb += hb1 + hb2;
            hub += q1;
            hvb += q2;
        }
    } else {
        const float u = hu / hsum, v = hv / hsum;
        const float s = sqrtf(u * u + v * v);
        const float C = dt * p.r * s / hsum;
        const float sb = Cb * dt * p.r / hsum;
        hsb += -Cb * C / hsum;
        if (s > 0.0f) {
            const float ub = sb * u / s, vb = sb * v / s;
            hub += ub / hsum;
            hvb += vb / hsum;
            hsb += -(ub * u + vb * v) / hsum;
        }
    }
}

// ---------------------------------------------------------------------------
// the tile
// ---------------------------------------------------------------------------

template <int W, int H, int NT, bool BORDER, bool HAS_FC>
struct AdjTile {
    using SM = AdjSmem<W, H, HAS_FC>;
    SM& A;
    Tile<W, H, NT, BORDER, SM>& T;
    const GocCdklmParams& p;
    const StepConst& k;

    // the slope adjoints of one direction at a time live in the flux planes Fx
    __device__ float (&Sxb(int c))[H][W] { return A.Fx[c]; }
    __device__ float (&Syb(int c))[H][W] { return A.Fx[c]; }

    // Reverse of one x face (east face of local cell (i, j)), adding to the
    // D-bar and x-slope-bar of cells i and i+1.
    template <bool CONST_F>
    __device__ void face_x_vjp(int i, int j, float F0b, float F1b, float F2b) {
        SM& S = A;
        const float ebm = S.D[0][j][i], ebp = S.D[0][j][i + 1];
        const bool dm = (ebm == kDryFlag), dp = (ebp == kDryFlag);
        const int gxp = T.x0 + i + 1;
        const float um = S.D[1][j][i], up = S.D[1][j][i + 1];
        float vm = S.D[2][j][i], vp = S.D[2][j][i + 1];
        const float Rpx = up - 0.5f * S.Sx[0][j][i + 1];
        const float Rpy = vp - 0.5f * S.Sx[1][j][i + 1];
        const float Rmx = um + 0.5f * S.Sx[0][j][i];
        const float Rmy = vm + 0.5f * S.Sx[1][j][i];
        const float Hf = 0.5f * (S.Hi[j][i + 1] + S.Hi[j + 1][i + 1]);
        float svm = 1.0f, svp = 1.0f;
        if (BORDER) {
            if (p.bc_west == 1 && gxp == 2) svm = -1.0f;
            if (p.bc_east == 1 && gxp == p.nx + 2) svp = -1.0f;
        }
        vm *= svm;
        vp *= svp;
        const float fp = T.F(j, i + 1, CONST_F), fm = T.F(j, i, CONST_F);
        const float vpn = up * T.nX + vp * T.nY;
        const float vmn = um * T.nX + vm * T.nY;
        const float xp = ebp - (S.Sx[2][j][i + 1] + p.dx * fp * vpn) * k.inv_2g;
        const float xm = ebm + (S.Sx[2][j][i] + p.dx * fm * vmn) * k.inv_2g;
        const float etap = fmaxf(-Hf, xp);
        const float etam = fmaxf(-Hf, xm);
        // the wet face on every lane; a face with a land side (rare) is redone
        // under a branch that a warp takes only when one of its lanes has one
        float etapb, etamb, Rpxb, Rpyb, Rmxb, Rmyb;
        cdklm_flux_vjp(p, k, etam, Rmx, Rmy, etap, Rpx, Rpy, Hf, F0b, F1b, F2b, etamb, Rmxb, Rmyb, etapb, Rpxb, Rpyb);
        if (__any_sync(__activemask(), dm || dp)) {
            if (dm || dp) {
                Rpxb = 0.f; Rpyb = 0.f; Rmxb = 0.f; Rmyb = 0.f;
                etapb = (dm && !dp) ? F1b * p.g * (etap + Hf) : 0.f;
                etamb = (dp && !dm) ? F1b * p.g * (etam + Hf) : 0.f;
            }
        }
        // etap = max(-Hf, xp): xp-bar only where xp is taken
        const float xpb = etapb * (xp > -Hf ? 1.0f : (xp == -Hf ? 0.5f : 0.0f));
        const float xmb = etamb * (xm > -Hf ? 1.0f : (xm == -Hf ? 0.5f : 0.0f));
        const float vpnb = -xpb * k.inv_2g * p.dx * fp;
        const float vmnb = xmb * k.inv_2g * p.dx * fm;
        // cell i (minus side)
        A.Db[0][j][i] += xmb;
        A.Db[1][j][i] += Rmxb + vmnb * T.nX;
        A.Db[2][j][i] += Rmyb + vmnb * T.nY * svm;
        Sxb(0)[j][i] += 0.5f * Rmxb;
        Sxb(1)[j][i] += 0.5f * Rmyb;
        Sxb(2)[j][i] += xmb * k.inv_2g;
        // cell i+1 (plus side)
        A.Db[0][j][i + 1] += xpb;
        A.Db[1][j][i + 1] += Rpxb + vpnb * T.nX;
        A.Db[2][j][i + 1] += Rpyb + vpnb * T.nY * svp;
        Sxb(0)[j][i + 1] += -0.5f * Rpxb;
        Sxb(1)[j][i + 1] += -0.5f * Rpyb;
        Sxb(2)[j][i + 1] += -xpb * k.inv_2g;
    }

    // Reverse of one y face (north face of local cell (i, j)).
    template <bool CONST_F>
    __device__ void face_y_vjp(int i, int j, float G0b, float G1b, float G2b) {
        SM& S = A;
        const float ebm = S.D[0][j][i], ebp = S.D[0][j + 1][i];
        const bool dm = (ebm == kDryFlag), dp = (ebp == kDryFlag);
        const int gyp = T.y0 + j + 1;
        const float eX = T.nY, eY = -T.nX;
        float um = S.D[1][j][i], up = S.D[1][j + 1][i];
        const float vm = S.D[2][j][i], vp = S.D[2][j + 1][i];
        const float Rpx = up - 0.5f * S.Sy[0][j + 1][i];
        const float Rpy = vp - 0.5f * S.Sy[1][j + 1][i];
        const float Rmx = um + 0.5f * S.Sy[0][j][i];
        const float Rmy = vm + 0.5f * S.Sy[1][j][i];
        const float Hf = 0.5f * (S.Hi[j + 1][i] + S.Hi[j + 1][i + 1]);
        float sum = 1.0f, sup = 1.0f;
        if (BORDER) {
            if (p.bc_south == 1 && gyp == 2) sum = -1.0f;
            if (p.bc_north == 1 && gyp == p.ny + 2) sup = -1.0f;
        }
        um *= sum;
        up *= sup;
        const float fp = T.F(j + 1, i, CONST_F), fm = T.F(j, i, CONST_F);
        const float upe = up * eX + vp * eY;
        const float ume = um * eX + vm * eY;
        const float xp = ebp - (S.Sy[2][j + 1][i] - p.dy * fp * upe) * k.inv_2g;
        const float xm = ebm + (S.Sy[2][j][i] - p.dy * fm * ume) * k.inv_2g;
        const float etap = fmaxf(-Hf, xp);
        const float etam = fmaxf(-Hf, xm);
        // forward: cdklm_flux(etam, Rmy, Rmx, etap, Rpy, Rpx) -> (a0, a1, a2), G = (a0, a2, a1);
        // the wet face on every lane, land faces under a warp vote
        float etapb, etamb, Rpxb, Rpyb, Rmxb, Rmyb;
        cdklm_flux_vjp(p, k, etam, Rmy, Rmx, etap, Rpy, Rpx, Hf, G0b, G2b, G1b, etamb, Rmyb, Rmxb, etapb, Rpyb, Rpxb);
        if (__any_sync(__activemask(), dm || dp)) {
            if (dm || dp) {
                Rpxb = 0.f; Rpyb = 0.f; Rmxb = 0.f; Rmyb = 0.f;
                etapb = (dm && !dp) ? G2b * p.g * (etap + Hf) : 0.f;
                etamb = (dp && !dm) ? G2b * p.g * (etam + Hf) : 0.f;
            }
        }
        const float xpb = etapb * (xp > -Hf ? 1.0f : (xp == -Hf ? 0.5f : 0.0f));
        const float xmb = etamb * (xm > -Hf ? 1.0f : (xm == -Hf ? 0.5f : 0.0f));
        const float upeb = xpb * k.inv_2g * p.dy * fp;
        const float umeb = -xmb * k.inv_2g * p.dy * fm;
        A.Db[0][j][i] += xmb;
        A.Db[1][j][i] += Rmxb + umeb * eX * sum;
        A.Db[2][j][i] += Rmyb + umeb * eY;
        Syb(0)[j][i] += 0.5f * Rmxb;
        Syb(1)[j][i] += 0.5f * Rmyb;
        Syb(2)[j][i] += xmb * k.inv_2g;
        A.Db[0][j + 1][i] += xpb;
        A.Db[1][j + 1][i] += Rpxb + upeb * eX * sup;
        A.Db[2][j + 1][i] += Rpyb + upeb * eY;
        Syb(0)[j + 1][i] += -0.5f * Rpxb;
        Syb(1)[j + 1][i] += -0.5f * Rpyb;
        Syb(2)[j + 1][i] += -xpb * k.inv_2g;
    }

    // Reverse of the x slopes of local cell (i, j): adds to D-bar of i-1, i, i+1.
    template <bool CONST_F>
    __device__ void slope_x_vjp(int i, int j) {
        SM& S = A;
        const float g0 = Sxb(0)[j][i], g1 = Sxb(1)[j][i], g2 = Sxb(2)[j][i];
        if (g0 == 0.0f && g1 == 0.0f && g2 == 0.0f) return;
        const float th = p.theta;
        const int gx = T.x0 + i;
        const float eL = S.D[0][j][i - 1], eC = S.D[0][j][i], eR = S.D[0][j][i + 1];
        const float uL = S.D[1][j][i - 1], uC = S.D[1][j][i], uR = S.D[1][j][i + 1];
        const float vL = S.D[2][j][i - 1], vC = S.D[2][j][i], vR = S.D[2][j][i + 1];
        float eLb = 0.f, eCb = 0.f, eRb = 0.f, uLb, uCb, uRb, vLb, vCb, vRb;
        minmod_slope_vjp(uL, uC, uR, th, g0, uLb, uCb, uRb);
        minmod_slope_vjp(vL, vC, vR, th, g1, vLb, vCb, vRb);
        float sl = 1.f, sc = 1.f, sr = 1.f, sa = 1.f;
        if (BORDER) {
            if (p.bc_west == 1) { if (gx < 3) sl = -1.f; if (gx < 2) sc = -1.f; }
            if (p.bc_east == 1) { if (gx > p.nx) sr = -1.f; if (gx > p.nx + 1) sc = -1.f; }
            if (p.bc_west == 1 && gx < 2) sa = -1.f;
            if (p.bc_east == 1 && gx > p.nx + 2) sa = -1.f;
        }
        const float fL = T.F(j, i - 1, CONST_F), fC = T.F(j, i, CONST_F), fR = T.F(j, i + 1, CONST_F);
        const float nX = T.nX, nY = T.nY;
        const float lfv = (nX * uL + nY * (sl * vL)) * fL;
        const float cfv = (nX * uC + nY * (sc * vC)) * fC;
        const float rfv = (nX * uR + nY * (sr * vR)) * fR;
        const float back = k.theta_g * (eC - eL - k.Vc * (cfv + lfv));
        const float cent = k.half_g * (eR - eL - k.Vc * (rfv + 2.0f * cfv + lfv));
        const float fwd = k.theta_g * (eR - eC - k.Vc * (cfv + rfv));
        const float K0 = minmod_raw(back, cent, fwd);
        const float dxfv = p.dx * fC * (sa * vC);
        const float Hw = 0.5f * (S.Hi[j][i] + S.Hi[j + 1][i]);
        const float He = 0.5f * (S.Hi[j][i + 1] + S.Hi[j + 1][i + 1]);
        const float t = (K0 + dxfv) * k.inv_2g;
        const float hw = eC + Hw - t;
        const float he = eC + He + t;
        // the clamps of adjustSlopes in reverse (selects)
        const bool pe = he > 0.0f, pw = hw > 0.0f;
        const float K1b = pe ? g2 : 0.f;
        const float K0b = pw ? K1b : 0.f;
        const float dxfvb = (pe ? 0.f : -g2) - (pw ? 0.f : K1b);
        eCb += (pe ? 0.f : -k.two_g * g2) + (pw ? 0.f : k.two_g * K1b);
        vCb += dxfvb * p.dx * fC * sa;
        float bb, cb, fb;
        minmod_raw_vjp(back, cent, fwd, K0b, bb, cb, fb);
        eCb += k.theta_g * bb - k.theta_g * fb;
        eLb += -k.theta_g * bb - k.half_g * cb;
        eRb += k.half_g * cb + k.theta_g * fb;
        const float cfvb = -k.Vc * (k.theta_g * bb + 2.0f * k.half_g * cb + k.theta_g * fb);
        const float lfvb = -k.Vc * (k.theta_g * bb + k.half_g * cb);
        const float rfvb = -k.Vc * (k.half_g * cb + k.theta_g * fb);
        uLb += lfvb * fL * nX; vLb += lfvb * fL * nY * sl;
        uCb += cfvb * fC * nX; vCb += cfvb * fC * nY * sc;
        uRb += rfvb * fR * nX; vRb += rfvb * fR * nY * sr;
        A.Db[0][j][i - 1] += eLb; A.Db[1][j][i - 1] += uLb; A.Db[2][j][i - 1] += vLb;
        A.Db[0][j][i] += eCb;     A.Db[1][j][i] += uCb;     A.Db[2][j][i] += vCb;
        A.Db[0][j][i + 1] += eRb; A.Db[1][j][i + 1] += uRb; A.Db[2][j][i + 1] += vRb;
    }

    // Reverse of the y slopes of local cell (i, j): adds to D-bar of j-1, j, j+1.
    template <bool CONST_F>
    __device__ void slope_y_vjp(int i, int j) {
        SM& S = A;
        const float g0 = Syb(0)[j][i], g1 = Syb(1)[j][i], g2 = Syb(2)[j][i];
        if (g0 == 0.0f && g1 == 0.0f && g2 == 0.0f) return;
        const float th = p.theta;
        const int gy = T.y0 + j;
        const float eL = S.D[0][j - 1][i], eC = S.D[0][j][i], eU = S.D[0][j + 1][i];
        const float uL = S.D[1][j - 1][i], uC = S.D[1][j][i], uU = S.D[1][j + 1][i];
        const float vL = S.D[2][j - 1][i], vC = S.D[2][j][i], vU = S.D[2][j + 1][i];
        float eLb = 0.f, eCb = 0.f, eUb = 0.f, uLb, uCb, uUb, vLb, vCb, vUb;
        minmod_slope_vjp(uL, uC, uU, th, g0, uLb, uCb, uUb);
        minmod_slope_vjp(vL, vC, vU, th, g1, vLb, vCb, vUb);
        float sl = 1.f, sc = 1.f, su = 1.f, sa = 1.f;
        if (BORDER) {
            if (p.bc_south == 1) { if (gy < 3) sl = -1.f; if (gy < 2) sc = -1.f; }
            if (p.bc_north == 1) { if (gy > p.ny) su = -1.f; if (gy > p.ny + 1) sc = -1.f; }
            if (p.bc_south == 1 && gy < 2) sa = -1.f;
            if (p.bc_north == 1 && gy > p.ny + 2) sa = -1.f;
        }
        const float eX = T.nY, eY = -T.nX;
        const float fL = T.F(j - 1, i, CONST_F), fC = T.F(j, i, CONST_F), fU = T.F(j + 1, i, CONST_F);
        const float lfu = (eX * (sl * uL) + eY * vL) * fL;
        const float cfu = (eX * (sc * uC) + eY * vC) * fC;
        const float ufu = (eX * (su * uU) + eY * vU) * fU;
        const float back = k.theta_g * (eC - eL + k.Uc * (cfu + lfu));
        const float cent = k.half_g * (eU - eL + k.Uc * (ufu + 2.0f * cfu + lfu));
        const float fwd = k.theta_g * (eU - eC + k.Uc * (cfu + ufu));
        const float L0 = minmod_raw(back, cent, fwd);
        const float dyfu = p.dy * fC * (sa * uC);
        const float Hs = 0.5f * (S.Hi[j][i] + S.Hi[j][i + 1]);
        const float Hn = 0.5f * (S.Hi[j + 1][i] + S.Hi[j + 1][i + 1]);
        const float t = (L0 - dyfu) * k.inv_2g;
        const float hs = eC + Hs - t;
        const float hn = eC + Hn + t;
        // the clamps of adjustSlopes in reverse (selects)
        const bool pn = hn > 0.0f, ps = hs > 0.0f;
        const float L1b = pn ? g2 : 0.f;
        const float L0b = ps ? L1b : 0.f;
        const float dyfub = (pn ? 0.f : g2) + (ps ? 0.f : L1b);
        eCb += (pn ? 0.f : -k.two_g * g2) + (ps ? 0.f : k.two_g * L1b);
        uCb += dyfub * p.dy * fC * sa;
        float bb, cb, fb;
        minmod_raw_vjp(back, cent, fwd, L0b, bb, cb, fb);
        eCb += k.theta_g * bb - k.theta_g * fb;
        eLb += -k.theta_g * bb - k.half_g * cb;
        eUb += k.half_g * cb + k.theta_g * fb;
        const float cfub = k.Uc * (k.theta_g * bb + 2.0f * k.half_g * cb + k.theta_g * fb);
        const float lfub = k.Uc * (k.theta_g * bb + k.half_g * cb);
        const float ufub = k.Uc * (k.half_g * cb + k.theta_g * fb);
        uLb += lfub * fL * eX * sl; vLb += lfub * fL * eY;
        uCb += cfub * fC * eX * sc; vCb += cfub * fC * eY;
        uUb += ufub * fU * eX * su; vUb += ufub * fU * eY;
        A.Db[0][j - 1][i] += eLb; A.Db[1][j - 1][i] += uLb; A.Db[2][j - 1][i] += vLb;
        A.Db[0][j][i] += eCb;     A.Db[1][j][i] += uCb;     A.Db[2][j][i] += vCb;
        A.Db[0][j + 1][i] += eUb; A.Db[1][j + 1][i] += uUb; A.Db[2][j + 1][i] += vUb;
    }
};

}  // namespace goc
