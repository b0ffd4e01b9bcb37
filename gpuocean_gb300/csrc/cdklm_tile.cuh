// CDKLM16 step kernels for sm_103a.
//
// One CTA owns an output tile of TX x TY interior cells and stages a halo of
// 2 cells per Runge-Kutta stage in shared memory:
//   * the fused RK2 kernel (NSTAGE = 2) loads Q^n on the tile + 4 cells,
//     recomputes the first stage on the tile + 2 cells (including the periodic
//     ghost images and the mirrored wall ghosts), then the second stage on the
//     tile, and writes Q^{n+1} (+ periodic ghost images) once.  One launch
//     replaces two step launches and two periodic boundary launches per step
//     (S/CDKLM16.py:519-572).
//   * the single-stage kernel (NSTAGE = 1) evaluates one stage with the
//     reference's buffer semantics (K/CDKLM16_kernel.cu:475-1090).
// Every face flux is evaluated once per stage and shared by the two cells
// beside it (the reference evaluates each face twice).
//
// The per-cell arithmetic follows the reference kernel:
//   desingularisation          K/CDKLM16_kernel.cu:614-656, K/common.cu:664-666
//   x slopes + Kx + wall fixes :673-737, adjustSlopes_x :160-203
//   x face flux                computeFFaceFlux :260-340, CDKLM16_flux :104-151
//   y slopes + Ly              :779-842, adjustSlopes_y :211-254
//   y face flux                computeGFaceFlux :346-416
//   sources, friction, RK      :874-1089
// Constant divisions of the reference (/(2g), /DX, /DY, /(ap-am)) are
// multiplications by precomputed reciprocals here.
#pragma once

#include <type_traits>

#include "common.cuh"
#include "f32x2.cuh"
#include "noise_transfer.cuh"
#include "tma.cuh"

namespace goc {

// Per-launch constants derived on the host.
struct StepConst {
    float inv_dx, inv_dy, inv_2g;
    float half_g, two_g;
    float theta_g;        // theta * g
    float Vc, Uc;         // dx/(2g), dy/(2g)
    float inv_atm_x, inv_atm_y;  // 1/(2 dx rho), 1/(2 dy rho)
    int periodic_x, periodic_y;
    float one;            // 1, a run-time value for the paired sums (f32x2.cuh)
    // operands of the paired arithmetic as pairs of equal halves, so that
    // each is one 64-bit operand read instead of two register moves
    float2 one2, none2;   // (1, 1), (-1, -1)
    float2 quarter2, half2;
    float2 theta2, theta_g2, half_g2, g2, Vc2, Uc2;
};

template <int W, int H>
struct TileSmem {
    float D[3][H][W];    // (eta, u, v) after desingularisation
    float Hmb[H][W];     // cell mean depth (initBm semantics); [j][i + 2] holds cell (i, j)
    float Fc[H][W];      // Coriolis f per cell
    float Sx[3][H][W];   // u_x, v_x, dx*Kx at each cell
    float Sy[3][H][W];   // u_y, v_y, dy*Ly at each cell
    float Fx[3][H][W];   // flux through the east face of each cell
    float Gy[3][H][W];   // flux through the north face of each cell
    // depth at the south-west corner of each cell, land -> kDryFlag (the
    // stage code reads corners (j, i) with j < H, i < W only: the corners
    // north and east of the last row and column are not needed)
    float Hi[H][W];
};

// The single-stage kernel with a north-angle texture: each cell sees the
// faces around it with its own north vector (K/CDKLM16_kernel.cu:744-765),
// so every face flux exists twice, once per adjacent cell: Fx / Gy hold the
// faces as their minus (west / south) cell sees them, Fx2 / Gy2 as their
// plus cell does.
template <int W, int H>
struct TileSmemAngle : TileSmem<W, H> {
    float Fx2[3][H][W];
    float Gy2[3][H][W];
};

// 0.25 sb (sb + sc) (sc + sf) min(|b|, |c|, |f|) with sb, sc, sf the signs
// (+-1) of b, c, f, evaluated on the sign bits: with all three signs equal
// the product is sb * min exactly; otherwise it is a zero whose sign the
// product's factors give - + when sb = sc, - when sb != sc = sf, sb's sign
// when sb != sc != sf.  The same bits as the floating-point expression for
// finite arguments.
__device__ __forceinline__ float minmod_raw(float b, float c, float f) {
    const float m = fminf(fminf(fabsf(b), fabsf(c)), fabsf(f));
    const unsigned B = __float_as_uint(b), C = __float_as_uint(c), F = __float_as_uint(f);
    const unsigned x1 = B ^ C, x2 = C ^ F;
    const unsigned zero = (x1 & (~x2 | B)) & 0x80000000u;
    const unsigned same = __float_as_uint(m) | (B & 0x80000000u);
    return __uint_as_float(((x1 | x2) & 0x80000000u) ? zero : same);
}

__device__ __forceinline__ float minmod_slope(float l, float c, float r, float theta) {
    return minmod_raw((c - l) * theta, (r - l) * 0.5f, (r - c) * theta);
}

// minmod_raw and minmod_slope of two independent triples at once (paired
// arithmetic, the same roundings; the unit factors and constants as pairs
// from the step constants).
__device__ __forceinline__ float2 minmod_raw2(float2 b, float2 c, float2 f, const StepConst& k) {
    const float2 sb = pr(copysignf(1.0f, b.x), copysignf(1.0f, b.y));
    const float2 sc = pr(copysignf(1.0f, c.x), copysignf(1.0f, c.y));
    const float2 sf = pr(copysignf(1.0f, f.x), copysignf(1.0f, f.y));
    const float2 m = pr(fminf(fminf(fabsf(b.x), fabsf(c.x)), fabsf(f.x)),
                        fminf(fminf(fabsf(b.y), fabsf(c.y)), fabsf(f.y)));
    return mul2(mul2(mul2(mul2(k.quarter2, sb), add2(sb, sc, k.one2)), add2(sc, sf, k.one2)), m);
}

// with theta = p.theta (StepConst::theta2)
__device__ __forceinline__ float2 minmod_slope2(float2 l, float2 c, float2 r, const StepConst& k) {
    return minmod_raw2(mul2(sub2n(c, l, k.none2), k.theta2), mul2(sub2n(r, l, k.none2), k.half2),
                       mul2(sub2n(r, c, k.none2), k.theta2), k);
}

// K/common.cu:664-666.  The reference's literal 0.5*eps is a double.
__device__ __forceinline__ float desing(float h, float hu, float eps) {
    const float a = (float)((double)(h * h / (2.0f * eps)) + 0.5 * (double)eps);
    return hu / fmaxf(fminf(a, eps), fabsf(h));
}

// Desingularised (eta, u, v) of a raw state, K/CDKLM16_kernel.cu:614-656.
// Every lane evaluates the wet cell's division; land and shallow cells
// (rare) are redone under a branch that a warp takes only when one of its
// lanes has such a cell, so the common case runs without a divergent branch.
__device__ __forceinline__ void desingularize_cell(const GocCdklmParams& p, float eta, float hu, float hv,
                                                   float Hm, float& oe, float& ou, float& ov) {
    const float h = eta + Hm;
    const float ih = 1.0f / h;
    oe = eta; ou = hu * ih; ov = hv * ih;
    const bool land = fabsf(Hm - p.land_value) <= kDryEps;
    const bool shallow = h < p.desing_eps;
    if (__any_sync(__activemask(), land || shallow)) {
        if (land) {
            oe = kDryFlag; ou = 0.0f; ov = 0.0f;
        } else if (shallow) {
            if (h <= p.depth_cutoff) {
                oe = -Hm + p.depth_cutoff; ou = 0.0f; ov = 0.0f;
            } else {
                ou = desing(h, hu, p.desing_eps);
                ov = desing(h, hv, p.desing_eps);
            }
        }
    }
}

// Central-upwind flux with the flux balancer, K/CDKLM16_kernel.cu:82-151.
// Q = (eta, u_normal, v_transverse).  Returns true where both wave speeds
// vanish (near-dry faces, rare): the reference's flux is zero there, and the
// caller replaces the general expression computed here.
__device__ __forceinline__ bool cdklm_flux(const GocCdklmParams& p, const StepConst& k,
                                           float em, float um_, float vm_, float ep, float up_, float vp_,
                                           float H, float& F0, float& F1, float& F2) {
    // the plus and minus sides in pairs (x: plus, y: minus); a dry side (h at
    // or below the cutoff) contributes no flux and no wave speed
    const float2 h = add2(pr(ep, em), pr(H), k.one2);
    const float2 hu = mul2(h, pr(up_, um_));
    const float2 f1 = add2(mul2(hu, pr(up_, um_)), mul2(mul2(k.half_g2, h), h), k.one2);
    const float2 f2 = mul2(hu, pr(vp_, vm_));
    const float2 gh = mul2(k.g2, h);
    const bool wp = h.x > p.depth_cutoff, wm = h.y > p.depth_cutoff;
    const float Fp0 = wp ? hu.x : 0.f, Fp1 = wp ? f1.x : 0.f, Fp2 = wp ? f2.x : 0.f;
    const float Fm0 = wm ? hu.y : 0.f, Fm1 = wm ? f1.y : 0.f, Fm2 = wm ? f2.y : 0.f;
    const float up = wp ? up_ : 0.f, cp = wp ? sqrtf(gh.x) : 0.f;
    const float um = wm ? um_ : 0.f, cm = wm ? sqrtf(gh.y) : 0.f;
    const float2 lo = sub2n(pr(um, up), pr(cm, cp), k.none2);
    const float2 hi = add2(pr(um, up), pr(cm, cp), k.one2);
    const float am = fminf(fminf(lo.x, lo.y), 0.0f);
    const float ap = fmaxf(fmaxf(hi.x, hi.y), 0.0f);
    const bool still = fabsf(ap - am) < p.flux_slope_eps;
    const float inv = 1.0f / (ap - am);
    const float apam = ap * am;
    // (F0, F1) = ((ap Fm - am Fp) + apam (ep - em, Fp0 - Fm0)) inv
    const float2 t = sub2n(mul2(pr(ap), pr(Fm0, Fm1)), mul2(pr(am), pr(Fp0, Fp1)), k.none2);
    const float2 F01 = mul2(add2(t, mul2(pr(apam), sub2n(pr(ep, Fp0), pr(em, Fm0), k.none2)), k.one2), pr(inv));
    F0 = F01.x;
    F1 = F01.y;
    const float fb = p.flux_balancer;
    const float2 s2 = mul2(pr(ap, am), pr(Fm2, Fp2));
    const float2 hv = mul2(h, pr(vp_, vm_));
    float g2 = (um_ > -up_) ? fb * Fm2 : fb * Fp2;
    g2 += (1.0f - fb) * (((s2.x - s2.y) + apam * (hv.x - hv.y)) * inv);
    F2 = g2;
    return still;
}

// Issue the TMA copies of the input boxes of the tile whose staged region
// starts at (x + 2, y) (x a multiple of 4): eta, hu, hv into the planes
// Sx[0], Sx[1], Sy[0] (columns x .. x + W) and the edge area (columns
// x + W .. x + W + 4); with `aux` also the cell-mean depth into the Hmb
// plane and the Coriolis f into Sy[1] (the same column origin x), with their
// east boxes.  The caller is one thread, after a barrier that ended every
// generic access of those planes.
template <int W, int H>
__device__ __forceinline__ void tma_stage_tile(TileTma& t, TileSmem<W, H>& S, int x, int y, bool aux) {
    constexpr uint32_t kBox = W * H * sizeof(float), kEdge = 4 * H * sizeof(float);
    const int naux = aux ? (t.aux_coriolis ? 2 : 1) : 0;
    fence_proxy_async_shared();
    mbar_arrive_expect_tx(t.bar, (uint32_t)(3 + naux) * (kBox + kEdge));
    float* const dst[5] = {&S.Sx[0][0][0], &S.Sx[1][0][0], &S.Sy[0][0][0], &S.Hmb[0][0], &S.Sy[1][0][0]};
    for (int c = 0; c < 3; ++c) {
        tma_load_2d(dst[c], t.in_maps + c, x, y, t.bar);
        tma_load_2d(t.edge + c * 4 * H, t.edge_maps + c, x + W, y, t.bar);
    }
    for (int c = 0; c < naux; ++c) {
        tma_load_2d(dst[3 + c], t.aux_maps + 2 * c, x, y, t.bar);
        tma_load_2d(t.edge + (3 + c) * 4 * H, t.aux_maps + 2 * c + 1, x + W, y, t.bar);
    }
}

// Cell (i, j) of item `idx` of a loop over an NX x ny block of cells.  The
// tile planes are 8 floats wider than most loops, so a warp that ran on
// across the end of a row would meet its own banks again at the next row
// (two shared-memory wavefronts instead of one).  The block is therefore
// walked as its first M = 32 * floor(NX / 32) columns row by row (each warp
// one run of 32 consecutive cells), then its last NX - M columns packed row
// after row.  Loops narrower than 32 cells walk the block row by row.
template <int NX>
__device__ __forceinline__ void block_cell(int idx, int ny, int& i, int& j) {
    constexpr int M = NX < 32 ? NX : 32 * (NX / 32), R = NX - M;
    if (R == 0 || idx < M * ny) {
        i = idx % M; j = idx / M;
    } else {
        const int q = idx - M * ny;
        i = M + q % (R > 0 ? R : 1); j = q / (R > 0 ? R : 1);
    }
}

// SM: the shared-memory layout; any struct with the members of TileSmem that
// the stage code reads (D, Sx, Sy, Fx, Gy, Hi and, with a Coriolis texture, Fc).
// ANGLE: the north vector varies by cell (angle texture; SM then has the
// Fx2 / Gy2 planes of TileSmemAngle).
template <int W, int H, int NT, bool BORDER, class SM = TileSmem<W, H>, bool ANGLE = false>
struct Tile {
    SM& S;
    const GocCdklmParams& p;
    const StepConst& k;
    int x0, y0;               // global cell of local (0,0)
    float nX, nY;             // north vector (constant angle)
    float f0;                 // Coriolis f of a 1x1 texture
    float wind_X, wind_Y;     // scaled wind stress of 1x1 textures

    __device__ float F(int j, int i, bool const_f) const { return const_f ? f0 : S.Fc[j][i]; }

    // North vector of local cell (i, j): the angle texture at the cell's
    // (unwrapped) global index, as getNorth evaluates it
    // (K/CDKLM16_kernel.cu:70-79), or the constant one.
    __device__ __forceinline__ void north(int i, int j, float& ax, float& ay) const {
        if constexpr (ANGLE) {
            const float s = (x0 + i + 0.5f) / (p.nx + 4.0f);
            const float t = (y0 + j + 0.5f) / (p.ny + 4.0f);
            const float a = tex_bilinear(p.angle, p.angle_nx, p.angle_ny, s, t);
            ax = __sinf(a);
            ay = __cosf(a);
        } else {
            ax = nX;
            ay = nY;
        }
    }

    // Start thread of the second loop of a phase whose first loop has n_first
    // items: the warps that take one item more in the first loop (from thread
    // 0) start the second loop at its end, so no warp takes the extra item of
    // both loops (the phase ends at a barrier, so its slowest warp sets its
    // length).  Whole warps are rotated, so each warp still reads one run of
    // consecutive cells.
    __device__ static int second_loop_thread(int n_first) {
        const int tail = ((n_first % NT) + 31) & ~31;
        return (int)((threadIdx.x + NT - tail) % NT);
    }

    // x slopes on [ux0-1, ux1+1) x [uy0, uy1) and y slopes on
    // [ux0, ux1) x [uy0-1, uy1+1); `skip` leading rows are left out
    template <int UX0, int UX1, int UY0, int UY1, bool CONST_F>
    __device__ void slopes(int skip = 0) {
        slopes_boxes<UX0 - 1, UX1 + 1, UY0, UY1, UX0, UX1, UY0 - 1, UY1 + 1, CONST_F>(skip);
    }

    // x slopes on [xx0, xx1) x [xy0, xy1), y slopes on [yx0, yx1) x
    // [yy0, yy1); `skip` leading rows of each are left out
    template <int XX0, int XX1, int XY0, int XY1, int YX0, int YX1, int YY0, int YY1, bool CONST_F>
    __device__ void slopes_boxes(int skip = 0) {
        constexpr int NXS = XX1 - XX0, NYS = XY1 - XY0;
        for (int idx = threadIdx.x; idx < NXS * (NYS - skip); idx += NT) {
            int i, j;
            block_cell<NXS>(idx, NYS - skip, i, j);
            i += XX0; j += XY0 + skip;
            const int gx = x0 + i;
            const float eL = S.D[0][j][i - 1], eC = S.D[0][j][i], eR = S.D[0][j][i + 1];
            const float uL = S.D[1][j][i - 1], uC = S.D[1][j][i], uR = S.D[1][j][i + 1];
            const float vL = S.D[2][j][i - 1], vC = S.D[2][j][i], vR = S.D[2][j][i + 1];
            const float2 suv = minmod_slope2(pr(uL, vL), pr(uC, vC), pr(uR, vR), k);
            S.Sx[0][j][i] = suv.x;
            S.Sx[1][j][i] = suv.y;
            float lv = vL, cv = vC, rv = vR;
            if (BORDER) {
                if (p.bc_west == 1) { if (gx < 3) lv = -lv; if (gx < 2) cv = -cv; }
                if (p.bc_east == 1) { if (gx > p.nx) rv = -rv; if (gx > p.nx + 1) cv = -cv; }
            }
            const float fL = F(j, i - 1, CONST_F), fC = F(j, i, CONST_F), fR = F(j, i + 1, CONST_F);
            float cnX, cnY;
            north(i, j, cnX, cnY);
            // (left, right) in pairs
            const float2 lrfv =
                mul2(add2(mul2(pr(cnX), pr(uL, uR)), mul2(pr(cnY), pr(lv, rv)), k.one2), pr(fL, fR));
            const float lfv = lrfv.x, rfv = lrfv.y;
            const float cfv = (cnX * uC + cnY * cv) * fC;
            // (backward, forward) in pairs
            const float2 bf = mul2(k.theta_g2, sub2n(sub2n(pr(eC, eR), pr(eL, eC), k.none2),
                                                     mul2(k.Vc2, add2(pr(cfv), pr(lfv, rfv), k.one2)), k.none2));
            const float cent = k.half_g * (eR - eL - k.Vc * (rfv + 2.0f * cfv + lfv));
            float Kx = minmod_raw(bf.x, cent, bf.y);
            float va = vC;
            if (BORDER) {
                if (p.bc_west == 1 && gx < 2) va = -va;
                if (p.bc_east == 1 && gx > p.nx + 2) va = -va;
            }
            const float dxfv = p.dx * fC * va;
            const float Hw = 0.5f * (S.Hi[j][i] + S.Hi[j + 1][i]);
            const float He = 0.5f * (S.Hi[j][i + 1] + S.Hi[j + 1][i + 1]);
            const float t = (Kx + dxfv) * k.inv_2g;
            const float hw = eC + Hw - t;
            const float he = eC + He + t;
            Kx = (hw > 0.0f) ? Kx : -dxfv + k.two_g * (eC + Hw);
            Kx = (he > 0.0f) ? Kx : -dxfv - k.two_g * (eC + He);
            S.Sx[2][j][i] = Kx;
        }
        constexpr int NXY = YX1 - YX0, NYY = YY1 - YY0;
        for (int idx = second_loop_thread(NXS * (NYS - skip)); idx < NXY * (NYY - skip); idx += NT) {
            int i, j;
            block_cell<NXY>(idx, NYY - skip, i, j);
            i += YX0; j += YY0 + skip;
            float cnX, cnY;
            north(i, j, cnX, cnY);
            const float eX = cnY, eY = -cnX;  // east vector
            const int gy = y0 + j;
            const float eL = S.D[0][j - 1][i], eC = S.D[0][j][i], eU = S.D[0][j + 1][i];
            const float uL = S.D[1][j - 1][i], uC = S.D[1][j][i], uU = S.D[1][j + 1][i];
            const float vL = S.D[2][j - 1][i], vC = S.D[2][j][i], vU = S.D[2][j + 1][i];
            const float2 suv = minmod_slope2(pr(uL, vL), pr(uC, vC), pr(uU, vU), k);
            S.Sy[0][j][i] = suv.x;
            S.Sy[1][j][i] = suv.y;
            float lu = uL, cu = uC, uu = uU;
            if (BORDER) {
                if (p.bc_south == 1) { if (gy < 3) lu = -lu; if (gy < 2) cu = -cu; }
                if (p.bc_north == 1) { if (gy > p.ny) uu = -uu; if (gy > p.ny + 1) cu = -cu; }
            }
            const float fL = F(j - 1, i, CONST_F), fC = F(j, i, CONST_F), fU = F(j + 1, i, CONST_F);
            // (lower, upper) in pairs
            const float2 lufu =
                mul2(add2(mul2(pr(eX), pr(lu, uu)), mul2(pr(eY), pr(vL, vU)), k.one2), pr(fL, fU));
            const float lfu = lufu.x, ufu = lufu.y;
            const float cfu = (eX * cu + eY * vC) * fC;
            // (backward, forward) in pairs
            const float2 bf = mul2(k.theta_g2, add2(sub2n(pr(eC, eU), pr(eL, eC), k.none2),
                                                    mul2(k.Uc2, add2(pr(cfu), pr(lfu, ufu), k.one2)), k.one2));
            const float cent = k.half_g * (eU - eL + k.Uc * (ufu + 2.0f * cfu + lfu));
            float Ly = minmod_raw(bf.x, cent, bf.y);
            float ua = uC;
            if (BORDER) {
                if (p.bc_south == 1 && gy < 2) ua = -ua;
                if (p.bc_north == 1 && gy > p.ny + 2) ua = -ua;
            }
            const float dyfu = p.dy * fC * ua;
            const float Hs = 0.5f * (S.Hi[j][i] + S.Hi[j][i + 1]);
            const float Hn = 0.5f * (S.Hi[j + 1][i] + S.Hi[j + 1][i + 1]);
            const float t = (Ly - dyfu) * k.inv_2g;
            const float hs = eC + Hs - t;
            const float hn = eC + Hn + t;
            Ly = (hs > 0.0f) ? Ly : dyfu + k.two_g * (eC + Hs);
            Ly = (hn > 0.0f) ? Ly : dyfu - k.two_g * (eC + Hn);
            S.Sy[2][j][i] = Ly;
        }
    }

    // east faces of cells [ux0-1, ux1) x [uy0, uy1); north faces of cells
    // [ux0, ux1) x [uy0-1, uy1); `skip` leading rows are left out
    template <int UX0, int UX1, int UY0, int UY1, bool CONST_F>
    __device__ void faces(int skip = 0) {
        constexpr int NXF = UX1 - UX0 + 1, NYF = UY1 - UY0;
        for (int idx = threadIdx.x; idx < NXF * (NYF - skip); idx += NT) {
            int i, j;
            block_cell<NXF>(idx, NYF - skip, i, j);
            i += UX0 - 1; j += UY0 + skip;
            const int gxp = x0 + i + 1;  // global column of the plus cell
            const float ebm = S.D[0][j][i], ebp = S.D[0][j][i + 1];
            float F0 = 0.f, F1 = 0.f, F2 = 0.f;
            const bool dm = (ebm == kDryFlag), dp = (ebp == kDryFlag);
            if constexpr (!ANGLE) {
                // the wet face's flux on every lane; a face with a dry side
                // (rare) is redone under a branch that a warp takes only when
                // one of its lanes has one (values of a dry side's
                // reconstruction are not used)
                const float um = S.D[1][j][i], up = S.D[1][j][i + 1];
                float vm = S.D[2][j][i], vp = S.D[2][j][i + 1];
                const float Rpx = up - 0.5f * S.Sx[0][j][i + 1];
                const float Rpy = vp - 0.5f * S.Sx[1][j][i + 1];
                const float Rmx = um + 0.5f * S.Sx[0][j][i];
                const float Rmy = vm + 0.5f * S.Sx[1][j][i];
                const float Hf = 0.5f * (S.Hi[j][i + 1] + S.Hi[j + 1][i + 1]);
                if (BORDER) {
                    if (p.bc_west == 1 && gxp == 2) vm = -vm;
                    if (p.bc_east == 1 && gxp == p.nx + 2) vp = -vp;
                }
                float ax, ay;
                north(i, j, ax, ay);
                const float vpn = up * ax + vp * ay;
                const float vmn = um * ax + vm * ay;
                const float etap =
                    fmaxf(-Hf, ebp - (S.Sx[2][j][i + 1] + p.dx * F(j, i + 1, CONST_F) * vpn) * k.inv_2g);
                const float etam = fmaxf(-Hf, ebm + (S.Sx[2][j][i] + p.dx * F(j, i, CONST_F) * vmn) * k.inv_2g);
                const bool still = cdklm_flux(p, k, etam, Rmx, Rmy, etap, Rpx, Rpy, Hf, F0, F1, F2);
                // vanishing wave speeds: no flux; a land side: no flux but
                // the pressure of the other side (both rare)
                if (__any_sync(__activemask(), dm || dp || still)) {
                    if (still) {
                        F0 = 0.f; F1 = 0.f; F2 = 0.f;
                    }
                    if (dm || dp) {
                        F0 = 0.f; F2 = 0.f;
                        F1 = (dm && dp) ? 0.f
                             : dm ? k.half_g * (etap + Hf) * (etap + Hf) : k.half_g * (etam + Hf) * (etam + Hf);
                    }
                }
            } else if (!(dm && dp)) {
                const float um = S.D[1][j][i], up = S.D[1][j][i + 1];
                float vm = S.D[2][j][i], vp = S.D[2][j][i + 1];
                const float Rpx = up - 0.5f * S.Sx[0][j][i + 1];
                const float Rpy = vp - 0.5f * S.Sx[1][j][i + 1];
                const float Rmx = um + 0.5f * S.Sx[0][j][i];
                const float Rmy = vm + 0.5f * S.Sx[1][j][i];
                const float Hf = 0.5f * (S.Hi[j][i + 1] + S.Hi[j + 1][i + 1]);
                if (BORDER) {
                    if (p.bc_west == 1 && gxp == 2) vm = -vm;
                    if (p.bc_east == 1 && gxp == p.nx + 2) vp = -vp;
                }
                // the face as a cell with north vector (ax, ay) sees it
                auto face = [&](float ax, float ay, float& G0, float& G1, float& G2) {
                    const float vpn = up * ax + vp * ay;
                    const float vmn = um * ax + vm * ay;
                    const float etap =
                        fmaxf(-Hf, ebp - (S.Sx[2][j][i + 1] + p.dx * F(j, i + 1, CONST_F) * vpn) * k.inv_2g);
                    const float etam = fmaxf(-Hf, ebm + (S.Sx[2][j][i] + p.dx * F(j, i, CONST_F) * vmn) * k.inv_2g);
                    if (dm) {
                        G1 = k.half_g * (etap + Hf) * (etap + Hf);
                    } else if (dp) {
                        G1 = k.half_g * (etam + Hf) * (etam + Hf);
                    } else {
                        if (cdklm_flux(p, k, etam, Rmx, Rmy, etap, Rpx, Rpy, Hf, G0, G1, G2)) {
                            G0 = 0.f; G1 = 0.f; G2 = 0.f;
                        }
                    }
                };
                float ax, ay;
                north(i, j, ax, ay);
                face(ax, ay, F0, F1, F2);
                if constexpr (ANGLE) {
                    float P0 = 0.f, P1 = 0.f, P2 = 0.f;
                    north(i + 1, j, ax, ay);
                    face(ax, ay, P0, P1, P2);
                    S.Fx2[0][j][i] = P0; S.Fx2[1][j][i] = P1; S.Fx2[2][j][i] = P2;
                }
            } else if constexpr (ANGLE) {
                S.Fx2[0][j][i] = 0.f; S.Fx2[1][j][i] = 0.f; S.Fx2[2][j][i] = 0.f;
            }
            S.Fx[0][j][i] = F0; S.Fx[1][j][i] = F1; S.Fx[2][j][i] = F2;
        }
        constexpr int NXG = UX1 - UX0, NYG = UY1 - UY0 + 1;
        for (int idx = second_loop_thread(NXF * (NYF - skip)); idx < NXG * (NYG - skip); idx += NT) {
            int i, j;
            block_cell<NXG>(idx, NYG - skip, i, j);
            i += UX0; j += UY0 - 1 + skip;
            const int gyp = y0 + j + 1;
            const float ebm = S.D[0][j][i], ebp = S.D[0][j + 1][i];
            float G0 = 0.f, G1 = 0.f, G2 = 0.f;
            const bool dm = (ebm == kDryFlag), dp = (ebp == kDryFlag);
            if constexpr (!ANGLE) {
                float um = S.D[1][j][i], up = S.D[1][j + 1][i];
                const float vm = S.D[2][j][i], vp = S.D[2][j + 1][i];
                const float Rpx = up - 0.5f * S.Sy[0][j + 1][i];
                const float Rpy = vp - 0.5f * S.Sy[1][j + 1][i];
                const float Rmx = um + 0.5f * S.Sy[0][j][i];
                const float Rmy = vm + 0.5f * S.Sy[1][j][i];
                const float Hf = 0.5f * (S.Hi[j + 1][i] + S.Hi[j + 1][i + 1]);
                if (BORDER) {
                    if (p.bc_south == 1 && gyp == 2) um = -um;
                    if (p.bc_north == 1 && gyp == p.ny + 2) up = -up;
                }
                float ax, ay;
                north(i, j, ax, ay);
                const float eX = ay, eY = -ax;
                const float upe = up * eX + vp * eY;
                const float ume = um * eX + vm * eY;
                const float etap =
                    fmaxf(-Hf, ebp - (S.Sy[2][j + 1][i] - p.dy * F(j + 1, i, CONST_F) * upe) * k.inv_2g);
                const float etam = fmaxf(-Hf, ebm + (S.Sy[2][j][i] - p.dy * F(j, i, CONST_F) * ume) * k.inv_2g);
                float a0, a1, a2;
                const bool still = cdklm_flux(p, k, etam, Rmy, Rmx, etap, Rpy, Rpx, Hf, a0, a1, a2);
                G0 = a0; G1 = a2; G2 = a1;
                if (__any_sync(__activemask(), dm || dp || still)) {
                    if (still) {
                        G0 = 0.f; G1 = 0.f; G2 = 0.f;
                    }
                    if (dm || dp) {
                        G0 = 0.f; G1 = 0.f;
                        G2 = (dm && dp) ? 0.f
                             : dm ? k.half_g * (etap + Hf) * (etap + Hf) : k.half_g * (etam + Hf) * (etam + Hf);
                    }
                }
            } else if (!(dm && dp)) {
                float um = S.D[1][j][i], up = S.D[1][j + 1][i];
                const float vm = S.D[2][j][i], vp = S.D[2][j + 1][i];
                const float Rpx = up - 0.5f * S.Sy[0][j + 1][i];
                const float Rpy = vp - 0.5f * S.Sy[1][j + 1][i];
                const float Rmx = um + 0.5f * S.Sy[0][j][i];
                const float Rmy = vm + 0.5f * S.Sy[1][j][i];
                const float Hf = 0.5f * (S.Hi[j + 1][i] + S.Hi[j + 1][i + 1]);
                if (BORDER) {
                    if (p.bc_south == 1 && gyp == 2) um = -um;
                    if (p.bc_north == 1 && gyp == p.ny + 2) up = -up;
                }
                // the face as a cell with east vector (eX, eY) sees it
                auto face = [&](float eX, float eY, float& H0, float& H1, float& H2) {
                    const float upe = up * eX + vp * eY;
                    const float ume = um * eX + vm * eY;
                    const float etap =
                        fmaxf(-Hf, ebp - (S.Sy[2][j + 1][i] - p.dy * F(j + 1, i, CONST_F) * upe) * k.inv_2g);
                    const float etam = fmaxf(-Hf, ebm + (S.Sy[2][j][i] - p.dy * F(j, i, CONST_F) * ume) * k.inv_2g);
                    if (dm) {
                        H2 = k.half_g * (etap + Hf) * (etap + Hf);
                    } else if (dp) {
                        H2 = k.half_g * (etam + Hf) * (etam + Hf);
                    } else {
                        // u and v swap roles along y
                        float a0, a1, a2;
                        if (cdklm_flux(p, k, etam, Rmy, Rmx, etap, Rpy, Rpx, Hf, a0, a1, a2)) {
                            a0 = 0.f; a1 = 0.f; a2 = 0.f;
                        }
                        H0 = a0; H1 = a2; H2 = a1;
                    }
                };
                float ax, ay;
                north(i, j, ax, ay);
                face(ay, -ax, G0, G1, G2);
                if constexpr (ANGLE) {
                    float P0 = 0.f, P1 = 0.f, P2 = 0.f;
                    north(i, j + 1, ax, ay);
                    face(ay, -ax, P0, P1, P2);
                    S.Gy2[0][j][i] = P0; S.Gy2[1][j][i] = P1; S.Gy2[2][j][i] = P2;
                }
            } else if constexpr (ANGLE) {
                S.Gy2[0][j][i] = 0.f; S.Gy2[1][j][i] = 0.f; S.Gy2[2][j][i] = 0.f;
            }
            S.Gy[0][j][i] = G0; S.Gy[1][j][i] = G1; S.Gy[2][j][i] = G2;
        }
    }

    // The state of cell (i,j) that the RK combination starts from: eta,
    // the re-singularised momenta, the cell-mean depth and the water depth.
    __device__ __forceinline__ void cell_state(int i, int j, float& ec, float& hu, float& hv, float& Hm,
                                               float& hsum) const {
        ec = S.D[0][j][i];
        const float uc = S.D[1][j][i], vc = S.D[2][j][i];
        Hm = 0.25f * (S.Hi[j][i] + S.Hi[j + 1][i] + S.Hi[j][i + 1] + S.Hi[j + 1][i + 1]);
        hsum = ec + Hm;
        hu = 0.0f; hv = 0.0f;
        if (hsum > p.depth_cutoff) { hu = uc * hsum; hv = vc * hsum; }
    }

    // Right-hand side L(Q) of the cell (i,j) plus the quantities the RK
    // combination needs; K/CDKLM16_kernel.cu:739-966.
    template <bool CONST_F, bool SIMPLE_FORCING>
    __device__ void rhs(int i, int j, int gxs, int gys, float& L1, float& L2, float& L3,
                        float& ec, float& hu, float& hv, float& Hm, float& hsum) const {
        cell_state(i, j, ec, hu, hv, Hm, hsum);
        const float uc = S.D[1][j][i], vc = S.D[2][j][i];
        const float fc = F(j, i, CONST_F);
        // the west / south faces as this cell sees them: with a north-angle
        // texture the plus-cell versions of the neighbours' faces
        auto WF = [&](int c) -> float {
            if constexpr (ANGLE) return S.Fx2[c][j][i - 1]; else return S.Fx[c][j][i - 1];
        };
        auto SF = [&](int c) -> float {
            if constexpr (ANGLE) return S.Gy2[c][j - 1][i]; else return S.Gy[c][j - 1][i];
        };
        float fd0 = (S.Fx[0][j][i] - WF(0)) * k.inv_dx;
        float fd1 = (S.Fx[1][j][i] - WF(1)) * k.inv_dx;
        float fd2 = (S.Fx[2][j][i] - WF(2)) * k.inv_dx;
        if (!p.one_dimensional) {
            fd0 = fd0 + (S.Gy[0][j][i] - SF(0)) * k.inv_dy;
            fd1 = fd1 + (S.Gy[1][j][i] - SF(1)) * k.inv_dy;
            fd2 = fd2 + (S.Gy[2][j][i] - SF(2)) * k.inv_dy;
        }
        // source terms of a wet cell, evaluated on every lane; dry and land
        // cells (rare) have none
        const bool wet = hsum >= p.depth_cutoff && ec != kDryFlag;
        float st1, st2;
        {
            const float tx = (S.Sx[2][j][i] + p.dx * fc * vc) * k.inv_2g;
            const float ty = (S.Sy[2][j][i] - p.dy * fc * uc) * k.inv_2g;
            const float eta_we = 0.5f * ((ec - tx) + (ec + tx));
            const float eta_sn = 0.5f * ((ec + ty) + (ec - ty));
            const float RHxp = 0.5f * (S.Hi[j][i + 1] + S.Hi[j + 1][i + 1]);
            const float RHxm = 0.5f * (S.Hi[j][i] + S.Hi[j + 1][i]);
            const float RHyp = 0.5f * (S.Hi[j + 1][i] + S.Hi[j + 1][i + 1]);
            const float RHym = 0.5f * (S.Hi[j][i] + S.Hi[j][i + 1]);
            float nX, nY;
            north(i, j, nX, nY);
            const float eX = nY, eY = -nX;
            const float hu_e = hu * eX + hv * eY;
            const float hv_n = hu * nX + hv * nY;
            const float hu_ec = fc * hv_n;
            const float hv_nc = -fc * hu_e;
            const float upx = -nX, upy = nY;
            const float hu_cor = upy * hu_ec + (-upx) * hv_nc;
            const float hv_cor = upx * hu_ec + upy * hv_nc;
            float X, Y, ax = 0.0f, ay = 0.0f;
            if (SIMPLE_FORCING) {
                X = wind_X; Y = wind_Y;
            } else {
                const float s = ((float)gxs + 0.5f) / (float)(p.nx + 4);
                const float t = ((float)gys + 0.5f) / (float)(p.ny + 4);
                const float wxc = tex_bilinear(p.wind_x_cur, p.wind_x_nx, p.wind_x_ny, s, t);
                const float wxn = tex_bilinear(p.wind_x_next, p.wind_x_nx, p.wind_x_ny, s, t);
                const float wyc = tex_bilinear(p.wind_y_cur, p.wind_y_nx, p.wind_y_ny, s, t);
                const float wyn = tex_bilinear(p.wind_y_next, p.wind_y_nx, p.wind_y_ny, s, t);
                X = p.wind_stress_factor * (p.wind_t * wxn + (1.0f - p.wind_t) * wxc);
                Y = p.wind_stress_factor * (p.wind_t * wyn + (1.0f - p.wind_t) * wyc);
                if (p.atm_p_nx * p.atm_p_ny > 1) {
                    const float pt = p.atm_p_t;
                    const float dxn = 1.0f / (float)(p.nx + 4), dyn = 1.0f / (float)(p.ny + 4);
                    auto P = [&](float ss, float tt) {
                        const float c = tex_bilinear(p.atm_p_cur, p.atm_p_nx, p.atm_p_ny, ss, tt);
                        const float n = tex_bilinear(p.atm_p_next, p.atm_p_nx, p.atm_p_ny, ss, tt);
                        return pt * n + (1.0f - pt) * c;
                    };
                    const float pe = P(s + dxn, t), pw = P(s - dxn, t);
                    const float pn = P(s, t + dyn), ps = P(s, t - dyn);
                    ax = -(pe - pw) * hsum * k.inv_atm_x;
                    ay = -(pn - ps) * hsum * k.inv_atm_y;
                }
            }
            const float bath1 = p.g * (eta_we + Hm) * (RHxp - RHxm);
            const float bath2 = p.g * (eta_sn + Hm) * (RHyp - RHym);
            st1 = X + hu_cor + ax + bath1 * k.inv_dx;
            st2 = Y + hv_cor + ay + bath2 * k.inv_dy;
        }
        if (!wet) {
            st1 = 0.0f; st2 = 0.0f;
        }
        L1 = -fd0;
        L2 = -fd1 + st1;
        L3 = -fd2 + st2;
    }

    // Whether the semi-implicit friction term acts (the same for every cell
    // of a launch).  Without it C = 0 and the reference's division of the
    // updated momenta by 1 + C (or 1 + C / 2) is a division by one, which
    // the fused step leaves out: the approximate division (-prec-div=false)
    // returns its dividend exactly for a divisor of one.
    __device__ __forceinline__ bool has_friction() const { return p.r > 0.0f && p.rk_order < 3; }

    // Semi-implicit friction coefficient C (K/CDKLM16_kernel.cu:971-983).
    __device__ float friction(float dt, float hsum, float hu, float hv) const {
        if (!(p.r > 0.0f) || p.rk_order >= 3) return 0.0f;
        if (hsum < p.desing_eps) {
            const float u = desing(hsum, hu, p.desing_eps);
            const float v = desing(hsum, hv, p.desing_eps);
            return dt * p.r * desing(hsum, sqrtf(u * u + v * v), p.desing_eps);
        }
        const float u = hu / hsum, v = hv / hsum;
        return dt * p.r * sqrtf(u * u + v * v) / hsum;
    }
};

// Final clamp of an updated state (K/CDKLM16_kernel.cu:1069-1088).
__device__ __forceinline__ void finish_cell(const GocCdklmParams& p, float Hm, float& e, float& hu, float& hv) {
    if (e + Hm <= p.depth_cutoff) {
        e = -Hm + p.depth_cutoff; hu = 0.0f; hv = 0.0f;
    }
    e = fmaxf(-Hm + p.depth_cutoff, e);
}

__device__ __forceinline__ void store_with_images(const GocCdklmParams& p, const StepConst& k, float* e_out,
                                                  float* hu_out, float* hv_out, int pitch, int gx, int gy,
                                                  float e, float hu, float hv) {
    int xs[2] = {gx, -1}, ys[2] = {gy, -1};
    if (k.periodic_x) {
        if (gx < 4) xs[1] = gx + p.nx;
        else if (gx >= p.nx) xs[1] = gx - p.nx;
    }
    if (k.periodic_y) {
        if (gy < 4) ys[1] = gy + p.ny;
        else if (gy >= p.ny) ys[1] = gy - p.ny;
    }
#pragma unroll
    for (int a = 0; a < 2; ++a) {
        if (ys[a] < 0) continue;
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            if (xs[b] < 0) continue;
            const size_t o = (size_t)ys[a] * pitch + xs[b];
            e_out[o] = e; hu_out[o] = hu; hv_out[o] = hv;
        }
    }
}

// Model error fused into the step (ensemble launches that perturb): the
// SOAR coarse field of the member (already computed for this block) is
// up-sampled on the tile and its balanced perturbation is added to
// Q^{n+1} before the write, the work of the stand-alone transfer kernel
// (noise_transfer.cu) without its read-modify-write pass.  With `spare`,
// the unperturbed Q^{n+1} is also written there (interior cells and
// periodic images), for the drifters of the block's last step, which move
// with the state before the model error.
struct TileNoise {
    const GocNoiseDesc* d;          // the member's descriptor (shared memory)
    float* spare_e; float* spare_u; float* spare_v;   // unperturbed copy, or null
};

// Launch constants of a parameter set.
// IEEE division on host and device alike, so that launch constants do not
// depend on where they were derived (device code is built with
// -prec-div=false).
__host__ __device__ inline float exact_div(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}

__host__ __device__ inline StepConst make_step_const(const GocCdklmParams& p) {
    StepConst k;
    k.inv_dx = exact_div(1.0f, p.dx);
    k.inv_dy = exact_div(1.0f, p.dy);
    k.inv_2g = exact_div(1.0f, 2.0f * p.g);
    k.half_g = 0.5f * p.g;
    k.two_g = 2.0f * p.g;
    k.theta_g = p.theta * p.g;
    k.Vc = exact_div(p.dx, 2.0f * p.g);
    k.Uc = exact_div(p.dy, 2.0f * p.g);
    k.inv_atm_x = exact_div(1.0f, 2.0f * p.dx * p.rho_o);
    k.inv_atm_y = exact_div(1.0f, 2.0f * p.dy * p.rho_o);
    k.periodic_x = (p.bc_east == 2);
    k.periodic_y = (p.bc_north == 2);
    // 1 for every valid grid, from a run-time value so that the device
    // compiler cannot treat it as a constant
    k.one = p.nx >= 0 ? 1.0f : -1.0f;
    k.one2 = make_float2(k.one, k.one);
    k.none2 = make_float2(-k.one, -k.one);
    k.quarter2 = make_float2(0.25f, 0.25f);
    k.half2 = make_float2(0.5f, 0.5f);
    k.theta2 = make_float2(p.theta, p.theta);
    k.theta_g2 = make_float2(k.theta_g, k.theta_g);
    k.half_g2 = make_float2(k.half_g, k.half_g);
    k.g2 = make_float2(p.g, p.g);
    k.Vc2 = make_float2(k.Vc, k.Vc);
    k.Uc2 = make_float2(k.Uc, k.Uc);
    return k;
}

// One output tile (tile_x, tile_y) of one stage (NSTAGE = 1) or of a full
// fused RK2 step (NSTAGE = 2).  Called by the single-simulator kernel and by
// the persistent ensemble kernel; the caller synchronises the block before
// the shared memory is reused.
// Rows of stage-1 results a tile of a column strip hands to the next tile of
// the strip (TY rows further north): the tile's local rows [H - 6, H - 2) are
// the next tile's rows [2, 6).
constexpr int kHandRows = 4;

// Copy kHandRows consecutive rows of each of the three state planes (width
// W, plane strides dst_plane / src_plane floats) between a tile's planes and
// a packed hand-over buffer [3][kHandRows][W].  The rows of one plane are
// contiguous, so with W and H even every block starts on a 16-byte boundary
// and moves as float4.  Items are taken from the last thread down: the first
// warps carry the extra items of the loops the copy runs beside.
template <int W, int H, int NT>
__device__ __forceinline__ void copy_hand_rows(float* dst, int dst_plane, const float* src, int src_plane) {
    constexpr int NH = kHandRows * W;
    if constexpr (W % 2 == 0 && H % 2 == 0) {
        constexpr int N4 = NH / 4;
        for (int q = NT - 1 - (int)threadIdx.x; q < 3 * N4; q += NT) {
            const int c = q / N4, r = q - c * N4;
            reinterpret_cast<float4*>(dst + c * dst_plane)[r] = reinterpret_cast<const float4*>(src + c * src_plane)[r];
        }
    } else {
        for (int q = NT - 1 - (int)threadIdx.x; q < 3 * NH; q += NT) {
            const int c = q / NH, r = q - c * NH;
            dst[c * dst_plane + r] = src[c * src_plane + r];
        }
    }
}

// s1: first local row of the stage-1 region the body computes (2: all of it;
// 6: the rows [2, 6) come from `side_in`, the previous tile of the strip).
// side_out (if not null) receives the stage-1 rows the next tile of the strip
// reuses.  Only the RK2 fused path (NSTAGE = 2) streams.  s1 is a run-time
// value so that one instantiation serves both kinds of tile (the kernel's
// code stays within the instruction cache).
// p: the scalar parameters the stage loops read; pm: the member's own
// parameters, whose texture pointers the tile's set-up reads (the same
// object for a single simulator; for an ensemble whose members share their
// scalars, p can then live in the kernel's parameter space, where the loops
// read it as instruction operands instead of shared-memory loads).
template <int TX, int TY, int NSTAGE, int NT, bool CONST_F, bool SIMPLE_FORCING, bool BORDER, bool NOISE = false,
          bool ANGLE = false>
__device__ __forceinline__ bool cdklm_tile_body(const GocCdklmParams& p, const GocCdklmParams& pm,
                                                const StepConst& k, float dt, int rk_step,
                                                int tile_x, int tile_y,
                                                const float* __restrict__ e_in, const float* __restrict__ hu_in,
                                                const float* __restrict__ hv_in, float* e_out, float* hu_out,
                                                float* hv_out, float* e_alt, float* hu_alt, float* hv_alt, int pitch,
                                                const float* __restrict__ Hi_g, int hi_pitch,
                                                const float* __restrict__ Hm_g, int hm_pitch, float* smem_raw,
                                                int s1 = 2, const float* side_in = nullptr,
                                                float* side_out = nullptr, TileTma* tma = nullptr,
                                                const TileNoise* nz = nullptr) {
    constexpr int HALO = 2 * NSTAGE;
    constexpr int W = TX + 2 * HALO, H = TY + 2 * HALO;
    static_assert(!ANGLE || NSTAGE == 1, "a north-angle texture is stepped stage by stage");
    using SMT = std::conditional_t<ANGLE, TileSmemAngle<W, H>, TileSmem<W, H>>;
    SMT& S = *reinterpret_cast<SMT*>(smem_raw);

    Tile<W, H, NT, BORDER, SMT, ANGLE> T{S, p, k, 2 + tile_x * TX - HALO, 2 + tile_y * TY - HALO, 0.f, 1.f, 0.f, 0.f,
                                         0.f};
    {
        // uniform one-value textures are read once per thread; the north
        // vector with the fast sine / cosine getNorth uses (K/CDKLM16_kernel.cu:78)
        const float a = __ldg(pm.angle);
        T.nX = __sinf(a);
        T.nY = __cosf(a);
        if (CONST_F) T.f0 = __ldg(pm.coriolis_f);
        if (SIMPLE_FORCING) {
            const float wt = pm.wind_t;
            T.wind_X = pm.wind_stress_factor * (wt * __ldg(pm.wind_x_next) + (1.0f - wt) * __ldg(pm.wind_x_cur));
            T.wind_Y = pm.wind_stress_factor * (wt * __ldg(pm.wind_y_next) + (1.0f - wt) * __ldg(pm.wind_y_cur));
        }
    }
    const int nx = p.nx, ny = p.ny;
    const bool px = k.periodic_x, py = k.periodic_y;

    // A tile whose first stage-1 rows come from the previous tile of its
    // strip (s1 = 6) reads its halo's south rows only in part: stage 1 reads
    // Q^n from row 4 on (rows [2, 6) then take the handed-over stage-1
    // values), stage 2's south-most y slopes read corner-depth rows from 3 on
    // and Coriolis rows (with a per-cell Coriolis f) from 2 on.  All fields
    // are loaded from row 2 on (the rows below are not loaded): one row start
    // for every field costs less than a test per cell and field.
    const int r0 = (NSTAGE == 2 && s1 != 2) ? 2 : 0;

    // Q^n of an interior tile may have been staged by TMA into the planes
    // Sx[0], Sx[1], Sy[0] (box from column x0 - 2: TMA boxes start on 16-byte
    // boundaries): wait for it.  Every thread waits (each thus sees the
    // copy's writes) and the CTA uses the staged tile only if all of them saw
    // it land.  A wait that runs out sets the error flag the host reads and
    // stops the CTA's staging; the tile then loads Q^n itself, once the late
    // copy has landed (a second bounded wait) so that it cannot overwrite the
    // planes afterwards.  If it never lands the CTA gives up (returns false).
    bool staged = false;
    if (!BORDER && tma && tma->staged) {
        staged = __syncthreads_and(mbar_wait_bounded(tma->bar, tma->phase, kTmaWaitLimitNs)) != 0;
        if (!staged) {
            if (threadIdx.x == 0) {
                *tma->off = 1;
                atomicExch(tma->err, 1);
            }
            if (!__syncthreads_and(mbar_wait_bounded(tma->bar, tma->phase, kTmaWaitLimitNs))) return false;
        }
        tma->phase ^= 1u;
    }
    // staged depth and Coriolis boxes (launches whose last phase does not
    // use their planes as model-error scratch)
    const bool aux = staged && tma->aux;
    const bool aux_f = aux && tma->aux_coriolis;
    // field c of local cell (i, j) from its staged boxes: the main box holds
    // columns from x0 - 2 (plane column i + 2), the east box the last two
    auto staged_at = [&](const float (&P)[H][W], int c, int i, int j) -> float {
        const bool east = i >= W - 2;
        const float* a = east ? tma->edge + (c * H + j) * 4 + (i - (W - 2)) : &P[j][i + 2];
        return *a;
    };

    // 2. Q^n with wall mirrors and periodic images, desingularised with the
    //    cell-mean depth of the (unmirrored) cell (K/CDKLM16_kernel.cu:614-656)
    //    One loop over the cells from row r0 also loads each cell's corner
    //    depth (land marked with the dry flag, K/CDKLM16_kernel.cu:571-587)
    //    and Coriolis f.
    for (int idx = threadIdx.x; idx < (H - r0) * W; idx += NT) {
        const int i = idx % W, j = r0 + idx / W;
        {
            const int gc = T.x0 + i, gr = T.y0 + j;
            const int cc = !BORDER ? gc : px ? wrap_interior(gc, nx) : clampi(gc, 0, nx + 4);
            const int cr = !BORDER ? gr : py ? wrap_interior(gr, ny) : clampi(gr, 0, ny + 4);
            float v = __ldg(Hi_g + (size_t)cr * hi_pitch + cc);
            if (fabsf(v - p.land_value) < kDryEps) v = kDryFlag;
            S.Hi[j][i] = v;
        }
        int gx = T.x0 + i, gy = T.y0 + j;
        int mx = gx, my = gy;
        float su = 1.0f, sv = 1.0f;
        if (BORDER) {
            if (px) gx = wrap_interior(gx, nx);
            if (py) gy = wrap_interior(gy, ny);
            const bool inx = (gx >= 2 && gx < nx + 2), iny = (gy >= 2 && gy < ny + 2);
            mx = gx;
            my = gy;
            if (iny) {
                if (p.bc_east == 1 && (gx == nx + 2 || gx == nx + 3)) { mx = 2 * nx + 3 - gx; su = -1.0f; }
                if (p.bc_west == 1 && (gx == 0 || gx == 1)) { mx = 3 - gx; su = -1.0f; }
            }
            if (inx) {
                if (p.bc_north == 1 && (gy == ny + 2 || gy == ny + 3)) { my = 2 * ny + 3 - gy; sv = -1.0f; }
                if (p.bc_south == 1 && (gy == 0 || gy == 1)) { my = 3 - gy; sv = -1.0f; }
            }
            mx = clampi(mx, 0, nx + 3);
            my = clampi(my, 0, ny + 3);
            gx = clampi(gx, 0, nx + 3);
            gy = clampi(gy, 0, ny + 3);
        }
        {
            float e, hu, hv, hmb;
            if (!BORDER && staged) {
                e = staged_at(S.Sx[0], 0, i, j);
                hu = staged_at(S.Sx[1], 1, i, j);
                hv = staged_at(S.Sy[0], 2, i, j);
            } else {
                const size_t o = (size_t)my * pitch + mx;
                e = __ldg(e_in + o);
                hu = su * __ldg(hu_in + o);
                hv = sv * __ldg(hv_in + o);
            }
            if (!BORDER && aux) {
                hmb = staged_at(S.Hmb, 3, i, j);
            } else {
                hmb = __ldg(Hm_g + (size_t)gy * hm_pitch + gx);
                if (i < W - 2) S.Hmb[j][i + 2] = hmb;
            }
            float oe, ou, ov;
            desingularize_cell(p, e, hu, hv, hmb, oe, ou, ov);
            S.D[0][j][i] = oe; S.D[1][j][i] = ou; S.D[2][j][i] = ov;
        }
        if (!CONST_F) {
            if (!BORDER && aux_f) {
                S.Fc[j][i] = staged_at(S.Sy[1], 4, i, j);
            } else if (pm.coriolis_cell) {
                S.Fc[j][i] = __ldg(pm.coriolis_cell + (size_t)gy * (pm.coriolis_cell_pitch / 4) + gx);
            } else {
                const int fx = (BORDER && !px) ? T.x0 + i : gx, fy = (BORDER && !py) ? T.y0 + j : gy;
                const float s = (fx + 0.5f) / (nx + 4.0f);
                const float t = (fy + 0.5f) / (ny + 4.0f);
                S.Fc[j][i] = tex_bilinear(pm.coriolis_f, pm.coriolis_nx, pm.coriolis_ny, s, t);
            }
        }
    }
    __syncthreads();

    if (NSTAGE == 2) {
        // ---- stage 1 on the tile + 2 cells (rows from s1) ----
        T.template slopes<2, W - 2, 2, H - 2, CONST_F>(s1 - 2);
        __syncthreads();
        T.template faces<2, W - 2, 2, H - 2, CONST_F>(s1 - 2);
        __syncthreads();
        const int nu = (W - 4) * (H - 2 - s1);
        // The update of a cell reads D^n of that cell only (its neighbours
        // enter through the flux and slope planes), so each result is
        // desingularised into D* at once; the wall mirrors write ghost cells,
        // whose own update is skipped.  A rolled loop keeps one copy of the
        // cell update in the kernel (the step is sensitive to the instruction
        // cache).  The previous tile's stage-1 rows become this tile's rows
        // [2, 6) meanwhile: the update neither reads nor writes them (its
        // rows start at s1 = 6 and read the state planes at their own cell).
        if (s1 != 2) copy_hand_rows<W, H, NT>(&S.D[0][2][0], H * W, side_in, kHandRows * W);
        for (int idx = threadIdx.x; idx < nu; idx += NT) {
            int i, j;
            block_cell<W - 4>(idx, H - 2 - s1, i, j);
            i += 2; j += s1;
            int gx = T.x0 + i, gy = T.y0 + j;
            const int gxs = (BORDER && px) ? wrap_interior(gx, nx) : gx;
            const int gys = (BORDER && py) ? wrap_interior(gy, ny) : gy;
            const bool ok = !BORDER || ((px || (gx >= 2 && gx < nx + 2)) && (py || (gy >= 2 && gy < ny + 2)));
            if (!ok) continue;
            float L1, L2, L3, ec, hu, hv, Hm, hsum;
            T.template rhs<CONST_F, SIMPLE_FORCING>(i, j, gxs, gys, L1, L2, L3, ec, hu, hv, Hm, hsum);
            float qe = ec + dt * L1;
            float qu = hu + dt * L2;
            float qv = hv + dt * L3;
            if (T.has_friction()) {
                const float C = T.friction(dt, hsum, hu, hv);
                qu = qu / (1.0f + C);
                qv = qv / (1.0f + C);
            }
            finish_cell(p, Hm, qe, qu, qv);
            // the first-stage state of the tile's own cells, when asked for
            // (the adjoint's second-stage VJP reads it)
            if (e_alt && i >= HALO && i < HALO + TX && j >= HALO && j < HALO + TY && gx < nx + 2 && gy < ny + 2) {
                const size_t os = (size_t)gy * pitch + gx;
                e_alt[os] = qe; hu_alt[os] = qu; hv_alt[os] = qv;
            }
            float oe, ou, ov;
            desingularize_cell(p, qe, qu, qv, S.Hmb[j][i + 2], oe, ou, ov);
            S.D[0][j][i] = oe; S.D[1][j][i] = ou; S.D[2][j][i] = ov;
            if (BORDER) {
                // wall ghosts of the stage result (K/CDKLM16_kernel.cu:420-470)
                auto mirror = [&](int ii, int jj, float me0, float mu0, float mv0) {
                    if (ii < 2 || ii >= W - 2 || jj < 2 || jj >= H - 2) return;
                    float me, mu, mv;
                    desingularize_cell(p, me0, mu0, mv0, S.Hmb[jj][ii + 2], me, mu, mv);
                    S.D[0][jj][ii] = me; S.D[1][jj][ii] = mu; S.D[2][jj][ii] = mv;
                };
                if (p.bc_north == 1) {
                    if (gys == ny + 1) mirror(i, j + 1, qe, qu, -qv);
                    if (gys == ny) mirror(i, j + 3, qe, qu, -qv);
                }
                if (p.bc_south == 1) {
                    if (gys == 2) mirror(i, j - 1, qe, qu, -qv);
                    if (gys == 3) mirror(i, j - 3, qe, qu, -qv);
                }
                if (p.bc_east == 1) {
                    if (gxs == nx + 1) mirror(i + 1, j, qe, -qu, qv);
                    if (gxs == nx) mirror(i + 3, j, qe, -qu, qv);
                }
                if (p.bc_west == 1) {
                    if (gxs == 2) mirror(i - 1, j, qe, -qu, qv);
                    if (gxs == 3) mirror(i - 3, j, qe, -qu, qv);
                }
            }
        }
        __syncthreads();
        // this tile's stage-1 rows [H - 6, H - 2) for the next tile of the
        // strip, beside the slopes below (which only read the state planes)
        if (side_out) copy_hand_rows<W, H, NT>(side_out, kHandRows * W, &S.D[0][H - 2 - kHandRows][0], H * W);
        // ---- stage 2 on the tile ----
        T.template slopes<4, W - 4, 4, H - 4, CONST_F>();
        __syncthreads();
        T.template faces<4, W - 4, 4, H - 4, CONST_F>();
        __syncthreads();
        // the last phase reads neither Sx[0..1] nor Sy[0..1]: stage the next
        // tile of the strip there meanwhile
        if (tma && tma->next_tile_y >= 0 && threadIdx.x == 0 && *tma->off == 0)
            tma_stage_tile<W, H>(*tma, S, T.x0 - 2, 2 + tma->next_tile_y * TY - HALO, tma->next_aux);
        // model error: the eta perturbation on the tile + 1 ring, into Sy[1]
        // (dead after the faces; the staging above does not touch it), with
        // the cell-mean depths' plane (dead since stage 1) as scratch
        constexpr int DW = TX + 2, DH = TY + 2;
        float* de = &S.Sy[1][0][0];
        if constexpr (NOISE) {
            if (nz) {
                noise_tile_field<DW, DH, NT>(*nz->d, p.dx, p.dy, T.x0 + HALO - 1, T.y0 + HALO - 1, de,
                                             &S.Hmb[0][0], W * H, threadIdx.x);
                __syncthreads();
            }
        }
        // A rolled loop keeps one copy of the cell update; Q^n of the cell is
        // loaded first, so its latency overlaps the update.
        for (int idx = threadIdx.x; idx < TX * TY; idx += NT) {
            const int i = 4 + idx % TX, j = 4 + idx / TX;
            const int gx = T.x0 + i, gy = T.y0 + j;
            if (BORDER && (gx >= nx + 2 || gy >= ny + 2)) continue;
            const size_t o = (size_t)gy * pitch + gx;
            const float ea = __ldg(e_in + o), hua = __ldg(hu_in + o), hva = __ldg(hv_in + o);
            float L1, L2, L3, ec, hu, hv, Hm, hsum;
            T.template rhs<CONST_F, SIMPLE_FORCING>(i, j, gx, gy, L1, L2, L3, ec, hu, hv, Hm, hsum);
            float ne = 0.5f * (ea + (ec + dt * L1));
            float nhu = 0.5f * (hua + (hu + dt * L2));
            float nhv = 0.5f * (hva + (hv + dt * L3));
            if (T.has_friction()) {
                const float C = T.friction(dt, hsum, hu, hv);
                nhu = nhu / (1.0f + 0.5f * C);
                nhv = nhv / (1.0f + 0.5f * C);
            }
            finish_cell(p, Hm, ne, nhu, nhv);
            if constexpr (NOISE) {
                if (nz) {
                    if (nz->spare_e) {
                        if (BORDER) {
                            store_with_images(p, k, nz->spare_e, nz->spare_u, nz->spare_v, pitch, gx, gy, ne, nhu,
                                              nhv);
                        } else {
                            nz->spare_e[o] = ne; nz->spare_u[o] = nhu; nz->spare_v[o] = nhv;
                        }
                    }
                    // the cell's corner depths from the tile's plane (land
                    // corners hold the dry flag there)
                    const float hc[4] = {S.Hi[j][i], S.Hi[j][i + 1], S.Hi[j + 1][i], S.Hi[j + 1][i + 1]};
                    const int ox = T.x0 + HALO - 1, oy = T.y0 + HALO - 1;
                    perturbed_state(*nz->d, nx, ny, p.dx, p.dy, kDryFlag, gx, gy, nz->d->interpolation_factor <= 1,
                                    [&](int jj, int ii) { return de[(jj - oy) * DW + (ii - ox)]; }, ne, nhu, nhv, hc);
                }
            }
            if (BORDER) {
                store_with_images(p, k, e_out, hu_out, hv_out, pitch, gx, gy, ne, nhu, nhv);
            } else {
                e_out[o] = ne; hu_out[o] = nhu; hv_out[o] = nhv;
            }
        }
    } else {
        // ---- one stage with the reference's buffer semantics ----
        T.template slopes<2, W - 2, 2, H - 2, CONST_F>();
        __syncthreads();
        T.template faces<2, W - 2, 2, H - 2, CONST_F>();
        __syncthreads();
        for (int idx = threadIdx.x; idx < TX * TY; idx += NT) {
            const int i = 2 + idx % TX, j = 2 + idx / TX;
            const int gx = T.x0 + i, gy = T.y0 + j;
            if (BORDER && (gx >= nx + 2 || gy >= ny + 2)) continue;
            float L1, L2, L3, ec, hu, hv, Hm, hsum;
            T.template rhs<CONST_F, SIMPLE_FORCING>(i, j, gx, gy, L1, L2, L3, ec, hu, hv, Hm, hsum);
            const size_t o = (size_t)gy * pitch + gx;
            float ne, nhu, nhv;
            float* de = e_out; float* du = hu_out; float* dv = hv_out;
            if (p.rk_order < 3) {
                const float C = T.friction(dt, hsum, hu, hv);
                if (rk_step == 0) {
                    ne = ec + dt * L1;
                    nhu = (hu + dt * L2) / (1.0f + C);
                    nhv = (hv + dt * L3) / (1.0f + C);
                } else {
                    ne = 0.5f * (e_out[o] + (ec + dt * L1));
                    nhu = 0.5f * (hu_out[o] + (hu + dt * L2)) / (1.0f + 0.5f * C);
                    nhv = 0.5f * (hv_out[o] + (hv + dt * L3)) / (1.0f + 0.5f * C);
                }
            } else {
                if (rk_step == 0) {
                    ne = ec + dt * L1; nhu = hu + dt * L2; nhv = hv + dt * L3;
                } else if (rk_step == 1) {
                    ne = 0.75f * e_out[o] + 0.25f * (ec + dt * L1);
                    nhu = 0.75f * hu_out[o] + 0.25f * (hu + dt * L2);
                    nhv = 0.75f * hv_out[o] + 0.25f * (hv + dt * L3);
                    de = e_alt; du = hu_alt; dv = hv_alt;
                } else {
                    ne = (e_out[o] + 2.0f * (ec + dt * L1)) / 3.0f;
                    nhu = (hu_out[o] + 2.0f * (hu + dt * L2)) / 3.0f;
                    nhv = (hv_out[o] + 2.0f * (hv + dt * L3)) / 3.0f;
                }
            }
            finish_cell(p, Hm, ne, nhu, nhv);
            de[o] = ne; du[o] = nhu; dv[o] = nhv;
        }
    }
    return true;
}

// A tile needs the boundary logic (periodic wrap, wall mirrors, clamping,
// periodic ghost images of the output) when its staged region reaches
// outside the interior.
template <int TX, int TY, int NSTAGE>
__device__ __forceinline__ bool tile_on_border(const GocCdklmParams& p, int tile_x, int tile_y) {
    constexpr int HALO = 2 * NSTAGE;
    const int x0 = 2 + tile_x * TX - HALO, y0 = 2 + tile_y * TY - HALO;
    return x0 < 2 || y0 < 2 || x0 + TX + 2 * HALO > p.nx + 2 || y0 + TY + 2 * HALO > p.ny + 2;
}

template <int TX, int TY, int NSTAGE, int NT, bool CONST_F, bool SIMPLE_FORCING, bool ANGLE = false>
__device__ __forceinline__ void cdklm_tile(const GocCdklmParams& p, const StepConst& k, float dt, int rk_step,
                                           int tile_x, int tile_y,
                                           const float* __restrict__ e_in, const float* __restrict__ hu_in,
                                           const float* __restrict__ hv_in, float* e_out, float* hu_out,
                                           float* hv_out, float* e_alt, float* hu_alt, float* hv_alt, int pitch,
                                           const float* __restrict__ Hi_g, int hi_pitch,
                                           const float* __restrict__ Hm_g, int hm_pitch, float* smem_raw) {
    if (tile_on_border<TX, TY, NSTAGE>(p, tile_x, tile_y))
        cdklm_tile_body<TX, TY, NSTAGE, NT, CONST_F, SIMPLE_FORCING, true, false, ANGLE>(
            p, p, k, dt, rk_step, tile_x, tile_y, e_in, hu_in, hv_in, e_out, hu_out, hv_out, e_alt, hu_alt, hv_alt,
            pitch, Hi_g, hi_pitch, Hm_g, hm_pitch, smem_raw);
    else
        cdklm_tile_body<TX, TY, NSTAGE, NT, CONST_F, SIMPLE_FORCING, false, false, ANGLE>(
            p, p, k, dt, rk_step, tile_x, tile_y, e_in, hu_in, hv_in, e_out, hu_out, hv_out, e_alt, hu_alt, hv_alt,
            pitch, Hi_g, hi_pitch, Hm_g, hm_pitch, smem_raw);
}

// Tile `tile_y` of the column strip `tile_x` in a run of consecutive tiles
// of one strip (fused RK2): reuse = the previous tile of the run handed over
// its last stage-1 rows through side_in; side_out (or null for the run's last
// tile) receives this tile's.  Returns false when the CTA has to give up (a
// TMA copy of its input that never landed).  A tile whose staged rows reach outside the
// interior rows computes all of its stage-1 rows: the north/south wall
// mirrors of its first rows land in rows it does not take over.  East/west
// borders keep the hand-over (their mirrors stay within a row).
template <int TX, int TY, int NT, bool CONST_F, bool SIMPLE_FORCING, bool NOISE = false>
__device__ __forceinline__ bool cdklm_strip_tile(const GocCdklmParams& p, const GocCdklmParams& pm,
                                                 const StepConst& k, float dt, int tile_x,
                                                 int tile_y, bool reuse, const float* __restrict__ e_in,
                                                 const float* __restrict__ hu_in, const float* __restrict__ hv_in,
                                                 float* e_out, float* hu_out, float* hv_out, int pitch,
                                                 const float* __restrict__ Hi_g, int hi_pitch,
                                                 const float* __restrict__ Hm_g, int hm_pitch, float* smem_raw,
                                                 const float* side_in, float* side_out, TileTma* tma,
                                                 const TileNoise* nz = nullptr) {
    const bool border = tile_on_border<TX, TY, 2>(p, tile_x, tile_y);
    const int y0 = 2 + tile_y * TY - 4;
    const int s1 = (reuse && y0 >= 2 && y0 + TY + 8 <= p.ny + 2) ? 2 + kHandRows : 2;
    if (border)
        return cdklm_tile_body<TX, TY, 2, NT, CONST_F, SIMPLE_FORCING, true, NOISE>(
            p, pm, k, dt, 1, tile_x, tile_y, e_in, hu_in, hv_in, e_out, hu_out, hv_out, nullptr, nullptr, nullptr,
            pitch, Hi_g, hi_pitch, Hm_g, hm_pitch, smem_raw, s1, side_in, side_out, tma, nz);
    return cdklm_tile_body<TX, TY, 2, NT, CONST_F, SIMPLE_FORCING, false, NOISE>(
        p, pm, k, dt, 1, tile_x, tile_y, e_in, hu_in, hv_in, e_out, hu_out, hv_out, nullptr, nullptr, nullptr,
        pitch, Hi_g, hi_pitch, Hm_g, hm_pitch, smem_raw, s1, side_in, side_out, tma, nz);
}

template <int TX, int TY, int NSTAGE, int NT, bool CONST_F, bool SIMPLE_FORCING, bool ANGLE = false>
__global__ void __launch_bounds__(NT, ANGLE ? 2 : 3)
cdklm_tile_kernel(const GocCdklmParams p, const StepConst k, float dt, int rk_step,
                  const float* __restrict__ e_in, const float* __restrict__ hu_in,
                  const float* __restrict__ hv_in, float* e_out, float* hu_out, float* hv_out,
                  float* e_alt, float* hu_alt, float* hv_alt, int pitch,
                  const float* __restrict__ Hi_g, int hi_pitch, const float* __restrict__ Hm_g, int hm_pitch) {
    extern __shared__ __align__(16) float smem_raw[];
    cdklm_tile<TX, TY, NSTAGE, NT, CONST_F, SIMPLE_FORCING, ANGLE>(p, k, dt, rk_step, blockIdx.x, blockIdx.y, e_in,
                                                                   hu_in, hv_in, e_out, hu_out, hv_out, e_alt,
                                                                   hu_alt, hv_alt, pitch, Hi_g, hi_pitch, Hm_g,
                                                                   hm_pitch, smem_raw);
}

// Output tile of the step kernels and threads per CTA.
constexpr int kTX = 32, kTY = 16, kNT = 256;

// Host-side validation of a parameter set (shared by all entry points).
// allow_open: open (sponge) boundaries, flags 3 and 4, whose ghost cells the
// stage reads as stored - only the single-stage entry takes them, since the
// sponge kernels act between the stages.
// allow_angle: a north-angle texture (more than one value), which only the
// single-stage entry steps.
inline int validate_params(const GocCdklmParams* p, const char* who, bool allow_open = false,
                           bool allow_angle = false) {
    if (!p) return set_error(GOC_ERR_ARG, "%s: null params", who);
    if (p->nx < 1 || p->ny < 1) return set_error(GOC_ERR_ARG, "%s: nx, ny must be >= 1 (got %d, %d)", who, p->nx, p->ny);
    if (!(p->dx > 0.0f) || !(p->dy > 0.0f) || !(p->g > 0.0f))
        return set_error(GOC_ERR_ARG, "%s: dx, dy, g must be positive", who);
    if (p->rk_order < 1 || p->rk_order > 3) return set_error(GOC_ERR_ARG, "%s: rk_order must be 1, 2 or 3", who);
    if (p->rk_order == 3 && p->r != 0.0f)
        return set_error(GOC_ERR_ARG, "%s: 3rd order Runge Kutta supported only without friction", who);
    const int b[4] = {p->bc_north, p->bc_east, p->bc_south, p->bc_west};
    for (int i = 0; i < 4; ++i)
        if (b[i] != 1 && b[i] != 2 && !(allow_open && (b[i] == 3 || b[i] == 4)))
            return set_error(GOC_ERR_UNSUPPORTED, "%s: boundary flag %d not supported here (1 = wall, 2 = periodic%s)",
                             who, b[i], allow_open ? ", 3, 4 = sponge" : "; sponges need the single-stage entry");
    if ((p->bc_north == 2) != (p->bc_south == 2) || (p->bc_east == 2) != (p->bc_west == 2))
        return set_error(GOC_ERR_ARG, "%s: periodic boundaries must come in opposite pairs", who);
    if (!p->coriolis_f || p->coriolis_nx < 1 || p->coriolis_ny < 1)
        return set_error(GOC_ERR_ARG, "%s: Coriolis texture missing", who);
    if (!p->angle || p->angle_nx < 1 || p->angle_ny < 1)
        return set_error(GOC_ERR_ARG, "%s: angle texture missing", who);
    if (!allow_angle && (p->angle_nx != 1 || p->angle_ny != 1))
        return set_error(GOC_ERR_UNSUPPORTED,
                         "%s: a north-angle texture is stepped stage by stage (goc_cdklm_stage); this entry takes a "
                         "constant (1x1) angle", who);
    if (!p->wind_x_cur || !p->wind_x_next || !p->wind_y_cur || !p->wind_y_next ||
        p->wind_x_nx < 1 || p->wind_x_ny < 1 || p->wind_y_nx < 1 || p->wind_y_ny < 1)
        return set_error(GOC_ERR_ARG, "%s: wind stress textures missing", who);
    if (!p->atm_p_cur || !p->atm_p_next || p->atm_p_nx < 1 || p->atm_p_ny < 1)
        return set_error(GOC_ERR_ARG, "%s: atmospheric pressure textures missing", who);
    if ((p->bc_north == 2 && p->ny < 4) || (p->bc_east == 2 && p->nx < 4))
        return set_error(GOC_ERR_ARG, "%s: periodic directions need at least 4 interior cells", who);
    return GOC_OK;
}

}  // namespace goc
