// Adjoint of the CDKLM16 RK2 step: stage VJP kernels and their host entry
// points.  Built with FMA contraction (7 % fewer instructions than without):
// the forward quantities the VJP recomputes (slopes, reconstructions,
// fluxes) then differ from the forward kernel's by rounding, so where the
// forward's limiter or clamp arguments tie to the last bit the VJP may take
// the other side's subgradient.  Single-simulator and member-batched VJPs
// run one kernel and agree bit for bit.
#include <cstdio>
#include <type_traits>

#include "cdklm_adjoint.cuh"

namespace goc {

constexpr int kAX = 32, kAY = 16, kANT = 256;   // x-bar tile and threads per CTA
constexpr int kAYSmall = 8;                      // tile height for grids that fill few SMs
constexpr int kAHalo = 4;

// HAS_Y: the stage output y (ye, yu, yv) is given.  The cell pass then takes
// the updated state from it instead of from the forward fluxes, and the
// forward recompute stops after the slopes (the face pass recomputes each
// flux it differentiates anyway).
template <int TX, int TY, int NT, bool CONST_F, bool BORDER, bool HAS_Y>
__device__ void stage_vjp_body(const GocCdklmParams& p, const StepConst& k, float dt, int rk_step, int tile_x,
                               int tile_y, const float* __restrict__ xe, const float* __restrict__ xu,
                               const float* __restrict__ xv, const float* __restrict__ ae,
                               const float* __restrict__ au, const float* __restrict__ av,
                               const float* __restrict__ ye, const float* __restrict__ yu,
                               const float* __restrict__ yv, const float* __restrict__ ybe, const float* __restrict__ ybu,
                               const float* __restrict__ ybv, const float* __restrict__ bbe,
                               const float* __restrict__ bbu, const float* __restrict__ bbv, float* xbe, float* xbu,
                               float* xbv, float* abe, float* abu, float* abv, int pitch,
                               const float* __restrict__ Hi_g, int hi_pitch, const float* __restrict__ Hm_g,
                               int hm_pitch, float* wind_partials, float* smem_raw) {
    constexpr int W = TX + 2 * kAHalo, H = TY + 2 * kAHalo;
    using SM = AdjSmem<W, H, !CONST_F>;
    SM& A = *reinterpret_cast<SM*>(smem_raw);
    SM& S = A;
    Tile<W, H, NT, BORDER, SM> T{S, p, k, 2 + tile_x * TX - kAHalo, 2 + tile_y * TY - kAHalo, 0.f, 1.f, 0.f, 0.f, 0.f};
    {
        const float a = __ldg(p.angle);
        T.nX = sinf(a);
        T.nY = cosf(a);
        if (CONST_F) T.f0 = __ldg(p.coriolis_f);
        const float wt = p.wind_t;
        T.wind_X = p.wind_stress_factor * (wt * __ldg(p.wind_x_next) + (1.0f - wt) * __ldg(p.wind_x_cur));
        T.wind_Y = p.wind_stress_factor * (wt * __ldg(p.wind_y_next) + (1.0f - wt) * __ldg(p.wind_y_cur));
    }
    AdjTile<W, H, NT, BORDER, !CONST_F> R{A, T, p, k};
    const int nx = p.nx, ny = p.ny;
    const bool px = k.periodic_x, py = k.periodic_y;

    // staged position -> memory cell it reads, with the wall-mirror signs
    auto source = [&](int i, int j, int& mx, int& my, int& hx, int& hy, float& su, float& sv) {
        int gx = T.x0 + i, gy = T.y0 + j;
        mx = gx; my = gy; su = 1.0f; sv = 1.0f;
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
        hx = gx; hy = gy;
    };
    // 1. x on the tile + 4, desingularised, and the corner depths (as the
    //    forward kernel); adjoint accumulators cleared
    for (int idx = threadIdx.x; idx < H * W; idx += NT) {
        const int i = idx % W, j = idx / W;
        {
            const int gc = T.x0 + i, gr = T.y0 + j;
            const int cc = !BORDER ? gc : px ? wrap_interior(gc, nx) : clampi(gc, 0, nx + 4);
            const int cr = !BORDER ? gr : py ? wrap_interior(gr, ny) : clampi(gr, 0, ny + 4);
            float v = __ldg(Hi_g + (size_t)cr * hi_pitch + cc);
            if (fabsf(v - p.land_value) < kDryEps) v = kDryFlag;
            S.Hi[j][i] = v;
        }
        int mx, my, hx, hy;
        float su, sv;
        source(i, j, mx, my, hx, hy, su, sv);
        const size_t o = (size_t)my * pitch + mx;
        const float e = __ldg(xe + o);
        const float hu = su * __ldg(xu + o);
        const float hv = sv * __ldg(xv + o);
        const float hmb = __ldg(Hm_g + (size_t)hy * hm_pitch + hx);
        float oe, ou, ov;
        desingularize_cell(p, e, hu, hv, hmb, oe, ou, ov);
        S.D[0][j][i] = oe; S.D[1][j][i] = ou; S.D[2][j][i] = ov;
        if (!CONST_F) {
            if (p.coriolis_cell) {
                S.Fc[j][i] = __ldg(p.coriolis_cell + (size_t)hy * (p.coriolis_cell_pitch / 4) + hx);
            } else {
                const int fx = (BORDER && !px) ? T.x0 + i : hx, fy = (BORDER && !py) ? T.y0 + j : hy;
                const float s = (fx + 0.5f) / (nx + 4.0f);
                const float t = (fy + 0.5f) / (ny + 4.0f);
                S.Fc[j][i] = tex_bilinear(p.coriolis_f, p.coriolis_nx, p.coriolis_ny, s, t);
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) A.Db[c][j][i] = 0.0f;
    }
    __syncthreads();

    // 2. forward recompute of the stage on the tile + 2 (without y: with the
    //    fluxes, which the cell pass needs for the updated state).  With y
    //    only the slopes the face passes read: x slopes on the tile's rows
    //    (cells two beyond it in x), y slopes on its columns
    if constexpr (HAS_Y) {
        T.template slopes_boxes<kAHalo - 2, kAHalo + TX + 2, kAHalo, kAHalo + TY, kAHalo, kAHalo + TX,
                                kAHalo - 2, kAHalo + TY + 2, CONST_F>();
        __syncthreads();
    } else {
        T.template slopes<2, W - 2, 2, H - 2, CONST_F>();
        __syncthreads();
        T.template faces<2, W - 2, 2, H - 2, CONST_F>();
        __syncthreads();
    }

    // 3. cell pass: RK combination, friction and source terms in reverse.
    //    The flux-divergence adjoints stay in registers until every cell has
    //    read the fluxes, then replace them in the Gy planes.
    float wXb = 0.0f, wYb = 0.0f;
    constexpr int NCELL = (W - 4) * (H - 4);
    constexpr int PER = (NCELL + NT - 1) / NT;
    // A rolled loop keeps one copy of the cell pass in the kernel (it is
    // sensitive to the instruction cache); fdb then lives in local memory.
    float fdb[PER][3];
#pragma unroll
    for (int r = 0; r < PER; ++r) { fdb[r][0] = 0.f; fdb[r][1] = 0.f; fdb[r][2] = 0.f; }
#pragma unroll 1
    for (int r = 0; r < PER; ++r) {
        const int idx = threadIdx.x + r * NT;
        if (idx >= NCELL) continue;
        int i, j;
        block_cell<W - 4>(idx, H - 4, i, j);
        i += 2; j += 2;
        const int gx = T.x0 + i, gy = T.y0 + j;
        const int gxs = (BORDER && px) ? wrap_interior(gx, nx) : gx;
        const int gys = (BORDER && py) ? wrap_interior(gy, ny) : gy;
        const bool ok = !BORDER || ((px || (gx >= 2 && gx < nx + 2)) && (py || (gy >= 2 && gy < ny + 2)));
        if (!ok) continue;
        const bool core = (i >= kAHalo && i < kAHalo + TX && j >= kAHalo && j < kAHalo + TY &&
                           gx < nx + 2 && gy < ny + 2);
        const size_t o = (size_t)gys * pitch + gxs;
        const float yb0 = __ldg(ybe + o), yb1 = __ldg(ybu + o), yb2 = __ldg(ybv + o);
        float L1 = 0.f, L2 = 0.f, L3 = 0.f, ec, hu, hv, Hm, hsum;
        if constexpr (HAS_Y)
            T.cell_state(i, j, ec, hu, hv, Hm, hsum);
        else
            T.template rhs<CONST_F, true>(i, j, gxs, gys, L1, L2, L3, ec, hu, hv, Hm, hsum);
        const float C = T.friction(dt, hsum, hu, hv);
        // the updated state before the final clamp, and whether the clamp
        // dried the cell.  From y: a cell the clamp dried holds exactly
        // (-Hm + cutoff, 0, 0) (finish_cell); a wet cell holds its updated
        // momenta.  (A wet cell at rest whose eta the clamp raised to the
        // same value reads as dry: a tie at the clamp's kink.)
        bool ydry = false;
        float ynu = 0.f, ynv = 0.f;
        if constexpr (HAS_Y) {
            const float ye0 = __ldg(ye + o);
            ynu = __ldg(yu + o);
            ynv = __ldg(yv + o);
            ydry = (ynu == 0.0f && ynv == 0.0f && ye0 == -Hm + p.depth_cutoff);
        }
        float nhu, nhv, ecb, hub, hvb, L1b, L2b, L3b, Cb;
        float eab = 0.f, huab = 0.f, hvab = 0.f;
        if (rk_step == 0) {
            bool dry;
            if constexpr (HAS_Y) {
                nhu = ynu; nhv = ynv; dry = ydry;
            } else {
                const float ne = ec + dt * L1;
                nhu = (hu + dt * L2) / (1.0f + C);
                nhv = (hv + dt * L3) / (1.0f + C);
                dry = (ne + Hm <= p.depth_cutoff);
            }
            if (dry) continue;
            const float ic = 1.0f / (1.0f + C);
            ecb = yb0;
            L1b = dt * yb0;
            hub = yb1 * ic;
            hvb = yb2 * ic;
            L2b = dt * hub;
            L3b = dt * hvb;
            Cb = -(yb1 * nhu + yb2 * nhv) * ic;
        } else {
            const float Dd = 1.0f + 0.5f * C;
            bool dry;
            if constexpr (HAS_Y) {
                nhu = ynu; nhv = ynv; dry = ydry;
            } else {
                const float ea = __ldg(ae + o), hua = __ldg(au + o), hva = __ldg(av + o);
                const float ne = 0.5f * (ea + (ec + dt * L1));
                nhu = 0.5f * (hua + (hu + dt * L2)) / Dd;
                nhv = 0.5f * (hva + (hv + dt * L3)) / Dd;
                dry = (ne + Hm <= p.depth_cutoff);
            }
            if (dry) {
                if (core) {
                    abe[o] = 0.0f; abu[o] = 0.0f; abv[o] = 0.0f;
                }
                continue;
            }
            const float iD = 1.0f / Dd;
            const float Bu = yb1 * iD, Bv = yb2 * iD;
            eab = 0.5f * yb0;
            ecb = 0.5f * yb0;
            L1b = 0.5f * dt * yb0;
            huab = 0.5f * Bu;
            hvab = 0.5f * Bv;
            hub = 0.5f * Bu;
            hvb = 0.5f * Bv;
            L2b = 0.5f * dt * Bu;
            L3b = 0.5f * dt * Bv;
            Cb = -0.5f * (yb1 * nhu + yb2 * nhv) * iD;
        }
        float hsb = 0.0f;
        friction_vjp(p, dt, hsum, hu, hv, Cb, hsb, hub, hvb);
        fdb[r][0] = -L1b;
        fdb[r][1] = -L2b;
        fdb[r][2] = -L3b;
        const float uc = S.D[1][j][i], vc = S.D[2][j][i];
        if (hsum >= p.depth_cutoff && ec != kDryFlag) {
            const float st1b = L2b, st2b = L3b;
            if (core) { wXb += st1b; wYb += st2b; }
            const float RHxp = 0.5f * (S.Hi[j][i + 1] + S.Hi[j + 1][i + 1]);
            const float RHxm = 0.5f * (S.Hi[j][i] + S.Hi[j + 1][i]);
            const float RHyp = 0.5f * (S.Hi[j + 1][i] + S.Hi[j + 1][i + 1]);
            const float RHym = 0.5f * (S.Hi[j][i] + S.Hi[j][i + 1]);
            ecb += st1b * k.inv_dx * p.g * (RHxp - RHxm) + st2b * k.inv_dy * p.g * (RHyp - RHym);
            const float fc = T.F(j, i, CONST_F);
            const float nX = T.nX, nY = T.nY, eX = nY, eY = -nX;
            const float hu_ecb = nY * st1b - nX * st2b;
            const float hv_ncb = nX * st1b + nY * st2b;
            const float hv_nb = fc * hu_ecb;
            const float hu_eb = -fc * hv_ncb;
            hub += eX * hu_eb + nX * hv_nb;
            hvb += eY * hu_eb + nY * hv_nb;
        }
        float ucb = 0.0f, vcb = 0.0f;
        if (hsum > p.depth_cutoff) {
            ucb = hub * hsum;
            vcb = hvb * hsum;
            hsb += hub * uc + hvb * vc;
        }
        ecb += hsb;
        A.Db[0][j][i] = ecb;
        A.Db[1][j][i] = ucb;
        A.Db[2][j][i] = vcb;
        if (rk_step == 1 && core) {
            abe[o] = eab; abu[o] = huab; abv[o] = hvab;
        }
    }
    __syncthreads();
    // the fluxes are dead: Gy takes the flux-divergence adjoints (zero outside
    // the cells of the pass), Fx the slope adjoints
    for (int idx = threadIdx.x; idx < H * W; idx += NT) {
        const int i = idx % W, j = idx / W;
#pragma unroll
        for (int c = 0; c < 3; ++c) { S.Fx[c][j][i] = 0.0f; S.Gy[c][j][i] = 0.0f; }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < PER; ++r) {
        const int idx = threadIdx.x + r * NT;
        if (idx >= NCELL) continue;
        int i, j;
        block_cell<W - 4>(idx, H - 4, i, j);
        i += 2; j += 2;
        S.Gy[0][j][i] = fdb[r][0]; S.Gy[1][j][i] = fdb[r][1]; S.Gy[2][j][i] = fdb[r][2];
    }
    __syncthreads();
    auto FDb = [&](int c) -> float (&)[H][W] { return S.Gy[c]; };

    // The reverse passes cover only what reaches the x-bar of the tile's
    // cells (and of the wall-mirror positions that fold onto them): an x face
    // or x slope changes the adjoints of its own row only, a y face or y
    // slope those of its own column.  x faces and slopes therefore run on
    // the tile's rows, y faces and slopes on its columns; along the pass
    // direction the faces reach two cells beyond the tile, the slopes one.
    // Faces between two ghost cells of a wall carry no adjoint (the cell
    // pass leaves ghost cells out), so walls need no more.
    constexpr int T0X = kAHalo, T1X = kAHalo + TX, T0Y = kAHalo, T1Y = kAHalo + TY;

    // 4. faces in reverse, two colours each.  x faces are coloured as a
    //    checkerboard ((i + j) even / odd): faces of one row never share a
    //    cell.  A warp takes 16 faces of a row and 16 of the next: the
    //    stride-2 accesses of one half-warp cover 32 consecutive floats, and
    //    the checkerboard puts the two rows on even and odd banks, so they do
    //    not conflict; the remaining faces of each row come afterwards.
    constexpr int FX0 = T0X - 2;                 // east faces of cells [T0X - 2, T1X + 1) on the tile's rows
    constexpr int NXF = TX + 3, NYF = TY;
    constexpr int FPR = (NXF + 1) / 2;          // faces of one colour per row
    constexpr int FM = FPR < 16 ? FPR : 16, FR = FPR - FM;
    constexpr int NITEM = FM == 16 ? ((NYF + 1) / 2) * 32 + FR * NYF : FPR * NYF;
#pragma unroll 1
    for (int colour = 0; colour < 2; ++colour) {
        for (int idx = threadIdx.x; idx < NITEM; idx += NT) {
            int row, kf;
            if (idx < ((NYF + 1) / 2) * 32 && FM == 16) {
                const int lane = idx & 31;
                row = 2 * (idx >> 5) + (lane >> 4);
                kf = lane & 15;
                if (row >= NYF) continue;
            } else {
                const int q = idx - (FM == 16 ? ((NYF + 1) / 2) * 32 : 0);
                if (FM != 16) {
                    row = idx / FPR; kf = idx % FPR;
                } else {
                    if (q >= FR * NYF) continue;
                    row = q / (FR > 0 ? FR : 1); kf = FM + q % (FR > 0 ? FR : 1);
                }
            }
            const int j = T0Y + row;
            const int i = FX0 + 2 * kf + ((j + colour) & 1);
            if (i >= T1X + 1) continue;
            const float F0b = (FDb(0)[j][i] - FDb(0)[j][i + 1]) * k.inv_dx;
            const float F1b = (FDb(1)[j][i] - FDb(1)[j][i + 1]) * k.inv_dx;
            const float F2b = (FDb(2)[j][i] - FDb(2)[j][i + 1]) * k.inv_dx;
            if (F0b == 0.0f && F1b == 0.0f && F2b == 0.0f) continue;
            R.template face_x_vjp<CONST_F>(i, j, F0b, F1b, F2b);
        }
        __syncthreads();
    }
    // 5. x slopes in reverse (three colours); their adjoints are complete
    //    once the x faces are done
    constexpr int NXS = TX + 2, NYS = TY;       // x slopes of cells [T0X - 1, T1X + 1) on the tile's rows
#pragma unroll 1
    for (int colour = 0; colour < 3; ++colour) {
        constexpr int PERROW = (NXS + 2) / 3;
        for (int idx = threadIdx.x; idx < PERROW * NYS; idx += NT) {
            const int i = T0X - 1 + colour + 3 * (idx % PERROW);
            const int j = T0Y + idx / PERROW;
            if (i >= T1X + 1) continue;
            R.template slope_x_vjp<CONST_F>(i, j);
        }
        __syncthreads();
    }
    // Fx is cleared again for the y-slope adjoints
    for (int idx = threadIdx.x; idx < H * W; idx += NT) {
        const int i = idx % W, j = idx / W;
#pragma unroll
        for (int c = 0; c < 3; ++c) S.Fx[c][j][i] = 0.0f;
    }
    __syncthreads();
    // 6. y faces and y slopes in reverse
    if (!p.one_dimensional) {
        constexpr int NXG = TX, NYG = TY + 3;     // north faces of rows [T0Y - 2, T1Y + 1) on the tile's columns
#pragma unroll 1
        for (int colour = 0; colour < 2; ++colour) {
            for (int idx = threadIdx.x; idx < NXG * ((NYG + 1) / 2); idx += NT) {
                const int i = T0X + idx % NXG;
                const int j = T0Y - 2 + colour + 2 * (idx / NXG);
                if (j >= T1Y + 1) continue;
                const float G0b = (FDb(0)[j][i] - FDb(0)[j + 1][i]) * k.inv_dy;
                const float G1b = (FDb(1)[j][i] - FDb(1)[j + 1][i]) * k.inv_dy;
                const float G2b = (FDb(2)[j][i] - FDb(2)[j + 1][i]) * k.inv_dy;
                if (G0b == 0.0f && G1b == 0.0f && G2b == 0.0f) continue;
                R.template face_y_vjp<CONST_F>(i, j, G0b, G1b, G2b);
            }
            __syncthreads();
        }
    }

    constexpr int NXY = TX, NYY = TY + 2;       // y slopes of rows [T0Y - 1, T1Y + 1) on the tile's columns
#pragma unroll 1
    for (int colour = 0; colour < 3; ++colour) {
        constexpr int PERCOL = (NYY + 2) / 3;
        for (int idx = threadIdx.x; idx < NXY * PERCOL; idx += NT) {
            const int i = T0X + idx % NXY;
            const int j = T0Y - 1 + colour + 3 * (idx / NXY);
            if (j >= T1Y + 1) continue;
            R.template slope_y_vjp<CONST_F>(i, j);
        }
        __syncthreads();
    }

    // 7. desingularisation in reverse at the tile's positions (border tiles:
    //    also the two rings around it, where the wall mirrors of its cells
    //    lie), as the adjoint of the memory cell each read (signs of the wall
    //    mirrors); the result per position goes to the Gy planes
    constexpr int DR = BORDER ? 2 : 0, DW = TX + 2 * DR, DH = TY + 2 * DR;
    for (int idx = threadIdx.x; idx < DW * DH; idx += NT) {
        const int i = T0X - DR + idx % DW, j = T0Y - DR + idx / DW;
        const float d0 = A.Db[0][j][i], d1 = A.Db[1][j][i], d2 = A.Db[2][j][i];
        float eb = 0.f, hub = 0.f, hvb = 0.f;
        if (d0 != 0.0f || d1 != 0.0f || d2 != 0.0f) {
            int mx, my, hx, hy;
            float su, sv;
            source(i, j, mx, my, hx, hy, su, sv);
            const size_t o = (size_t)my * pitch + mx;
            const float e = __ldg(xe + o);
            const float hu = su * __ldg(xu + o);
            const float hv = sv * __ldg(xv + o);
            const float hmb = __ldg(Hm_g + (size_t)hy * hm_pitch + hx);
            desingularize_cell_vjp(p, e, hu, hv, hmb, d0, d1, d2, eb, hub, hvb);
            hub *= su;
            hvb *= sv;
        }
        S.Gy[0][j][i] = eb; S.Gy[1][j][i] = hub; S.Gy[2][j][i] = hvb;
    }
    __syncthreads();

    // 8. x-bar of the tile's interior cells: own position plus the wall
    //    mirror positions that read it
    for (int idx = threadIdx.x; idx < TX * TY; idx += NT) {
        const int i = kAHalo + idx % TX, j = kAHalo + idx / TX;
        const int gx = T.x0 + i, gy = T.y0 + j;
        if (gx >= nx + 2 || gy >= ny + 2) continue;
        float s0 = S.Gy[0][j][i], s1 = S.Gy[1][j][i], s2 = S.Gy[2][j][i];
        if (BORDER) {
            int mi = -1;
            if (p.bc_west == 1 && (gx == 2 || gx == 3)) mi = i - (2 * gx - 3);
            if (p.bc_east == 1 && (gx == nx || gx == nx + 1)) mi = i + (2 * nx + 3 - 2 * gx);
            if (mi >= 0 && mi < W) { s0 += S.Gy[0][j][mi]; s1 += S.Gy[1][j][mi]; s2 += S.Gy[2][j][mi]; }
            int mj = -1;
            if (p.bc_south == 1 && (gy == 2 || gy == 3)) mj = j - (2 * gy - 3);
            if (p.bc_north == 1 && (gy == ny || gy == ny + 1)) mj = j + (2 * ny + 3 - 2 * gy);
            if (mj >= 0 && mj < H) { s0 += S.Gy[0][mj][i]; s1 += S.Gy[1][mj][i]; s2 += S.Gy[2][mj][i]; }
        }
        const size_t o = (size_t)gy * pitch + gx;
        if (bbe) { s0 += __ldg(bbe + o); s1 += __ldg(bbu + o); s2 += __ldg(bbv + o); }
        xbe[o] = s0; xbu[o] = s1; xbv[o] = s2;
    }

    // 9. wind-stress adjoint of the tile's cells
    if (wind_partials) {
        __shared__ float red[2][NT / 32];
        for (int off = 16; off > 0; off >>= 1) {
            wXb += __shfl_xor_sync(0xffffffffu, wXb, off);
            wYb += __shfl_xor_sync(0xffffffffu, wYb, off);
        }
        if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = wXb; red[1][threadIdx.x >> 5] = wYb; }
        __syncthreads();
        if (threadIdx.x == 0) {
            float sx = 0.f, sy = 0.f;
            for (int w = 0; w < NT / 32; ++w) { sx += red[0][w]; sy += red[1][w]; }
            // each tile owns its two slots: accumulate across calls
            const int t = tile_y * ((p.nx + TX - 1) / TX) + tile_x;
            wind_partials[2 * t] += sx;
            wind_partials[2 * t + 1] += sy;
        }
    }
}

// Tile of position q when the ntx x nty tiles are taken interior tiles first
// (the rectangle [ix0, ix1) x [iy0, iy1), row by row), then the border frame
// (the rows below and above the rectangle, then the columns beside it).
__device__ __forceinline__ void interior_first_tile(int q, int ntx, int nty, int ix0, int ix1, int iy0, int iy1,
                                                    int& tx, int& ty) {
    const int iw = ix1 - ix0, ih = iy1 - iy0;
    if (iw <= 0 || ih <= 0) {
        tx = q % ntx; ty = q / ntx;
        return;
    }
    if (q < iw * ih) {
        tx = ix0 + q % iw; ty = iy0 + q / iw;
        return;
    }
    q -= iw * ih;
    if (q < iy0 * ntx) {
        tx = q % ntx; ty = q / ntx;
        return;
    }
    q -= iy0 * ntx;
    const int nb = (nty - iy1) * ntx;
    if (q < nb) {
        tx = q % ntx; ty = iy1 + q / ntx;
        return;
    }
    q -= nb;
    const int side = ntx - iw > 0 ? ntx - iw : 1;
    const int c = q % side;
    ty = iy0 + q / side;
    tx = c < ix0 ? c : ix1 + (c - ix0);
}

// Members sharing parameters and bathymetry.  Block b works on member
// m = b % n_members at offset m * member_stride (states and adjoints),
// m * wind_stride (wind) and m * partials_stride (wind partials), on tile
// position b / n_members of the interior-first order: while the interior
// tiles of all members last, every CTA runs the interior code (the kernel is
// sensitive to the instruction cache).
template <bool CONST_F, bool HAS_Y, int TY>
__global__ void __launch_bounds__(kANT, CONST_F ? 3 : 2)
stage_vjp_members_kernel(const GocCdklmParams p, const StepConst k, float dt, int rk_step, const float* xe,
                         const float* xu, const float* xv, const float* ae, const float* au, const float* av,
                         const float* ye, const float* yu, const float* yv, const float* ybe, const float* ybu, const float* ybv, const float* bbe, const float* bbu,
                         const float* bbv, float* xbe, float* xbu, float* xbv, float* abe, float* abu, float* abv,
                         int pitch, long long member_stride, int wind_stride, const float* Hi_g, int hi_pitch,
                         const float* Hm_g, int hm_pitch, float* wind_partials, int partials_stride,
                         int n_members, int4 inner) {
    extern __shared__ __align__(16) float smem_raw[];
    const int member = (int)(blockIdx.x % (unsigned)n_members);
    int tx, ty;
    interior_first_tile((int)(blockIdx.x / (unsigned)n_members), (p.nx + kAX - 1) / kAX, (p.ny + TY - 1) / TY,
                        inner.x, inner.y, inner.z, inner.w, tx, ty);
    const size_t o = (size_t)member * (size_t)member_stride;
    GocCdklmParams pm = p;
    if (wind_stride) {
        const size_t wo = (size_t)member * wind_stride;
        pm.wind_x_cur += wo; pm.wind_x_next += wo; pm.wind_y_cur += wo; pm.wind_y_next += wo;
    }
    auto sh = [&](const float* q) { return q ? q + o : q; };
    auto shw = [&](float* q) { return q ? q + o : q; };
    float* wp = wind_partials ? wind_partials + (size_t)member * partials_stride : nullptr;
    const int x0 = 2 + tx * kAX - kAHalo, y0 = 2 + ty * TY - kAHalo;
    const bool border = x0 < 2 || y0 < 2 || x0 + kAX + 2 * kAHalo > p.nx + 2 || y0 + TY + 2 * kAHalo > p.ny + 2;
    if (border)
        stage_vjp_body<kAX, TY, kANT, CONST_F, true, HAS_Y>(
            pm, k, dt, rk_step, tx, ty, sh(xe), sh(xu), sh(xv), sh(ae), sh(au), sh(av), sh(ye), sh(yu), sh(yv),
            sh(ybe), sh(ybu), sh(ybv), sh(bbe), sh(bbu), sh(bbv), shw(xbe), shw(xbu), shw(xbv), shw(abe), shw(abu),
            shw(abv), pitch, Hi_g, hi_pitch, Hm_g, hm_pitch, wp, smem_raw);
    else
        stage_vjp_body<kAX, TY, kANT, CONST_F, false, HAS_Y>(
            pm, k, dt, rk_step, tx, ty, sh(xe), sh(xu), sh(xv), sh(ae), sh(au), sh(av), sh(ye), sh(yu), sh(yv),
            sh(ybe), sh(ybu), sh(ybv), sh(bbe), sh(bbu), sh(bbv), shw(xbe), shw(xbu), shw(xbv), shw(abe), shw(abu),
            shw(abv), pitch, Hi_g, hi_pitch, Hm_g, hm_pitch, wp, smem_raw);
}

static int vjp_check(const GocCdklmParams* p, int pitch, int Hi_pitch, int Hm_pitch, const char* who) {
    int rc = validate_params(p, who);
    if (rc) return rc;
    if (p->rk_order != 2) return set_error(GOC_ERR_UNSUPPORTED, "%s: the adjoint covers RK2 only", who);
    if (!(p->wind_x_nx == 1 && p->wind_x_ny == 1 && p->wind_y_nx == 1 && p->wind_y_ny == 1))
        return set_error(GOC_ERR_UNSUPPORTED, "%s: the adjoint needs uniform (1x1) wind stress", who);
    if (!(p->atm_p_nx == 1 && p->atm_p_ny == 1))
        return set_error(GOC_ERR_UNSUPPORTED, "%s: the adjoint does not cover atmospheric pressure fields", who);
    // a periodic image must never fall inside the tile that owns its cell
    if (p->bc_east == 2 && p->nx < kAX + 2 * kAHalo)
        return set_error(GOC_ERR_UNSUPPORTED, "%s: periodic x needs nx >= %d for the adjoint", who, kAX + 2 * kAHalo);
    if (p->bc_north == 2 && p->ny < kAY + 2 * kAHalo)
        return set_error(GOC_ERR_UNSUPPORTED, "%s: periodic y needs ny >= %d for the adjoint", who, kAY + 2 * kAHalo);
    if (pitch < (p->nx + 4) * 4 || pitch % 4 || Hm_pitch < (p->nx + 4) * 4 || Hm_pitch % 4 ||
        Hi_pitch < (p->nx + 5) * 4 || Hi_pitch % 4)
        return set_error(GOC_ERR_ARG, "%s: bad pitch", who);
    return GOC_OK;
}

// Dynamic shared memory above 48 KB is opted into once per kernel.
template <class K>
static int configure_smem(K kern, size_t smem) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return set_error(GOC_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(e));
    return GOC_OK;
}

// The buffers of one stage VJP call (device pointers; y may be null).
struct VjpBuffers {
    const float *xe, *xu, *xv, *ae, *au, *av, *ye, *yu, *yv, *ybe, *ybu, *ybv, *bbe, *bbu, *bbv;
    float *xbe, *xbu, *xbv, *abe, *abu, *abv;
};

static int vjp_args(const GocCdklmParams* p, int rk_step, const VjpBuffers& b, int pitch, int Hi_pitch,
                    int Hm_pitch, const float* Hi, const float* Hm, const char* who) {
    int rc = vjp_check(p, pitch, Hi_pitch, Hm_pitch, who);
    if (rc) return rc;
    if (rk_step != 0 && rk_step != 1) return set_error(GOC_ERR_ARG, "%s: rk_step must be 0 or 1", who);
    if (!b.xe || !b.xu || !b.xv || !b.ybe || !b.ybu || !b.ybv || !b.xbe || !b.xbu || !b.xbv || !Hi || !Hm)
        return set_error(GOC_ERR_ARG, "%s: null buffer", who);
    if (rk_step == 1 && (!b.ae || !b.au || !b.av || !b.abe || !b.abu || !b.abv))
        return set_error(GOC_ERR_ARG, "%s: the second stage needs Q^n and its adjoint output", who);
    if ((b.bbe || b.bbu || b.bbv) && !(b.bbe && b.bbu && b.bbv))
        return set_error(GOC_ERR_ARG, "%s: base must be all three arrays or none", who);
    if ((b.ye || b.yu || b.yv) && !(b.ye && b.yu && b.yv))
        return set_error(GOC_ERR_ARG, "%s: the stage output must be all three arrays or none", who);
    if (b.xbe == b.ybe || b.xbe == b.xe)
        return set_error(GOC_ERR_ARG, "%s: x-bar must not alias x or y-bar", who);
    return GOC_OK;
}

// Calls f(CF, HY, TY) with the three as compile-time constants
// (std::integral_constant values): constant Coriolis, stage output given,
// tile height.
template <class F>
static int dispatch_vjp(bool cf, bool hy, bool small, F&& f) {
    using T = std::true_type;
    using N = std::false_type;
    using S = std::integral_constant<int, kAYSmall>;
    using L = std::integral_constant<int, kAY>;
    if (cf) {
        if (hy) return small ? f(T{}, T{}, S{}) : f(T{}, T{}, L{});
        return small ? f(T{}, N{}, S{}) : f(T{}, N{}, L{});
    }
    if (hy) return small ? f(N{}, T{}, S{}) : f(N{}, T{}, L{});
    return small ? f(N{}, N{}, S{}) : f(N{}, N{}, L{});
}

// Tiles of kAY rows fill the GPU's SMs less than twice over: the launch
// then takes tiles of kAYSmall rows, twice as many CTAs, each with about
// 0.6 of the work (a launch of a few CTAs per SM is bound by one CTA's
// latency, not by throughput).
static bool small_tiles(const GocCdklmParams* p, int n_members) {
    static int sms[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    int& n = sms[dev & 63];
    if (n == 0 && cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) n = 0;
    const long long tiles = (long long)((p->nx + kAX - 1) / kAX) * ((p->ny + kAY - 1) / kAY) * n_members;
    return n > 0 && tiles < 2LL * n;
}

// Wind partials: one (x, y) pair per tile of the smaller tile height, so the
// count covers either launch.
static int goc_cdklm_vjp_partials_count(int nx, int ny) {
    if (nx < 1 || ny < 1) return 0;
    return 2 * ((nx + kAX - 1) / kAX) * ((ny + kAYSmall - 1) / kAYSmall);
}

static int stage_vjp_members_impl(const GocCdklmParams* p, float dt, int rk_step, const VjpBuffers& b, int pitch,
                                  long long member_stride, int n_members, int wind_stride, const float* Hi,
                                  int Hi_pitch, const float* Hm, int Hm_pitch, float* wind_partials, void* stream,
                                  const char* who) {
    int rc = vjp_args(p, rk_step, b, pitch, Hi_pitch, Hm_pitch, Hi, Hm, who);
    if (rc) return rc;
    if (n_members < 1 || n_members > 65535 || member_stride < (long long)(p->ny + 4) * (pitch / 4) || wind_stride < 0)
        return set_error(GOC_ERR_ARG, "%s: bad member count or stride", who);
    const StepConst k = make_step_const(*p);
    const bool cf = (p->coriolis_nx == 1 && p->coriolis_ny == 1);
    cudaStream_t st = as_stream(stream);
    const int partials = goc_cdklm_vjp_partials_count(p->nx, p->ny);
    const int pf = pitch / 4, hip = Hi_pitch / 4, hmp = Hm_pitch / 4;
    return dispatch_vjp(cf, b.ye != nullptr, small_tiles(p, n_members), [&](auto CF, auto HY, auto TY) -> int {
        constexpr int ty = decltype(TY)::value;
        // interior tile rectangle (contiguous in x and in y)
        const int ntx = (p->nx + kAX - 1) / kAX, nty = (p->ny + ty - 1) / ty;
        int4 inner = make_int4(0, 0, 0, 0);
        for (int t = 0, first = -1; t < ntx; ++t) {
            const int x0 = 2 + t * kAX - kAHalo;
            if (x0 >= 2 && x0 + kAX + 2 * kAHalo <= p->nx + 2) {
                if (first < 0) first = inner.x = t;
                inner.y = t + 1;
            }
        }
        for (int t = 0, first = -1; t < nty; ++t) {
            const int y0 = 2 + t * ty - kAHalo;
            if (y0 >= 2 && y0 + ty + 2 * kAHalo <= p->ny + 2) {
                if (first < 0) first = inner.z = t;
                inner.w = t + 1;
            }
        }
        constexpr int W = kAX + 2 * kAHalo, H = ty + 2 * kAHalo;
        constexpr size_t smem = sizeof(AdjSmem<W, H, !decltype(CF)::value>);
        auto kern = stage_vjp_members_kernel<decltype(CF)::value, decltype(HY)::value, ty>;
        static bool configured = false;
        if (!configured) {
            if (int e = configure_smem(kern, smem)) return e;
            configured = true;
        }
        const dim3 grid((unsigned)(ntx * nty) * (unsigned)n_members);
        kern<<<grid, kANT, smem, st>>>(*p, k, dt, rk_step, b.xe, b.xu, b.xv, b.ae, b.au, b.av, b.ye, b.yu, b.yv,
                                       b.ybe, b.ybu, b.ybv, b.bbe, b.bbu, b.bbv, b.xbe, b.xbu, b.xbv, b.abe, b.abu,
                                       b.abv, pf, member_stride, wind_stride, Hi, hip, Hm, hmp, wind_partials,
                                       partials, n_members, inner);
        count_launch();
        return check_launch("stage_vjp_members_kernel");
    });
}

// One simulator: the member-batched kernel with one member, so that single
// and batched VJPs run the same code and agree bit for bit.
static int stage_vjp_impl(const GocCdklmParams* p, float dt, int rk_step, const VjpBuffers& b, int pitch,
                          const float* Hi, int Hi_pitch, const float* Hm, int Hm_pitch, float* wind_partials,
                          void* stream, const char* who) {
    const long long plane = (long long)(p->ny + 4) * (pitch / 4);
    return stage_vjp_members_impl(p, dt, rk_step, b, pitch, plane, 1, 0, Hi, Hi_pitch, Hm, Hm_pitch, wind_partials,
                                  stream, who);
}

}  // namespace goc

using namespace goc;

extern "C" int goc_cdklm_vjp_partials(int nx, int ny) { return goc_cdklm_vjp_partials_count(nx, ny); }

extern "C" int goc_cdklm_stage_vjp(const GocCdklmParams* p, float dt, int rk_step, const float* x_eta,
                                   const float* x_hu, const float* x_hv, const float* a_eta, const float* a_hu,
                                   const float* a_hv, const float* yb_eta, const float* yb_hu, const float* yb_hv,
                                   const float* base_eta, const float* base_hu, const float* base_hv,
                                   float* xb_eta, float* xb_hu, float* xb_hv, float* ab_eta, float* ab_hu,
                                   float* ab_hv, int pitch, const float* Hi, int Hi_pitch, const float* Hm,
                                   int Hm_pitch, float* wind_partials, void* stream) {
    const VjpBuffers b{x_eta, x_hu, x_hv, a_eta, a_hu, a_hv, nullptr, nullptr, nullptr, yb_eta, yb_hu, yb_hv,
                       base_eta, base_hu, base_hv, xb_eta, xb_hu, xb_hv, ab_eta, ab_hu, ab_hv};
    return stage_vjp_impl(p, dt, rk_step, b, pitch, Hi, Hi_pitch, Hm, Hm_pitch, wind_partials, stream,
                          "goc_cdklm_stage_vjp");
}

extern "C" int goc_cdklm_stage_vjp_out(const GocCdklmParams* p, float dt, int rk_step, const float* x_eta,
                                       const float* x_hu, const float* x_hv, const float* a_eta, const float* a_hu,
                                       const float* a_hv, const float* y_eta, const float* y_hu, const float* y_hv,
                                       const float* yb_eta, const float* yb_hu, const float* yb_hv,
                                       const float* base_eta, const float* base_hu, const float* base_hv,
                                       float* xb_eta, float* xb_hu, float* xb_hv, float* ab_eta, float* ab_hu,
                                       float* ab_hv, int pitch, const float* Hi, int Hi_pitch, const float* Hm,
                                       int Hm_pitch, float* wind_partials, void* stream) {
    if (!y_eta || !y_hu || !y_hv) return set_error(GOC_ERR_ARG, "goc_cdklm_stage_vjp_out: null stage output");
    const VjpBuffers b{x_eta, x_hu, x_hv, a_eta, a_hu, a_hv, y_eta, y_hu, y_hv, yb_eta, yb_hu, yb_hv,
                       base_eta, base_hu, base_hv, xb_eta, xb_hu, xb_hv, ab_eta, ab_hu, ab_hv};
    return stage_vjp_impl(p, dt, rk_step, b, pitch, Hi, Hi_pitch, Hm, Hm_pitch, wind_partials, stream,
                          "goc_cdklm_stage_vjp_out");
}

extern "C" int goc_cdklm_stage_vjp_members(const GocCdklmParams* p, float dt, int rk_step, const float* x_eta,
                                           const float* x_hu, const float* x_hv, const float* a_eta,
                                           const float* a_hu, const float* a_hv, const float* yb_eta,
                                           const float* yb_hu, const float* yb_hv, const float* base_eta,
                                           const float* base_hu, const float* base_hv, float* xb_eta, float* xb_hu,
                                           float* xb_hv, float* ab_eta, float* ab_hu, float* ab_hv, int pitch,
                                           long long member_stride, int n_members, int wind_stride,
                                           const float* Hi, int Hi_pitch, const float* Hm, int Hm_pitch,
                                           float* wind_partials, void* stream) {
    const VjpBuffers b{x_eta, x_hu, x_hv, a_eta, a_hu, a_hv, nullptr, nullptr, nullptr, yb_eta, yb_hu, yb_hv,
                       base_eta, base_hu, base_hv, xb_eta, xb_hu, xb_hv, ab_eta, ab_hu, ab_hv};
    return stage_vjp_members_impl(p, dt, rk_step, b, pitch, member_stride, n_members, wind_stride, Hi, Hi_pitch,
                                  Hm, Hm_pitch, wind_partials, stream, "goc_cdklm_stage_vjp_members");
}

extern "C" int goc_cdklm_stage_vjp_members_out(const GocCdklmParams* p, float dt, int rk_step, const float* x_eta,
                                               const float* x_hu, const float* x_hv, const float* a_eta,
                                               const float* a_hu, const float* a_hv, const float* y_eta,
                                               const float* y_hu, const float* y_hv, const float* yb_eta,
                                               const float* yb_hu, const float* yb_hv, const float* base_eta,
                                               const float* base_hu, const float* base_hv, float* xb_eta,
                                               float* xb_hu, float* xb_hv, float* ab_eta, float* ab_hu, float* ab_hv,
                                               int pitch, long long member_stride, int n_members, int wind_stride,
                                               const float* Hi, int Hi_pitch, const float* Hm, int Hm_pitch,
                                               float* wind_partials, void* stream) {
    if (!y_eta || !y_hu || !y_hv)
        return set_error(GOC_ERR_ARG, "goc_cdklm_stage_vjp_members_out: null stage output");
    const VjpBuffers b{x_eta, x_hu, x_hv, a_eta, a_hu, a_hv, y_eta, y_hu, y_hv, yb_eta, yb_hu, yb_hv,
                       base_eta, base_hu, base_hv, xb_eta, xb_hu, xb_hv, ab_eta, ab_hu, ab_hv};
    return stage_vjp_members_impl(p, dt, rk_step, b, pitch, member_stride, n_members, wind_stride, Hi, Hi_pitch,
                                  Hm, Hm_pitch, wind_partials, stream, "goc_cdklm_stage_vjp_members_out");
}
