// Adjoint of the CDKLM16 RK2 step: stage VJP kernels and their host entry
// points.  Compiled like the step (no FMA contraction) so that the forward
// recompute inside the VJP reproduces the forward step bit for bit.
#include <cstdio>

#include "cdklm_adjoint.cuh"

namespace goc {

constexpr int kAX = 32, kAY = 16, kANT = 256;   // x-bar tile and threads per CTA
constexpr int kAHalo = 4;

template <int TX, int TY, int NT, bool CONST_F, bool BORDER>
__device__ void stage_vjp_body(const GocCdklmParams& p, const StepConst& k, float dt, int rk_step, int tile_x,
                               int tile_y, const float* __restrict__ xe, const float* __restrict__ xu,
                               const float* __restrict__ xv, const float* __restrict__ ae,
                               const float* __restrict__ au, const float* __restrict__ av,
                               const float* __restrict__ ybe, const float* __restrict__ ybu,
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

    // 1. corner depths (as the forward kernel)
    for (int idx = threadIdx.x; idx < (H + 1) * (W + 1); idx += NT) {
        const int i = idx % (W + 1), j = idx / (W + 1);
        const int gc = T.x0 + i, gr = T.y0 + j;
        const int cc = !BORDER ? gc : px ? wrap_interior(gc, nx) : clampi(gc, 0, nx + 4);
        const int cr = !BORDER ? gr : py ? wrap_interior(gr, ny) : clampi(gr, 0, ny + 4);
        float v = __ldg(Hi_g + (size_t)cr * hi_pitch + cc);
        if (fabsf(v - p.land_value) < kDryEps) v = kDryFlag;
        S.Hi[j][i] = v;
    }
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
    // 2. x on the tile + 4, desingularised; adjoint accumulators cleared
    for (int idx = threadIdx.x; idx < H * W; idx += NT) {
        const int i = idx % W, j = idx / W;
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

    // 3. forward recompute of the stage on the tile + 2
    T.template slopes<2, W - 2, 2, H - 2, CONST_F>();
    __syncthreads();
    T.template faces<2, W - 2, 2, H - 2, CONST_F>();
    __syncthreads();

    // 4. cell pass: RK combination, friction and source terms in reverse.
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
        float L1, L2, L3, ec, hu, hv, Hm, hsum;
        T.template rhs<CONST_F, true>(i, j, gxs, gys, L1, L2, L3, ec, hu, hv, Hm, hsum);
        const float C = T.friction(dt, hsum, hu, hv);
        float ne, nhu, nhv, ecb, hub, hvb, L1b, L2b, L3b, Cb;
        float eab = 0.f, huab = 0.f, hvab = 0.f;
        if (rk_step == 0) {
            ne = ec + dt * L1;
            nhu = (hu + dt * L2) / (1.0f + C);
            nhv = (hv + dt * L3) / (1.0f + C);
            const bool dry = (ne + Hm <= p.depth_cutoff);
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
            const float ea = __ldg(ae + o), hua = __ldg(au + o), hva = __ldg(av + o);
            const float Dd = 1.0f + 0.5f * C;
            ne = 0.5f * (ea + (ec + dt * L1));
            nhu = 0.5f * (hua + (hu + dt * L2)) / Dd;
            nhv = 0.5f * (hva + (hv + dt * L3)) / Dd;
            const bool dry = (ne + Hm <= p.depth_cutoff);
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

    // 5. faces in reverse, two colours each.  x faces are coloured as a
    //    checkerboard ((i + j) even / odd): faces of one row never share a
    //    cell.  A warp takes 16 faces of a row and 16 of the next: the
    //    stride-2 accesses of one half-warp cover 32 consecutive floats, and
    //    the checkerboard puts the two rows on even and odd banks, so they do
    //    not conflict; the remaining faces of each row come afterwards.
    constexpr int NXF = W - 3, NYF = H - 4;     // east faces of cells [1, W-2) on rows [2, H-2)
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
            const int j = 2 + row;
            const int i = 1 + 2 * kf + ((j + colour) & 1);
            if (i >= W - 2) continue;
            const float F0b = (FDb(0)[j][i] - FDb(0)[j][i + 1]) * k.inv_dx;
            const float F1b = (FDb(1)[j][i] - FDb(1)[j][i + 1]) * k.inv_dx;
            const float F2b = (FDb(2)[j][i] - FDb(2)[j][i + 1]) * k.inv_dx;
            if (F0b == 0.0f && F1b == 0.0f && F2b == 0.0f) continue;
            R.template face_x_vjp<CONST_F>(i, j, F0b, F1b, F2b);
        }
        __syncthreads();
    }
    // 6. x slopes in reverse (three colours); their adjoints are complete
    //    once the x faces are done
    constexpr int NXS = W - 2, NYS = H - 4;     // x slopes of cells [1, W-1) on rows [2, H-2)
#pragma unroll 1
    for (int colour = 0; colour < 3; ++colour) {
        constexpr int PERROW = (NXS + 2) / 3;
        for (int idx = threadIdx.x; idx < PERROW * NYS; idx += NT) {
            const int i = 1 + colour + 3 * (idx % PERROW);
            const int j = 2 + idx / PERROW;
            if (i >= W - 1) continue;
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
    // 7. y faces and y slopes in reverse
    if (!p.one_dimensional) {
        constexpr int NXG = W - 4, NYG = H - 3;   // north faces of cells [2, W-2) on rows [1, H-2)
#pragma unroll 1
        for (int colour = 0; colour < 2; ++colour) {
            for (int idx = threadIdx.x; idx < NXG * ((NYG + 1) / 2); idx += NT) {
                const int i = 2 + idx % NXG;
                const int j = 1 + colour + 2 * (idx / NXG);
                if (j >= H - 2) continue;
                const float G0b = (FDb(0)[j][i] - FDb(0)[j + 1][i]) * k.inv_dy;
                const float G1b = (FDb(1)[j][i] - FDb(1)[j + 1][i]) * k.inv_dy;
                const float G2b = (FDb(2)[j][i] - FDb(2)[j + 1][i]) * k.inv_dy;
                if (G0b == 0.0f && G1b == 0.0f && G2b == 0.0f) continue;
                R.template face_y_vjp<CONST_F>(i, j, G0b, G1b, G2b);
            }
            __syncthreads();
        }
    }

    constexpr int NXY = W - 4, NYY = H - 2;     // y slopes of cells [2, W-2) on rows [1, H-1)
#pragma unroll 1
    for (int colour = 0; colour < 3; ++colour) {
        constexpr int PERCOL = (NYY + 2) / 3;
        for (int idx = threadIdx.x; idx < NXY * PERCOL; idx += NT) {
            const int i = 2 + idx % NXY;
            const int j = 1 + colour + 3 * (idx / NXY);
            if (j >= H - 1) continue;
            R.template slope_y_vjp<CONST_F>(i, j);
        }
        __syncthreads();
    }

    // 8. desingularisation in reverse at every staged position, as the
    //    adjoint of the memory cell it read (signs of the wall mirrors); the
    //    result per position goes to the Gy planes
    for (int idx = threadIdx.x; idx < H * W; idx += NT) {
        const int i = idx % W, j = idx / W;
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

    // 9. x-bar of the tile's interior cells: own position plus the wall
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

    // 10. wind-stress adjoint of the tile's cells
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

template <bool CONST_F>
__global__ void __launch_bounds__(kANT, CONST_F ? 3 : 2)
stage_vjp_kernel(const GocCdklmParams p, const StepConst k, float dt, int rk_step, const float* xe, const float* xu,
                 const float* xv, const float* ae, const float* au, const float* av, const float* ybe,
                 const float* ybu, const float* ybv, const float* bbe, const float* bbu, const float* bbv,
                 float* xbe, float* xbu, float* xbv, float* abe, float* abu, float* abv, int pitch,
                 const float* Hi_g, int hi_pitch, const float* Hm_g, int hm_pitch, float* wind_partials) {
    extern __shared__ __align__(16) float smem_raw[];
    const int tx = blockIdx.x, ty = blockIdx.y;
    const int x0 = 2 + tx * kAX - kAHalo, y0 = 2 + ty * kAY - kAHalo;
    const bool border = x0 < 2 || y0 < 2 || x0 + kAX + 2 * kAHalo > p.nx + 2 || y0 + kAY + 2 * kAHalo > p.ny + 2;
    if (border)
        stage_vjp_body<kAX, kAY, kANT, CONST_F, true>(p, k, dt, rk_step, tx, ty, xe, xu, xv, ae, au, av, ybe, ybu,
                                                      ybv, bbe, bbu, bbv, xbe, xbu, xbv, abe, abu, abv, pitch, Hi_g,
                                                      hi_pitch, Hm_g, hm_pitch, wind_partials, smem_raw);
    else
        stage_vjp_body<kAX, kAY, kANT, CONST_F, false>(p, k, dt, rk_step, tx, ty, xe, xu, xv, ae, au, av, ybe, ybu,
                                                       ybv, bbe, bbu, bbv, xbe, xbu, xbv, abe, abu, abv, pitch, Hi_g,
                                                       hi_pitch, Hm_g, hm_pitch, wind_partials, smem_raw);
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
template <bool CONST_F>
__global__ void __launch_bounds__(kANT, CONST_F ? 3 : 2)
stage_vjp_members_kernel(const GocCdklmParams p, const StepConst k, float dt, int rk_step, const float* xe,
                         const float* xu, const float* xv, const float* ae, const float* au, const float* av,
                         const float* ybe, const float* ybu, const float* ybv, const float* bbe, const float* bbu,
                         const float* bbv, float* xbe, float* xbu, float* xbv, float* abe, float* abu, float* abv,
                         int pitch, long long member_stride, int wind_stride, const float* Hi_g, int hi_pitch,
                         const float* Hm_g, int hm_pitch, float* wind_partials, int partials_stride,
                         int n_members, int4 inner) {
    extern __shared__ __align__(16) float smem_raw[];
    const int member = (int)(blockIdx.x % (unsigned)n_members);
    int tx, ty;
    interior_first_tile((int)(blockIdx.x / (unsigned)n_members), (p.nx + kAX - 1) / kAX, (p.ny + kAY - 1) / kAY,
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
    const int x0 = 2 + tx * kAX - kAHalo, y0 = 2 + ty * kAY - kAHalo;
    const bool border = x0 < 2 || y0 < 2 || x0 + kAX + 2 * kAHalo > p.nx + 2 || y0 + kAY + 2 * kAHalo > p.ny + 2;
    if (border)
        stage_vjp_body<kAX, kAY, kANT, CONST_F, true>(pm, k, dt, rk_step, tx, ty, sh(xe), sh(xu), sh(xv), sh(ae),
                                                      sh(au), sh(av), sh(ybe), sh(ybu), sh(ybv), sh(bbe), sh(bbu),
                                                      sh(bbv), shw(xbe), shw(xbu), shw(xbv), shw(abe), shw(abu),
                                                      shw(abv), pitch, Hi_g, hi_pitch, Hm_g, hm_pitch, wp, smem_raw);
    else
        stage_vjp_body<kAX, kAY, kANT, CONST_F, false>(pm, k, dt, rk_step, tx, ty, sh(xe), sh(xu), sh(xv), sh(ae),
                                                       sh(au), sh(av), sh(ybe), sh(ybu), sh(ybv), sh(bbe), sh(bbu),
                                                       sh(bbv), shw(xbe), shw(xbu), shw(xbv), shw(abe), shw(abu),
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

template <bool CF>
static int launch_vjp(const GocCdklmParams* p, const StepConst& k, float dt, int rk, const float* xe,
                      const float* xu, const float* xv, const float* ae, const float* au, const float* av,
                      const float* ybe, const float* ybu, const float* ybv, const float* bbe, const float* bbu,
                      const float* bbv, float* xbe, float* xbu, float* xbv, float* abe, float* abu, float* abv,
                      int pitch_f, const float* Hi, int hip_f, const float* Hm, int hmp_f, float* wind,
                      cudaStream_t st) {
    constexpr int W = kAX + 2 * kAHalo, H = kAY + 2 * kAHalo;
    constexpr size_t smem = sizeof(AdjSmem<W, H, !CF>);
    auto kern = stage_vjp_kernel<CF>;
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return set_error(GOC_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(e));
        configured = true;
    }
    dim3 grid((p->nx + kAX - 1) / kAX, (p->ny + kAY - 1) / kAY);
    kern<<<grid, kANT, smem, st>>>(*p, k, dt, rk, xe, xu, xv, ae, au, av, ybe, ybu, ybv, bbe, bbu, bbv, xbe, xbu,
                                   xbv, abe, abu, abv, pitch_f, Hi, hip_f, Hm, hmp_f, wind);
    count_launch();
    return check_launch("stage_vjp_kernel");
}

}  // namespace goc

using namespace goc;

extern "C" int goc_cdklm_vjp_partials(int nx, int ny) {
    if (nx < 1 || ny < 1) return 0;
    return 2 * ((nx + kAX - 1) / kAX) * ((ny + kAY - 1) / kAY);
}

extern "C" int goc_cdklm_stage_vjp(const GocCdklmParams* p, float dt, int rk_step, const float* x_eta,
                                   const float* x_hu, const float* x_hv, const float* a_eta, const float* a_hu,
                                   const float* a_hv, const float* yb_eta, const float* yb_hu, const float* yb_hv,
                                   const float* base_eta, const float* base_hu, const float* base_hv,
                                   float* xb_eta, float* xb_hu, float* xb_hv, float* ab_eta, float* ab_hu,
                                   float* ab_hv, int pitch, const float* Hi, int Hi_pitch, const float* Hm,
                                   int Hm_pitch, float* wind_partials, void* stream) {
    int rc = vjp_check(p, pitch, Hi_pitch, Hm_pitch, "goc_cdklm_stage_vjp");
    if (rc) return rc;
    if (rk_step != 0 && rk_step != 1) return set_error(GOC_ERR_ARG, "goc_cdklm_stage_vjp: rk_step must be 0 or 1");
    if (!x_eta || !x_hu || !x_hv || !yb_eta || !yb_hu || !yb_hv || !xb_eta || !xb_hu || !xb_hv || !Hi || !Hm)
        return set_error(GOC_ERR_ARG, "goc_cdklm_stage_vjp: null buffer");
    if (rk_step == 1 && (!a_eta || !a_hu || !a_hv || !ab_eta || !ab_hu || !ab_hv))
        return set_error(GOC_ERR_ARG, "goc_cdklm_stage_vjp: the second stage needs Q^n and its adjoint output");
    if ((base_eta || base_hu || base_hv) && !(base_eta && base_hu && base_hv))
        return set_error(GOC_ERR_ARG, "goc_cdklm_stage_vjp: base must be all three arrays or none");
    if (xb_eta == yb_eta || xb_eta == x_eta)
        return set_error(GOC_ERR_ARG, "goc_cdklm_stage_vjp: x-bar must not alias x or y-bar");
    const StepConst k = make_step_const(*p);
    const bool cf = (p->coriolis_nx == 1 && p->coriolis_ny == 1);
    cudaStream_t st = as_stream(stream);
    const int pf = pitch / 4, hip = Hi_pitch / 4, hmp = Hm_pitch / 4;
    if (cf)
        return launch_vjp<true>(p, k, dt, rk_step, x_eta, x_hu, x_hv, a_eta, a_hu, a_hv, yb_eta, yb_hu, yb_hv,
                                base_eta, base_hu, base_hv, xb_eta, xb_hu, xb_hv, ab_eta, ab_hu, ab_hv, pf, Hi, hip,
                                Hm, hmp, wind_partials, st);
    return launch_vjp<false>(p, k, dt, rk_step, x_eta, x_hu, x_hv, a_eta, a_hu, a_hv, yb_eta, yb_hu, yb_hv,
                             base_eta, base_hu, base_hv, xb_eta, xb_hu, xb_hv, ab_eta, ab_hu, ab_hv, pf, Hi, hip, Hm,
                             hmp, wind_partials, st);
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
    int rc = vjp_check(p, pitch, Hi_pitch, Hm_pitch, "goc_cdklm_stage_vjp_members");
    if (rc) return rc;
    if (rk_step != 0 && rk_step != 1)
        return set_error(GOC_ERR_ARG, "goc_cdklm_stage_vjp_members: rk_step must be 0 or 1");
    if (!x_eta || !x_hu || !x_hv || !yb_eta || !yb_hu || !yb_hv || !xb_eta || !xb_hu || !xb_hv || !Hi || !Hm)
        return set_error(GOC_ERR_ARG, "goc_cdklm_stage_vjp_members: null buffer");
    if (rk_step == 1 && (!a_eta || !a_hu || !a_hv || !ab_eta || !ab_hu || !ab_hv))
        return set_error(GOC_ERR_ARG, "goc_cdklm_stage_vjp_members: the second stage needs Q^n and its adjoint");
    if ((base_eta || base_hu || base_hv) && !(base_eta && base_hu && base_hv))
        return set_error(GOC_ERR_ARG, "goc_cdklm_stage_vjp_members: base must be all three arrays or none");
    if (xb_eta == yb_eta || xb_eta == x_eta)
        return set_error(GOC_ERR_ARG, "goc_cdklm_stage_vjp_members: x-bar must not alias x or y-bar");
    if (n_members < 1 || n_members > 65535 || member_stride < (long long)(p->ny + 4) * (pitch / 4) || wind_stride < 0)
        return set_error(GOC_ERR_ARG, "goc_cdklm_stage_vjp_members: bad member count or stride");
    const StepConst k = make_step_const(*p);
    const bool cf = (p->coriolis_nx == 1 && p->coriolis_ny == 1);
    cudaStream_t st = as_stream(stream);
    constexpr int W = kAX + 2 * kAHalo, H = kAY + 2 * kAHalo;
    const size_t smem = cf ? sizeof(AdjSmem<W, H, false>) : sizeof(AdjSmem<W, H, true>);
    const int partials = goc_cdklm_vjp_partials(p->nx, p->ny);
    // interior tile rectangle (contiguous in x and in y)
    const int ntx = (p->nx + kAX - 1) / kAX, nty = (p->ny + kAY - 1) / kAY;
    int4 inner = make_int4(0, 0, 0, 0);
    for (int t = 0, first = -1; t < ntx; ++t) {
        const int x0 = 2 + t * kAX - kAHalo;
        if (x0 >= 2 && x0 + kAX + 2 * kAHalo <= p->nx + 2) {
            if (first < 0) first = inner.x = t;
            inner.y = t + 1;
        }
    }
    for (int t = 0, first = -1; t < nty; ++t) {
        const int y0 = 2 + t * kAY - kAHalo;
        if (y0 >= 2 && y0 + kAY + 2 * kAHalo <= p->ny + 2) {
            if (first < 0) first = inner.z = t;
            inner.w = t + 1;
        }
    }
    const dim3 grid((unsigned)(ntx * nty) * (unsigned)n_members);
    static bool configured[2] = {false, false};
    if (!configured[cf]) {
        cudaError_t e = cf ? cudaFuncSetAttribute(stage_vjp_members_kernel<true>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                           : cudaFuncSetAttribute(stage_vjp_members_kernel<false>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return set_error(GOC_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(e));
        configured[cf] = true;
    }
    const int pf = pitch / 4, hip = Hi_pitch / 4, hmp = Hm_pitch / 4;
    if (cf)
        stage_vjp_members_kernel<true><<<grid, kANT, smem, st>>>(
            *p, k, dt, rk_step, x_eta, x_hu, x_hv, a_eta, a_hu, a_hv, yb_eta, yb_hu, yb_hv, base_eta, base_hu,
            base_hv, xb_eta, xb_hu, xb_hv, ab_eta, ab_hu, ab_hv, pf, member_stride, wind_stride, Hi, hip, Hm, hmp,
            wind_partials, partials, n_members, inner);
    else
        stage_vjp_members_kernel<false><<<grid, kANT, smem, st>>>(
            *p, k, dt, rk_step, x_eta, x_hu, x_hv, a_eta, a_hu, a_hv, yb_eta, yb_hu, yb_hv, base_eta, base_hu,
            base_hv, xb_eta, xb_hu, xb_hv, ab_eta, ab_hu, ab_hv, pf, member_stride, wind_stride, Hi, hip, Hm, hmp,
            wind_partials, partials, n_members, inner);
    count_launch();
    return check_launch("stage_vjp_members_kernel");
}
