// Transfer of the SOAR coarse field to the ocean state: the bicubic
// up-sampling of the coarse eta perturbation and its geostrophically balanced
// momentum (K/ocean_noise.cu:256-666, applied by S/OceanStateNoise.py:418-459).
//
// Two callers share this code and must give the same bits: the stand-alone
// perturbation kernels (noise_transfer.cu) and the epilogue of the fused
// ensemble step (ensemble.cuh), which adds the perturbation to Q^{n+1} before
// writing it.  Both translation units are compiled with the same arithmetic
// options (flush-to-zero, the fast division/square root of -prec-div=false /
// -prec-sqrt=false, no FMA contraction), so one source gives one rounding.
// The reference builds these kernels with --use_fast_math (contracting
// multiply-adds); the difference is a few float32 ulps of the perturbation.
#pragma once

#include "common.cuh"

namespace goc {

struct OceanRef {
    int nx, ny;
    float dx, dy;
    float* eta; float* hu; float* hv; int pitch;    // floats
    const float* Hi; int hi_pitch;                  // floats
    float land;
    int images_ns, images_ew;                       // write periodic ghost images
};

__device__ __forceinline__ OceanRef ocean_of(const GocMemberDesc& m, int images) {
    return OceanRef{m.p.nx, m.p.ny, m.p.dx, m.p.dy, m.eta[0], m.hu[0], m.hv[0], m.pitch / 4, m.Hi, m.Hi_pitch / 4,
                    m.p.land_value, images && m.p.bc_north == 2, images && m.p.bc_east == 2};
}

// Write a perturbed interior cell and, for periodic boundaries, its ghost
// images (the boundary fill the reference runs after perturbState,
// S/CDKLM16.py:571-572).
__device__ __forceinline__ void store_cell(const OceanRef& o, int ti, int tj, float e, float u, float v) {
    int xs[2] = {ti, -1}, ys[2] = {tj, -1};
    if (o.images_ew) xs[1] = (ti < 4) ? ti + o.nx : (ti >= o.nx ? ti - o.nx : -1);
    if (o.images_ns) ys[1] = (tj < 4) ? tj + o.ny : (tj >= o.ny ? tj - o.ny : -1);
    for (int a = 0; a < 2; ++a) {
        if (ys[a] < 0) continue;
        for (int b = 0; b < 2; ++b) {
            if (xs[b] < 0) continue;
            const size_t k = (size_t)ys[a] * o.pitch + xs[b];
            o.eta[k] = e; o.hu[k] = u; o.hv[k] = v;
        }
    }
}

// Coriolis parameter of cell (ti, tj) as the noise kernels see it: f plus the
// beta-plane term along the north vector, or the Coriolis texture when f = 0.
template <class D>
__device__ __forceinline__ float noise_coriolis(const D& d, int nx, int ny, float dx, float dy, int ti, int tj) {
    float c = d.f + d.beta * ((ti + 0.5f) * dx * d.north_x + (tj + 0.5f) * dy * d.north_y);
    if (d.f == 0.0f && d.coriolis_f) {
        const float s = (ti + 0.5f) / (nx + 4.0f), t = (tj + 0.5f) / (ny + 4.0f);
        c = tex_bilinear(d.coriolis_f, d.coriolis_nx, d.coriolis_ny, s, t);
    }
    return c;
}

template <class D>
__device__ __forceinline__ float noise_coriolis(const D& d, const OceanRef& o, int ti, int tj) {
    return noise_coriolis(d, o.nx, o.ny, o.dx, o.dy, ti, tj);
}

__device__ __forceinline__ float coarse_at(const GocNoiseDesc& d, int j, int i) {
    j = clampi(j, 0, d.coarse_ny + 3);
    i = clampi(i, 0, d.coarse_nx + 3);
    return d.coarse[(size_t)j * (d.coarse_pitch / 4) + i];
}

// Bicubic up-sampling of the coarse field (K/ocean_noise.cu:497-586), split in
// three parts so that a tile computes the coefficient matrix of each coarse
// cell once and evaluates it at every fine cell inside: the coarse cell (ci, cj)
// of fine cell (ti, tj) with the fractional position (rx, ry) in it, the 4x4
// coefficients A of coarse cell (ci, cj), and the polynomial.
__device__ __forceinline__ int bicubic_ci(const GocNoiseDesc& d, float dx, int ti, float* rx) {
    const float x = (ti - 2 + 0.5f + d.offset_i) * dx;
    int ci = (int)floorf(x / d.coarse_dx + 2 - 0.5f);
    if (ci > d.coarse_nx + 1) ci -= 1;
    *rx = (x - (ci - 2 + 0.5f) * d.coarse_dx) / d.coarse_dx;
    return ci;
}

__device__ __forceinline__ int bicubic_cj(const GocNoiseDesc& d, float dy, int tj, float* ry) {
    const float y = (tj - 2 + 0.5f + d.offset_j) * dy;
    int cj = (int)floorf(y / d.coarse_dy + 2 - 0.5f);
    if (cj > d.coarse_ny + 1) cj -= 1;
    *ry = (y - (cj - 2 + 0.5f) * d.coarse_dy) / d.coarse_dy;
    return cj;
}

__device__ __forceinline__ void bicubic_coeffs(const GocNoiseDesc& d, int ci, int cj, float* A /* [16], row-major */) {
    float c[4][4];  // c[row][col] = coarse[cj-1+row][ci-1+col]
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) c[r][q] = coarse_at(d, cj - 1 + r, ci - 1 + q);
    // values, x/y derivatives and cross derivatives at the 4 corners
    float F[4][4];
    F[0][0] = c[1][1]; F[0][1] = c[2][1]; F[1][0] = c[1][2]; F[1][1] = c[2][2];
    F[2][0] = (c[1][2] - c[1][0]) / 2.0f; F[2][1] = (c[2][2] - c[2][0]) / 2.0f;
    F[3][0] = (c[1][3] - c[1][1]) / 2.0f; F[3][1] = (c[2][3] - c[2][1]) / 2.0f;
    F[0][2] = (c[2][1] - c[0][1]) / 2.0f; F[0][3] = (c[3][1] - c[1][1]) / 2.0f;
    F[1][2] = (c[2][2] - c[0][2]) / 2.0f; F[1][3] = (c[3][2] - c[1][2]) / 2.0f;
    const float fy_10 = (c[2][0] - c[0][0]) / 2.0f, fy_11 = (c[3][0] - c[1][0]) / 2.0f;
    const float fy20 = (c[2][3] - c[0][3]) / 2.0f, fy21 = (c[3][3] - c[1][3]) / 2.0f;
    F[2][2] = (F[1][2] - fy_10) / 2.0f; F[2][3] = (F[1][3] - fy_11) / 2.0f;
    F[3][2] = (fy20 - F[0][2]) / 2.0f; F[3][3] = (fy21 - F[0][3]) / 2.0f;
    const float B[4][4] = {{1, 0, 0, 0}, {0, 0, 1, 0}, {-3, 3, -2, -1}, {2, -2, 1, 1}};
    float FB[4][4];   // FB = F B^T, A = B FB
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q)
            FB[r][q] = F[r][0] * B[q][0] + F[r][1] * B[q][1] + F[r][2] * B[q][2] + F[r][3] * B[q][3];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q)
            A[4 * r + q] = B[r][0] * FB[0][q] + B[r][1] * FB[1][q] + B[r][2] * FB[2][q] + B[r][3] * FB[3][q];
}

__device__ __forceinline__ float bicubic_eval(const float* A, float rx, float ry) {
    const float xv[4] = {1.0f, rx, rx * rx, rx * rx * rx};
    const float yv[4] = {1.0f, ry, ry * ry, ry * ry * ry};
    float v = 0.0f;
#pragma unroll
    for (int r = 0; r < 4; ++r)
        v += xv[r] * (A[4 * r] * yv[0] + A[4 * r + 1] * yv[1] + A[4 * r + 2] * yv[2] + A[4 * r + 3] * yv[3]);
    return v;
}

// Bicubic value of the coarse field at fine cell (ti, tj).
__device__ __forceinline__ float bicubic_value(const GocNoiseDesc& d, float dx, float dy, int ti, int tj) {
    float rx, ry, A[16];
    const int ci = bicubic_ci(d, dx, ti, &rx), cj = bicubic_cj(d, dy, tj, &ry);
    bicubic_coeffs(d, ci, cj, A);
    return bicubic_eval(A, rx, ry);
}

// The eta perturbation on an NX x NY block of fine cells with origin (gi0,
// gj0) (full-array indices) into de[NY][NX] (shared memory), computed by the
// NT threads of the block together (`t`: this thread's index in [0, NT)).
// `scratch` (shared, `scratch_floats` floats) holds the coefficient matrices
// of the coarse cells under the block when they fit; otherwise every fine
// cell evaluates its own (same values).  The block's threads must all call
// this; it ends without a barrier.
template <int NX, int NY, int NT>
__device__ __forceinline__ void noise_tile_field(const GocNoiseDesc& d, float dx, float dy, int gi0, int gj0,
                                                 float* de, float* scratch, int scratch_floats, int t) {
    if (d.interpolation_factor <= 1) {
        for (int c = t; c < NX * NY; c += NT) de[c] = coarse_at(d, gj0 + c / NX, gi0 + c % NX);
        return;
    }
    // the coarse cells under the block: the index is monotone in the fine index
    float r;
    const int ci0 = bicubic_ci(d, dx, gi0, &r), ci1 = bicubic_ci(d, dx, gi0 + NX - 1, &r);
    const int cj0 = bicubic_cj(d, dy, gj0, &r), cj1 = bicubic_cj(d, dy, gj0 + NY - 1, &r);
    const int ncx = ci1 - ci0 + 1, ncy = cj1 - cj0 + 1;
    if (ncx * ncy * 17 + 2 * (NX + NY) > scratch_floats) {
        for (int c = t; c < NX * NY; c += NT) de[c] = bicubic_value(d, dx, dy, gi0 + c % NX, gj0 + c / NX);
        return;
    }
    float* A = scratch;                            // [ncx * ncy][17]
    int* s_ci = reinterpret_cast<int*>(scratch + ncx * ncy * 17);
    int* s_cj = s_ci + NX;
    float* s_rx = reinterpret_cast<float*>(s_cj + NY);
    float* s_ry = s_rx + NX;
    for (int c = t; c < ncx * ncy; c += NT) bicubic_coeffs(d, ci0 + c % ncx, cj0 + c / ncx, A + 17 * c);
    for (int c = t; c < NX + NY; c += NT) {
        if (c < NX) {
            s_ci[c] = clampi(bicubic_ci(d, dx, gi0 + c, &s_rx[c]) - ci0, 0, ncx - 1);
        } else {
            const int j = c - NX;
            s_cj[j] = clampi(bicubic_cj(d, dy, gj0 + j, &s_ry[j]) - cj0, 0, ncy - 1);
        }
    }
    __syncthreads();
    for (int c = t; c < NX * NY; c += NT) {
        const int j = c / NX, i = c % NX;
        de[c] = bicubic_eval(A + 17 * (s_cj[j] * ncx + s_ci[i]), s_rx[i], s_ry[j]);
    }
}

// The perturbed state of interior cell (ti, tj) from its state (e, u, v) and
// corner depths hc = (Hi[tj][ti], Hi[tj][ti+1], Hi[tj+1][ti], Hi[tj+1][ti+1]).
// `factor1`: the coarse grid is the computational grid (geostrophicBalance,
// the state's own depth in h and land cells zeroed); otherwise bicubic
// up-sampling (bicubicInterpolation, land cells unperturbed).  `de(jj, ii)`
// gives the perturbation of eta.
template <typename DE>
__device__ __forceinline__ void perturbed_state(const GocNoiseDesc& d, int nx, int ny, float dx, float dy, float land,
                                                int ti, int tj, bool factor1, DE de, float& e, float& u, float& v,
                                                const float* hc) {
    const bool dry = (hc[0] == land) || (hc[1] == land) || (hc[2] == land) || (hc[3] == land);
    const float H_mid = 0.25f * (hc[0] + hc[1] + hc[2] + hc[3]);
    const float cor = noise_coriolis(d, nx, ny, dx, dy, ti, tj);
    const float dc = de(tj, ti);
    const float ex = (de(tj, ti + 1) - de(tj, ti - 1)) / (2.0f * dx);
    const float ey = (de(tj + 1, ti) - de(tj - 1, ti)) / (2.0f * dy);
    if (factor1) {
        const float h_mid = dc + H_mid + e;
        const float dhu = -(d.g / cor) * h_mid * ey;
        const float dhv = (d.g / cor) * h_mid * ex;
        if (dry) {
            e = 0.0f; u = 0.0f; v = 0.0f;
        } else {
            e += dc; u += dhu; v += dhv;
        }
    } else if (!dry) {
        e += dc;
        u += -(d.g / cor) * (H_mid + dc) * ey;
        v += (d.g / cor) * (H_mid + dc) * ex;
    }
}

// Host-side validation and set-up of an OceanRef.
inline int make_ocean(int nx, int ny, float dx, float dy, float* eta, float* hu, float* hv, int pitch,
                      const float* Hi, int Hi_pitch, float land, int images_ns, int images_ew, OceanRef* o,
                      const char* who) {
    if (nx < 1 || ny < 1 || !eta || !hu || !hv || !Hi) return set_error(GOC_ERR_ARG, "%s: bad ocean arguments", who);
    if (pitch < (nx + 4) * 4 || Hi_pitch < (nx + 5) * 4 || pitch % 4 || Hi_pitch % 4)
        return set_error(GOC_ERR_ARG, "%s: pitch too small", who);
    if ((images_ns && ny < 4) || (images_ew && nx < 4))
        return set_error(GOC_ERR_ARG, "%s: periodic directions need at least 4 cells", who);
    *o = OceanRef{nx, ny, dx, dy, eta, hu, hv, pitch / 4, Hi, Hi_pitch / 4, land, images_ns, images_ew};
    return GOC_OK;
}

// Tiles of the stand-alone transfer kernels (noise_transfer.cu): kPX x kPY
// interior cells, kPT thread rows of kPX threads.
constexpr int kPX = 32, kPY = 32, kPT = 8;

// Stand-alone transfer of every member's coarse field after RK2 step
// `substep` of a block (substep < 0: between blocks), one tile per item
// (member, tile column, tile row, -) (noise_transfer.cu).
int launch_perturb_batched(const GocNoiseDesc* noise, const GocMemberDesc* members, const int4* items, int n_items,
                           const int* nsub, int substep, cudaStream_t stream);

// substep < 0: between blocks, the state of member m is buffer set 0 of the
// ensemble's device member table (-1: every member; -2: the members that
// take model error in the block just ended).  substep = k: right after RK2
// step k of a block, members that took step k hold their state in set
// (k + 1) % 2.  nsub: per member the block's steps if it takes model error,
// else 0.
__device__ __forceinline__ bool member_set(const int* nsub, int m, int substep, int* set) {
    if (substep < 0) {
        *set = 0;
        return substep == -1 || nsub[m] > 0;
    }
    if (substep >= nsub[m]) return false;
    *set = (substep + 1) & 1;
    return true;
}

}  // namespace goc
