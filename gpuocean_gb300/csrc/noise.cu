// Stochastic model error: random numbers, SOAR-correlated coarse field and
// its geostrophically balanced (bicubic) transfer to the ocean state.
//
// Semantics follow the reference kernels (K/ocean_noise.cu:126-666,
// K/random_number_generators.cu:1-134, K/interpolation.cu) and their build
// flags (--use_fast_math, S/OceanStateNoise.py:214-217): this translation
// unit is compiled with -use_fast_math as well.
#include <curand_kernel.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "noise_transfer.cuh"

namespace goc {

// ---------------------------------------------------------------------------
// random numbers
// ---------------------------------------------------------------------------

__device__ __forceinline__ unsigned long long lcg_next(unsigned long long s) {
    return (s * 1103515245ULL + 12345ULL) % 2147483647ULL;
}

// Two uniforms per seed (K/random_number_generators.cu:5-22); `normal`
// applies Box-Muller with a redraw when the first uniform is 0 (:35-52).
__global__ void lcg_kernel(int seed_nx, int seed_ny, int random_nx, unsigned long long* seeds, int seed_pitch,
                           float* random, int random_pitch, int normal) {
    const int ti = blockIdx.x * blockDim.x + threadIdx.x;
    const int tj = blockIdx.y * blockDim.y + threadIdx.y;
    if (ti >= seed_nx || tj >= seed_ny) return;
    unsigned long long* srow = seeds + (size_t)tj * seed_pitch;
    float* rrow = random + (size_t)tj * random_pitch;
    unsigned long long s = srow[ti];
    s = lcg_next(s);
    float u1 = (float)(s / 2147483648.0);
    s = lcg_next(s);
    float u2 = (float)(s / 2147483648.0);
    float a = u1, b = u2;
    if (normal) {
        if (u1 == 0.0f) {
            s = lcg_next(s);
            u1 = (float)(s / 2147483648.0);
            s = lcg_next(s);
            u2 = (float)(s / 2147483648.0);
        }
        const float r = sqrtf(-2.0f * logf(u1));
        a = r * cospif(2 * u2);
        b = r * sinpif(2 * u2);
    }
    srow[ti] = s;
    if (2 * ti < random_nx) rrow[2 * ti] = a;
    if (2 * ti + 1 < random_nx) rrow[2 * ti + 1] = b;
}

__global__ void xorwow_init_kernel(curandStateXORWOW_t* states, int n, unsigned long long seed) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) curand_init(seed, (unsigned long long)i, 0ULL, states + i);
}

__global__ void xorwow_normal_kernel(curandStateXORWOW_t* states, int nx, int ny, float* random, int pitch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx * ny) return;
    curandStateXORWOW_t st = states[i];
    random[(size_t)(i / nx) * pitch + (i % nx)] = curand_normal(&st);
    states[i] = st;
}

// ---------------------------------------------------------------------------
// SOAR coarse field (K/ocean_noise.cu:126-247)
// ---------------------------------------------------------------------------

__device__ __forceinline__ float soar_cov(int ax, int ay, int bx, int by, float dx, float dy, float q0, float L) {
    const float dist = sqrtf(dx * dx * (ax - bx) * (ax - bx) + dy * dy * (ay - by) * (ay - by));
    return q0 * (1.0f + dist / L) * expf(-dist / L);
}

__device__ __forceinline__ void soar_cell(const GocNoiseDesc& d, float scale, int additive, int ti, int tj,
                                          const float* __restrict__ random, float* coarse) {
    const int cnx = d.coarse_nx, cny = d.coarse_ny;
    if (ti >= cnx + 4 || tj >= cny + 4) return;
    float q = 0.0f;
    for (int b = 0; b < 5; ++b) {
        // xi row read by stencil row b of coarse cell tj
        const int r = d.periodic_ns ? ((tj + b - 4) % cny + cny) % cny : min(tj + b, cny + 7);
        const float* row = random + (size_t)r * (d.random_pitch / 4);
        for (int a = 0; a < 5; ++a) {
            const int c = d.periodic_ew ? ((ti + a - 4) % cnx + cnx) % cnx : min(ti + a, cnx + 7);
            q += soar_cov(2, 2, a, b, d.coarse_dx, d.coarse_dy, d.soar_q0, d.soar_L) * row[c];
        }
    }
    float* out = coarse + (size_t)tj * (d.coarse_pitch / 4) + ti;
    if (additive) *out += scale * q;
    else *out = scale * q;
}

__global__ void soar_kernel(GocNoiseDesc d, float scale, int additive) {
    soar_cell(d, scale, additive, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y,
              d.random, d.coarse);
}

// ---------------------------------------------------------------------------
// batched: the SOAR fields of all members in one launch (the transfer to the
// state is in noise_transfer.cu, or fused into the ensemble step)
// ---------------------------------------------------------------------------

constexpr int kNB = 16;                            // SOAR tile edge (coarse cells)

__global__ void soar_batched_active_kernel(const GocNoiseDesc* __restrict__ nd, const int4* __restrict__ items,
                                           const int* __restrict__ nsub, int substep, float scale) {
    const int4 it = items[blockIdx.x];
    int set;
    if (!member_set(nsub, it.x, substep, &set)) return;
    const GocNoiseDesc& d = nd[it.x];
    soar_cell(d, scale, 0, it.y * kNB + threadIdx.x, it.z * kNB + threadIdx.y, d.random, d.coarse);
}

// XORWOW normals for every member's random field; one state per element.
__global__ void xorwow_batched_kernel(const GocNoiseDesc* __restrict__ nd, const int4* __restrict__ chunks,
                                      curandStateXORWOW_t* states, const int* __restrict__ nsub, int substep) {
    const int4 c = chunks[blockIdx.x];   // (member, first element, count, first state)
    int set;
    if (!member_set(nsub, c.x, substep, &set)) return;
    const GocNoiseDesc& d = nd[c.x];
    const int rnx = d.periodic_ew ? d.coarse_nx : d.coarse_nx + 8;
    for (int q = threadIdx.x; q < c.z; q += blockDim.x) {
        const int e = c.y + q;
        curandStateXORWOW_t st = states[c.w + q];
        const float v = curand_normal(&st);
        states[c.w + q] = st;
        const_cast<float*>(d.random)[(size_t)(e / rnx) * (d.random_pitch / 4) + (e % rnx)] = v;
    }
}

__global__ void xorwow_batched_init_kernel(curandStateXORWOW_t* states, int n, unsigned long long seed) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) curand_init(seed, (unsigned long long)i, 0ULL, states + i);
}

// ---------------------------------------------------------------------------
// Karhunen-Loeve model error (K/ocean_noise.cu:666-954)
// ---------------------------------------------------------------------------
//
// The reference sums 2 Nx Ny terms per cell, each with two powers and two
// sines or cosines.  The sum separates: with a_n = n^-decay,
//   d_eta(x, y) = sum_j a_m(j) [ sin(2 pi m y_s) Bs_j(x) + cos(2 pi m y_c) Bc_j(x) ],
//   Bs_j(x) = sum_i r_sin[j][i] a_n(i) sin(2 pi n x_s)   (Bc likewise),
// so one launch tabulates Bs, Bc per column and the y factors per row, and
// the perturbation costs 2 Ny multiply-adds per cell.  Table layout (floats):
// Bs, Bc: [Ny][nx + 2]; As, Ac: [Ny][ny + 2]; column / row t stands for the
// full-array cell t + 1 (the interior plus one ghost cell on each side).

struct KLRoll {
    float xs, ys, xc, yc;
};

__host__ __device__ __forceinline__ int kl_count_x(const GocKLDesc& d) { return d.basis_x_end - d.basis_x_start + 1; }
__host__ __device__ __forceinline__ int kl_count_y(const GocKLDesc& d) { return d.basis_y_end - d.basis_y_start + 1; }

__device__ void kl_table_entry(const GocKLDesc& d, KLRoll r, int nx, int ny, int part, int t) {
    const int NX = kl_count_x(d), NY = kl_count_y(d);
    const int CX = nx + 2, RY = ny + 2;
    float* Bs = d.table;
    float* Bc = Bs + (size_t)NY * CX;
    float* As = Bc + (size_t)NY * CX;
    float* Ac = As + (size_t)NY * RY;
    const float* rns = d.random;
    const int rp = d.random_pitch / 4;
    if (part == 0) {
        if (t >= CX) return;
        // unit-square coordinate of full-array column t + 1, evaluated in
        // double as (ti + 0.5 - 2) / nx is in K/ocean_noise.cu:826
        const float x = (float)((t + 1 + 0.5 - 2) / nx);
        const float xs = x + r.xs, xc = x + r.xc;
        for (int j = 0; j < NY; ++j) {
            float bs = 0.0f, bc = 0.0f;
            for (int i = 0; i < NX; ++i) {
                const int n = d.basis_x_start + i;
                const float an = powf((float)n, -d.kl_decay);
                bs += rns[(size_t)j * rp + i] * an * sinpif(2 * n * xs);
                bc += rns[(size_t)(NY + j) * rp + i] * an * cospif(2 * n * xc);
            }
            Bs[(size_t)j * CX + t] = d.include_sin ? bs : 0.0f;
            Bc[(size_t)j * CX + t] = d.include_cos ? bc : 0.0f;
        }
    } else {
        if (t >= RY) return;
        const float y = (float)((t + 1 + 0.5 - 2) / ny);
        const float ys = y + r.ys, yc = y + r.yc;
        for (int j = 0; j < NY; ++j) {
            const int m = d.basis_y_start + j;
            const float am = powf((float)m, -d.kl_decay);
            As[(size_t)j * RY + t] = am * sinpif(2 * m * ys);
            Ac[(size_t)j * RY + t] = am * cospif(2 * m * yc);
        }
    }
}

constexpr int kKX = 32, kKY = 32;  // KL perturbation tile (interior cells)
constexpr int kKT = 8;             // thread rows: each thread owns kKY / kKT cells of a column
constexpr int kKR = kKY / kKT;
constexpr int kKLMaxRows = 32;     // basis rows staged in shared memory (more: read from the tables directly)

// kl_sample_eta / kl_sample_ocean_state on one tile with interior origin
// (bx, by): d_eta on the tile + 1 ring from the tables, then (unless
// eta_only) the geostrophically balanced hu, hv of K/ocean_noise.cu:901-947.
// The reference computes a dry-cell flag there and does not use it: land
// cells are perturbed as well.  Every thread loads the state and corner
// depths of its kKR cells first and the tile's slices of the tables are
// staged in shared memory, so the DRAM and L2 round trips overlap.
__device__ void kl_perturb_tile(const GocKLDesc& d, const OceanRef& o, float scale, int eta_only, int bx, int by) {
    __shared__ float s_d[kKY + 2][kKX + 2];
    __shared__ float s_bx[2][kKLMaxRows][kKX + 2];
    __shared__ float s_ay[2][kKLMaxRows][kKY + 2];
    const int NY = kl_count_y(d), CX = o.nx + 2, RY = o.ny + 2;
    const float* Bs = d.table;
    const float* Bc = Bs + (size_t)NY * CX;
    const float* As = Bc + (size_t)NY * CX;
    const float* Ac = As + (size_t)NY * RY;
    const float amp = scale * d.kl_scaling;
    const int tx = threadIdx.x, t = threadIdx.y * kKX + tx;
    const int ti = 2 + bx + tx;
    float e0[kKR], u0[kKR], v0[kKR], H_mid[kKR];
#pragma unroll
    for (int r = 0; r < kKR; ++r) {
        const int ty = threadIdx.y + r * kKT, tj = 2 + by + ty;
        e0[r] = u0[r] = v0[r] = H_mid[r] = 0.0f;
        if (ti < o.nx + 2 && tj < o.ny + 2) {
            const size_t k = (size_t)tj * o.pitch + ti;
            e0[r] = o.eta[k];
            if (!eta_only) {
                u0[r] = o.hu[k];
                v0[r] = o.hv[k];
                const float* h0 = o.Hi + (size_t)tj * o.hi_pitch + ti;
                const float* h1 = h0 + o.hi_pitch;
                H_mid[r] = 0.25f * (h0[0] + h0[1] + h1[0] + h1[1]);
            }
        }
    }
    const bool staged = NY <= kKLMaxRows;
    if (staged) {
        // rows (sine block, then cosine block) over the thread rows, columns over the lanes
        for (int wr = threadIdx.y; wr < 2 * NY; wr += kKT) {
            const int w = wr >= NY, r = wr - w * NY;
            const float* B = (w ? Bc : Bs) + (size_t)r * CX;
            const float* A = (w ? Ac : As) + (size_t)r * RY;
            for (int c = tx; c < kKX + 2; c += kKX) s_bx[w][r][c] = bx + c < CX ? B[bx + c] : 0.0f;
            for (int c = tx; c < kKY + 2; c += kKX) s_ay[w][r][c] = by + c < RY ? A[by + c] : 0.0f;
        }
        __syncthreads();
    }
    for (int q = t; q < (kKY + 2) * (kKX + 2); q += kKX * kKT) {
        const int i = q % (kKX + 2), j = q / (kKX + 2);
        const int cx = bx + i, ry = by + j;   // table column / row of full-array cell (1 + bx + i, 1 + by + j)
        float v = 0.0f;
        if (cx < CX && ry < RY) {
            if (staged) {
#pragma unroll 4
                for (int r = 0; r < NY; ++r) v += s_ay[0][r][j] * s_bx[0][r][i] + s_ay[1][r][j] * s_bx[1][r][i];
            } else {
                for (int r = 0; r < NY; ++r)
                    v += As[(size_t)r * RY + ry] * Bs[(size_t)r * CX + cx] + Ac[(size_t)r * RY + ry] * Bc[(size_t)r * CX + cx];
            }
            v *= amp;
        }
        s_d[j][i] = v;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kKR; ++r) {
        const int ty = threadIdx.y + r * kKT, tj = 2 + by + ty;
        if (ti >= o.nx + 2 || tj >= o.ny + 2) continue;
        const float de = s_d[ty + 1][tx + 1];
        if (eta_only) {
            o.eta[(size_t)tj * o.pitch + ti] = e0[r] + de;
        } else {
            const float cor = noise_coriolis(d, o, ti, tj);
            const float ex = (s_d[ty + 1][tx + 2] - s_d[ty + 1][tx]) / (2.0f * o.dx);
            const float ey = (s_d[ty + 2][tx + 1] - s_d[ty][tx + 1]) / (2.0f * o.dy);
            const float dhu = -(d.g / cor) * (H_mid[r] + de) * ey;
            const float dhv = (d.g / cor) * (H_mid[r] + de) * ex;
            store_cell(o, ti, tj, e0[r] + de, u0[r] + dhu, v0[r] + dhv);
        }
    }
    __syncthreads();
}

__global__ void kl_table_kernel(GocKLDesc d, int nx, int ny) {
    kl_table_entry(d, KLRoll{d.roll_x_sin, d.roll_y_sin, d.roll_x_cos, d.roll_y_cos}, nx, ny, blockIdx.y,
                   blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void __launch_bounds__(kKX * kKT, 4) kl_perturb_kernel(GocKLDesc d, OceanRef o, float scale, int eta_only) {
    kl_perturb_tile(d, o, scale, eta_only, blockIdx.x * kKX, blockIdx.y * kKY);
}

// batched: member m uses the normals and rollers of member src[m]
__global__ void kl_table_batched_kernel(const GocKLDesc* __restrict__ kl, const int* __restrict__ src,
                                        const float4* __restrict__ rollers, int n, int roll_set,
                                        const GocMemberDesc* __restrict__ mem, const int4* __restrict__ items,
                                        const int* __restrict__ nsub, int substep) {
    const int4 it = items[blockIdx.x];   // (member, part, first entry, 0)
    int set;
    if (!member_set(nsub, it.x, substep, &set)) return;
    const float4 r = rollers[(size_t)roll_set * n + src[it.x]];
    kl_table_entry(kl[it.x], KLRoll{r.x, r.y, r.z, r.w}, mem[it.x].p.nx, mem[it.x].p.ny, it.y, it.z + threadIdx.x);
}

__global__ void __launch_bounds__(kKX * kKT, 4)
kl_perturb_batched_kernel(const GocKLDesc* __restrict__ kl, const GocMemberDesc* __restrict__ mem,
                                          const int4* __restrict__ items, const int* __restrict__ nsub, int substep,
                                          float scale) {
    const int4 it = items[blockIdx.x];   // (member, tile x, tile y, 0)
    int set;
    if (!member_set(nsub, it.x, substep, &set)) return;
    const GocMemberDesc& m = mem[it.x];
    const OceanRef o{m.p.nx, m.p.ny, m.p.dx, m.p.dy, m.eta[set], m.hu[set], m.hv[set], m.pitch / 4, m.Hi,
                     m.Hi_pitch / 4, m.p.land_value, m.p.bc_north == 2, m.p.bc_east == 2};
    kl_perturb_tile(kl[it.x], o, scale, 0, it.y * kKX, it.z * kKY);
}

// XORWOW normals into the source members' fields; chunk = (member, first
// element, count, first state)
__global__ void kl_xorwow_batched_kernel(const GocKLDesc* __restrict__ kl, const int4* __restrict__ chunks,
                                         curandStateXORWOW_t* states, const int* __restrict__ nsub, int substep) {
    const int4 c = chunks[blockIdx.x];
    int set;
    if (!member_set(nsub, c.x, substep, &set)) return;
    const GocKLDesc& d = kl[c.x];
    const int NX = kl_count_x(d);
    float* rnd = const_cast<float*>(d.random);
    for (int q = threadIdx.x; q < c.z; q += blockDim.x) {
        const int e = c.y + q;
        curandStateXORWOW_t st = states[c.w + q];
        rnd[(size_t)(e / NX) * (d.random_pitch / 4) + e % NX] = curand_normal(&st);
        states[c.w + q] = st;
    }
}

// Roller set of a perturbation at `substep`: 0 for the perturbations after a
// block (substep -1: all members, -2: the members that stepped), k + 1 after
// RK2 step k of a block.
__host__ __device__ __forceinline__ int kl_roll_set(int substep) { return substep < 0 ? 0 : substep + 1; }

// Rollers of the source members that perturb at `substep`, drawn on the
// device (one XORWOW state per member) into roller set kl_roll_set(substep).
__global__ void kl_roll_batched_kernel(const int* __restrict__ src, curandStateXORWOW_t* states, float4* rollers,
                                       int n, const int* __restrict__ nsub, int substep) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    int set;
    if (m >= n || src[m] != m || !member_set(nsub, m, substep, &set)) return;
    curandStateXORWOW_t st = states[m];
    const float a = curand_uniform(&st), b = curand_uniform(&st), c = curand_uniform(&st), d = curand_uniform(&st);
    rollers[(size_t)kl_roll_set(substep) * n + m] = make_float4(a, b, c, d);
    states[m] = st;
}

}  // namespace goc

using namespace goc;

static int check_noise(const GocNoiseDesc* d, const char* who) {
    if (!d) return set_error(GOC_ERR_ARG, "%s: null noise descriptor", who);
    if (d->coarse_nx < 1 || d->coarse_ny < 1 || !(d->coarse_dx > 0) || !(d->coarse_dy > 0) || !(d->soar_L > 0))
        return set_error(GOC_ERR_ARG, "%s: bad coarse grid", who);
    if (!d->random || !d->coarse) return set_error(GOC_ERR_ARG, "%s: null random/coarse buffer", who);
    if (d->coarse_pitch < (d->coarse_nx + 4) * 4 || d->random_pitch < 4)
        return set_error(GOC_ERR_ARG, "%s: pitch too small", who);
    if (d->interpolation_factor < 1) return set_error(GOC_ERR_ARG, "%s: interpolation factor must be >= 1", who);
    return GOC_OK;
}

extern "C" int goc_lcg_fill(int seed_nx, int seed_ny, int random_nx, unsigned long long* seeds, int seed_pitch,
                            float* random, int random_pitch, int normal, void* stream) {
    if (seed_nx < 1 || seed_ny < 1 || random_nx < 1 || random_nx > 2 * seed_nx || !seeds || !random ||
        seed_pitch < seed_nx * 8 || random_pitch < random_nx * 4 || seed_pitch % 8 || random_pitch % 4)
        return set_error(GOC_ERR_ARG, "goc_lcg_fill: bad arguments");
    dim3 blk(16, 16), grd((seed_nx + 15) / 16, (seed_ny + 15) / 16);
    lcg_kernel<<<grd, blk, 0, as_stream(stream)>>>(seed_nx, seed_ny, random_nx, seeds, seed_pitch / 8, random,
                                                   random_pitch / 4, normal);
    count_launch();
    return check_launch("lcg_kernel");
}

extern "C" size_t goc_xorwow_state_bytes(int n) { return (size_t)(n > 0 ? n : 0) * sizeof(curandStateXORWOW_t); }

extern "C" int goc_xorwow_init(void* states, int n, unsigned long long seed, void* stream) {
    if (!states || n < 1) return set_error(GOC_ERR_ARG, "goc_xorwow_init: bad arguments");
    xorwow_init_kernel<<<(n + 127) / 128, 128, 0, as_stream(stream)>>>((curandStateXORWOW_t*)states, n, seed);
    count_launch();
    return check_launch("xorwow_init_kernel");
}

extern "C" int goc_xorwow_normal(void* states, int nx, int ny, float* random, int random_pitch, void* stream) {
    if (!states || !random || nx < 1 || ny < 1 || random_pitch < nx * 4 || random_pitch % 4)
        return set_error(GOC_ERR_ARG, "goc_xorwow_normal: bad arguments");
    const int n = nx * ny;
    xorwow_normal_kernel<<<(n + 127) / 128, 128, 0, as_stream(stream)>>>((curandStateXORWOW_t*)states, nx, ny,
                                                                         random, random_pitch / 4);
    count_launch();
    return check_launch("xorwow_normal_kernel");
}

extern "C" int goc_soar(const GocNoiseDesc* d, float perturbation_scale, int additive, void* stream) {
    int rc = check_noise(d, "goc_soar");
    if (rc) return rc;
    dim3 blk(kNB, kNB), grd((d->coarse_nx + 4 + kNB - 1) / kNB, (d->coarse_ny + 4 + kNB - 1) / kNB);
    soar_kernel<<<grd, blk, 0, as_stream(stream)>>>(*d, perturbation_scale, additive);
    count_launch();
    return check_launch("soar_kernel");
}

// ---------------------------------------------------------------------------
// batched handle
// ---------------------------------------------------------------------------

struct NoiseBatch {
    int n = 0;
    GocNoiseDesc* d_noise = nullptr;
    int4* d_soar_items = nullptr;
    int4* d_pert_items = nullptr;
    int4* d_rng_chunks = nullptr;
    curandStateXORWOW_t* d_states = nullptr;
    int n_soar = 0, n_pert = 0, n_rng = 0, n_states = 0;
};

extern "C" int goc_noise_batch_create(void* ensemble, const GocNoiseDesc* noise, void** out) {
    if (!out || !noise || !ensemble) return set_error(GOC_ERR_ARG, "goc_noise_batch_create: bad arguments");
    *out = nullptr;
    int n_members = 0;
    const GocMemberDesc* members = ensemble_host_members(ensemble, &n_members);
    NoiseBatch* b = new NoiseBatch();
    b->n = n_members;
    std::vector<int4> soar, pert, rng;
    int states = 0;
    for (int m = 0; m < n_members; ++m) {
        int rc = check_noise(&noise[m], "goc_noise_batch_create");
        const GocMemberDesc& md = members[m];
        if (!rc && noise[m].interpolation_factor <= 1 &&
            (noise[m].coarse_nx != md.p.nx || noise[m].coarse_ny != md.p.ny))
            rc = set_error(GOC_ERR_ARG, "goc_noise_batch_create: member %d: factor 1 needs the coarse grid = the grid", m);
        if (rc) {
            delete b;
            return rc;
        }
        for (int j = 0; j < (noise[m].coarse_ny + 4 + kNB - 1) / kNB; ++j)
            for (int i = 0; i < (noise[m].coarse_nx + 4 + kNB - 1) / kNB; ++i) soar.push_back(make_int4(m, i, j, 0));
        for (int j = 0; j < (md.p.ny + kPY - 1) / kPY; ++j)
            for (int i = 0; i < (md.p.nx + kPX - 1) / kPX; ++i) pert.push_back(make_int4(m, i, j, 0));
        const int rnx = noise[m].periodic_ew ? noise[m].coarse_nx : noise[m].coarse_nx + 8;
        const int rny = noise[m].periodic_ns ? noise[m].coarse_ny : noise[m].coarse_ny + 8;
        for (int f = 0; f < rnx * rny; f += 256) {
            const int cnt = std::min(256, rnx * rny - f);
            rng.push_back(make_int4(m, f, cnt, states));
            states += cnt;
        }
    }
    b->n_soar = (int)soar.size();
    b->n_pert = (int)pert.size();
    b->n_rng = (int)rng.size();
    b->n_states = states;
    cudaError_t e = cudaMalloc(&b->d_noise, sizeof(GocNoiseDesc) * n_members);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_soar_items, sizeof(int4) * soar.size());
    if (e == cudaSuccess) e = cudaMalloc(&b->d_pert_items, sizeof(int4) * pert.size());
    if (e == cudaSuccess) e = cudaMalloc(&b->d_rng_chunks, sizeof(int4) * rng.size());
    if (e == cudaSuccess) e = cudaMemcpy(b->d_noise, noise, sizeof(GocNoiseDesc) * n_members, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_soar_items, soar.data(), sizeof(int4) * soar.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_pert_items, pert.data(), sizeof(int4) * pert.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_rng_chunks, rng.data(), sizeof(int4) * rng.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(b->d_noise); cudaFree(b->d_soar_items); cudaFree(b->d_pert_items); cudaFree(b->d_rng_chunks);
        delete b;
        return set_error(GOC_ERR_CUDA, "goc_noise_batch_create: %s", cudaGetErrorString(e));
    }
    *out = b;
    return GOC_OK;
}

namespace goc {
const GocNoiseDesc* noise_batch_device_desc(void* batch, int* n_members) {
    NoiseBatch* b = static_cast<NoiseBatch*>(batch);
    if (n_members) *n_members = b->n;
    return b->d_noise;
}
}  // namespace goc

extern "C" int goc_noise_batch_destroy(void* batch) {
    if (!batch) return GOC_OK;
    NoiseBatch* b = static_cast<NoiseBatch*>(batch);
    cudaFree(b->d_noise);
    cudaFree(b->d_soar_items);
    cudaFree(b->d_pert_items);
    cudaFree(b->d_rng_chunks);
    cudaFree(b->d_states);
    delete b;
    return GOC_OK;
}

extern "C" int goc_noise_batch_seed(void* batch, unsigned long long seed, void* stream) {
    if (!batch) return set_error(GOC_ERR_ARG, "goc_noise_batch_seed: null handle");
    NoiseBatch* b = static_cast<NoiseBatch*>(batch);
    if (!b->d_states) {
        cudaError_t e = cudaMalloc(&b->d_states, sizeof(curandStateXORWOW_t) * (size_t)b->n_states);
        if (e != cudaSuccess) return set_error(GOC_ERR_CUDA, "goc_noise_batch_seed: %s", cudaGetErrorString(e));
    }
    xorwow_batched_init_kernel<<<(b->n_states + 127) / 128, 128, 0, as_stream(stream)>>>(b->d_states, b->n_states, seed);
    count_launch();
    return check_launch("xorwow_batched_init_kernel");
}

extern "C" int goc_noise_batch_generate(void* batch, void* ensemble, int substep, void* stream) {
    if (!batch || !ensemble) return set_error(GOC_ERR_ARG, "goc_noise_batch_generate: null handle");
    NoiseBatch* b = static_cast<NoiseBatch*>(batch);
    if (!b->d_states) return set_error(GOC_ERR_ARG, "goc_noise_batch_generate: call goc_noise_batch_seed first");
    xorwow_batched_kernel<<<b->n_rng, 256, 0, as_stream(stream)>>>(b->d_noise, b->d_rng_chunks, b->d_states,
                                                                 ensemble_device_noise_steps(ensemble), substep);
    count_launch();
    return check_launch("xorwow_batched_kernel");
}

extern "C" int goc_noise_batch_field(void* batch, void* ensemble, float perturbation_scale, int substep,
                                     void* stream) {
    if (!batch || !ensemble) return set_error(GOC_ERR_ARG, "goc_noise_batch_field: null handle");
    NoiseBatch* b = static_cast<NoiseBatch*>(batch);
    int n = 0;
    ensemble_host_members(ensemble, &n);
    if (n != b->n) return set_error(GOC_ERR_ARG, "goc_noise_batch_field: ensemble has %d members, batch %d", n, b->n);
    soar_batched_active_kernel<<<b->n_soar, dim3(kNB, kNB), 0, as_stream(stream)>>>(
        b->d_noise, b->d_soar_items, ensemble_device_noise_steps(ensemble), substep, perturbation_scale);
    count_launch();
    return check_launch("soar_batched_active_kernel");
}

extern "C" int goc_noise_batch_perturb(void* batch, void* ensemble, float perturbation_scale, int substep,
                                       void* stream) {
    if (!batch || !ensemble) return set_error(GOC_ERR_ARG, "goc_noise_batch_perturb: null handle");
    NoiseBatch* b = static_cast<NoiseBatch*>(batch);
    int n = 0;
    ensemble_host_members(ensemble, &n);
    if (n != b->n) return set_error(GOC_ERR_ARG, "goc_noise_batch_perturb: ensemble has %d members, batch %d", n, b->n);
    cudaStream_t st = as_stream(stream);
    const int* nsub = ensemble_device_noise_steps(ensemble);
    soar_batched_active_kernel<<<b->n_soar, dim3(kNB, kNB), 0, st>>>(b->d_noise, b->d_soar_items, nsub, substep,
                                                                     perturbation_scale);
    count_launch();
    int rc = check_launch("soar_batched_active_kernel");
    if (rc) return rc;
    return launch_perturb_batched(b->d_noise, ensemble_device_members(ensemble), b->d_pert_items, b->n_pert, nsub,
                                  substep, st);
}

// ---------------------------------------------------------------------------
// Karhunen-Loeve model error: entry points
// ---------------------------------------------------------------------------

static int cuda_rc(cudaError_t e, const char* what) {
    return e == cudaSuccess ? GOC_OK : set_error(GOC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

static int check_kl(const GocKLDesc* d, int nx, int ny, const char* who) {
    if (!d) return set_error(GOC_ERR_ARG, "%s: null descriptor", who);
    if (nx < 1 || ny < 1) return set_error(GOC_ERR_ARG, "%s: bad grid", who);
    if (d->basis_x_start < 0 || d->basis_y_start < 0 || kl_count_x(*d) < 1 || kl_count_y(*d) < 1)
        return set_error(GOC_ERR_ARG, "%s: bad basis ranges", who);
    if (kl_count_x(*d) * kl_count_y(*d) > 1 << 20) return set_error(GOC_ERR_ARG, "%s: too many basis functions", who);
    return GOC_OK;
}

extern "C" long long goc_kl_table_floats(int nx, int ny, const GocKLDesc* kl) {
    if (check_kl(kl, nx, ny, "goc_kl_table_floats")) return GOC_ERR_ARG;
    return 2LL * kl_count_y(*kl) * ((long long)(nx + 2) + (ny + 2));
}

extern "C" int goc_kl_perturb(const GocKLDesc* kl, int nx, int ny, float dx, float dy, float perturbation_scale,
                              int eta_only, float* eta, float* hu, float* hv, int pitch, const float* Hi, int Hi_pitch,
                              int periodic_ns, int periodic_ew, void* stream) {
    int rc = check_kl(kl, nx, ny, "goc_kl_perturb");
    if (rc) return rc;
    if (!kl->table || !kl->random || kl->random_pitch < 4 * kl_count_x(*kl) || kl->random_pitch % 4)
        return set_error(GOC_ERR_ARG, "goc_kl_perturb: table or random field missing");
    if (!eta_only && !kl->coriolis_f && kl->f == 0.0f)
        return set_error(GOC_ERR_ARG, "goc_kl_perturb: f = 0 needs the Coriolis texture");
    OceanRef o;
    if (eta_only) {
        if (!eta || pitch < (nx + 4) * 4 || pitch % 4) return set_error(GOC_ERR_ARG, "goc_kl_perturb: bad eta");
        o = OceanRef{nx, ny, dx, dy, eta, nullptr, nullptr, pitch / 4, nullptr, 0, 0.0f, 0, 0};
    } else if ((rc = make_ocean(nx, ny, dx, dy, eta, hu, hv, pitch, Hi, Hi_pitch, 0.0f, periodic_ns, periodic_ew, &o,
                                "goc_kl_perturb"))) {
        return rc;
    }
    cudaStream_t st = as_stream(stream);
    const int ntab = std::max(nx, ny) + 2;
    kl_table_kernel<<<dim3((ntab + 127) / 128, 2), 128, 0, st>>>(*kl, nx, ny);
    count_launch();
    if ((rc = check_launch("kl_table_kernel"))) return rc;
    dim3 grd((nx + kKX - 1) / kKX, (ny + kKY - 1) / kKY);
    kl_perturb_kernel<<<grd, dim3(kKX, kKT), 0, st>>>(*kl, o, perturbation_scale, eta_only);
    count_launch();
    return check_launch("kl_perturb_kernel");
}

struct KLBatch {
    int n = 0, max_sets = 0;
    GocKLDesc* d_kl = nullptr;
    int* d_src = nullptr;
    float4* d_rollers = nullptr;
    float* d_arena = nullptr;                   // tables and random fields
    int4* d_tab_items = nullptr;
    int4* d_tile_items = nullptr;
    int4* d_rng_chunks = nullptr;
    curandStateXORWOW_t* d_states = nullptr;       // normals, then one roller state per member
    int n_tab = 0, n_tile = 0, n_rng = 0, n_states = 0;
    std::vector<GocKLDesc> host;
    std::vector<int> src;
};

static void kl_batch_free(KLBatch* b) {
    cudaFree(b->d_kl); cudaFree(b->d_src); cudaFree(b->d_rollers); cudaFree(b->d_arena);
    cudaFree(b->d_tab_items); cudaFree(b->d_tile_items); cudaFree(b->d_rng_chunks); cudaFree(b->d_states);
    delete b;
}

extern "C" int goc_kl_batch_create(void* ensemble, const GocKLDesc* kl, const int* source, int max_sets, void** out) {
    if (!out || !kl || !source || !ensemble || max_sets < 1)
        return set_error(GOC_ERR_ARG, "goc_kl_batch_create: bad arguments");
    *out = nullptr;
    int n = 0;
    const GocMemberDesc* members = ensemble_host_members(ensemble, &n);
    for (int m = 0; m < n; ++m) {
        const GocKLDesc& d = kl[m];
        int rc = check_kl(&d, members[m].p.nx, members[m].p.ny, "goc_kl_batch_create");
        if (rc) return rc;
        const int s = source[m];
        if (s < 0 || s >= n || source[s] != s)
            return set_error(GOC_ERR_ARG, "goc_kl_batch_create: member %d: source %d is not its own source", m, s);
        if (kl_count_x(kl[s]) != kl_count_x(d) || kl_count_y(kl[s]) != kl_count_y(d))
            return set_error(GOC_ERR_ARG, "goc_kl_batch_create: member %d and its source differ in basis size", m);
        if (d.f == 0.0f && !d.coriolis_f)
            return set_error(GOC_ERR_ARG, "goc_kl_batch_create: member %d: f = 0 needs the Coriolis texture", m);
    }
    KLBatch* b = new KLBatch();
    b->n = n;
    b->max_sets = max_sets;
    b->host.assign(kl, kl + n);
    b->src.assign(source, source + n);
    // arena: every member's tables, then the source members' random fields
    std::vector<size_t> tab_off(n), rnd_off(n, 0);
    size_t off = 0;
    for (int m = 0; m < n; ++m) {
        tab_off[m] = off;
        off += (size_t)goc_kl_table_floats(members[m].p.nx, members[m].p.ny, &kl[m]);
        off = (off + 31) & ~(size_t)31;
    }
    std::vector<int4> tab, tile, rng;
    int states = 0;
    for (int m = 0; m < n; ++m) {
        if (source[m] == m) {
            rnd_off[m] = off;
            const int cnt = 2 * kl_count_y(kl[m]) * kl_count_x(kl[m]);
            off += ((size_t)cnt + 31) & ~(size_t)31;
            for (int f = 0; f < cnt; f += 256) {
                const int c = std::min(256, cnt - f);
                rng.push_back(make_int4(m, f, c, states));
                states += c;
            }
        }
        const int nx = members[m].p.nx, ny = members[m].p.ny;
        for (int t = 0; t < nx + 2; t += 128) tab.push_back(make_int4(m, 0, t, 0));
        for (int t = 0; t < ny + 2; t += 128) tab.push_back(make_int4(m, 1, t, 0));
        for (int j = 0; j < (ny + kKY - 1) / kKY; ++j)
            for (int i = 0; i < (nx + kKX - 1) / kKX; ++i) tile.push_back(make_int4(m, i, j, 0));
    }
    b->n_tab = (int)tab.size();
    b->n_tile = (int)tile.size();
    b->n_rng = (int)rng.size();
    b->n_states = states;
    cudaError_t e = cudaMalloc(&b->d_arena, off * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(b->d_arena, 0, off * sizeof(float));
    for (int m = 0; m < n; ++m) {
        b->host[m].table = b->d_arena + tab_off[m];
        b->host[m].random = b->d_arena + rnd_off[source[m]];
        b->host[m].random_pitch = 4 * kl_count_x(kl[m]);
    }
    if (e == cudaSuccess) e = cudaMalloc(&b->d_kl, sizeof(GocKLDesc) * n);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_src, sizeof(int) * n);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_rollers, sizeof(float4) * (size_t)n * max_sets);
    if (e == cudaSuccess) e = cudaMemset(b->d_rollers, 0, sizeof(float4) * (size_t)n * max_sets);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_tab_items, sizeof(int4) * tab.size());
    if (e == cudaSuccess) e = cudaMalloc(&b->d_tile_items, sizeof(int4) * tile.size());
    if (e == cudaSuccess && !rng.empty()) e = cudaMalloc(&b->d_rng_chunks, sizeof(int4) * rng.size());
    if (e == cudaSuccess) e = cudaMemcpy(b->d_kl, b->host.data(), sizeof(GocKLDesc) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_src, source, sizeof(int) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_tab_items, tab.data(), sizeof(int4) * tab.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_tile_items, tile.data(), sizeof(int4) * tile.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !rng.empty())
        e = cudaMemcpy(b->d_rng_chunks, rng.data(), sizeof(int4) * rng.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        kl_batch_free(b);
        return set_error(GOC_ERR_CUDA, "goc_kl_batch_create: %s", cudaGetErrorString(e));
    }
    *out = b;
    return GOC_OK;
}

extern "C" int goc_kl_batch_destroy(void* batch) {
    if (batch) kl_batch_free(static_cast<KLBatch*>(batch));
    return GOC_OK;
}

extern "C" int goc_kl_batch_seed(void* batch, unsigned long long seed, void* stream) {
    if (!batch) return set_error(GOC_ERR_ARG, "goc_kl_batch_seed: null handle");
    KLBatch* b = static_cast<KLBatch*>(batch);
    const int total = b->n_states + b->n;
    if (!b->d_states) {
        cudaError_t e = cudaMalloc(&b->d_states, sizeof(curandStateXORWOW_t) * (size_t)total);
        if (e != cudaSuccess) return set_error(GOC_ERR_CUDA, "goc_kl_batch_seed: %s", cudaGetErrorString(e));
    }
    xorwow_batched_init_kernel<<<(total + 127) / 128, 128, 0, as_stream(stream)>>>(b->d_states, total, seed);
    count_launch();
    return check_launch("xorwow_batched_init_kernel");
}

extern "C" int goc_kl_batch_generate(void* batch, void* ensemble, int substep, void* stream) {
    if (!batch || !ensemble) return set_error(GOC_ERR_ARG, "goc_kl_batch_generate: null handle");
    KLBatch* b = static_cast<KLBatch*>(batch);
    if (!b->d_states) return set_error(GOC_ERR_ARG, "goc_kl_batch_generate: call goc_kl_batch_seed first");
    if (substep < -2 || kl_roll_set(substep) >= b->max_sets)
        return set_error(GOC_ERR_ARG, "goc_kl_batch_generate: substep %d outside the roller sets", substep);
    cudaStream_t st = as_stream(stream);
    const int* nsub = ensemble_device_noise_steps(ensemble);
    if (b->n_rng > 0) {
        kl_xorwow_batched_kernel<<<b->n_rng, 256, 0, st>>>(b->d_kl, b->d_rng_chunks, b->d_states, nsub, substep);
        count_launch();
        int rc = check_launch("kl_xorwow_batched_kernel");
        if (rc) return rc;
    }
    kl_roll_batched_kernel<<<(b->n + 127) / 128, 128, 0, st>>>(b->d_src, b->d_states + b->n_states, b->d_rollers,
                                                               b->n, nsub, substep);
    count_launch();
    return check_launch("kl_roll_batched_kernel");
}

extern "C" int goc_kl_batch_set_rollers(void* batch, const float* rollers, int n_sets, void* stream) {
    if (!batch || !rollers) return set_error(GOC_ERR_ARG, "goc_kl_batch_set_rollers: null argument");
    KLBatch* b = static_cast<KLBatch*>(batch);
    if (n_sets < 1 || n_sets > b->max_sets)
        return set_error(GOC_ERR_ARG, "goc_kl_batch_set_rollers: %d sets, room for %d", n_sets, b->max_sets);
    return cuda_rc(cudaMemcpyAsync(b->d_rollers, rollers, sizeof(float4) * (size_t)b->n * n_sets,
                                   cudaMemcpyHostToDevice, as_stream(stream)),
                   "goc_kl_batch_set_rollers");
}

extern "C" int goc_kl_batch_set_random(void* batch, int member, const float* host_normals, void* stream) {
    if (!batch || !host_normals) return set_error(GOC_ERR_ARG, "goc_kl_batch_set_random: null argument");
    KLBatch* b = static_cast<KLBatch*>(batch);
    if (member < 0 || member >= b->n) return set_error(GOC_ERR_ARG, "goc_kl_batch_set_random: bad member");
    const GocKLDesc& d = b->host[b->src[member]];
    const size_t bytes = sizeof(float) * 2 * kl_count_y(d) * kl_count_x(d);
    return cuda_rc(cudaMemcpyAsync(const_cast<float*>(d.random), host_normals, bytes, cudaMemcpyHostToDevice,
                                   as_stream(stream)),
                   "goc_kl_batch_set_random");
}

extern "C" int goc_kl_batch_perturb(void* batch, void* ensemble, float perturbation_scale, int substep, void* stream) {
    if (!batch || !ensemble) return set_error(GOC_ERR_ARG, "goc_kl_batch_perturb: null handle");
    KLBatch* b = static_cast<KLBatch*>(batch);
    int n = 0;
    ensemble_host_members(ensemble, &n);
    if (n != b->n) return set_error(GOC_ERR_ARG, "goc_kl_batch_perturb: ensemble has %d members, batch %d", n, b->n);
    if (substep < -2 || kl_roll_set(substep) >= b->max_sets)
        return set_error(GOC_ERR_ARG, "goc_kl_batch_perturb: substep %d outside the roller sets", substep);
    cudaStream_t st = as_stream(stream);
    const int* nsub = ensemble_device_noise_steps(ensemble);
    const GocMemberDesc* dm = ensemble_device_members(ensemble);
    kl_table_batched_kernel<<<b->n_tab, 128, 0, st>>>(b->d_kl, b->d_src, b->d_rollers, b->n, kl_roll_set(substep), dm,
                                                      b->d_tab_items, nsub, substep);
    count_launch();
    int rc = check_launch("kl_table_batched_kernel");
    if (rc) return rc;
    kl_perturb_batched_kernel<<<b->n_tile, dim3(kKX, kKT), 0, st>>>(b->d_kl, dm, b->d_tile_items, nsub, substep,
                                                                    perturbation_scale);
    count_launch();
    return check_launch("kl_perturb_batched_kernel");
}
