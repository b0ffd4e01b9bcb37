// Open (sponge) boundaries of an (eta, hu, hv) state with two ghost cells:
// linear interpolation (flag 4) and the flow relaxation scheme (flag 3),
// K/boundary_kernels.cu:250-541, called as BoundaryConditionsArakawaA.
// boundaryCondition calls them (U/Common.py:1310-1350): the north-south pair
// first, then east-west.
//
// The sponge of a side spans the outermost sponge_cells rows (columns) of the
// (ny+4) x (nx+4) array, ghost cells included.  Linear interpolation keeps
// the outermost row and the first row inside the sponge and interpolates the
// rows between them; the flow relaxation scheme blends every sponge row with
// the exterior solution, time-interpolated between two data sets and read
// from (2 x n x 3) channel-interleaved arrays by bilinear lookup.
//
// This translation unit is built with CUDA's default (IEEE) arithmetic, as the
// reference builds its boundary kernels.
#include "common.cuh"

namespace goc {

struct SpongeGrid {
    int nx, ny;          // interior cells
    int bc_north, bc_south, bc_east, bc_west;
    int sp_north, sp_south, sp_east, sp_west;
    float* eta; float* hu; float* hv;
    int pitch;           // floats
};

// Bilinear lookup of three interleaved channels, texel-centred normalised
// coordinates clamped to [0, 1] (K/interpolation.cu:193-262).
__device__ __forceinline__ float3 bilinear3(const float* __restrict__ data, int dnx, int dny, float s, float t) {
    s = __saturatef(s - 0.5f / dnx);
    t = __saturatef(t - 0.5f / dny);
    const float x = s * dnx, y = t * dny;
    const int x0 = min((int)floorf(x), dnx - 1), y0 = min((int)floorf(y), dny - 1);
    const float fx = x - x0, fy = y - y0;
    const int x1 = min(x0 + 1, dnx - 1), y1 = min(y0 + 1, dny - 1);
    float r[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float d00 = data[(y0 * dnx + x0) * 3 + c], d01 = data[(y0 * dnx + x1) * 3 + c];
        const float d10 = data[(y1 * dnx + x0) * 3 + c], d11 = data[(y1 * dnx + x1) * 3 + c];
        r[c] = d00 + fx * (d01 - d00) + fy * (d10 - d00) + fx * fy * (d00 + d11 - d01 - d10);
    }
    return make_float3(r[0], r[1], r[2]);
}

__device__ __forceinline__ float* at(float* p, int pitch, int j, int i) { return p + (size_t)j * pitch + i; }

// The reference's boundary kernels write p*q + r*s and get the first product
// rounded and the second fused into the sum: fma(r, s, p*q).
__device__ __forceinline__ float mul_add_mul(float p, float q, float r, float s) {
    return __fmaf_rn(r, s, __fmul_rn(p, q));
}
// (1 - w) * b + w * a (the relaxation, K/boundary_kernels.cu:467-469) and
// w * a + (1 - w) * b (the time interpolation of the exterior data, :457-459)
__device__ __forceinline__ float relax(float w, float a, float b) { return mul_add_mul(1.0f - w, b, w, a); }
__device__ __forceinline__ float time_interp(float w, float next, float cur) { return mul_add_mul(w, next, 1.0f - w, cur); }

// Relaxation weight 1 - tanh(max(0, d) / 2) of the cell d rows inside the sponge.
__device__ __forceinline__ float relaxation_weight(float d) { return 1.0f - tanhf(fmaxf(0.0f, d) / 2.0f); }

// linear interpolation between the outer row (0 or ny + 3) and the inner
// row sponge_cells (or ny + 3 - sponge_cells) of the same side
__global__ void sponge_linear_ns_kernel(SpongeGrid g) {
    const int ti = blockIdx.x * blockDim.x + threadIdx.x, tj = blockIdx.y * blockDim.y + threadIdx.y;
    const int top = g.ny + 3;
    const bool south = g.bc_south == 4 && tj < g.sp_south && tj > 0;
    const bool north = g.bc_north == 4 && tj > top - g.sp_north && tj < top;
    if (!((south || north) && ti > 0 && ti < g.nx + 3)) return;
    int inner = g.sp_south, outer = 0;
    if (tj > g.sp_south) {
        inner = top - g.sp_north;
        outer = top;
    }
    const float ratio = (float)(tj - outer) / (inner - outer);
    float* q[3] = {g.eta, g.hu, g.hv};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float vi = *at(q[c], g.pitch, inner, ti), vo = *at(q[c], g.pitch, outer, ti);
        *at(q[c], g.pitch, tj, ti) = vo + ratio * (vi - vo);
    }
}

__global__ void sponge_linear_ew_kernel(SpongeGrid g) {
    const int ti = blockIdx.x * blockDim.x + threadIdx.x, tj = blockIdx.y * blockDim.y + threadIdx.y;
    const int right = g.nx + 3;
    const bool west = g.bc_west == 4 && ti < g.sp_west && ti > 0;
    const bool east = g.bc_east == 4 && ti > right - g.sp_east && ti < right;
    if (!((west || east) && tj > 0 && tj < g.ny + 3)) return;
    int inner = g.sp_west, outer = 0;
    if (ti > g.sp_west) {
        inner = right - g.sp_east;
        outer = right;
    }
    const float ratio = (float)(ti - outer) / (inner - outer);
    float* q[3] = {g.eta, g.hu, g.hv};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float vi = *at(q[c], g.pitch, tj, inner), vo = *at(q[c], g.pitch, tj, outer);
        *at(q[c], g.pitch, tj, ti) = vo + ratio * (vi - vo);
    }
}

// flow relaxation: weight alpha = 1 - tanh(max(0, d) / 2) towards the
// exterior solution, d the distance from the outermost interior row
__global__ void sponge_frs_ns_kernel(SpongeGrid g, const float* __restrict__ cur, const float* __restrict__ next,
                                     int data_nx, float bt) {
    const int ti = blockIdx.x * blockDim.x + threadIdx.x, tj = blockIdx.y * blockDim.y + threadIdx.y;
    const bool south = g.bc_south == 3 && tj < g.sp_south && tj >= 0;
    const bool north = g.bc_north == 3 && tj > g.ny + 3 - g.sp_north && tj < g.ny + 4;
    if (!((south || north) && ti >= 0 && ti < g.nx + 4)) return;
    const float d = (tj <= g.sp_south) ? tj - 1 : ((g.ny + 2) - tj);
    const float alpha = relaxation_weight(d);
    const float s = ti / float(g.nx + 4);
    const float t = (tj < g.ny / 2.0) ? 0.25f : 0.75f;   // data row 0: south, row 1: north
    const float3 c0 = bilinear3(cur, data_nx, 2, s, t), c1 = bilinear3(next, data_nx, 2, s, t);
    const float ext[3] = {time_interp(bt, c1.x, c0.x), time_interp(bt, c1.y, c0.y), time_interp(bt, c1.z, c0.z)};
    float* q[3] = {g.eta, g.hu, g.hv};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float* p = at(q[c], g.pitch, tj, ti);
        *p = relax(alpha, ext[c], *p);
    }
}

__global__ void sponge_frs_ew_kernel(SpongeGrid g, const float* __restrict__ cur, const float* __restrict__ next,
                                     int data_ny, float bt) {
    const int ti = blockIdx.x * blockDim.x + threadIdx.x, tj = blockIdx.y * blockDim.y + threadIdx.y;
    const bool west = g.bc_west == 3 && ti < g.sp_west && ti >= 0;
    const bool east = g.bc_east == 3 && ti > g.nx + 3 - g.sp_east && ti < g.nx + 4;
    if (!((west || east) && tj >= 0 && tj < g.ny + 4)) return;
    const float d = (ti <= g.sp_west) ? ti - 1 : ((g.nx + 2) - ti);
    const float alpha = relaxation_weight(d);
    const float s = (ti < g.nx / 2.0) ? 0.25f : 0.75f;   // data column 0: west, column 1: east
    const float t = tj / float(g.ny + 4);
    const float3 c0 = bilinear3(cur, 2, data_ny, s, t), c1 = bilinear3(next, 2, data_ny, s, t);
    const float ext[3] = {time_interp(bt, c1.x, c0.x), time_interp(bt, c1.y, c0.y), time_interp(bt, c1.z, c0.z)};
    float* q[3] = {g.eta, g.hu, g.hv};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float* p = at(q[c], g.pitch, tj, ti);
        *p = relax(alpha, ext[c], *p);
    }
}

}  // namespace goc

using namespace goc;

extern "C" int goc_sponge_boundary(int nx, int ny, int bc_north, int bc_east, int bc_south, int bc_west,
                                   const int* sponge_cells, float* eta, float* hu, float* hv, int pitch,
                                   const float* ns_current, const float* ns_next, int ns_nx,
                                   const float* ew_current, const float* ew_next, int ew_ny, float bc_t,
                                   void* stream) {
    if (nx < 1 || ny < 1 || !sponge_cells) return set_error(GOC_ERR_ARG, "goc_sponge_boundary: bad grid");
    if (!eta || !hu || !hv || pitch < (nx + 4) * 4 || pitch % 4)
        return set_error(GOC_ERR_ARG, "goc_sponge_boundary: bad state buffers");
    SpongeGrid g{nx, ny, bc_north, bc_south, bc_east, bc_west,
                 sponge_cells[0], sponge_cells[2], sponge_cells[1], sponge_cells[3], eta, hu, hv, pitch / 4};
    const int sp[4] = {g.sp_north, g.sp_east, g.sp_south, g.sp_west};
    for (int k = 0; k < 4; ++k)
        if (sp[k] < 0 || sp[k] > (k % 2 ? nx : ny) + 3)
            return set_error(GOC_ERR_ARG, "goc_sponge_boundary: sponge width %d out of range", sp[k]);
    const bool frs_ns = bc_north == 3 || bc_south == 3, frs_ew = bc_east == 3 || bc_west == 3;
    if ((frs_ns && (!ns_current || !ns_next || ns_nx < 1)) || (frs_ew && (!ew_current || !ew_next || ew_ny < 1)))
        return set_error(GOC_ERR_ARG, "goc_sponge_boundary: flow relaxation needs the exterior data");
    // linear interpolation needs the inner row inside the array and apart from the outer row
    if ((bc_south == 4 && g.sp_south < 1) || (bc_north == 4 && g.sp_north < 1) || (bc_west == 4 && g.sp_west < 1) ||
        (bc_east == 4 && g.sp_east < 1))
        return set_error(GOC_ERR_ARG, "goc_sponge_boundary: linear interpolation needs sponge cells");
    cudaStream_t st = as_stream(stream);
    const dim3 blk(16, 16), grd((nx + 4 + 1 + 15) / 16, (ny + 4 + 1 + 15) / 16);   // U/Common.py:1170-1172
    int rc;
    if (bc_north != 2) {
        if (frs_ns) {
            sponge_frs_ns_kernel<<<grd, blk, 0, st>>>(g, ns_current, ns_next, ns_nx, bc_t);
            count_launch();
            if ((rc = check_launch("sponge_frs_ns_kernel"))) return rc;
        }
        if (bc_north == 4 || bc_south == 4) {
            sponge_linear_ns_kernel<<<grd, blk, 0, st>>>(g);
            count_launch();
            if ((rc = check_launch("sponge_linear_ns_kernel"))) return rc;
        }
    }
    if (bc_east != 2) {
        if (frs_ew) {
            sponge_frs_ew_kernel<<<grd, blk, 0, st>>>(g, ew_current, ew_next, ew_ny, bc_t);
            count_launch();
            if ((rc = check_launch("sponge_frs_ew_kernel"))) return rc;
        }
        if (bc_east == 4 || bc_west == 4) {
            sponge_linear_ew_kernel<<<grd, blk, 0, st>>>(g);
            count_launch();
            if ((rc = check_launch("sponge_linear_ew_kernel"))) return rc;
        }
    }
    return GOC_OK;
}
