// Stand-alone transfer of the SOAR coarse field to the ocean state (single
// simulator, and batched for moments outside the fused ensemble step):
// bicubic up-sampling + geostrophic balance, K/ocean_noise.cu:256-666.
//
// Compiled with the ensemble step's arithmetic options (no FMA contraction),
// so that these kernels and the fused step epilogue, which both use
// noise_transfer.cuh, round identically.
#include "noise_transfer.cuh"

namespace goc {

constexpr int kPR = kPY / kPT;   // cells per thread
// shared scratch of one tile: the coefficient matrices of up to 12 x 12
// coarse cells (factors >= 4 for the 34 fine cells of a tile + ring) and the
// per-column / per-row coarse indices and fractions
constexpr int kScratch = 12 * 12 * 17 + 2 * ((kPX + 2) + (kPY + 2));

// One kPX x kPY tile of interior cells (tile origin bx, by in interior
// cells).  Each thread owns kPR cells of one column; their state is loaded
// first so that the loads overlap the perturbation field (the corner depths,
// shared by the members and L2-resident, are read when used).
__device__ void perturb_tile(const GocNoiseDesc& d, const OceanRef& o, int bx, int by) {
    __shared__ float s_de[kPY + 2][kPX + 2];
    __shared__ float s_scratch[kScratch];
    const int tx = threadIdx.x, t = threadIdx.y * kPX + tx;
    constexpr int NT = kPX * kPT;
    const bool factor1 = d.interpolation_factor <= 1;
    const int ti = 2 + bx + tx;
    float q[kPR][3];
#pragma unroll
    for (int r = 0; r < kPR; ++r) {
        const int tj = 2 + by + threadIdx.y + r * kPT;
        q[r][0] = q[r][1] = q[r][2] = 0.0f;
        if (ti < o.nx + 2 && tj < o.ny + 2) {
            const size_t k = (size_t)tj * o.pitch + ti;
            q[r][0] = o.eta[k];
            q[r][1] = o.hu[k];
            q[r][2] = o.hv[k];
        }
    }
    // d_eta on the tile + 1 ring (interior origin at ghost offset 2)
    noise_tile_field<kPX + 2, kPY + 2, NT>(d, o.dx, o.dy, 2 + bx - 1, 2 + by - 1, &s_de[0][0], s_scratch, kScratch, t);
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kPR; ++r) {
        const int tj = 2 + by + threadIdx.y + r * kPT;
        if (ti < o.nx + 2 && tj < o.ny + 2) {
            const float* h0 = o.Hi + (size_t)tj * o.hi_pitch + ti;
            const float hc[4] = {__ldg(h0), __ldg(h0 + 1), __ldg(h0 + o.hi_pitch), __ldg(h0 + o.hi_pitch + 1)};
            float e = q[r][0], u = q[r][1], v = q[r][2];
            perturbed_state(d, o.nx, o.ny, o.dx, o.dy, o.land, ti, tj, factor1,
                            [&](int jj, int ii) { return s_de[jj - (2 + by) + 1][ii - (2 + bx) + 1]; }, e, u, v, hc);
            store_cell(o, ti, tj, e, u, v);
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kPX * kPT, 3) perturb_kernel(GocNoiseDesc d, OceanRef o) {
    perturb_tile(d, o, blockIdx.x * kPX, blockIdx.y * kPY);
}

__global__ void __launch_bounds__(kPX * kPT, 3)
perturb_batched_kernel(const GocNoiseDesc* __restrict__ nd, const GocMemberDesc* __restrict__ mem,
                       const int4* __restrict__ items, const int* __restrict__ nsub, int substep) {
    const int4 it = items[blockIdx.x];
    int set;
    if (!member_set(nsub, it.x, substep, &set)) return;
    const GocMemberDesc& m = mem[it.x];
    const OceanRef o{m.p.nx, m.p.ny, m.p.dx, m.p.dy, m.eta[set], m.hu[set], m.hv[set], m.pitch / 4, m.Hi,
                     m.Hi_pitch / 4, m.p.land_value, m.p.bc_north == 2, m.p.bc_east == 2};
    perturb_tile(nd[it.x], o, it.y * kPX, it.z * kPY);
}

int launch_perturb_batched(const GocNoiseDesc* noise, const GocMemberDesc* members, const int4* items, int n_items,
                           const int* nsub, int substep, cudaStream_t stream) {
    perturb_batched_kernel<<<n_items, dim3(kPX, kPT), 0, stream>>>(noise, members, items, nsub, substep);
    count_launch();
    return check_launch("perturb_batched_kernel");
}

}  // namespace goc

using namespace goc;

static int check_transfer(const GocNoiseDesc* d) {
    if (!d) return set_error(GOC_ERR_ARG, "goc_perturb_ocean: null noise descriptor");
    if (d->coarse_nx < 1 || d->coarse_ny < 1 || !(d->coarse_dx > 0) || !(d->coarse_dy > 0) || !d->coarse ||
        d->coarse_pitch < (d->coarse_nx + 4) * 4 || d->interpolation_factor < 1)
        return set_error(GOC_ERR_ARG, "goc_perturb_ocean: bad coarse grid");
    return GOC_OK;
}

extern "C" int goc_perturb_ocean(const GocNoiseDesc* d, int nx, int ny, float dx, float dy, float* eta, float* hu,
                                 float* hv, int pitch, const float* Hi, int Hi_pitch, float land_value,
                                 int periodic_ghosts, void* stream) {
    int rc = check_transfer(d);
    if (rc) return rc;
    OceanRef o;
    if ((rc = make_ocean(nx, ny, dx, dy, eta, hu, hv, pitch, Hi, Hi_pitch, land_value,
                         periodic_ghosts && d->periodic_ns, periodic_ghosts && d->periodic_ew, &o, "goc_perturb_ocean")))
        return rc;
    dim3 blk(kPX, kPT), grd((nx + kPX - 1) / kPX, (ny + kPY - 1) / kPY);
    perturb_kernel<<<grd, blk, 0, as_stream(stream)>>>(*d, o);
    count_launch();
    return check_launch("perturb_kernel");
}
