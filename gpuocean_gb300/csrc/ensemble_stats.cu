// Observation operator and ensemble statistics on the device.
//
// The reference observes and averages its ensembles from Python, member by
// member: observeParticles launches observeUnderlyingFlow once per particle
// (or downloads every state and indexes it in NumPy), and estimate /
// estimateVelocity download every member and reduce with NumPy
// (E/BaseOceanStateEnsemble.py:79-160, E/MultiLevelOceanEnsemble.py:143-267;
// E/ = src/gpuocean/ensembles).  Here one launch observes every member, one
// pass over HBM gives mean and variance of a member group, and the multi-level
// estimator is assembled on the finest grid in one more launch.
#include <algorithm>
#include <vector>

#include "common.cuh"

namespace goc {

// ---------------------------------------------------------------------------
// observation operator (K/observationKernels.cu:29-83)
// ---------------------------------------------------------------------------

// Cell of a position in metres from the south-west interior corner, as the
// reference computes it (IEEE division - its observation kernels are built
// with default options - floor, then the zero-reference offset), clamped to
// the (nx+4) x (ny+4) array.  The library's default is approximate division,
// so the rounding is spelled out.
__device__ __forceinline__ int observed_cell(float pos, float d, int zero_ref, int n) {
    return clampi((int)(floorf(__fdiv_rn(pos, d)) + zero_ref), 0, n + 3);
}

__global__ void observe_flow_kernel(int nx, int ny, float dx, float dy, int x_zero_ref, int y_zero_ref,
                                    const float* __restrict__ hu, int hu_pitch, const float* __restrict__ hv,
                                    int hv_pitch, int num_drifters, const float* __restrict__ pos, int pos_pitch,
                                    float* __restrict__ obs, int obs_pitch) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= num_drifters) return;
    const float* p = pos + (size_t)d * pos_pitch;
    const int cx = observed_cell(p[0], dx, x_zero_ref, nx), cy = observed_cell(p[1], dy, y_zero_ref, ny);
    float* o = obs + (size_t)d * obs_pitch;
    o[0] = hu[(size_t)cy * hu_pitch + cx];
    o[1] = hv[(size_t)cy * hv_pitch + cx];
}

// (eta, hu, hv) of member `first + blockIdx.y` at every position; positions
// are shared (member stride 0) or per member.
__global__ void observe_members_kernel(const GocMemberDesc* __restrict__ mem, int first, int num_positions,
                                       const float* __restrict__ pos, int pos_pitch, long long pos_member_stride,
                                       float* __restrict__ out) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (d >= num_positions) return;
    const GocMemberDesc& m = mem[first + i];
    const float* p = pos + i * pos_member_stride + (size_t)d * pos_pitch;
    const int cx = observed_cell(p[0], m.p.dx, 2, m.p.nx), cy = observed_cell(p[1], m.p.dy, 2, m.p.ny);
    const size_t k = (size_t)cy * (m.pitch / 4) + cx;
    float* o = out + ((size_t)i * num_positions + d) * 3;
    o[0] = m.eta[0][k];
    o[1] = m.hu[0][k];
    o[2] = m.hv[0][k];
}

// ---------------------------------------------------------------------------
// ensemble moments
// ---------------------------------------------------------------------------

constexpr int kMX = 32, kMY = 8;       // cells per block
constexpr int kMChunk = 128;           // member pointers staged in shared memory at a time

struct MomentSrc {
    const float* a; const float* b; const float* c;  // eta, hu, hv of buffer set 0
    const float* Hm;
    int pitch, Hm_pitch;                             // floats
};

// desingularise (U/OceanographicUtilities.py:413-414) in float32 with IEEE
// division, as NumPy evaluates it on float32 arrays.
__device__ __forceinline__ float desingularised_velocity(float h, float hu, float eps) {
    if (eps <= 0.0f) return __fdiv_rn(hu, h);
    const float a = __fadd_rn(__fdiv_rn(__fmul_rn(h, h), 2.0f * eps), 0.5f * eps);
    return __fdiv_rn(hu, fmaxf(fminf(a, eps), fabsf(h)));
}

// The quantities of one member at one interior cell: (eta, hu, hv) or (u, v).
template <int Q>
__device__ __forceinline__ void member_values(const MomentSrc& s, int x, int y, float eps, float* v) {
    const size_t k = (size_t)(y + 2) * s.pitch + (x + 2);
    if (Q == 0) {
        v[0] = __ldg(s.a + k); v[1] = __ldg(s.b + k); v[2] = __ldg(s.c + k);
    } else {
        const float h = __fadd_rn(__ldg(s.a + k), __ldg(s.Hm + (size_t)(y + 2) * s.Hm_pitch + (x + 2)));
        v[0] = desingularised_velocity(h, __ldg(s.b + k), eps);
        v[1] = desingularised_velocity(h, __ldg(s.c + k), eps);
    }
}

// One slice of the members: shifted sums s1 = sum(x - K), s2 = sum((x - K)^2)
// with K the first member's value.  With one slice the moments are written
// directly; otherwise the per-slice sums go to `part` (slice, 2P, cells).
template <int Q>
__global__ void __launch_bounds__(kMX * kMY) moments_kernel(const GocMemberDesc* __restrict__ mem, int first, int n,
                                                            int per_slice, int nx, int ny, float eps, int ddof,
                                                            float* __restrict__ mean, float* __restrict__ var,
                                                            float* __restrict__ part) {
    constexpr int P = Q == 0 ? 3 : 2;
    __shared__ MomentSrc s_src[kMChunk];
    const int x = blockIdx.x * kMX + threadIdx.x, y = blockIdx.y * kMY + threadIdx.y;
    const int t = threadIdx.y * kMX + threadIdx.x;
    const bool inside = x < nx && y < ny;
    const int m0 = blockIdx.z * per_slice, m1 = min(n, m0 + per_slice);
    float K[P], s1[P], s2[P];
    {
        const GocMemberDesc& d = mem[first];
        const MomentSrc s{d.eta[0], d.hu[0], d.hv[0], d.Hm, d.pitch / 4, d.Hm_pitch / 4};
        if (inside) member_values<Q>(s, x, y, eps, K);
    }
#pragma unroll
    for (int q = 0; q < P; ++q) s1[q] = s2[q] = 0.0f;
    for (int c0 = m0; c0 < m1; c0 += kMChunk) {
        const int cn = min(kMChunk, m1 - c0);
        __syncthreads();
        for (int i = t; i < cn; i += kMX * kMY) {
            const GocMemberDesc& d = mem[first + c0 + i];
            s_src[i] = MomentSrc{d.eta[0], d.hu[0], d.hv[0], d.Hm, d.pitch / 4, d.Hm_pitch / 4};
        }
        __syncthreads();
        if (!inside) continue;
        int i = 0;
        for (; i + 4 <= cn; i += 4) {   // four members' loads in flight
            float v[4][P];
#pragma unroll
            for (int u = 0; u < 4; ++u) member_values<Q>(s_src[i + u], x, y, eps, v[u]);
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int q = 0; q < P; ++q) {
                    const float e = v[u][q] - K[q];
                    s1[q] += e;
                    s2[q] += e * e;
                }
        }
        for (; i < cn; ++i) {
            float v[P];
            member_values<Q>(s_src[i], x, y, eps, v);
#pragma unroll
            for (int q = 0; q < P; ++q) {
                const float e = v[q] - K[q];
                s1[q] += e;
                s2[q] += e * e;
            }
        }
    }
    if (!inside) return;
    const size_t cells = (size_t)nx * ny, c = (size_t)y * nx + x;
    if (part) {
        float* o = part + (size_t)blockIdx.z * 2 * P * cells + c;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            o[(2 * q) * cells] = s1[q];
            o[(2 * q + 1) * cells] = s2[q];
        }
        return;
    }
#pragma unroll
    for (int q = 0; q < P; ++q) {
        if (mean) mean[q * cells + c] = K[q] + __fdiv_rn(s1[q], (float)n);
        if (var) var[q * cells + c] = __fdiv_rn(s2[q] - __fdiv_rn(s1[q] * s1[q], (float)n), (float)(n - ddof));
    }
}

// Sums the slices in order and writes the moments.
template <int Q>
__global__ void moments_finish_kernel(const GocMemberDesc* __restrict__ mem, int first, int n, int slices, int nx,
                                      int ny, float eps, int ddof, const float* __restrict__ part,
                                      float* __restrict__ mean, float* __restrict__ var) {
    constexpr int P = Q == 0 ? 3 : 2;
    const int x = blockIdx.x * kMX + threadIdx.x, y = blockIdx.y * kMY + threadIdx.y;
    if (x >= nx || y >= ny) return;
    const GocMemberDesc& d = mem[first];
    const MomentSrc s{d.eta[0], d.hu[0], d.hv[0], d.Hm, d.pitch / 4, d.Hm_pitch / 4};
    float K[P];
    member_values<Q>(s, x, y, eps, K);
    const size_t cells = (size_t)nx * ny, c = (size_t)y * nx + x;
#pragma unroll
    for (int q = 0; q < P; ++q) {
        float s1 = 0.0f, s2 = 0.0f;
        for (int z = 0; z < slices; ++z) {
            const float* o = part + (size_t)z * 2 * P * cells + c;
            s1 += o[(2 * q) * cells];
            s2 += o[(2 * q + 1) * cells];
        }
        if (mean) mean[q * cells + c] = K[q] + __fdiv_rn(s1, (float)n);
        if (var) var[q * cells + c] = __fdiv_rn(s2 - __fdiv_rn(s1 * s1, (float)n), (float)(n - ddof));
    }
}

// ---------------------------------------------------------------------------
// multi-level estimator (E/MultiLevelOceanEnsemble.py:258-267)
// ---------------------------------------------------------------------------

constexpr int kMaxLevels = 8;

struct MLLevels {
    const float* fine[kMaxLevels];
    const float* coarse[kMaxLevels];
    int nx[kMaxLevels], ny[kMaxLevels];
    int n_levels, planes;
};

// est = level-0 statistic + sum over levels of (fine - coarse), each term
// held constant over the finest cells it covers.  The level differences are
// formed in float32 and accumulated in float64, in level order, as NumPy
// does on the reference's float32 statistics and float64 accumulator.
__global__ void ml_combine_kernel(MLLevels L, double* __restrict__ out) {
    const int top = L.n_levels - 1;
    const int NX = L.nx[top], NY = L.ny[top];
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const int p = blockIdx.z;
    if (x >= NX || y >= NY) return;
    double est = 0.0;
    est += (double)L.fine[0][((size_t)p * L.ny[0] + (y >> top)) * L.nx[0] + (x >> top)];
    for (int l = 1; l <= top; ++l) {
        const int s = top - l;
        const int cnx = L.nx[l] / 2, cny = L.ny[l] / 2;
        const float f = L.fine[l][((size_t)p * L.ny[l] + (y >> s)) * L.nx[l] + (x >> s)];
        const float c = L.coarse[l][((size_t)p * cny + (y >> (s + 1))) * cnx + (x >> (s + 1))];
        est += (double)(f - c);
    }
    out[((size_t)p * NY + y) * NX + x] = est;
}

// Scratch for the per-slice sums, owned by the library (one per process).
struct StatsScratch {
    float* ptr = nullptr;
    size_t bytes = 0;
};
StatsScratch g_scratch;

}  // namespace goc

using namespace goc;

extern "C" int goc_observe_underlying_flow(int nx, int ny, float dx, float dy, int x_zero_ref, int y_zero_ref,
                                           const float* eta, int eta_pitch, const float* hu, int hu_pitch,
                                           const float* hv, int hv_pitch, float H, int num_drifters,
                                           const float* positions, int positions_pitch, float* observations,
                                           int observation_pitch, void* stream) {
    (void)eta; (void)eta_pitch; (void)H;   // the reference reads neither
    if (nx < 1 || ny < 1 || !(dx > 0.0f) || !(dy > 0.0f) || num_drifters < 0)
        return set_error(GOC_ERR_ARG, "goc_observe_underlying_flow: bad grid or count");
    if (num_drifters == 0) return GOC_OK;
    if (!hu || !hv || !positions || !observations)
        return set_error(GOC_ERR_ARG, "goc_observe_underlying_flow: null buffer");
    if (hu_pitch < (nx + 4) * 4 || hv_pitch < (nx + 4) * 4 || hu_pitch % 4 || hv_pitch % 4 || positions_pitch < 8 ||
        positions_pitch % 4 || observation_pitch < 8 || observation_pitch % 4)
        return set_error(GOC_ERR_ARG, "goc_observe_underlying_flow: bad pitch");
    observe_flow_kernel<<<(num_drifters + 127) / 128, 128, 0, as_stream(stream)>>>(
        nx, ny, dx, dy, x_zero_ref, y_zero_ref, hu, hu_pitch / 4, hv, hv_pitch / 4, num_drifters, positions,
        positions_pitch / 4, observations, observation_pitch / 4);
    count_launch();
    return check_launch("observe_flow_kernel");
}

extern "C" int goc_ensemble_observe(void* ensemble, int first_member, int n_members, const float* positions,
                                    int positions_pitch, long long positions_member_stride, int num_positions,
                                    float* out, void* stream) {
    int total = 0;
    if (!ensemble || !ensemble_host_members(ensemble, &total))
        return set_error(GOC_ERR_ARG, "goc_ensemble_observe: null ensemble");
    if (first_member < 0 || n_members < 0 || first_member + n_members > total || n_members > 65535)
        return set_error(GOC_ERR_ARG, "goc_ensemble_observe: member range outside the ensemble");
    if (num_positions < 0) return set_error(GOC_ERR_ARG, "goc_ensemble_observe: negative position count");
    if (n_members == 0 || num_positions == 0) return GOC_OK;
    if (!positions || !out) return set_error(GOC_ERR_ARG, "goc_ensemble_observe: null buffer");
    if (positions_pitch < 8 || positions_pitch % 4 || positions_member_stride < 0 || positions_member_stride % 4)
        return set_error(GOC_ERR_ARG, "goc_ensemble_observe: bad position pitch or stride");
    dim3 grd((num_positions + 127) / 128, n_members);
    observe_members_kernel<<<grd, 128, 0, as_stream(stream)>>>(ensemble_device_members(ensemble), first_member,
                                                               num_positions, positions, positions_pitch / 4,
                                                               positions_member_stride / 4, out);
    count_launch();
    return check_launch("observe_members_kernel");
}

extern "C" int goc_ensemble_moments(void* ensemble, int first_member, int n_members, int quantity, float desing_eps,
                                    int ddof, float* mean, float* var, void* stream) {
    int total = 0;
    const GocMemberDesc* host = ensemble ? ensemble_host_members(ensemble, &total) : nullptr;
    if (!host) return set_error(GOC_ERR_ARG, "goc_ensemble_moments: null ensemble");
    if (first_member < 0 || n_members < 1 || first_member + n_members > total)
        return set_error(GOC_ERR_ARG, "goc_ensemble_moments: member range outside the ensemble");
    if (quantity != 0 && quantity != 1) return set_error(GOC_ERR_ARG, "goc_ensemble_moments: quantity must be 0 or 1");
    if (!mean && !var) return set_error(GOC_ERR_ARG, "goc_ensemble_moments: no output");
    if (ddof < 0) return set_error(GOC_ERR_ARG, "goc_ensemble_moments: negative ddof");
    const int nx = host[first_member].p.nx, ny = host[first_member].p.ny;
    for (int m = first_member; m < first_member + n_members; ++m)
        if (host[m].p.nx != nx || host[m].p.ny != ny)
            return set_error(GOC_ERR_ARG, "goc_ensemble_moments: members %d and %d differ in grid size", first_member, m);
    const int P = quantity == 0 ? 3 : 2;
    const size_t cells = (size_t)nx * ny;
    dim3 blk(kMX, kMY), grd((nx + kMX - 1) / kMX, (ny + kMY - 1) / kMY);
    // split the members over slices until about four waves of blocks cover the device
    const long long blocks = (long long)grd.x * grd.y;
    int slices = (int)std::min<long long>(std::max<long long>(1, (152LL * 8 * 4 + blocks - 1) / blocks),
                                          std::max(1, n_members / 16));
    slices = std::min(slices, 65535);
    const int per_slice = (n_members + slices - 1) / slices;
    slices = (n_members + per_slice - 1) / per_slice;
    cudaStream_t st = as_stream(stream);
    float* part = nullptr;
    if (slices > 1) {
        const size_t need = (size_t)slices * 2 * P * cells * sizeof(float);
        if (g_scratch.bytes < need) {
            cudaError_t err = cudaStreamSynchronize(st);
            if (err == cudaSuccess) err = cudaFree(g_scratch.ptr);
            g_scratch.ptr = nullptr;
            g_scratch.bytes = 0;
            if (err == cudaSuccess) err = cudaMalloc(&g_scratch.ptr, need);
            if (err != cudaSuccess)
                return set_error(GOC_ERR_CUDA, "goc_ensemble_moments: scratch: %s", cudaGetErrorString(err));
            g_scratch.bytes = need;
        }
        part = g_scratch.ptr;
    }
    grd.z = slices;
    const GocMemberDesc* dm = ensemble_device_members(ensemble);
    if (quantity == 0)
        moments_kernel<0><<<grd, blk, 0, st>>>(dm, first_member, n_members, per_slice, nx, ny, desing_eps, ddof,
                                               mean, var, part);
    else
        moments_kernel<1><<<grd, blk, 0, st>>>(dm, first_member, n_members, per_slice, nx, ny, desing_eps, ddof,
                                               mean, var, part);
    count_launch();
    int rc = check_launch("moments_kernel");
    if (rc || slices == 1) return rc;
    grd.z = 1;
    if (quantity == 0)
        moments_finish_kernel<0><<<grd, blk, 0, st>>>(dm, first_member, n_members, slices, nx, ny, desing_eps, ddof,
                                                      part, mean, var);
    else
        moments_finish_kernel<1><<<grd, blk, 0, st>>>(dm, first_member, n_members, slices, nx, ny, desing_eps, ddof,
                                                      part, mean, var);
    count_launch();
    return check_launch("moments_finish_kernel");
}

extern "C" int goc_ml_combine(int n_levels, const float* const* fine, const float* const* coarse, const int* nx,
                              const int* ny, int n_planes, double* out, void* stream) {
    if (n_levels < 1 || n_levels > kMaxLevels || !fine || !nx || !ny || !out || n_planes < 1 || n_planes > 65535)
        return set_error(GOC_ERR_ARG, "goc_ml_combine: bad arguments");
    if (n_levels > 1 && !coarse) return set_error(GOC_ERR_ARG, "goc_ml_combine: coarse statistics missing");
    MLLevels L{};
    L.n_levels = n_levels;
    L.planes = n_planes;
    const int top = n_levels - 1;
    for (int l = 0; l < n_levels; ++l) {
        if (!fine[l] || (l > 0 && !coarse[l])) return set_error(GOC_ERR_ARG, "goc_ml_combine: null level %d", l);
        if (nx[l] < 1 || ny[l] < 1 || (long long)nx[l] << (top - l) != nx[top] ||
            (long long)ny[l] << (top - l) != ny[top] || (l > 0 && (nx[l] % 2 || ny[l] % 2)))
            return set_error(GOC_ERR_ARG, "goc_ml_combine: level %d is not the finest grid coarsened by 2^%d", l,
                             top - l);
        L.fine[l] = fine[l];
        L.coarse[l] = l > 0 ? coarse[l] : nullptr;
        L.nx[l] = nx[l];
        L.ny[l] = ny[l];
    }
    dim3 blk(32, 8), grd((nx[top] + 31) / 32, (ny[top] + 7) / 8, n_planes);
    ml_combine_kernel<<<grd, blk, 0, as_stream(stream)>>>(L, out);
    count_launch();
    return check_launch("ml_combine_kernel");
}
