// Per-cell CFL limit shared by the single-simulator and ensemble reductions.
#pragma once

#include "common.cuh"

namespace goc {

constexpr int kDtBX = 32, kDtBY = 8;

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ float cell_dt(int nx, int ny, float dx, float dy, float g, const float* __restrict__ e,
                                         const float* __restrict__ hu, const float* __restrict__ hv, int pitch,
                                         const float* __restrict__ Hm, int mp, float land, int i, int j) {
    if (i >= nx + 2 || j >= ny + 2) return kMaxDt;
    const float eta = e[(size_t)j * pitch + i];
    const float H = Hm[(size_t)j * mp + i];
    const float h = eta + H;
    if (h <= 0.0f || fabsf(H - land) < kDryEps) return kMaxDt;
    const float u = __fdiv_rn(hu[(size_t)j * pitch + i], h);
    const float v = __fdiv_rn(hv[(size_t)j * pitch + i], h);
    const float c = __fsqrt_rn(g * h);
    const float qx = 0.25f * dx, qy = 0.25f * dy;
    float d = __fdiv_rn(qx, fabsf(u + c));
    d = fminf(d, __fdiv_rn(qx, fabsf(u - c)));
    d = fminf(d, __fdiv_rn(qy, fabsf(v + c)));
    d = fminf(d, __fdiv_rn(qy, fabsf(v - c)));
    return d;
}

}  // namespace goc
