// Shared helpers of the gpuocean_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gpuocean_gb300.h"

namespace goc {

// Land / dry markers shared by every kernel of the scheme
// (the reference keeps them in K/CDKLM16_kernel.cu:34-35, K/max_dt.cu:33-34,
// K/initHm_kernel.cu:28-29).
constexpr float kDryFlag = 1.0e-30f;
constexpr float kDryEps = 1.0e-3f;
constexpr float kMaxDt = 100000.0f;

// Error reporting and launch accounting (runtime.cu).
int set_error(int code, const char* fmt, ...);
int check_launch(const char* what);
void count_launch(int n = 1);

// Member tables of an ensemble handle (ensemble.cu): the descriptors as
// created (host) and the device copy whose buffer set 0 is the current state.
const GocMemberDesc* ensemble_host_members(void* ensemble, int* n_members);
const GocMemberDesc* ensemble_device_members(void* ensemble);
const int* ensemble_device_nsub(void* ensemble);
// per member the block's step count if the member takes model error, else 0
const int* ensemble_device_noise_steps(void* ensemble);

// Device table of the members' SOAR descriptors of a noise batch handle
// (noise.cu); n_members receives the batch's member count.
const GocNoiseDesc* noise_batch_device_desc(void* batch, int* n_members);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Clamped, texel-centred bilinear lookup in normalised coordinates, the
// arithmetic of tex2D-style lookups used throughout the scheme
// (K/interpolation.cu:137-190).  The base index is clamped so that a
// coordinate of exactly 1.0 stays inside the array.
__device__ __forceinline__ float tex_bilinear(const float* __restrict__ data, int dnx, int dny,
                                              float s, float t) {
    s = __saturatef(s - 0.5f / dnx);
    t = __saturatef(t - 0.5f / dny);
    const float x = s * dnx;
    const float y = t * dny;
    const int x0 = min((int)floorf(x), dnx - 1);
    const int y0 = min((int)floorf(y), dny - 1);
    const float fx = x - x0;
    const float fy = y - y0;
    const int x1 = min(x0 + 1, dnx - 1);
    const int y1 = min(y0 + 1, dny - 1);
    const float d00 = __ldg(data + y0 * dnx + x0);
    const float d01 = __ldg(data + y0 * dnx + x1);
    const float d10 = __ldg(data + y1 * dnx + x0);
    const float d11 = __ldg(data + y1 * dnx + x1);
    return d00 + fx * (d01 - d00) + fy * (d10 - d00) + fx * fy * (d00 + d11 - d01 - d10);
}

// Periodic index map onto the interior range [2, n+2) of a grid with two
// ghost cells: cell k and k +- n are the same cell.
// Interior index (2 .. n+1) of the periodic image of index k.  Callers'
// indices lie within a tile's halo of the interior, at most one period away,
// so one conditional add or subtract does it; the remainder (an integer
// division, ~20 instructions) is left for grids narrower than a tile.
__device__ __forceinline__ int wrap_interior(int k, int n) {
    int m = k - 2;
    if (m < 0) m += n;
    else if (m >= n) m -= n;
    if ((unsigned)m >= (unsigned)n) {
        m %= n;
        if (m < 0) m += n;
    }
    return m + 2;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(max(v, lo), hi); }

}  // namespace goc
