// Bathymetry set-up, periodic ghost fill and the CFL time-step reduction.
#include "cfl.cuh"

namespace goc {

// ---------------------------------------------------------------------------
// bathymetry (U/Common.py:1438-1491, K/boundary_kernels.cu:122-247,
// K/initHm_kernel.cu:38-106)
// ---------------------------------------------------------------------------

// Ghost rows of the corner depths: periodic copies or closed mirrors.
__global__ void hi_rows_kernel(int nx, int ny, int mode, float* Hi, int pitch) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nx + 5) return;
    if (mode == 2) {
        // rows 0,1 <- ny, ny+1 ; rows ny+2..ny+4 <- 2..4
        for (int r = 0; r < 2; ++r) Hi[(size_t)r * pitch + c] = Hi[(size_t)(r + ny) * pitch + c];
        for (int r = ny + 2; r < ny + 5; ++r) Hi[(size_t)r * pitch + c] = Hi[(size_t)(r - ny) * pitch + c];
    } else {
        // mirror about the boundary corner rows 2 and ny+2
        Hi[(size_t)0 * pitch + c] = Hi[(size_t)4 * pitch + c];
        Hi[(size_t)1 * pitch + c] = Hi[(size_t)3 * pitch + c];
        Hi[(size_t)(ny + 4) * pitch + c] = Hi[(size_t)ny * pitch + c];
        Hi[(size_t)(ny + 3) * pitch + c] = Hi[(size_t)(ny + 1) * pitch + c];
    }
}

// Ghost columns of the corner depths.
__global__ void hi_cols_kernel(int nx, int ny, int mode, float* Hi, int pitch) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= ny + 5) return;
    float* row = Hi + (size_t)r * pitch;
    if (mode == 2) {
        for (int c = 0; c < 2; ++c) row[c] = row[c + nx];
        for (int c = nx + 2; c < nx + 5; ++c) row[c] = row[c - nx];
    } else {
        row[0] = row[4];
        row[1] = row[3];
        row[nx + 4] = row[nx];
        row[nx + 3] = row[nx + 1];
    }
}

// Cell means: sum of the wet corners / number of wet corners; land where
// all four corners are land.
__global__ void cell_mean_kernel(int nx, int ny, float land, const float* __restrict__ Hi, int hp,
                                 float* __restrict__ Hm, int mp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= nx + 4 || j >= ny + 4) return;
    auto corner = [&](int r, int c) {
        float v = Hi[(size_t)r * hp + c];
        return (fabsf(v - land) <= kDryEps) ? kDryFlag : v;
    };
    const float a = corner(j, i), b = corner(j + 1, i), c = corner(j, i + 1), d = corner(j + 1, i + 1);
    const float wet = 4.0f - (float)(a == kDryFlag) - (float)(b == kDryFlag) - (float)(c == kDryFlag) -
                      (float)(d == kDryFlag);
    Hm[(size_t)j * mp + i] = (wet == 0.0f) ? land : __fdiv_rn(((a + b) + c) + d, wet);
}

// ---------------------------------------------------------------------------
// periodic ghost cells of the state (K/boundary_kernels.cu:36-110)
// ---------------------------------------------------------------------------

__global__ void periodic_rows_kernel(int nx, int ny, float* e, float* hu, float* hv, int pitch) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int g = blockIdx.y;  // 0..3: ghost rows 0, 1, ny+2, ny+3
    if (c >= nx + 4) return;
    const int r = (g < 2) ? g : ny + g;
    const int src = (g < 2) ? r + ny : r - ny;
    const size_t o = (size_t)r * pitch + c, s = (size_t)src * pitch + c;
    e[o] = e[s]; hu[o] = hu[s]; hv[o] = hv[s];
}

__global__ void periodic_cols_kernel(int nx, int ny, float* e, float* hu, float* hv, int pitch) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int g = blockIdx.y;  // ghost columns 0, 1, nx+2, nx+3
    if (r >= ny + 4) return;
    const int c = (g < 2) ? g : nx + g;
    const int src = (g < 2) ? c + nx : c - nx;
    const size_t o = (size_t)r * pitch + c, s = (size_t)r * pitch + src;
    e[o] = e[s]; hu[o] = hu[s]; hv[o] = hv[s];
}

// ---------------------------------------------------------------------------
// CFL limit (K/max_dt.cu:42-195): per-block minimum into `partials`, then a
// single-block minimum of the partials.  IEEE divide and square root, as the
// reference builds max_dt.cu with default flags.
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kDtBX * kDtBY)
dt_partials_kernel(int nx, int ny, float dx, float dy, float g, const float* __restrict__ e,
                   const float* __restrict__ hu, const float* __restrict__ hv, int pitch,
                   const float* __restrict__ Hm, int mp, float land, float* __restrict__ partials) {
    __shared__ float wmin[kDtBX * kDtBY / 32];
    const int i = 2 + blockIdx.x * kDtBX + threadIdx.x;
    const int j = 2 + blockIdx.y * kDtBY + threadIdx.y;
    float d = cell_dt(nx, ny, dx, dy, g, e, hu, hv, pitch, Hm, mp, land, i, j);
    d = warp_min(d);
    const int tid = threadIdx.y * kDtBX + threadIdx.x;
    if ((tid & 31) == 0) wmin[tid >> 5] = d;
    __syncthreads();
    if (tid < 32) {
        float v = (tid < kDtBX * kDtBY / 32) ? wmin[tid] : kMaxDt;
        v = warp_min(v);
        if (tid == 0) partials[blockIdx.y * gridDim.x + blockIdx.x] = v;
    }
}

__global__ void __launch_bounds__(1024) dt_final_kernel(const float* __restrict__ partials, int n,
                                                        float* __restrict__ out) {
    __shared__ float wmin[32];
    float v = kMaxDt;
    for (int k = threadIdx.x; k < n; k += blockDim.x) v = fminf(v, partials[k]);
    v = warp_min(v);
    if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = (threadIdx.x < (blockDim.x + 31) / 32) ? wmin[threadIdx.x] : kMaxDt;
        v = warp_min(v);
        if (threadIdx.x == 0) out[0] = v;
    }
}

}  // namespace goc

using namespace goc;

extern "C" int goc_bathymetry_init(int nx, int ny, int bc_north, int bc_east, int bc_south, int bc_west,
                                   float land_value, float* Hi, int Hi_pitch, float* Hm, int Hm_pitch,
                                   void* stream) {
    if (nx < 1 || ny < 1) return set_error(GOC_ERR_ARG, "goc_bathymetry_init: nx, ny must be >= 1");
    if (!Hi || !Hm) return set_error(GOC_ERR_ARG, "goc_bathymetry_init: null buffer");
    if (Hi_pitch < (nx + 5) * 4 || Hi_pitch % 4 || Hm_pitch < (nx + 4) * 4 || Hm_pitch % 4)
        return set_error(GOC_ERR_ARG, "goc_bathymetry_init: pitch too small");
    if ((bc_north == 2 && ny < 3) || (bc_east == 2 && nx < 3))
        return set_error(GOC_ERR_ARG, "goc_bathymetry_init: periodic directions need at least 3 cells");
    cudaStream_t st = as_stream(stream);
    const int hp = Hi_pitch / 4, mp = Hm_pitch / 4;
    int rc;
    // north-south first, then east-west (U/Common.py:1538-1561); the closed
    // east-west branch is taken on the north/south flags, as the reference does.
    if (bc_north == 2 && bc_south == 2) {
        hi_rows_kernel<<<(nx + 5 + 127) / 128, 128, 0, st>>>(nx, ny, 2, Hi, hp);
        count_launch();
        if ((rc = check_launch("hi_rows_kernel"))) return rc;
    } else if (bc_north == 1 && bc_south == 1) {
        hi_rows_kernel<<<(nx + 5 + 127) / 128, 128, 0, st>>>(nx, ny, 1, Hi, hp);
        count_launch();
        if ((rc = check_launch("hi_rows_kernel"))) return rc;
    }
    if (bc_east == 2 && bc_west == 2) {
        hi_cols_kernel<<<(ny + 5 + 127) / 128, 128, 0, st>>>(nx, ny, 2, Hi, hp);
        count_launch();
        if ((rc = check_launch("hi_cols_kernel"))) return rc;
    } else if (bc_north == 1 && bc_south == 1) {
        hi_cols_kernel<<<(ny + 5 + 127) / 128, 128, 0, st>>>(nx, ny, 1, Hi, hp);
        count_launch();
        if ((rc = check_launch("hi_cols_kernel"))) return rc;
    }
    dim3 blk(32, 8), grd((nx + 4 + 31) / 32, (ny + 4 + 7) / 8);
    cell_mean_kernel<<<grd, blk, 0, st>>>(nx, ny, land_value, Hi, hp, Hm, mp);
    count_launch();
    return check_launch("cell_mean_kernel");
}

extern "C" int goc_periodic_ghosts(int nx, int ny, int bc_north, int bc_east, float* eta, float* hu, float* hv,
                                   int pitch, void* stream) {
    if (nx < 1 || ny < 1) return set_error(GOC_ERR_ARG, "goc_periodic_ghosts: nx, ny must be >= 1");
    if (!eta || !hu || !hv) return set_error(GOC_ERR_ARG, "goc_periodic_ghosts: null buffer");
    if (pitch < (nx + 4) * 4 || pitch % 4) return set_error(GOC_ERR_ARG, "goc_periodic_ghosts: pitch too small");
    if ((bc_north == 2 && ny < 2) || (bc_east == 2 && nx < 2))
        return set_error(GOC_ERR_ARG, "goc_periodic_ghosts: periodic directions need at least 2 cells");
    cudaStream_t st = as_stream(stream);
    int rc;
    if (bc_north == 2) {
        periodic_rows_kernel<<<dim3((nx + 4 + 127) / 128, 4), 128, 0, st>>>(nx, ny, eta, hu, hv, pitch / 4);
        count_launch();
        if ((rc = check_launch("periodic_rows_kernel"))) return rc;
    }
    if (bc_east == 2) {
        periodic_cols_kernel<<<dim3((ny + 4 + 127) / 128, 4), 128, 0, st>>>(nx, ny, eta, hu, hv, pitch / 4);
        count_launch();
        if ((rc = check_launch("periodic_cols_kernel"))) return rc;
    }
    return GOC_OK;
}

// Reduction blocks of the CFL kernels for an nx x ny grid; -1 when the grid
// is too large for one launch (block rows beyond the grid's y limit, or a
// count beyond INT_MAX).  The counts are formed in 64 bits.
extern "C" int goc_max_dt_partials(int nx, int ny) {
    if (nx < 1 || ny < 1) return 0;
    const long long bx = ((long long)nx + kDtBX - 1) / kDtBX, by = ((long long)ny + kDtBY - 1) / kDtBY;
    if (by > 65535 || bx * by > INT_MAX) return -1;
    return (int)(bx * by);
}

extern "C" int goc_max_dt(int nx, int ny, float dx, float dy, float g, const float* eta, const float* hu,
                          const float* hv, int pitch, const float* Hm, int Hm_pitch, float land_value,
                          float* partials, int partials_capacity, float* dt_out, void* stream) {
    if (nx < 1 || ny < 1) return set_error(GOC_ERR_ARG, "goc_max_dt: nx, ny must be >= 1");
    if (!eta || !hu || !hv || !Hm || !partials || !dt_out) return set_error(GOC_ERR_ARG, "goc_max_dt: null buffer");
    if (pitch < (nx + 4) * 4 || pitch % 4 || Hm_pitch < (nx + 4) * 4 || Hm_pitch % 4)
        return set_error(GOC_ERR_ARG, "goc_max_dt: pitch too small");
    const int need = goc_max_dt_partials(nx, ny);
    if (need < 0) return set_error(GOC_ERR_ARG, "goc_max_dt: a %d x %d grid is too large for one launch", nx, ny);
    if (partials_capacity < need)
        return set_error(GOC_ERR_ARG, "goc_max_dt: partials holds %d floats, %d needed", partials_capacity, need);
    cudaStream_t st = as_stream(stream);
    dim3 blk(kDtBX, kDtBY), grd((nx + kDtBX - 1) / kDtBX, (ny + kDtBY - 1) / kDtBY);
    dt_partials_kernel<<<grd, blk, 0, st>>>(nx, ny, dx, dy, g, eta, hu, hv, pitch / 4, Hm, Hm_pitch / 4,
                                            land_value, partials);
    count_launch();
    int rc = check_launch("dt_partials_kernel");
    if (rc) return rc;
    dt_final_kernel<<<1, 1024, 0, st>>>(partials, need, dt_out);
    count_launch();
    return check_launch("dt_final_kernel");
}

// ---------------------------------------------------------------------------
// CFL limit without allocation: the per-block partial minima live in a
// file-scope device array instead of caller-provided scratch.
// ---------------------------------------------------------------------------

#include <cuda.h>

#include <climits>
#include <mutex>

namespace goc {

// Room for the partial minima of grids up to 65536 reduction blocks of
// 32 x 8 cells (16.7 M interior cells, e.g. 4096 x 4096).  Every GPU that
// loads the library holds these 256 KiB until the process exits.
constexpr int kNoAllocPartials = 65536;
static __device__ __align__(256) float g_dt_partials[kNoAllocPartials];

// Device address of g_dt_partials, looked up once per device and context.
// In host code the array's name is only a host-side stand-in, so the address
// must come from cudaGetSymbolAddress with the device current.  The address
// belongs to the device's current context: when that context is replaced
// (cudaDeviceReset and a new primary context, or another context made
// current) the module is loaded anew and the address is looked up again.
// Contexts are told apart by their driver-assigned ID, which is never reused
// within a process.
constexpr int kMaxDevices = 64;
struct NoAllocSlot {
    float* addr = nullptr;
    unsigned long long ctx_id = 0;
};
static NoAllocSlot g_dt_partials_slot[kMaxDevices];
static std::mutex g_dt_partials_mutex;

// ID of the calling thread's current context (cuCtxGetCurrent + cuCtxGetId
// through the runtime's driver entry points, so the library need not link
// libcuda); false if the driver does not provide them.
static bool current_context_id(unsigned long long* id) {
    typedef CUresult (*GetCurrentFn)(CUcontext*);
    typedef CUresult (*GetIdFn)(CUcontext, unsigned long long*);
    static GetCurrentFn get_current = nullptr;
    static GetIdFn get_id = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrentFn>(p);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetIdFn>(p);
        cudaGetLastError();
    }
    CUcontext ctx = nullptr;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
    return get_id(ctx, id) == CUDA_SUCCESS;
}

static int noalloc_partials(float** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(GOC_ERR_CUDA, "goc_max_dt_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return set_error(GOC_ERR_UNSUPPORTED, "goc_max_dt_noalloc: device %d", dev);
    unsigned long long id = 0;
    bool have_id = current_context_id(&id);
    std::lock_guard<std::mutex> lock(g_dt_partials_mutex);
    NoAllocSlot& slot = g_dt_partials_slot[dev];
    if (!slot.addr || !have_id || slot.ctx_id != id) {
        // (also makes the device's primary context current if none is)
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_dt_partials);
        if (e != cudaSuccess)
            return set_error(GOC_ERR_CUDA, "goc_max_dt_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        slot.addr = static_cast<float*>(p);
        have_id = current_context_id(&id);
        slot.ctx_id = have_id ? id : 0;
    }
    *out = slot.addr;
    return GOC_OK;
}

}  // namespace goc

extern "C" int goc_max_dt_noalloc_capacity(void) { return goc::kNoAllocPartials; }

extern "C" int goc_max_dt_noalloc(int nx, int ny, float dx, float dy, float g, const float* eta, const float* hu,
                                  const float* hv, int pitch, const float* Hm, int Hm_pitch, float land_value,
                                  float* dt_out, void* stream) {
    if (nx < 1 || ny < 1) return set_error(GOC_ERR_ARG, "goc_max_dt_noalloc: nx, ny must be >= 1");
    const int need = goc_max_dt_partials(nx, ny);
    if (need < 0 || need > goc::kNoAllocPartials)
        return set_error(GOC_ERR_ARG,
                         "goc_max_dt_noalloc: a %d x %d grid needs %d partial minima, the built-in scratch holds %d "
                         "(at most %d reduction blocks of %d x %d cells); use goc_max_dt with caller scratch",
                         nx, ny, need, goc::kNoAllocPartials, goc::kNoAllocPartials, goc::kDtBX, goc::kDtBY);
    float* partials = nullptr;
    int rc = goc::noalloc_partials(&partials);
    if (rc) return rc;
    return goc_max_dt(nx, ny, dx, dy, g, eta, hu, hv, pitch, Hm, Hm_pitch, land_value, partials, need, dt_out,
                      stream);
}
