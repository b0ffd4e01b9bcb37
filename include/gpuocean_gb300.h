/*
 * gpuocean_gb300 - C ABI of the GB300 (sm_103a) CDKLM16 engine.
 *
 * Every entry point takes plain pointers and sizes, returns 0 on success and a
 * negative GOC_ERR_* code on failure; goc_last_error() then holds a message.
 * Device arrays are float32, row-major, one row = `pitch` bytes.  A state
 * array (eta, hu, hv) has (ny+4) rows of nx+4 cells (two ghost cells per
 * side); a corner-depth array Hi has (ny+5) rows of nx+5 values.
 *
 * Streams are opaque `void*` (a cudaStream_t; NULL = legacy default stream).
 *
 * Each kernel entry point below names the reference interface it replaces,
 * as a path relative to the GPU Ocean source tree:
 *   K/ = src/gpuocean/gpu_kernels, S/ = src/gpuocean/SWEsimulators,
 *   U/ = src/gpuocean/utils, D/ = src/gpuocean/drifters.
 */
#ifndef GPUOCEAN_GB300_H
#define GPUOCEAN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    GOC_OK = 0,
    GOC_ERR_ARG = -1,       /* invalid size / pointer / flag */
    GOC_ERR_CUDA = -2,      /* CUDA runtime error */
    GOC_ERR_UNSUPPORTED = -3,
    GOC_ERR_TIMEOUT = -4    /* a bounded device-side wait gave up */
};

/* Boundary flags as in U/Common.py:920-945: 1 = wall, 2 = periodic. */
enum { GOC_BC_WALL = 1, GOC_BC_PERIODIC = 2 };

/*
 * Parameters of one CDKLM16 simulator.  Replaces the compile-time #defines
 * of S/CDKLM16.py:242-269 and the scalar/texture kernel arguments of
 * S/CDKLM16.py:688-723 (cdklm_swe_2D, prepared format
 * "fiPiPiPiPiPiPiPiPifPPPPfPPPPfi").  Textures are device arrays of
 * (ny_tex, nx_tex) float32, looked up with clamped texel-centred bilinear
 * interpolation (K/interpolation.cu:137-190).
 */
typedef struct GocCdklmParams {
    int32_t nx, ny;                 /* interior cells */
    float dx, dy;                   /* cell size [m] */
    float g;                        /* gravity */
    float r;                        /* bottom friction (quadratic form) */
    float theta;                    /* minmod theta */
    float desing_eps;               /* desingularisation eps */
    float flux_slope_eps;           /* symmetric Riemann fan threshold */
    float depth_cutoff;             /* dry-cell depth */
    float flux_balancer;            /* upwind share of the transverse flux */
    float rho_o;                    /* water density (pressure forcing) */
    float wind_stress_factor;
    int32_t rk_order;               /* 1, 2 or 3 */
    int32_t one_dimensional;        /* skip y fluxes */
    int32_t bc_north, bc_east, bc_south, bc_west;
    float land_value;               /* corner depth that marks land (1e20) */
    const float* coriolis_f; int32_t coriolis_nx, coriolis_ny;
    const float* angle;      int32_t angle_nx, angle_ny;
    const float* wind_x_cur; const float* wind_x_next; int32_t wind_x_nx, wind_x_ny;
    const float* wind_y_cur; const float* wind_y_next; int32_t wind_y_nx, wind_y_ny;
    float wind_t;                   /* time interpolation weight in [0,1] */
    const float* atm_p_cur;  const float* atm_p_next; int32_t atm_p_nx, atm_p_ny;
    float atm_p_t;
} GocCdklmParams;

/* ---------------- runtime plumbing (device memory, streams, timing) ------ */

int goc_version(void);
int goc_last_error(char* buf, int len);
int goc_device_count(int* count);
int goc_set_device(int device);
int goc_device_synchronize(void);
int goc_malloc(void** ptr, size_t bytes);
int goc_free(void* ptr);
int goc_host_alloc(void** ptr, size_t bytes);   /* pinned host memory */
int goc_host_free(void* ptr);
int goc_memset_async(void* dst, int value, size_t bytes, void* stream);
int goc_memcpy_h2d_async(void* dst, const void* src, size_t bytes, void* stream);
int goc_memcpy_d2h_async(void* dst, const void* src, size_t bytes, void* stream);
int goc_memcpy_d2d_async(void* dst, const void* src, size_t bytes, void* stream);
int goc_stream_create(void** stream);
int goc_stream_destroy(void* stream);
int goc_stream_synchronize(void* stream);
int goc_event_create(void** event);
int goc_event_destroy(void* event);
int goc_event_record(void* event, void* stream);
int goc_event_elapsed_ms(void* start, void* stop, float* ms);
int goc_graph_begin_capture(void* stream);
int goc_graph_end_capture(void* stream, void** graph_exec);
int goc_graph_launch(void* graph_exec, void* stream);
int goc_graph_destroy(void* graph_exec);
/* Number of kernels this library has launched since load (all entry points). */
int64_t goc_kernel_launch_count(void);

/* ---------------- CDKLM16 step ------------------------------------------ */

/*
 * One full SSP-RK2 time step fused into a single launch.
 * Replaces, per step, S/CDKLM16.py:519-530 + :571-572: cdklm_swe_2D stage 0
 * (K/CDKLM16_kernel.cu:475), periodicBoundary_NS/EW on the stage buffer
 * (K/boundary_kernels.cu:36-110, U/Common.py:1310-1330), cdklm_swe_2D
 * stage 1 and the final periodic ghost fill.
 * Reads Q^n from (eta0, hu0, hv0), writes Q^{n+1} into (eta1, hu1, hv1):
 * interior cells, and for periodic boundaries also the ghost images.  The
 * two buffer sets must not overlap (the caller swaps them after the call).
 * Hi: corner depths after goc_bathymetry_init.
 */
int goc_cdklm_rk2_step(const GocCdklmParams* p, float dt,
                       const float* eta0, const float* hu0, const float* hv0,
                       float* eta1, float* hu1, float* hv1, int pitch,
                       const float* Hi, int Hi_pitch, void* stream);

/*
 * One Runge-Kutta stage, reference semantics: cdklm_swe_2D
 * (K/CDKLM16_kernel.cu:475-1090) with rk_step = step_.  Interior cells of
 * the output set are written; for RK2 stage 1 and RK3 stages 1-2 the output
 * set must hold Q^n on entry.  For RK3 stage 1 the result is written to
 * `q_alt` (the reference writes it back into the input buffer,
 * K/CDKLM16_kernel.cu:1076-1083); pass NULL elsewhere.
 */
int goc_cdklm_stage(const GocCdklmParams* p, float dt, int rk_step,
                    const float* eta_in, const float* hu_in, const float* hv_in,
                    float* eta_out, float* hu_out, float* hv_out,
                    float* eta_alt, float* hu_alt, float* hv_alt, int pitch,
                    const float* Hi, int Hi_pitch, void* stream);

/*
 * Periodic ghost-cell fill, north/south before east/west.
 * Replaces periodicBoundary_NS / periodicBoundary_EW
 * (K/boundary_kernels.cu:36-110) driven by
 * BoundaryConditionsArakawaA.boundaryCondition (U/Common.py:1310-1330).
 */
int goc_periodic_ghosts(int nx, int ny, int bc_north, int bc_east,
                        float* eta, float* hu, float* hv, int pitch, void* stream);

/*
 * Bathymetry set-up: makes the corner depths periodic or mirrored and
 * computes the cell means.  Replaces U/Common.py:1438-1491,1538-1561:
 * periodic/closed_boundary_intersections_NS/EW (K/boundary_kernels.cu:122-247)
 * and initBm (K/initHm_kernel.cu:38-106).  Hi is updated in place; Hm gets
 * (ny+4) x (nx+4) cell means (land_value where all corners are land).
 */
int goc_bathymetry_init(int nx, int ny, int bc_north, int bc_east, int bc_south,
                        int bc_west, float land_value, float* Hi, int Hi_pitch,
                        float* Hm, int Hm_pitch, void* stream);

/*
 * CFL limit: writes min over interior cells of
 * min(0.25 dx/|u +- sqrt(g h)|, 0.25 dy/|v +- sqrt(g h)|) (1e5 for dry or
 * land cells) to dt_out[0], before the Courant factor.
 * Replaces per_block_max_dt + max_dt_reduction (K/max_dt.cu:42-195,
 * S/CDKLM16.py:814-841).  `partials` is caller-provided scratch of at least
 * goc_max_dt_partials(nx, ny) floats.
 */
int goc_max_dt_partials(int nx, int ny);
int goc_max_dt(int nx, int ny, float dx, float dy, float g,
               const float* eta, const float* hu, const float* hv, int pitch,
               const float* Hm, int Hm_pitch, float land_value,
               float* partials, int partials_capacity, float* dt_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GPUOCEAN_GB300_H */
