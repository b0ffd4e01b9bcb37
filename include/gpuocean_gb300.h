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
    /* optional: the texture evaluated at every cell centre, (ny+4) x (nx+4)
     * with pitch coriolis_cell_pitch bytes (goc_cell_texture); NULL = look
     * the texture up in the kernel */
    const float* coriolis_cell; int32_t coriolis_cell_pitch;
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
/* Device-side ordering (no host wait): every stream of `waiters` waits for
 * the work queued so far on `signaller` (fan_out), or `waiter` waits for the
 * work queued so far on every stream of `signallers` (fan_in).  A batched
 * ensemble uses them to order its own stream with its members' streams. */
int goc_stream_fan_out(void* signaller, void* const* waiters, int n_waiters);
int goc_stream_fan_in(void* waiter, void* const* signallers, int n_signallers);
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
 * Hi, Hm: corner depths and cell means from goc_bathymetry_init (the
 * reference kernel takes the same pair, Hi_ptr_/Hm_ptr_).
 */
int goc_cdklm_rk2_step(const GocCdklmParams* p, float dt,
                       const float* eta0, const float* hu0, const float* hv0,
                       float* eta1, float* hu1, float* hv1, int pitch,
                       const float* Hi, int Hi_pitch, const float* Hm, int Hm_pitch,
                       void* stream);

/*
 * n_steps fused RK2 steps (dts in host memory), from buffer set 0
 * (eta0, hu0, hv0) alternating with set 1; the state ends in set
 * n_steps % 2.  The loop of CDKLM16.step (S/CDKLM16.py:493-509) for a run of
 * steps with nothing between them (no model error, drifters, sponge or
 * time-varying forcing), issued from the library.
 */
int goc_cdklm_rk2_steps(const GocCdklmParams* p, const float* dts, int n_steps, float* eta0, float* hu0,
                        float* hv0, float* eta1, float* hu1, float* hv1, int pitch, const float* Hi, int Hi_pitch,
                        const float* Hm, int Hm_pitch, void* stream);

/*
 * goc_cdklm_rk2_step that also writes the first-stage state Q* of the
 * interior cells to (eta_s, hu_s, hv_s): the same values goc_cdklm_stage
 * with rk_step 0 gives, at no extra launch.  For the adjoint's recompute of
 * a rollout segment (no counterpart in the reference).
 */
int goc_cdklm_rk2_step_stage(const GocCdklmParams* p, float dt,
                             const float* eta0, const float* hu0, const float* hv0,
                             float* eta1, float* hu1, float* hv1,
                             float* eta_s, float* hu_s, float* hv_s, int pitch,
                             const float* Hi, int Hi_pitch, const float* Hm, int Hm_pitch,
                             void* stream);

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
                    const float* Hi, int Hi_pitch, const float* Hm, int Hm_pitch,
                    void* stream);

/*
 * Evaluate a texture at every cell centre of an (ny+4) x (nx+4) grid,
 * s = (i+0.5)/(nx+4), t = (j+0.5)/(ny+4), with the kernels' bilinear lookup
 * (the positions coriolisF uses, K/CDKLM16_kernel.cu:49-57).  Fills
 * GocCdklmParams.coriolis_cell.
 */
int goc_cell_texture(const float* tex, int tex_nx, int tex_ny, int nx, int ny,
                     float* out, int out_pitch, void* stream);

/*
 * Periodic ghost-cell fill, north/south before east/west.
 * Replaces periodicBoundary_NS / periodicBoundary_EW
 * (K/boundary_kernels.cu:36-110) driven by
 * BoundaryConditionsArakawaA.boundaryCondition (U/Common.py:1310-1330).
 */
int goc_periodic_ghosts(int nx, int ny, int bc_north, int bc_east,
                        float* eta, float* hu, float* hv, int pitch, void* stream);

/*
 * Open (sponge) boundaries, BoundaryConditionsArakawaA.boundaryCondition for
 * flags 3 (flow relaxation scheme) and 4 (linear interpolation)
 * (U/Common.py:1310-1350, K/boundary_kernels.cu:250-541): north-south first,
 * then east-west; a periodic pair (flag 2) is skipped here (goc_periodic_ghosts
 * fills it).  sponge_cells = {north, east, south, west}: rows / columns of the
 * (ny+4) x (nx+4) array, ghost cells included, that each sponge spans.  The
 * flow relaxation reads the exterior solution from (2 x ns_nx x 3) float
 * arrays (row 0 south, row 1 north; channels eta, hu, hv) and
 * (ew_ny x 2 x 3) arrays (column 0 west, column 1 east), blended as
 * bc_t * next + (1 - bc_t) * current.  Device memory, pitch in bytes.
 */
int goc_sponge_boundary(int nx, int ny, int bc_north, int bc_east, int bc_south, int bc_west,
                        const int* sponge_cells, float* eta, float* hu, float* hv, int pitch,
                        const float* ns_current, const float* ns_next, int ns_nx,
                        const float* ew_current, const float* ew_next, int ew_ny, float bc_t, void* stream);

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
 * goc_max_dt_partials(nx, ny) floats (-1: the grid is too large for one
 * launch, and goc_max_dt rejects it with GOC_ERR_ARG).
 */
int goc_max_dt_partials(int nx, int ny);
int goc_max_dt(int nx, int ny, float dx, float dy, float g,
               const float* eta, const float* hu, const float* hv, int pitch,
               const float* Hm, int Hm_pitch, float land_value,
               float* partials, int partials_capacity, float* dt_out, void* stream);

/*
 * The CFL limit of goc_max_dt without any allocation by the caller or the
 * library: the per-block partial minima go to a scratch array that is part
 * of the library image (no counterpart in the reference, whose Python host
 * allocates its dt buffers with PyCUDA).  For callers that cannot allocate
 * device memory on their step path: a host model that owns all device memory
 * through its own pool and has no allocator to lend, or a loop that must not
 * pay the implicit device synchronisation of cudaMalloc/cudaFree.
 *  - Limit: goc_max_dt_noalloc_capacity() partial minima (65536, i.e. grids of
 *    up to 65536 blocks of 32 x 8 interior cells); larger grids are rejected
 *    with GOC_ERR_ARG.  The array (256 KiB) stays resident on every GPU that
 *    loads the library until the process exits.
 *  - The first call on a device looks up the array's device address with
 *    cudaGetSymbolAddress while that device is current; make that first call
 *    before any stream capture.  The address belongs to the device's current
 *    context: after that context is replaced (cudaDeviceReset and a new
 *    primary context, or another context made current) the next call looks
 *    the address up again, and that call too must come before any capture.
 *  - All calls share the one array: calls whose kernels overlap on the GPU
 *    (e.g. on two streams at once) race.  Each call overwrites every partial
 *    it reads, so nothing needs clearing between calls.
 *  - No cudaMalloc, cudaFree or allocating library routine is called.
 */
int goc_max_dt_noalloc_capacity(void);
int goc_max_dt_noalloc(int nx, int ny, float dx, float dy, float g,
                       const float* eta, const float* hu, const float* hv, int pitch,
                       const float* Hm, int Hm_pitch, float land_value, float* dt_out, void* stream);

/* ---------------- adjoint of the RK2 step --------------------------------- */

/*
 * Vector-Jacobian product of one RK2 stage (no counterpart in the reference,
 * which has no adjoint).  With y the stage output on interior cells,
 *   rk_step 0:  y = S1(x),     x = Q^n        (the first stage)
 *   rk_step 1:  y = S2(a, x),  x = Q*, a = Q^n (the second stage)
 * the call writes, on interior cells,
 *   xb = base + (dS/dx)^T yb      (base may be NULL)
 *   ab = (dS2/da)^T yb             (rk_step 1 only)
 * and, if wind_partials is not NULL, ADDS to its goc_cdklm_vjp_partials(nx, ny)
 * floats the per-tile partial sums (x, y interleaved) of (dS/dX_eff)^T yb
 * (the caller zeroes them; calls on one stream may share them), where
 * X_eff = wind_stress_factor * stress is the uniform wind stress the step
 * adds.  Ghost cells of the adjoint arrays are neither read nor written:
 * ghost cells of the state are periodic images or wall mirrors of interior
 * cells, and their adjoint is folded onto those cells.  Branches (limiter,
 * dry clamps, desingularisation) follow the recomputed forward state.
 * Requirements: rk_order 2, uniform (1x1) wind stress, no pressure field,
 * nx >= 40 with periodic x and ny >= 24 with periodic y.  An RK2 step's VJP
 * is the rk_step-1 call (x = Q*, a = Q^n, yb = lambda^{n+1}, xb = lambda*,
 * ab = lambda^n) followed by the rk_step-0 call (x = Q^n, yb = lambda*,
 * base = xb = lambda^n); Q* comes from goc_cdklm_stage with rk_step 0.
 */
int goc_cdklm_vjp_partials(int nx, int ny);

/*
 * Member-batched forms for ensembles that share parameters and bathymetry
 * but not their state (no counterpart in the reference): member z of one
 * launch works on the buffers at offset z * member_stride floats from the
 * given pointers, and reads its uniform wind stress at offset
 * z * wind_stride floats from the parameters' wind pointers (0 = shared).
 * goc_cdklm_rk2_step_members is goc_cdklm_rk2_step_stage for n_members
 * members (eta_s, hu_s, hv_s may be NULL); goc_cdklm_stage_vjp_members is
 * goc_cdklm_stage_vjp for n_members members, member z writing its
 * goc_cdklm_vjp_partials(nx, ny) wind partials at z times that count.
 */
int goc_cdklm_rk2_step_members(const GocCdklmParams* p, float dt,
                               const float* eta0, const float* hu0, const float* hv0,
                               float* eta1, float* hu1, float* hv1,
                               float* eta_s, float* hu_s, float* hv_s, int pitch,
                               long long member_stride, int n_members, int wind_stride,
                               const float* Hi, int Hi_pitch, const float* Hm, int Hm_pitch,
                               void* stream);
int goc_cdklm_stage_vjp_members(const GocCdklmParams* p, float dt, int rk_step,
                                const float* x_eta, const float* x_hu, const float* x_hv,
                                const float* a_eta, const float* a_hu, const float* a_hv,
                                const float* yb_eta, const float* yb_hu, const float* yb_hv,
                                const float* base_eta, const float* base_hu, const float* base_hv,
                                float* xb_eta, float* xb_hu, float* xb_hv,
                                float* ab_eta, float* ab_hu, float* ab_hv, int pitch,
                                long long member_stride, int n_members, int wind_stride,
                                const float* Hi, int Hi_pitch, const float* Hm, int Hm_pitch,
                                float* wind_partials, void* stream);
int goc_cdklm_stage_vjp(const GocCdklmParams* p, float dt, int rk_step,
                        const float* x_eta, const float* x_hu, const float* x_hv,
                        const float* a_eta, const float* a_hu, const float* a_hv,
                        const float* yb_eta, const float* yb_hu, const float* yb_hv,
                        const float* base_eta, const float* base_hu, const float* base_hv,
                        float* xb_eta, float* xb_hu, float* xb_hv,
                        float* ab_eta, float* ab_hu, float* ab_hv, int pitch,
                        const float* Hi, int Hi_pitch, const float* Hm, int Hm_pitch,
                        float* wind_partials, void* stream);

/*
 * The same VJPs given the stage output y as well (no counterpart in the
 * reference): rk_step 0 takes y = Q*, rk_step 1 y = Q^{n+1}, exactly as the
 * forward step wrote them (goc_cdklm_rk2_step_stage keeps both).  The
 * updated state and the dry clamp of each cell then come from y instead of
 * from a recompute of the stage's fluxes, which the kernel skips; results
 * are those of goc_cdklm_stage_vjp except where the final clamp ties (a wet
 * cell at rest that the clamp raised to exactly -Hm + depth_cutoff reads as
 * dried).  A rollout's backward sweep has y at hand.
 */
int goc_cdklm_stage_vjp_out(const GocCdklmParams* p, float dt, int rk_step,
                            const float* x_eta, const float* x_hu, const float* x_hv,
                            const float* a_eta, const float* a_hu, const float* a_hv,
                            const float* y_eta, const float* y_hu, const float* y_hv,
                            const float* yb_eta, const float* yb_hu, const float* yb_hv,
                            const float* base_eta, const float* base_hu, const float* base_hv,
                            float* xb_eta, float* xb_hu, float* xb_hv,
                            float* ab_eta, float* ab_hu, float* ab_hv, int pitch,
                            const float* Hi, int Hi_pitch, const float* Hm, int Hm_pitch,
                            float* wind_partials, void* stream);
int goc_cdklm_stage_vjp_members_out(const GocCdklmParams* p, float dt, int rk_step,
                                    const float* x_eta, const float* x_hu, const float* x_hv,
                                    const float* a_eta, const float* a_hu, const float* a_hv,
                                    const float* y_eta, const float* y_hu, const float* y_hv,
                                    const float* yb_eta, const float* yb_hu, const float* yb_hv,
                                    const float* base_eta, const float* base_hu, const float* base_hv,
                                    float* xb_eta, float* xb_hu, float* xb_hv,
                                    float* ab_eta, float* ab_hu, float* ab_hv, int pitch,
                                    long long member_stride, int n_members, int wind_stride,
                                    const float* Hi, int Hi_pitch, const float* Hm, int Hm_pitch,
                                    float* wind_partials, void* stream);

/* ---------------- drifters ---------------------------------------------- */

/*
 * Advect num_drifters + 1 positions (the last is the observation) by one
 * forward-Euler step with cell-centred bilinear velocities hu/(Hm + eta),
 * optional wind drift and periodic wrap.  Replaces passiveDrifterKernel
 * (K/driftKernels.cu:74-183) as launched by GPUDrifterCollection.drift
 * (D/GPUDrifterCollection.py:210-233, prepared "iifffiiPiPiPiPiiiiPifPPPPff").
 * Cell indices outside the grid are clamped.
 */
int goc_drift(int nx, int ny, float dx, float dy, float dt, int x_zero_ref, int y_zero_ref,
              const float* eta, const float* hu, const float* hv, int pitch,
              const float* Hm, int Hm_pitch, int periodic_north_south, int periodic_east_west,
              int num_drifters, float* positions, int positions_pitch, float sensitivity,
              const float* wind_x_cur, const float* wind_x_next,
              const float* wind_y_cur, const float* wind_y_next, int wind_nx, int wind_ny,
              float wind_t, float wind_drift_factor, void* stream);

/*
 * Adjoint of one goc_drift step without wind drift (no counterpart in the
 * reference).  positions: the positions before the step; positions_bar
 * holds the adjoint of the positions after the step on entry and of those
 * before it on return.  The adjoint of the state the step read (interior
 * cells; periodic ghost images folded onto their cells, wall ghosts carry
 * none) is ADDED to (eta_bar, hu_bar, hv_bar) with atomic additions, so the
 * summation order, and the last bits of the sums, vary between runs.
 */
int goc_drift_vjp(int nx, int ny, float dx, float dy, float dt, int x_zero_ref, int y_zero_ref,
                  const float* eta, const float* hu, const float* hv, int pitch,
                  const float* Hm, int Hm_pitch, int periodic_north_south, int periodic_east_west,
                  int num_positions, const float* positions, int positions_pitch,
                  float* positions_bar, int positions_bar_pitch, float sensitivity,
                  float* eta_bar, float* hu_bar, float* hv_bar, void* stream);

/* Periodic wrap of drifter positions; replaces enforceBoundaryConditions
 * (K/driftKernels.cu:187-223). */
int goc_drift_enforce_boundary(float domain_size_x, float domain_size_y, int periodic_north_south,
                               int periodic_east_west, int num_drifters, float* positions,
                               int positions_pitch, void* stream);

/* ---------------- stochastic model error (SOAR) --------------------------- */

/*
 * One SOAR model-error configuration (S/OceanStateNoise.py:47-272): a
 * coarse grid with interpolation_factor cells per coarse cell, a random
 * field of (cny, cnx) normals in each periodic direction and (cny+8, cnx+8)
 * otherwise, and the (cny+4, cnx+4) coarse buffer the SOAR field goes to.
 * f, beta, g, north_x/y feed the geostrophic balance
 * (K/ocean_noise.cu:361-378); with f == 0 the Coriolis texture is used.
 */
typedef struct GocNoiseDesc {
    int32_t coarse_nx, coarse_ny;
    float coarse_dx, coarse_dy;
    float soar_q0, soar_L;
    int32_t periodic_ns, periodic_ew;
    int32_t interpolation_factor;
    int32_t offset_i, offset_j;        /* coarse-grid alignment offsets */
    const float* random; int32_t random_pitch;   /* bytes */
    float* coarse; int32_t coarse_pitch;         /* bytes */
    float f, beta, g;
    float north_x, north_y;
    const float* coriolis_f; int32_t coriolis_nx, coriolis_ny;
} GocNoiseDesc;

/* LCG draws (K/random_number_generators.cu:58-134 uniformDistribution /
 * normalDistribution, launched by U/RandomNumbers.py:165-185): each uint64
 * seed advances twice and gives two numbers; normal = Box-Muller. */
int goc_lcg_fill(int seed_nx, int seed_ny, int random_nx, unsigned long long* seeds, int seed_pitch,
                 float* random, int random_pitch, int normal, void* stream);

/* curand XORWOW normals, the reference's default generator
 * (U/RandomNumbers.py:86-97 via pycuda.curandom).  `states` holds
 * goc_xorwow_state_bytes(nx*ny) bytes. */
size_t goc_xorwow_state_bytes(int n);
int goc_xorwow_init(void* states, int n, unsigned long long seed, void* stream);
int goc_xorwow_normal(void* states, int nx, int ny, float* random, int random_pitch, void* stream);

/* SOAR-correlated coarse field from the random field
 * (K/ocean_noise.cu:141-247, S/OceanStateNoise.py:394-416). */
int goc_soar(const GocNoiseDesc* noise, float perturbation_scale, int additive, void* stream);

/* Add the coarse field (bicubic up-sampled for factors > 1) and its
 * geostrophically balanced momentum to the interior of (eta, hu, hv);
 * replaces geostrophicBalance / bicubicInterpolation (K/ocean_noise.cu:256-666,
 * S/OceanStateNoise.py:418-459).  periodic_ghosts = 1 also refreshes the
 * periodic ghost images of the perturbed cells. */
int goc_perturb_ocean(const GocNoiseDesc* noise, int nx, int ny, float dx, float dy,
                      float* eta, float* hu, float* hv, int pitch, const float* Hi, int Hi_pitch,
                      float land_value, int periodic_ghosts, void* stream);

/* ---------------- batched ensemble engine -------------------------------- */

/*
 * One ensemble member: parameters, bathymetry and its two state buffer
 * sets.  Members may differ in grid size, spacing, physics and boundaries.
 * Replaces the per-member simulator objects that the reference's ensembles
 * step in Python loops (E/OceanNoiseEnsemble.py:517-543,
 * E/OceanModelEnsemble.py:138-150, E/MultiLevelOceanEnsemble.py:95-141;
 * E/ = src/gpuocean/ensembles).
 */
typedef struct GocMemberDesc {
    GocCdklmParams p;
    const float* Hi;  int32_t Hi_pitch;     /* corner depths (bytes pitch) */
    const float* Hm;  int32_t Hm_pitch;     /* cell means (for the CFL limit) */
    float* eta[2]; float* hu[2]; float* hv[2];  /* buffer set 0 holds the state */
    int32_t pitch;                          /* state pitch in bytes */
} GocMemberDesc;

/*
 * Build an ensemble handle: copies the member table to the device and
 * builds the member/tile work queue (member-major 32x16 tiles).  Up to
 * `max_substeps` RK2 steps can be scheduled per block.
 */
int goc_ensemble_create(const GocMemberDesc* members, int n_members, int max_substeps, void** ensemble);
int goc_ensemble_destroy(void* ensemble);
int goc_ensemble_size(void* ensemble, int* n_members, int* n_tiles);
/*
 * TMA staging of the step's input state: number of members whose interior
 * tiles load (eta, hu, hv) by tensor-map bulk copies (every buffer on a
 * 16-byte boundary and a row pitch that is a multiple of 16 bytes), the
 * number of tiles staged so far, and the device flag set when a staging wait
 * ran out (0 in normal operation; the CTA then loads with ordinary loads).
 * Reading the device counters synchronises.  Any output may be NULL.
 */
int goc_ensemble_tma_status(void* ensemble, int* staged_members, long long* staged_tiles, int* wait_errors);
/*
 * The staging error flag as of the last block that completed on the device,
 * without synchronising: goc_ensemble_end_block copies the device flag into
 * pinned host memory at the end of every block.  Nonzero means a CTA's
 * staged input never landed and that CTA stopped stepping: the states of
 * that block are not valid.  (Batched engine; no counterpart in the
 * reference.)
 */
int goc_ensemble_staging_errors(void* ensemble, int* errors);
/*
 * Self-test of the bounded wait that guards TMA staging: one CTA waits on an
 * mbarrier phase that nothing completes, for limit_ms (0 < limit_ms <= 1000)
 * of the GPU's global timer.  timed_out = 1 when the wait gave up as it
 * should; waited_ms = the time it waited.  Nothing faults and nothing hangs:
 * the kernel returns and the context stays usable.
 */
int goc_selftest_wait_timeout(double limit_ms, int* timed_out, double* waited_ms);

/*
 * Per-member step schedule of one block: dt_table is n_members x
 * max_substeps (row-major, host memory), member m takes n_substeps[m] steps.
 * This is the dt sequence of S/CDKLM16.py:493-509 (local_dt = min(dt,
 * t_end - t_now)) evaluated once per member on the host.
 */
int goc_ensemble_set_schedule(void* ensemble, const float* dt_table, const int* n_substeps, void* stream);

/*
 * Step k of the block for every member with k < n_substeps[m]: one
 * persistent launch over the member/tile work queue; each tile runs the
 * fused RK2 step (see goc_cdklm_rk2_step) from set (k % 2) into set
 * ((k + 1) % 2).  Graph-capturable.
 */
int goc_ensemble_rk2_substep(void* ensemble, int k, void* stream);

/*
 * Output tile shapes of the persistent kernel (no counterpart in the
 * reference).  goc_ensemble_tile_shape gives shape `index` in cells;
 * goc_ensemble_set_tile_shape rebuilds the member/tile work queue for it
 * (synchronises the device; call outside stream capture, and re-capture
 * graphs afterwards).  Every shape computes bit-identical states; the
 * autotuner (BatchedEnsemble.autotune) times them and keeps the fastest.
 */
int goc_ensemble_tile_shape_count(void);
int goc_ensemble_tile_shape(int index, int* tx, int* ty);
int goc_ensemble_set_tile_shape(void* ensemble, int index);
int goc_ensemble_get_tile_shape(void* ensemble, int* index);

/* Close a block of `n_launched` substeps: advects the drifters of the last
 * step of members that ran all of them, then makes buffer set 0 the current
 * state again (swaps members whose block had an odd number of steps).
 * Graph-capturable. */
int goc_ensemble_end_block(void* ensemble, int n_launched, void* stream);

/*
 * Attach drifters: positions[m] is member m's device array of
 * (num_drifters[m] + 1) x 2 floats (x, y in metres from the south-west
 * interior corner; the last row is the observation position), NULL for a
 * member without drifters.  Each RK2 substep then also advects the
 * drifters with the state after the previous substep, as
 * GPUDrifterCollection.driftFromSim does after every step
 * (D/GPUDrifterCollection.py:198-233, K/driftKernels.cu:74-183); wind drift
 * with goc_ensemble_set_drift_wind.
 */
int goc_ensemble_set_drifters(void* ensemble, float* const* positions, const int* num_drifters,
                              float sensitivity, void* stream);

/*
 * Wind drift of ensemble drifters (the wind branch of passiveDrifterKernel,
 * K/driftKernels.cu:151-157, as GPUDrifterCollection(wind=...,
 * wind_drift_factor=...) applies it): wind[m] gives member m's current and
 * next wind textures (device, nx x ny, both components read with that size
 * as the reference does) and factor (0: no wind drift).  Those members'
 * drifters then move in a launch of their own before each persistent step
 * (and at the end of the block), with the time weight of each step's drift
 * from goc_ensemble_set_wind_times: an n_members x max_substeps host table,
 * entry (m, k) for the drift after step k.  Call goc_ensemble_set_drift_wind
 * again after goc_ensemble_set_drifters.  Synchronise `stream`.
 */
typedef struct GocDriftWindDesc {
    const float* x_current; const float* x_next;
    const float* y_current; const float* y_next;
    int32_t nx, ny;
    float wind_drift_factor;
} GocDriftWindDesc;
int goc_ensemble_set_drift_wind(void* ensemble, const GocDriftWindDesc* wind, void* stream);
int goc_ensemble_set_wind_times(void* ensemble, const float* wind_t, void* stream);

/*
 * Every member's drifter rows (N_m positions and the observation row) in one
 * packed (rows x 2) float array, member by member, and the observation rows of
 * every member with drifters from an (n_members x 2) array: one launch each
 * instead of a copy per member (the reference reads and writes each
 * collection on its own, D/GPUDrifterCollection.py:179-200).  Device memory;
 * goc_ensemble_drifter_rows gives the packed row count.
 */
int goc_ensemble_drifter_rows(void* ensemble, long long* rows);
int goc_ensemble_gather_drifters(void* ensemble, float* dst, void* stream);
int goc_ensemble_scatter_observations(void* ensemble, const float* src, void* stream);

/* Copy member m's current descriptor (device pointers) to the host.
 * Synchronises `stream`. */
int goc_ensemble_get_member(void* ensemble, int m, GocMemberDesc* out, void* stream);

/*
 * CFL limit of every member into dt_out[0..n_members) (device memory), the
 * batched form of goc_max_dt.  Uses per-block partial minima held in
 * scratch owned by the ensemble handle.
 */
int goc_ensemble_max_dt(void* ensemble, float* dt_out, void* stream);

/*
 * Model error of every member in two launches (SOAR over all coarse grids,
 * then the balanced transfer into each member's state, with periodic ghost
 * images).  noise[m] configures member m of `ensemble`.  Replaces the
 * per-member OceanStateNoise.perturbSim calls of the reference's ensembles
 * (E/OceanNoiseEnsemble.py:517-543 via S/CDKLM16.py:567-568,726-733).
 * substep = -1 perturbs every member's current state between blocks;
 * substep = -2 only the members that took model error in the block just
 * ended (see goc_ensemble_set_noise_mask);
 * substep = k perturbs, right after RK2 step k of a block, the members that
 * took step k (the cadence of step(t, apply_stochastic_term=True)).
 * goc_noise_batch_generate draws new XORWOW normals into the members'
 * random fields (same substep rule) after goc_noise_batch_seed.
 */
int goc_noise_batch_create(void* ensemble, const GocNoiseDesc* noise, void** batch);
int goc_noise_batch_destroy(void* batch);
int goc_noise_batch_seed(void* batch, unsigned long long seed, void* stream);
int goc_noise_batch_generate(void* batch, void* ensemble, int substep, void* stream);
int goc_noise_batch_perturb(void* batch, void* ensemble, float perturbation_scale, int substep, void* stream);

/*
 * Model error fused into the ensemble step (the batched engine's form of
 * perturbState after a step, S/CDKLM16.py:567-568 and 786-790; no
 * counterpart kernel in the reference).  goc_noise_batch_field computes only
 * the SOAR coarse fields (same substep rule as goc_noise_batch_perturb).
 * goc_ensemble_set_block_noise(ensemble, batch, mode) then makes the
 * following goc_ensemble_rk2_substep launches add each member's up-sampled,
 * geostrophically balanced perturbation to Q^{n+1} inside the step, before
 * the write, instead of a separate read-modify-write pass:
 *   mode 0: members perturb after the last step of their block (the
 *           dataAssimilationStep cadence); the drifters of that last step
 *           move with the state before the perturbation, read from an
 *           unperturbed copy the step writes (allocated here, one buffer
 *           set per member with drifters);
 *   mode 1: members perturb after every step (the CDKLM16.step cadence),
 *           before their drifters move;
 *   mode -1: no fused model error.
 * The mode stays in force, also for goc_ensemble_end_block, until changed.
 * The coarse fields must be computed before the first perturbing launch and
 * stay unchanged until the last.  Results are bit-identical to stepping and
 * then calling goc_noise_batch_perturb.  Call outside stream capture.
 */
int goc_noise_batch_field(void* batch, void* ensemble, float perturbation_scale, int substep, void* stream);
int goc_ensemble_set_block_noise(void* ensemble, void* noise_batch, int mode);

/*
 * Which members take model error inside a block (mask[m] != 0), for a truth
 * and particles stepped with different stochastic flags
 * (E/OceanNoiseEnsemble.py:517-543; the reference calls step with
 * apply_stochastic_term per member).  NULL: every member.  Applies to every
 * later block (fused or not, SOAR or KL) until changed; perturbations
 * between blocks (substep -1) ignore it.  Synchronises `stream`.
 */
int goc_ensemble_set_noise_mask(void* ensemble, const int* mask, void* stream);

/* ------------------------------------------------------------------------
 * Karhunen-Loeve model error (S/ModelErrorKL.py:38-463, K/ocean_noise.cu:666-954)
 * ------------------------------------------------------------------------ */

/*
 * One KL model error: d_eta(x, y) = scale * kl_scaling * sum over basis rows
 * j (m = basis_y_start + j) and columns i (n = basis_x_start + i) of
 * m^-kl_decay n^-kl_decay (r_sin[j][i] sin(2 pi m y_s) sin(2 pi n x_s) +
 * r_cos[j][i] cos(2 pi m y_c) cos(2 pi n x_c)) on the unit square, with
 * x_s = x + roll_x_sin etc.; random holds the (2 Ny) x Nx normals (sine rows
 * first), pitch in bytes.  The sum is separable: per column a table of the
 * x sums, per row the y factors, so a cell costs 2 Ny multiply-adds instead
 * of 4 Nx Ny transcendental terms.  table: device scratch of
 * goc_kl_table_floats(nx, ny, kl) floats.  f, beta, g, north and the
 * Coriolis texture as for the SOAR noise.
 */
typedef struct GocKLDesc {
    int32_t basis_x_start, basis_x_end, basis_y_start, basis_y_end;
    int32_t include_cos, include_sin;
    float kl_decay, kl_scaling;
    float roll_x_sin, roll_y_sin, roll_x_cos, roll_y_cos;
    const float* random; int32_t random_pitch;
    float f, beta, g;
    float north_x, north_y;
    const float* coriolis_f; int32_t coriolis_nx, coriolis_ny;
    float* table;
} GocKLDesc;

/* Scratch size (floats) of the basis tables for an nx x ny grid; < 0 on bad
 * arguments. */
long long goc_kl_table_floats(int nx, int ny, const GocKLDesc* kl);

/*
 * kl_sample_eta (eta_only = 1) or kl_sample_ocean_state (eta_only = 0,
 * with the geostrophically balanced hu, hv of K/ocean_noise.cu:901-947):
 * adds the KL perturbation times perturbation_scale to the interior of the
 * (ny+4) x (nx+4) state.  With periodic_ns / periodic_ew the periodic ghost
 * images of the perturbed cells are written as well (the boundary fill the
 * reference runs after perturbState in CDKLM16.step).  Two launches: the
 * basis tables, then the perturbation.
 */
int goc_kl_perturb(const GocKLDesc* kl, int nx, int ny, float dx, float dy, float perturbation_scale,
                   int eta_only, float* eta, float* hu, float* hv, int pitch, const float* Hi, int Hi_pitch,
                   int periodic_ns, int periodic_ew, void* stream);

/*
 * KL model error of every member of an ensemble.  kl[m] configures member m
 * (its table and random pointers are ignored: the batch owns both);
 * source[m] is the member whose normals and rollers member m uses (m itself,
 * or the fine partner of a multi-level pair, the coupling of
 * perturbSimilarAs, S/CDKLM16.py:782-790).  goc_kl_batch_seed seeds XORWOW
 * states for every source member's normals and rollers; goc_kl_batch_generate draws new
 * normals and rollers on the device (substep rule of
 * goc_noise_batch_perturb; the rollers go to set 0 for substep -1 or -2,
 * set substep + 1 otherwise);
 * goc_kl_batch_set_rollers uploads n_sets x n_members x 4 rollers (host;
 * set 0 is used with substep -1 and -2, set k + 1 with substep k);
 * goc_kl_batch_set_random copies host normals for member m's source.
 */
int goc_kl_batch_create(void* ensemble, const GocKLDesc* kl, const int* source, int max_sets, void** batch);
int goc_kl_batch_destroy(void* batch);
int goc_kl_batch_seed(void* batch, unsigned long long seed, void* stream);
int goc_kl_batch_generate(void* batch, void* ensemble, int substep, void* stream);
int goc_kl_batch_set_rollers(void* batch, const float* rollers, int n_sets, void* stream);
int goc_kl_batch_set_random(void* batch, int member, const float* host_normals, void* stream);
int goc_kl_batch_perturb(void* batch, void* ensemble, float perturbation_scale, int substep, void* stream);

/* ------------------------------------------------------------------------
 * Observation operator and ensemble statistics
 * ------------------------------------------------------------------------ */

/*
 * Drop-in for the observeUnderlyingFlow kernel (K/observationKernels.cu:29-83,
 * launched from E/BaseOceanStateEnsemble.py:117-130 with the prepared format
 * "iiffiiPiPiPifiPiPi" of E/OceanNoiseEnsemble.py:333-339): for drifter d
 * at positions + d * positions_pitch (x, y in metres), observations + d *
 * observation_pitch receives (hu, hv) of the cell
 * (floor(x / dx) + x_zero_ref, floor(y / dy) + y_zero_ref).  Pitches in
 * bytes.  eta and H are accepted for signature parity and not read (the
 * reference reads neither).  Cell indices are clamped to the array (the
 * reference reads outside it for positions outside the domain).
 */
int goc_observe_underlying_flow(int nx, int ny, float dx, float dy, int x_zero_ref, int y_zero_ref,
                                const float* eta, int eta_pitch, const float* hu, int hu_pitch,
                                const float* hv, int hv_pitch, float H, int num_drifters,
                                const float* positions, int positions_pitch, float* observations,
                                int observation_pitch, void* stream);

/*
 * The observation operator over members [first_member, first_member +
 * n_members) of an ensemble in one launch (replaces the per-particle loop
 * of BaseOceanStateEnsemble.observeParticles, E/BaseOceanStateEnsemble.py:
 * 79-145).  For member i of the range and position d: out[(i *
 * num_positions + d) * 3 + {0, 1, 2}] = (eta, hu, hv) of the member's current
 * state at the cell holding the position (zero reference cell 2, as the
 * reference's ensembles pass).  Positions are (x, y) rows with a pitch in
 * bytes; member i reads them at positions + i * positions_member_stride
 * bytes (0: every member observes the same positions).  Device memory.
 */
int goc_ensemble_observe(void* ensemble, int first_member, int n_members, const float* positions,
                         int positions_pitch, long long positions_member_stride, int num_positions,
                         float* out, void* stream);

/*
 * Mean and variance over members [first_member, first_member + n_members)
 * of an ensemble, per interior cell, in one pass over the members' current
 * states (replaces the download-and-NumPy loops of estimate /
 * estimateVelocity, E/BaseOceanStateEnsemble.py:147-176 and
 * E/MultiLevelOceanEnsemble.py:143-250 with func = np.mean / np.var).
 * The members must share one grid.  quantity 0: planes (eta, hu, hv);
 * quantity 1: planes (u, v) = (hu, hv) / h with h = eta + Hm, desingularised
 * as U/OceanographicUtilities.py:413-414 does when desing_eps > 0 (plain
 * division otherwise).  mean / var: device arrays of planes x ny x nx
 * float32 (either may be NULL); var divides by n_members - ddof.  The sums
 * are shifted by the first member's value.  Large member groups on small
 * grids are split over slices whose sums go to scratch owned by the library
 * (grown on demand, which synchronises the stream; not graph-capturable).
 */
int goc_ensemble_moments(void* ensemble, int first_member, int n_members, int quantity, float desing_eps,
                         int ddof, float* mean, float* var, void* stream);

/*
 * The multi-level estimator of MultiLevelOceanEnsemble._estimate_pure
 * (E/MultiLevelOceanEnsemble.py:258-267) on the device.  Level l has a
 * statistic fine[l] on an ny[l] x nx[l] grid (planes x ny x nx float32) and,
 * for l > 0, the coarse partners' statistic coarse[l] on the grid of level
 * l - 1; every level is the finest grid coarsened by 2^(top - l).  out
 * (planes x ny[top] x nx[top] float64) = fine[0] + sum over l > 0 of
 * (fine[l] - coarse[l]), each held constant over the finest cells it covers;
 * the differences are formed in float32 and accumulated in float64 in level
 * order.  fine / coarse / nx / ny are host arrays of n_levels entries
 * (device pointers); at most 8 levels.
 */
int goc_ml_combine(int n_levels, const float* const* fine, const float* const* coarse, const int* nx,
                   const int* ny, int n_planes, double* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GPUOCEAN_GB300_H */
