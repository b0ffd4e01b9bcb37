// Batched ensemble engine: shared declarations of the host handle, the
// persistent member/tile kernel (templated on the tile shape) and its
// launchers.  Each tile shape is instantiated in a translation unit of its
// own (ensemble_shape_*.cu) so that the variants compile in parallel.
#pragma once

#include <algorithm>
#include <vector>

#include "cdklm_tile.cuh"
#include "cfl.cuh"
#include "drift.cuh"

namespace goc {

// Output tile shapes (cells) the engine can run; the autotuner picks one per
// ensemble.  Index 0 is the default.
struct TileShape { int tx, ty; };
constexpr TileShape kEnsembleShapes[] = {{32, 16}, {32, 8}, {16, 16}, {64, 8}, {32, 24}};
constexpr int kNumEnsembleShapes = sizeof(kEnsembleShapes) / sizeof(kEnsembleShapes[0]);
constexpr int kTmaMapsPerMember = 16;

// CTAs per SM the shared memory of a shape allows (at most 3), used as the
// launch-bounds occupancy target of its kernel.
template <int TX, int TY>
constexpr int shape_min_blocks() {
    constexpr size_t b = sizeof(TileSmem<TX + 8, TY + 8>) + 2 * 3 * kHandRows * (TX + 8) * sizeof(float) +
                         5 * (TY + 8) * 4 * sizeof(float) + 1024;
    return (int)(3 * b <= 228 * 1024 ? 3 : 2 * b <= 228 * 1024 ? 2 : 1);
}

struct Ensemble {
    int n_members = 0;
    int n_tiles = 0;                      // output tiles of all members
    int n_runs = 0;                       // work items: runs of consecutive tiles of a column strip
    int max_substeps = 0;
    int n_dt_items = 0;
    bool const_f = true, simple = true;
    // every member has the same scalar parameters (textures aside): the step
    // then reads them from the kernel's parameter space (pu, ku)
    bool uniform = false;
    GocCdklmParams pu{};
    StepConst ku{};
    std::vector<GocMemberDesc> host;      // descriptors as created (set 0 current)
    GocMemberDesc* d_members = nullptr;   // device copy, buffers swapped on device
    int4* d_tiles = nullptr;              // runs (member, tile_x, first tile_y, tiles)
    // [shape][member][kTmaMapsPerMember] TMA maps: eta, hu, hv main boxes of
    // buffer sets 0 and 1, their east boxes, then the cell-mean depth and the
    // Coriolis table (main, east)
    CUtensorMap* d_tmaps = nullptr;
    const float** d_tma_base = nullptr;   // per member: set-0 eta buffer (null: member not staged by TMA)
    int* d_tma_aux = nullptr;             // per member: bit 0 depth boxes staged, bit 1 Coriolis boxes too
    int* d_tma_err = nullptr;             // set when a staging wait ran out
    volatile int* h_tma_err = nullptr;    // pinned host copy, refreshed at the end of every block
    unsigned long long* d_tma_tiles = nullptr;  // tiles staged by TMA so far
    int* d_queue = nullptr;               // work items taken beyond the first gridDim.x (per launch)
    int n_tma_members = 0;
    float* d_dt = nullptr;                // n_members x max_substeps
    int* d_nsub = nullptr;                // n_substeps per member
    int4* d_dt_items = nullptr;           // CFL work: (member, bx, by, partial index)
    int2* d_dt_ranges = nullptr;          // per member [first partial, count)
    float* d_partials = nullptr;          // CFL scratch
    // drifters: one (N_m + 1) x 2 position array per member
    float** d_drift_pos = nullptr;        // per member, null = no drifters
    int4* d_drift_chunks = nullptr;       // (member, first row, count, packed row of the first row), all members
    int n_drift_chunks = 0;
    std::vector<int4> host_chunks;
    // chunks the persistent step advects (members without wind drift) and
    // those a launch of their own advects (members with wind drift)
    int4* d_step_chunks = nullptr;        // == d_drift_chunks when no member has wind drift
    int n_step_chunks = 0;
    int4* d_wind_chunks = nullptr;
    int n_wind_chunks = 0;
    std::vector<char> has_wind;           // per member
    DriftWind* d_wind = nullptr;          // per member (factor 0: none); t comes from d_wind_t
    float* d_wind_t = nullptr;            // n_members x max_substeps: wind time weight of each step's drift
    int* d_drift_n = nullptr;             // drifters per member (the observation row is row n)
    long long drift_rows = 0;             // rows of all members' position arrays, packed
    float drift_sensitivity = 1.0f;
    std::vector<char> has_drifters;       // per member
    // unperturbed copies of the block's last state, for members with
    // drifters (fused model error at the dataAssimilationStep cadence)
    float* d_spare_pool = nullptr;
    float** d_spare = nullptr;            // 3 per member (eta, hu, hv), null without drifters
    // model error fused into the block's launches (goc_ensemble_set_block_noise)
    int block_noise = -1;                 // NoiseMode, or -1: none
    void* noise_batch = nullptr;
    std::vector<int> nsub_host;           // steps per member of the current schedule
    // members that take model error in the current block: their step count,
    // 0 for members masked out (goc_ensemble_set_noise_mask); the batched
    // noise kernels gate on this instead of the step count
    std::vector<int> noise_mask;          // empty: every member
    std::vector<int> nsub_noise_host;
    int* d_nsub_noise = nullptr;
    int shape = 0;                        // index into kEnsembleShapes
};

constexpr int kDriftChunk = 256;

__device__ __forceinline__ DriftGrid member_drift_grid(const GocMemberDesc& d, int set) {
    return DriftGrid{d.p.nx, d.p.ny, d.p.dx, d.p.dy, 2, 2, d.eta[set], d.hu[set], d.hv[set], d.pitch / 4,
                     d.Hm, d.Hm_pitch / 4, d.p.bc_north == 2, d.p.bc_east == 2};
}

// Advect one chunk of a member's drifters with the state of buffer set `set`
// (or, with `copy`, the unperturbed copy of that state: the drift of the
// last step of a block whose model error was fused into that step).
__device__ __forceinline__ void drift_chunk(const GocMemberDesc& d, float* pos, int first, int count, int set,
                                           float dt, float sensitivity, float* const* copy = nullptr) {
    const DriftGrid g = member_drift_grid(d, set);
    for (int q = threadIdx.x; q < count; q += blockDim.x) {
        float* p = pos + 2 * (size_t)(first + q);
        float px = p[0], py = p[1];
        if (copy)
            drift_one_with(g, CopyVelocity{g, copy[0], copy[1], copy[2]}, nullptr, dt, sensitivity, px, py);
        else
            drift_one(g, nullptr, dt, sensitivity, px, py);
        p[0] = px;
        p[1] = py;
    }
}

// ---------------------------------------------------------------------------
// the persistent RK2 kernel
// ---------------------------------------------------------------------------

// Which members a launch with fused model error perturbs.
enum NoiseMode : int {
    kNoiseLastStep = 0,   // members taking the last step of their block (dataAssimilationStep cadence)
    kNoiseEveryStep = 1,  // every member taking a step (CDKLM16.step cadence)
};

// NOISE: the variant that adds the members' SOAR model error to Q^{n+1}
// (noise: one descriptor per member, coarse fields already computed;
// spare: per member three buffers (eta, hu, hv) for the unperturbed state,
// or null entries / a null table; noise_steps: per member the step count of
// the block if the member takes model error, else 0).
template <int TX, int TY, int MINB, bool CONST_F, bool SIMPLE_FORCING, bool NOISE, bool UNI>
__global__ void __launch_bounds__(kNT, MINB)
ensemble_rk2_kernel(const GocCdklmParams pu, const StepConst ku, const GocMemberDesc* __restrict__ members, const int4* __restrict__ tiles, int n_tiles,
                    const float* __restrict__ dt_table, const int* __restrict__ nsub, int max_sub, int k,
                    float* const* __restrict__ drift_pos, const int4* __restrict__ drift_chunks, int n_chunks,
                    float sensitivity, const CUtensorMap* __restrict__ tmaps,
                    const float* const* __restrict__ tma_base, const int* __restrict__ tma_aux, int* tma_err,
                    unsigned long long* tma_tiles, const GocNoiseDesc* __restrict__ noise,
                    float* const* __restrict__ spare, int noise_mode, const int* __restrict__ noise_steps,
                    int* queue) {
    extern __shared__ __align__(128) float smem_raw[];
    // TMA writes the staging planes on 128-byte boundaries: stage only if the
    // dynamic shared memory starts on one (the pointer itself stays the
    // shared array, so every access keeps shared-memory addressing)
    const bool smem_aligned = (smem_u32(smem_raw) & 127u) == 0;
    __shared__ GocMemberDesc md;
    __shared__ StepConst kc;
    __shared__ GocNoiseDesc nd;   // NOISE only
    __shared__ __align__(8) uint64_t tma_bar;
    __shared__ int tma_off;
    if (threadIdx.x == 0) {
        mbar_init(&tma_bar, 1);
        tma_off = 0;
    }
    __syncthreads();
    TileTma tma{nullptr, nullptr, nullptr, false, nullptr, &tma_bar, 0u, false, false, false, -1, &tma_off, tma_err};
    unsigned staged_tiles = 0;  // counted by thread 0
    int cur = -1;
    TileNoise tn{&nd, nullptr, nullptr, nullptr};
    bool perturb = false;   // the current member takes its model error in this launch
    // Work items: the RK2 tiles of step k, then (for k >= 1) the drifter
    // chunks of step k-1, which read the input state of step k (buffer set
    // k % 2) that no tile of this launch writes.  Each CTA takes item
    // blockIdx.x first, then the next untaken one from a counter (zeroed
    // before the launch): runs of different lengths and cost, and members
    // that take no step in this launch, then even out over the CTAs.
    __shared__ int s_next;
    auto next_item = [&]() {
        __syncthreads();
        if (threadIdx.x == 0) s_next = (int)gridDim.x + atomicAdd(queue, 1);
        __syncthreads();
        return s_next;
    };
    const int n_items = n_tiles + (k >= 1 ? n_chunks : 0);
    for (int item = blockIdx.x; item < n_items; item = next_item()) {
        if (item >= n_tiles) {
            const int4 c = drift_chunks[item - n_tiles];
            const int ns = __ldg(nsub + c.x);
            if (k - 1 >= ns) continue;
            // a member whose last step (k - 1 = ns - 1) wrote an unperturbed
            // copy of its state drifts with that copy, in a launch of its own
            // (ensemble_end_drift_kernel) that keeps this kernel's code small
            if (spare && k == ns && k == __ldg(noise_steps + c.x) && spare[3 * c.x]) continue;
            drift_chunk(members[c.x], drift_pos[c.x], c.y, c.z, k & 1,
                        __ldg(dt_table + (size_t)c.x * max_sub + (k - 1)), sensitivity);
            continue;
        }
        // a run of t.w consecutive tiles of the column strip t.y, from tile row t.z
        const int4 t = tiles[item];
        const int m = t.x;
        if (k >= __ldg(nsub + m)) continue;  // member already at the end of its block
        if (m != cur) {
            __syncthreads();
            if (threadIdx.x == 0) {
                md = members[m];
                kc = make_step_const(md.p);
                if constexpr (NOISE) {
                    if (noise) nd = noise[m];
                }
            }
            __syncthreads();
            cur = m;
            if constexpr (NOISE) {
                const int nn = __ldg(noise_steps + m);
                perturb = noise != nullptr && (noise_mode == kNoiseEveryStep ? k < nn : k == nn - 1);
                const bool keep = perturb && noise_mode == kNoiseLastStep && spare != nullptr;
                tn.spare_e = keep ? spare[3 * m] : nullptr;
                tn.spare_u = keep ? spare[3 * m + 1] : nullptr;
                tn.spare_v = keep ? spare[3 * m + 2] : nullptr;
            }
        }
        const int in = k & 1, out = in ^ 1;
        const float dt = __ldg(dt_table + (size_t)m * max_sub + k);
        float* side = smem_raw + sizeof(TileSmem<TX + 8, TY + 8>) / sizeof(float);
        constexpr int NSIDE = 3 * kHandRows * (TX + 8);
        // TMA staging of the member's input set (interior tiles only); tma_off
        // is read after a barrier, so the choice is the same in every thread
        const float* base = tma_base[m];
        const bool use_tma = base != nullptr && tma_off == 0 && smem_aligned;
        const CUtensorMap* mm = tmaps + (size_t)m * kTmaMapsPerMember;
        const int set = md.eta[in] == base ? 0 : 1;
        tma.in_maps = use_tma ? mm + set * 3 : nullptr;
        tma.edge_maps = mm + 6 + set * 3;
        const int auxf = use_tma ? __ldg(tma_aux + m) : 0;
        tma.aux_maps = (auxf & 1) ? mm + 12 : nullptr;
        tma.aux_coriolis = (auxf & 2) != 0;
        tma.edge = side + 2 * NSIDE;
        // depth and Coriolis boxes of a run's later tiles are staged during the
        // previous tile's last phase, whose planes the fused model error uses
        // as scratch when this member perturbs in this launch
        tma.next_aux = tma.aux_maps != nullptr && !perturb;
        bool pending = false;  // the previous tile of the run staged this one
        for (int r = 0; r < t.w; ++r) {
            const int ty = t.z + r;
            // tma_off is set by thread 0 only before the previous tile's
            // staging point and read here after a barrier: a copy of this
            // tile was issued exactly when `pending` and tma_off is still 0
            tma.staged = use_tma && tma_off == 0 && !tile_on_border<TX, TY, 2>(md.p, t.y, ty);
            // its depth / Coriolis boxes: staged with the first tile of a run,
            // or by the previous tile when that could
            tma.aux = tma.staged && tma.aux_maps != nullptr && (pending ? tma.next_aux : true);
            staged_tiles += tma.staged ? 1u : 0u;
            if (tma.staged && !pending && threadIdx.x == 0)
                tma_stage_tile<TX + 8, TY + 8>(tma, *reinterpret_cast<TileSmem<TX + 8, TY + 8>*>(smem_raw),
                                               t.y * TX - 4, 2 + ty * TY - 4, tma.aux);
            tma.next_tile_y =
                (use_tma && r + 1 < t.w && !tile_on_border<TX, TY, 2>(md.p, t.y, ty + 1)) ? ty + 1 : -1;
            // stage-1 rows handed along the run through two alternating buffers
            const float* side_in = side + ((r + 1) & 1) * NSIDE;
            float* side_out = r + 1 < t.w ? side + (r & 1) * NSIDE : nullptr;
            // every thread gets the same answer (it comes from a barrier
            // vote): a CTA whose staged input never landed stops here, with
            // the error flag set for the host
            // with UNI the stage loops read the shared scalar parameters
            // from the kernel's parameter space, the member's textures from md
            const GocCdklmParams& ps = UNI ? pu : md.p;
            const StepConst& ks = UNI ? ku : kc;
            if (!cdklm_strip_tile<TX, TY, kNT, CONST_F, SIMPLE_FORCING, NOISE>(
                    ps, md.p, ks, dt, t.y, ty, r > 0, md.eta[in], md.hu[in], md.hv[in], md.eta[out], md.hu[out],
                    md.hv[out], md.pitch / 4, md.Hi, md.Hi_pitch / 4, md.Hm, md.Hm_pitch / 4, smem_raw, side_in,
                    side_out, &tma, perturb ? &tn : nullptr))
                goto done;
            pending = tma.next_tile_y >= 0 && tma_off == 0;
            __syncthreads();
        }
    }
done:
    if (threadIdx.x == 0 && staged_tiles) atomicAdd(tma_tiles, (unsigned long long)staged_tiles);
}

// Dynamic shared memory of the persistent kernel: the tile planes, two
// hand-over buffers of stage-1 rows and the east boxes of the TMA staging
// (5 fields x rows x 4 columns).
template <int TX, int TY>
constexpr size_t ensemble_smem() {
    return sizeof(TileSmem<TX + 8, TY + 8>) + 2 * 3 * kHandRows * (TX + 8) * sizeof(float) +
           5 * (TY + 8) * 4 * sizeof(float);
}

// Kernel attributes and the persistent grid are set up once per variant,
// outside any stream capture (goc_ensemble_create calls this).
template <int TX, int TY, bool CF, bool SF, bool NOISE, bool UNI>
int configure_ensemble_kernel(int* grid_out) {
    constexpr size_t smem = ensemble_smem<TX, TY>();
    static int grid = 0;
    if (grid == 0) {
        auto kern = ensemble_rk2_kernel<TX, TY, shape_min_blocks<TX, TY>(), CF, SF, NOISE, UNI>;
        cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return set_error(GOC_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(err));
        int blocks = 0;
        err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kern, kNT, smem);
        if (err != cudaSuccess) return set_error(GOC_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(err));
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        grid = std::max(1, sms) * std::max(1, blocks);
    }
    *grid_out = grid;
    return GOC_OK;
}

// Model error fused into one launch: the members' descriptors (device), the
// spare-buffer table (or null) and the NoiseMode.
struct FusedNoise {
    const GocNoiseDesc* noise;
    float* const* spare;
    int mode;
};

template <int TX, int TY, bool CF, bool SF, bool NOISE, bool UNI>
int launch_ensemble(Ensemble* e, int k, cudaStream_t st, const FusedNoise* fn) {
    constexpr size_t smem = ensemble_smem<TX, TY>();
    auto kern = ensemble_rk2_kernel<TX, TY, shape_min_blocks<TX, TY>(), CF, SF, NOISE, UNI>;
    int full = 0;
    int rc = configure_ensemble_kernel<TX, TY, CF, SF, NOISE, UNI>(&full);
    if (rc) return rc;
    const int items = e->n_runs + (k >= 1 ? e->n_step_chunks : 0);
    const int grid = std::min(items, full);
    cudaError_t qe = cudaMemsetAsync(e->d_queue, 0, sizeof(int), st);
    if (qe != cudaSuccess) return set_error(GOC_ERR_CUDA, "ensemble work counter: %s", cudaGetErrorString(qe));
    kern<<<grid, kNT, smem, st>>>(e->pu, e->ku, e->d_members, e->d_tiles, e->n_runs, e->d_dt, e->d_nsub,
                                  e->max_substeps, k, e->d_drift_pos, e->d_step_chunks, e->n_step_chunks,
                                  e->drift_sensitivity,
                                  e->d_tmaps + (size_t)e->shape * e->n_members * kTmaMapsPerMember,
                                  e->d_tma_base, e->d_tma_aux, e->d_tma_err, e->d_tma_tiles, fn ? fn->noise : nullptr,
                                  fn ? fn->spare : nullptr, fn ? fn->mode : 0, e->d_nsub_noise, e->d_queue);
    count_launch();
    return check_launch(NOISE ? "ensemble_rk2_kernel (model error)" : "ensemble_rk2_kernel");
}

// The variants an ensemble can launch: constant or textured Coriolis,
// uniform or textured forcing, with or without fused model error, and (with
// uniform forcing) shared scalar parameters in parameter space.
template <int TX, int TY, bool CF, bool SF>
int configure_variants(const Ensemble* e, int* grid) {
    int g2 = 0;
    if (SF && e->uniform) {
        int rc = configure_ensemble_kernel<TX, TY, CF, SF, false, SF>(grid);
        return rc ? rc : configure_ensemble_kernel<TX, TY, CF, SF, true, SF>(&g2);
    }
    int rc = configure_ensemble_kernel<TX, TY, CF, SF, false, false>(grid);
    return rc ? rc : configure_ensemble_kernel<TX, TY, CF, SF, true, false>(&g2);
}

// Launchers of one tile shape (explicitly instantiated per shape).
template <int TX, int TY>
int ensemble_configure_shape(const Ensemble* e, int* grid) {
    if (e->const_f && e->simple) return configure_variants<TX, TY, true, true>(e, grid);
    if (e->const_f) return configure_variants<TX, TY, true, false>(e, grid);
    if (e->simple) return configure_variants<TX, TY, false, true>(e, grid);
    return configure_variants<TX, TY, false, false>(e, grid);
}

template <int TX, int TY, bool CF, bool SF>
int launch_variant(Ensemble* e, int k, cudaStream_t st, const FusedNoise* fn) {
    const bool noise = fn && fn->noise;
    if (SF && e->uniform)
        return noise ? launch_ensemble<TX, TY, CF, SF, true, SF>(e, k, st, fn)
                     : launch_ensemble<TX, TY, CF, SF, false, SF>(e, k, st, fn);
    return noise ? launch_ensemble<TX, TY, CF, SF, true, false>(e, k, st, fn)
                 : launch_ensemble<TX, TY, CF, SF, false, false>(e, k, st, fn);
}

// fn: the model error of this launch (null: none); fn->noise null means no
// member perturbs here but fn->spare still tells the drifter work which
// members drift with an unperturbed copy (the plain variant runs then).
template <int TX, int TY>
int ensemble_launch_shape(Ensemble* e, int k, cudaStream_t st, const FusedNoise* fn) {
    if (e->const_f && e->simple) return launch_variant<TX, TY, true, true>(e, k, st, fn);
    if (e->const_f) return launch_variant<TX, TY, true, false>(e, k, st, fn);
    if (e->simple) return launch_variant<TX, TY, false, true>(e, k, st, fn);
    return launch_variant<TX, TY, false, false>(e, k, st, fn);
}

#define GOC_ENSEMBLE_SHAPE_EXTERN(TX, TY)                                           \
    extern template int ensemble_configure_shape<TX, TY>(const Ensemble*, int*);     \
    extern template int ensemble_launch_shape<TX, TY>(Ensemble*, int, cudaStream_t, const FusedNoise*);
GOC_ENSEMBLE_SHAPE_EXTERN(32, 16)
GOC_ENSEMBLE_SHAPE_EXTERN(32, 8)
GOC_ENSEMBLE_SHAPE_EXTERN(16, 16)
GOC_ENSEMBLE_SHAPE_EXTERN(64, 8)
GOC_ENSEMBLE_SHAPE_EXTERN(32, 24)
#undef GOC_ENSEMBLE_SHAPE_EXTERN

}  // namespace goc
