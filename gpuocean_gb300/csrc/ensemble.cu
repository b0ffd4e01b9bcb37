// Batched ensemble engine: every member of an ensemble (grids of any size)
// advances in one persistent launch per RK2 step over a member/tile work
// queue, instead of one Python-driven launch sequence per member
// (E/OceanNoiseEnsemble.py:517-543, E/MultiLevelOceanEnsemble.py:95-141).
#include <cudaTypedefs.h>

#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "ensemble.cuh"

namespace goc {

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// Drift of the last step of members that ran all `n_launched` steps of the block.
// Drift of step s (state in buffer set (s + 1) % 2) outside the persistent
// step: members with nsub == s + 1 (last_only: their block ended with step
// s) or with s < nsub (every member that took step s).
// spare: the members' unperturbed copies of the last step's state (3 per
// member, null entries or a null table: drift with the state itself);
// copy_only: only the members that drift with such a copy.  wind: per member
// wind drift (factor 0: none), its time weight for step s in wind_t.
__global__ void ensemble_drift_kernel(const GocMemberDesc* __restrict__ members, const int* __restrict__ nsub,
                                      const float* __restrict__ dt_table, int max_sub, int s, int last_only,
                                      float* const* __restrict__ drift_pos, const int4* __restrict__ chunks,
                                      float sensitivity, float* const* __restrict__ spare,
                                      const int* __restrict__ noise_steps, int copy_only,
                                      const DriftWind* __restrict__ wind, const float* __restrict__ wind_t) {
    const int4 c = chunks[blockIdx.x];
    const int m = c.x, ns = nsub[m];
    if (s < 0 || (last_only ? ns != s + 1 : s >= ns)) return;
    // the copy holds the last step's state only if that step took model error
    float* const* copy = (spare && spare[3 * m] && ns == s + 1 && noise_steps[m] == s + 1) ? spare + 3 * m : nullptr;
    if (copy_only && !copy) return;
    DriftWind w;
    const bool windy = wind && wind[m].factor != 0.0f;
    if (windy) {
        w = wind[m];
        w.t = wind_t[(size_t)m * max_sub + s];
    }
    const GocMemberDesc& d = members[m];
    const DriftGrid g = member_drift_grid(d, (s + 1) & 1);
    const float dt = dt_table[(size_t)m * max_sub + s];
    float* pos = drift_pos[m];
    for (int q = threadIdx.x; q < c.z; q += blockDim.x) {
        float* p = pos + 2 * (size_t)(c.y + q);
        float px = p[0], py = p[1];
        if (copy)
            drift_one_with(g, CopyVelocity{g, copy[0], copy[1], copy[2]}, windy ? &w : nullptr, dt, sensitivity, px,
                           py);
        else
            drift_one(g, windy ? &w : nullptr, dt, sensitivity, px, py);
        p[0] = px;
        p[1] = py;
    }
}

__global__ void ensemble_end_block_kernel(GocMemberDesc* members, const int* nsub, int n) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n || (nsub[m] & 1) == 0) return;
    GocMemberDesc& d = members[m];
    float* t;
    t = d.eta[0]; d.eta[0] = d.eta[1]; d.eta[1] = t;
    t = d.hu[0]; d.hu[0] = d.hu[1]; d.hu[1] = t;
    t = d.hv[0]; d.hv[0] = d.hv[1]; d.hv[1] = t;
}

__global__ void __launch_bounds__(kDtBX * kDtBY)
ensemble_dt_partials_kernel(const GocMemberDesc* __restrict__ members, const int4* __restrict__ items,
                            float* __restrict__ partials) {
    __shared__ float wmin[kDtBX * kDtBY / 32];
    const int4 it = items[blockIdx.x];
    const GocMemberDesc& d = members[it.x];
    const int i = 2 + it.y * kDtBX + threadIdx.x;
    const int j = 2 + it.z * kDtBY + threadIdx.y;
    float v = cell_dt(d.p.nx, d.p.ny, d.p.dx, d.p.dy, d.p.g, d.eta[0], d.hu[0], d.hv[0], d.pitch / 4, d.Hm,
                      d.Hm_pitch / 4, d.p.land_value, i, j);
    v = warp_min(v);
    const int tid = threadIdx.y * kDtBX + threadIdx.x;
    if ((tid & 31) == 0) wmin[tid >> 5] = v;
    __syncthreads();
    if (tid < 32) {
        float w = (tid < kDtBX * kDtBY / 32) ? wmin[tid] : kMaxDt;
        w = warp_min(w);
        if (tid == 0) partials[it.w] = w;
    }
}

__global__ void __launch_bounds__(256) ensemble_dt_final_kernel(const float* __restrict__ partials,
                                                                const int2* __restrict__ ranges,
                                                                float* __restrict__ out) {
    __shared__ float wmin[8];
    const int2 r = ranges[blockIdx.x];
    float v = kMaxDt;
    for (int q = threadIdx.x; q < r.y; q += blockDim.x) v = fminf(v, partials[r.x + q]);
    v = warp_min(v);
    if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = (threadIdx.x < 8) ? wmin[threadIdx.x] : kMaxDt;
        v = warp_min(v);
        if (threadIdx.x == 0) out[blockIdx.x] = v;
    }
}

static void free_ensemble(Ensemble* e) {
    cudaFree(e->d_members);
    cudaFree(e->d_tiles);
    cudaFree(e->d_dt);
    cudaFree(e->d_nsub);
    cudaFree(e->d_dt_items);
    cudaFree(e->d_dt_ranges);
    cudaFree(e->d_partials);
    if (e->d_step_chunks != e->d_drift_chunks) cudaFree(e->d_step_chunks);
    cudaFree(e->d_wind_chunks);
    cudaFree(e->d_wind);
    cudaFree(e->d_wind_t);
    cudaFree(e->d_drift_pos);
    cudaFree(e->d_drift_chunks);
    cudaFree(e->d_drift_n);
    cudaFree(e->d_tmaps);
    cudaFree(e->d_tma_base);
    cudaFree(e->d_tma_aux);
    cudaFree(e->d_tma_err);
    if (e->h_tma_err) cudaFreeHost(const_cast<int*>(e->h_tma_err));
    cudaFree(e->d_tma_tiles);
    cudaFree(e->d_queue);
    cudaFree(e->d_spare_pool);
    cudaFree(e->d_spare);
    cudaFree(e->d_nsub_noise);
    delete e;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (null if
// the driver does not provide it).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

// TMA maps of every member's (eta, hu, hv) in both buffer sets, one main box
// per tile shape (the shape's tile + 4 cells on each side, from two columns
// west of it) and one east box of 4 columns; and of the cell-mean depth and
// the per-cell Coriolis table (main and east boxes), which the kernel stages
// with the state when it can.  A member is staged by TMA when every state
// buffer starts on a 16-byte boundary, its row pitch is a multiple of 16
// bytes and every map encodes; otherwise its tiles load Q^n with ordinary
// loads.  The depth (and Coriolis) boxes follow the same rules.
static int build_tma_maps(Ensemble* e) {
    const int n = e->n_members;
    std::vector<CUtensorMap> maps((size_t)kNumEnsembleShapes * n * kTmaMapsPerMember);
    std::vector<const float*> base(n, nullptr);
    std::vector<int> aux(n, 0);
    const PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    auto aligned = [](const void* p, size_t pitch) {
        return p != nullptr && reinterpret_cast<uintptr_t>(p) % 16 == 0 && pitch % 16 == 0;
    };
    e->n_tma_members = 0;
    for (int m = 0; m < n; ++m) {
        const GocMemberDesc& d = e->host[m];
        float* const buf[2][3] = {{d.eta[0], d.hu[0], d.hv[0]}, {d.eta[1], d.hu[1], d.hv[1]}};
        bool ok = encode != nullptr && d.pitch % 16 == 0;
        for (int set = 0; set < 2; ++set)
            for (int c = 0; c < 3; ++c) ok = ok && reinterpret_cast<uintptr_t>(buf[set][c]) % 16 == 0;
        bool depth = ok && aligned(d.Hm, (size_t)d.Hm_pitch);
        bool cor = depth && !e->const_f && aligned(d.p.coriolis_cell, (size_t)d.p.coriolis_cell_pitch);
        const cuuint64_t dims[2] = {(cuuint64_t)d.p.nx + 4, (cuuint64_t)d.p.ny + 4};
        const cuuint32_t unit[2] = {1, 1};
        auto enc = [&](CUtensorMap* map, const void* ptr, size_t pitch, cuuint32_t bx, cuuint32_t by) {
            const cuuint64_t strides[1] = {(cuuint64_t)pitch};
            const cuuint32_t box[2] = {bx, by};
            return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(ptr), dims, strides, box, unit,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
        };
        for (int sh = 0; ok && sh < kNumEnsembleShapes; ++sh) {
            CUtensorMap* mm = &maps[((size_t)sh * n + m) * kTmaMapsPerMember];
            const cuuint32_t bx = (cuuint32_t)kEnsembleShapes[sh].tx + 8, by = (cuuint32_t)kEnsembleShapes[sh].ty + 8;
            for (int set = 0; ok && set < 2; ++set)
                for (int c = 0; ok && c < 3; ++c)
                    ok = enc(mm + set * 3 + c, buf[set][c], (size_t)d.pitch, bx, by) &&
                         enc(mm + 6 + set * 3 + c, buf[set][c], (size_t)d.pitch, 4, by);
            if (depth)
                depth = enc(mm + 12, d.Hm, (size_t)d.Hm_pitch, bx, by) && enc(mm + 13, d.Hm, (size_t)d.Hm_pitch, 4, by);
            if (cor)
                cor = enc(mm + 14, d.p.coriolis_cell, (size_t)d.p.coriolis_cell_pitch, bx, by) &&
                      enc(mm + 15, d.p.coriolis_cell, (size_t)d.p.coriolis_cell_pitch, 4, by);
        }
        if (ok) {
            base[m] = d.eta[0];
            aux[m] = depth ? (cor ? 3 : 1) : 0;
            ++e->n_tma_members;
        }
    }
    cudaError_t err = cudaMalloc(&e->d_tmaps, sizeof(CUtensorMap) * maps.size());
    if (err == cudaSuccess) err = cudaMalloc(&e->d_tma_base, sizeof(const float*) * n);
    if (err == cudaSuccess) err = cudaMalloc(&e->d_tma_aux, sizeof(int) * n);
    if (err == cudaSuccess) err = cudaMalloc(&e->d_tma_err, sizeof(int));
    if (err == cudaSuccess) err = cudaMalloc(&e->d_tma_tiles, sizeof(unsigned long long));
    if (err == cudaSuccess)
        err = cudaMemcpy(e->d_tmaps, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice);
    if (err == cudaSuccess)
        err = cudaMemcpy(e->d_tma_base, base.data(), sizeof(const float*) * n, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemcpy(e->d_tma_aux, aux.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemset(e->d_tma_err, 0, sizeof(int));
    if (err == cudaSuccess) {
        int* h = nullptr;
        err = cudaHostAlloc(&h, sizeof(int), cudaHostAllocDefault);
        if (err == cudaSuccess) {
            *h = 0;
            e->h_tma_err = h;
        }
    }
    if (err == cudaSuccess) err = cudaMemset(e->d_tma_tiles, 0, sizeof(unsigned long long));
    if (err != cudaSuccess) return set_error(GOC_ERR_CUDA, "ensemble TMA maps: %s", cudaGetErrorString(err));
    return GOC_OK;
}

const GocMemberDesc* ensemble_host_members(void* ensemble, int* n_members) {
    Ensemble* e = static_cast<Ensemble*>(ensemble);
    if (n_members) *n_members = e->n_members;
    return e->host.data();
}

const GocMemberDesc* ensemble_device_members(void* ensemble) { return static_cast<Ensemble*>(ensemble)->d_members; }

const int* ensemble_device_nsub(void* ensemble) { return static_cast<Ensemble*>(ensemble)->d_nsub; }

const int* ensemble_device_noise_steps(void* ensemble) { return static_cast<Ensemble*>(ensemble)->d_nsub_noise; }

static int shape_configure(const Ensemble* e, int* grid) {
    switch (e->shape) {
        case 0: return ensemble_configure_shape<32, 16>(e, grid);
        case 1: return ensemble_configure_shape<32, 8>(e, grid);
        case 2: return ensemble_configure_shape<16, 16>(e, grid);
        case 3: return ensemble_configure_shape<64, 8>(e, grid);
        case 4: return ensemble_configure_shape<32, 24>(e, grid);
    }
    return set_error(GOC_ERR_ARG, "ensemble: tile shape %d out of range", e->shape);
}

static int shape_launch(Ensemble* e, int k, cudaStream_t st, const FusedNoise* fn) {
    switch (e->shape) {
        case 0: return ensemble_launch_shape<32, 16>(e, k, st, fn);
        case 1: return ensemble_launch_shape<32, 8>(e, k, st, fn);
        case 2: return ensemble_launch_shape<16, 16>(e, k, st, fn);
        case 3: return ensemble_launch_shape<64, 8>(e, k, st, fn);
        case 4: return ensemble_launch_shape<32, 24>(e, k, st, fn);
    }
    return set_error(GOC_ERR_ARG, "ensemble: tile shape %d out of range", e->shape);
}

// (Re)build the member/tile work queue for the ensemble's tile shape.
// Work queue: every member's column strips cut into runs of at most kRunTiles
// consecutive tiles; a CTA steps a run from south to north, handing the
// overlapping stage-1 rows from one tile to the next.  A run holds either
// interior tiles only or border tiles only (the two are different code), and
// all interior runs come before all border runs, longest first within each
// group: while the interior runs last, every CTA of an SM executes the same
// code, which keeps the instruction cache warm; the short border runs then
// even out the end of the launch.
constexpr int kRunTiles = 8;

static bool host_tile_on_border(const GocCdklmParams& p, int tx, int ty, int i, int j) {
    const int x0 = 2 + i * tx - 4, y0 = 2 + j * ty - 4;
    return x0 < 2 || y0 < 2 || x0 + tx + 8 > p.nx + 2 || y0 + ty + 8 > p.ny + 2;
}

static int build_tiles(Ensemble* e) {
    const TileShape sh = kEnsembleShapes[e->shape];
    std::vector<int4> inner, border;
    int n_tiles = 0;
    for (int m = 0; m < e->n_members; ++m) {
        const GocCdklmParams& p = e->host[m].p;
        const int tx = (p.nx + sh.tx - 1) / sh.tx, ty = (p.ny + sh.ty - 1) / sh.ty;
        for (int i = 0; i < tx; ++i)
            for (int j = 0; j < ty;) {
                // a maximal stretch of tiles of one kind, cut into balanced runs
                const bool b = host_tile_on_border(p, sh.tx, sh.ty, i, j);
                int end = j + 1;
                while (end < ty && host_tile_on_border(p, sh.tx, sh.ty, i, end) == b) ++end;
                const int len = end - j, runs = (len + kRunTiles - 1) / kRunTiles;
                for (int r = 0; r < runs; ++r) {
                    const int n = len / runs + (r < len % runs ? 1 : 0);
                    (b ? border : inner).push_back(make_int4(m, i, j, n));
                    j += n;
                }
            }
        n_tiles += tx * ty;
    }
    auto longest_first = [](const int4& a, const int4& b) { return a.w > b.w; };
    std::stable_sort(inner.begin(), inner.end(), longest_first);
    std::stable_sort(border.begin(), border.end(), longest_first);
    std::vector<int4> tiles(inner);
    tiles.insert(tiles.end(), border.begin(), border.end());
    cudaFree(e->d_tiles);
    e->d_tiles = nullptr;
    cudaError_t err = cudaMalloc(&e->d_tiles, sizeof(int4) * tiles.size());
    if (err == cudaSuccess)
        err = cudaMemcpy(e->d_tiles, tiles.data(), sizeof(int4) * tiles.size(), cudaMemcpyHostToDevice);
    if (err != cudaSuccess) return set_error(GOC_ERR_CUDA, "ensemble tile queue: %s", cudaGetErrorString(err));
    e->n_tiles = n_tiles;
    e->n_runs = (int)tiles.size();
    int grid = 0;
    return shape_configure(e, &grid);
}

}  // namespace goc

using namespace goc;

extern "C" int goc_ensemble_create(const GocMemberDesc* members, int n_members, int max_substeps, void** out) {
    if (!out) return set_error(GOC_ERR_ARG, "goc_ensemble_create: null out pointer");
    *out = nullptr;
    if (!members || n_members < 1) return set_error(GOC_ERR_ARG, "goc_ensemble_create: no members");
    if (max_substeps < 1) return set_error(GOC_ERR_ARG, "goc_ensemble_create: max_substeps must be >= 1");
    Ensemble* e = new Ensemble();
    e->n_members = n_members;
    e->max_substeps = max_substeps;
    e->host.assign(members, members + n_members);
    std::vector<int4> dt_items;
    std::vector<int2> ranges;
    for (int m = 0; m < n_members; ++m) {
        const GocMemberDesc& d = members[m];
        char who[64];
        snprintf(who, sizeof(who), "goc_ensemble_create: member %d", m);
        int rc = validate_params(&d.p, who);
        if (!rc && d.p.rk_order != 2) rc = set_error(GOC_ERR_ARG, "%s: rk_order must be 2", who);
        if (!rc && (!d.Hi || !d.Hm || !d.eta[0] || !d.eta[1] || !d.hu[0] || !d.hu[1] || !d.hv[0] || !d.hv[1]))
            rc = set_error(GOC_ERR_ARG, "%s: null buffer", who);
        if (!rc && (d.pitch < (d.p.nx + 4) * 4 || d.pitch % 4 || d.Hi_pitch < (d.p.nx + 5) * 4 || d.Hi_pitch % 4 ||
                    d.Hm_pitch < (d.p.nx + 4) * 4 || d.Hm_pitch % 4))
            rc = set_error(GOC_ERR_ARG, "%s: pitch too small", who);
        if (!rc && (d.eta[0] == d.eta[1] || d.hu[0] == d.hu[1] || d.hv[0] == d.hv[1]))
            rc = set_error(GOC_ERR_ARG, "%s: the two buffer sets must differ", who);
        if (rc) {
            delete e;
            return rc;
        }
        e->const_f = e->const_f && d.p.coriolis_nx == 1 && d.p.coriolis_ny == 1;
        e->simple = e->simple && d.p.wind_x_nx == 1 && d.p.wind_x_ny == 1 && d.p.wind_y_nx == 1 &&
                    d.p.wind_y_ny == 1 && d.p.atm_p_nx == 1 && d.p.atm_p_ny == 1;
        const int bx = (d.p.nx + kDtBX - 1) / kDtBX, by = (d.p.ny + kDtBY - 1) / kDtBY;
        ranges.push_back(make_int2((int)dt_items.size(), bx * by));
        for (int j = 0; j < by; ++j)
            for (int i = 0; i < bx; ++i) dt_items.push_back(make_int4(m, i, j, (int)dt_items.size()));
    }
    e->n_dt_items = (int)dt_items.size();
    // shared scalar parameters: every member's parameters equal member 0's
    // once the texture pointers are set aside (those stay per member)
    auto scalars = [](GocCdklmParams q) {
        q.coriolis_f = q.coriolis_cell = q.angle = nullptr;
        q.wind_x_cur = q.wind_x_next = q.wind_y_cur = q.wind_y_next = nullptr;
        q.atm_p_cur = q.atm_p_next = nullptr;
        q.wind_t = 0.0f;
        q.atm_p_t = 0.0f;
        return q;
    };
    e->pu = scalars(e->host[0].p);
    e->uniform = true;
    for (int m = 1; m < n_members && e->uniform; ++m) {
        const GocCdklmParams q = scalars(e->host[m].p);
        e->uniform = std::memcmp(&q, &e->pu, sizeof(q)) == 0;
    }
    e->ku = make_step_const(e->pu);
    cudaError_t err = cudaSuccess;
    auto alloc = [&](void** p, size_t bytes) {
        if (err == cudaSuccess) err = cudaMalloc(p, bytes);
    };
    alloc((void**)&e->d_members, sizeof(GocMemberDesc) * n_members);
    alloc((void**)&e->d_dt, sizeof(float) * (size_t)n_members * max_substeps);
    alloc((void**)&e->d_nsub, sizeof(int) * n_members);
    alloc((void**)&e->d_nsub_noise, sizeof(int) * n_members);
    alloc((void**)&e->d_dt_items, sizeof(int4) * dt_items.size());
    alloc((void**)&e->d_dt_ranges, sizeof(int2) * ranges.size());
    alloc((void**)&e->d_partials, sizeof(float) * dt_items.size());
    if (err == cudaSuccess)
        err = cudaMemcpy(e->d_members, members, sizeof(GocMemberDesc) * n_members, cudaMemcpyHostToDevice);
    if (err == cudaSuccess)
        err = cudaMemcpy(e->d_dt_items, dt_items.data(), sizeof(int4) * dt_items.size(), cudaMemcpyHostToDevice);
    if (err == cudaSuccess)
        err = cudaMemcpy(e->d_dt_ranges, ranges.data(), sizeof(int2) * ranges.size(), cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemset(e->d_nsub, 0, sizeof(int) * n_members);
    if (err == cudaSuccess) err = cudaMemset(e->d_nsub_noise, 0, sizeof(int) * n_members);
    if (err == cudaSuccess) err = cudaMemset(e->d_dt, 0, sizeof(float) * (size_t)n_members * max_substeps);
    if (err == cudaSuccess) err = cudaMalloc(&e->d_queue, sizeof(int));
    if (err == cudaSuccess) err = cudaMemset(e->d_queue, 0, sizeof(int));
    if (err != cudaSuccess) {
        free_ensemble(e);
        return set_error(GOC_ERR_CUDA, "goc_ensemble_create: %s", cudaGetErrorString(err));
    }
    int rc = build_tma_maps(e);
    if (!rc) rc = build_tiles(e);
    if (rc) {
        free_ensemble(e);
        return rc;
    }
    *out = e;
    return GOC_OK;
}

extern "C" int goc_ensemble_destroy(void* ensemble) {
    if (!ensemble) return GOC_OK;
    free_ensemble(static_cast<Ensemble*>(ensemble));
    return GOC_OK;
}

extern "C" int goc_ensemble_tma_status(void* ensemble, int* staged_members, long long* staged_tiles,
                                       int* wait_errors) {
    if (!ensemble) return set_error(GOC_ERR_ARG, "goc_ensemble_tma_status: null handle");
    Ensemble* e = static_cast<Ensemble*>(ensemble);
    if (staged_members) *staged_members = e->n_tma_members;
    if (staged_tiles) {
        unsigned long long v = 0;
        const cudaError_t err = cudaMemcpy(&v, e->d_tma_tiles, sizeof(v), cudaMemcpyDeviceToHost);
        if (err != cudaSuccess) return set_error(GOC_ERR_CUDA, "goc_ensemble_tma_status: %s", cudaGetErrorString(err));
        *staged_tiles = (long long)v;
    }
    if (wait_errors) {
        int v = 0;
        const cudaError_t err = cudaMemcpy(&v, e->d_tma_err, sizeof(int), cudaMemcpyDeviceToHost);
        if (err != cudaSuccess) return set_error(GOC_ERR_CUDA, "goc_ensemble_tma_status: %s", cudaGetErrorString(err));
        *wait_errors = v;
    }
    return GOC_OK;
}

extern "C" int goc_ensemble_size(void* ensemble, int* n_members, int* n_tiles) {
    if (!ensemble) return set_error(GOC_ERR_ARG, "goc_ensemble_size: null handle");
    Ensemble* e = static_cast<Ensemble*>(ensemble);
    if (n_members) *n_members = e->n_members;
    if (n_tiles) *n_tiles = e->n_tiles;
    return GOC_OK;
}

// Per member the steps of the block if it takes model error, else 0 (host
// copy and device table); synchronises the stream (the host copy is reused).
static int upload_noise_steps(Ensemble* e, cudaStream_t st) {
    e->nsub_noise_host.assign(e->n_members, 0);
    for (int m = 0; m < e->n_members && m < (int)e->nsub_host.size(); ++m)
        e->nsub_noise_host[m] = (e->noise_mask.empty() || e->noise_mask[m]) ? e->nsub_host[m] : 0;
    cudaError_t err = cudaMemcpyAsync(e->d_nsub_noise, e->nsub_noise_host.data(), sizeof(int) * e->n_members,
                                      cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    if (err != cudaSuccess) return set_error(GOC_ERR_CUDA, "ensemble noise steps: %s", cudaGetErrorString(err));
    return GOC_OK;
}

extern "C" int goc_ensemble_set_schedule(void* ensemble, const float* dt_table, const int* n_substeps, void* stream) {
    if (!ensemble || !dt_table || !n_substeps) return set_error(GOC_ERR_ARG, "goc_ensemble_set_schedule: null argument");
    Ensemble* e = static_cast<Ensemble*>(ensemble);
    for (int m = 0; m < e->n_members; ++m) {
        if (n_substeps[m] < 0 || n_substeps[m] > e->max_substeps)
            return set_error(GOC_ERR_ARG, "goc_ensemble_set_schedule: member %d has %d steps (max %d)", m,
                             n_substeps[m], e->max_substeps);
        for (int k = 0; k < n_substeps[m]; ++k)
            if (!(dt_table[(size_t)m * e->max_substeps + k] >= 0.0f))
                return set_error(GOC_ERR_ARG, "goc_ensemble_set_schedule: negative dt for member %d", m);
    }
    cudaStream_t st = as_stream(stream);
    cudaError_t err = cudaMemcpyAsync(e->d_dt, dt_table, sizeof(float) * (size_t)e->n_members * e->max_substeps,
                                      cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(e->d_nsub, n_substeps, sizeof(int) * e->n_members, cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);  // host arrays may be reused on return
    if (err != cudaSuccess) return set_error(GOC_ERR_CUDA, "goc_ensemble_set_schedule: %s", cudaGetErrorString(err));
    e->nsub_host.assign(n_substeps, n_substeps + e->n_members);
    return upload_noise_steps(e, st);
}

extern "C" int goc_ensemble_set_noise_mask(void* ensemble, const int* mask, void* stream) {
    if (!ensemble) return set_error(GOC_ERR_ARG, "goc_ensemble_set_noise_mask: null handle");
    Ensemble* e = static_cast<Ensemble*>(ensemble);
    if (mask) e->noise_mask.assign(mask, mask + e->n_members);
    else e->noise_mask.clear();
    return upload_noise_steps(e, as_stream(stream));
}

// The unperturbed copies of the members with drifters (one buffer set each,
// with the member's pitch), allocated once.
static int ensure_spares(Ensemble* e) {
    if (e->d_spare) return GOC_OK;
    std::vector<size_t> offset(e->n_members, 0);
    size_t total = 0;
    for (int m = 0; m < e->n_members; ++m) {
        if (m >= (int)e->has_drifters.size() || !e->has_drifters[m]) continue;
        const GocMemberDesc& d = e->host[m];
        offset[m] = total;
        total += 3 * (size_t)d.pitch * (d.p.ny + 4);
    }
    std::vector<float*> table(3 * (size_t)e->n_members, nullptr);
    cudaError_t err = cudaSuccess;
    if (total) {
        err = cudaMalloc(&e->d_spare_pool, total);
        // wall ghost cells are read from the state itself; the rest is written
        // before it is read, but keep the copy defined from the start
        if (err == cudaSuccess) err = cudaMemset(e->d_spare_pool, 0, total);
    }
    for (int m = 0; err == cudaSuccess && total && m < e->n_members; ++m) {
        if (m >= (int)e->has_drifters.size() || !e->has_drifters[m]) continue;
        const GocMemberDesc& d = e->host[m];
        char* base = reinterpret_cast<char*>(e->d_spare_pool) + offset[m];
        const size_t plane = (size_t)d.pitch * (d.p.ny + 4);
        for (int c = 0; c < 3; ++c) table[3 * (size_t)m + c] = reinterpret_cast<float*>(base + c * plane);
    }
    if (err == cudaSuccess) err = cudaMalloc(&e->d_spare, sizeof(float*) * table.size());
    if (err == cudaSuccess)
        err = cudaMemcpy(e->d_spare, table.data(), sizeof(float*) * table.size(), cudaMemcpyHostToDevice);
    if (err != cudaSuccess) {
        cudaFree(e->d_spare_pool);
        cudaFree(e->d_spare);
        e->d_spare_pool = nullptr;
        e->d_spare = nullptr;
        return set_error(GOC_ERR_CUDA, "goc_ensemble_set_block_noise: %s", cudaGetErrorString(err));
    }
    return GOC_OK;
}

extern "C" int goc_ensemble_set_block_noise(void* ensemble, void* noise_batch, int mode) {
    if (!ensemble) return set_error(GOC_ERR_ARG, "goc_ensemble_set_block_noise: null handle");
    Ensemble* e = static_cast<Ensemble*>(ensemble);
    if (mode < 0) {
        e->block_noise = -1;
        e->noise_batch = nullptr;
        return GOC_OK;
    }
    if (mode != kNoiseLastStep && mode != kNoiseEveryStep)
        return set_error(GOC_ERR_ARG, "goc_ensemble_set_block_noise: mode %d (0 = last step, 1 = every step)", mode);
    int n = 0;
    if (!noise_batch || !noise_batch_device_desc(noise_batch, &n) || n != e->n_members)
        return set_error(GOC_ERR_ARG, "goc_ensemble_set_block_noise: the noise batch must have one member per member");
    if (mode == kNoiseLastStep) {
        const int rc = ensure_spares(e);
        if (rc) return rc;
    }
    e->block_noise = mode;
    e->noise_batch = noise_batch;
    return GOC_OK;
}

// One launch of ensemble_drift_kernel over `chunks` (see there).
static int launch_drift(Ensemble* e, int s, int last_only, int copy_only, const int4* chunks, int n_chunks,
                        float* const* spare, void* stream) {
    if (n_chunks <= 0) return GOC_OK;
    ensemble_drift_kernel<<<n_chunks, kDriftChunk, 0, as_stream(stream)>>>(
        e->d_members, e->d_nsub, e->d_dt, e->max_substeps, s, last_only, e->d_drift_pos, chunks,
        e->drift_sensitivity, spare, e->d_nsub_noise, copy_only, e->d_wind, e->d_wind_t);
    count_launch();
    return check_launch("ensemble_drift_kernel");
}

extern "C" int goc_ensemble_rk2_substep(void* ensemble, int k, void* stream) {
    if (!ensemble) return set_error(GOC_ERR_ARG, "goc_ensemble_rk2_substep: null handle");
    Ensemble* e = static_cast<Ensemble*>(ensemble);
    if (k < 0 || k >= e->max_substeps) return set_error(GOC_ERR_ARG, "goc_ensemble_rk2_substep: k=%d out of range", k);
    if (k >= 1 && e->n_wind_chunks > 0) {
        // drifters with wind drift: the drift of step k - 1 in a launch of
        // its own (it reads set k % 2, which this step does not write)
        const int rc = launch_drift(e, k - 1, 0, 0, e->d_wind_chunks, e->n_wind_chunks,
                                    e->block_noise == kNoiseLastStep ? e->d_spare : nullptr, stream);
        if (rc) return rc;
    }
    if (e->block_noise < 0) return shape_launch(e, k, as_stream(stream), nullptr);
    // model error fused into this step for the members that take it here
    bool any = false;
    for (int m = 0; m < e->n_members && !any; ++m) {
        const int ns = m < (int)e->nsub_noise_host.size() ? e->nsub_noise_host[m] : 0;
        any = e->block_noise == kNoiseEveryStep ? k < ns : k == ns - 1;
    }
    const FusedNoise fn{noise_batch_device_desc(e->noise_batch, nullptr),
                        e->block_noise == kNoiseLastStep ? e->d_spare : nullptr, e->block_noise};
    if (fn.spare && k >= 1 && e->n_step_chunks > 0) {
        // members whose block ended with step k - 1: their drifters move with
        // the unperturbed copy of that step's state (the persistent launch
        // leaves them out)
        bool ended = false;
        for (int m = 0; m < e->n_members && !ended; ++m)
            ended = m < (int)e->has_drifters.size() && e->has_drifters[m] && e->nsub_host[m] == k &&
                    e->nsub_noise_host[m] == k;
        if (ended) {
            const int rc = launch_drift(e, k - 1, 1, 1, e->d_step_chunks, e->n_step_chunks, fn.spare, stream);
            if (rc) return rc;
        }
    }
    if (any) return shape_launch(e, k, as_stream(stream), &fn);
    // no member perturbs here, but drifters of members whose block ended
    // with a perturbed step read that step's unperturbed copy
    const FusedNoise plain{nullptr, fn.spare, fn.mode};
    return fn.spare ? shape_launch(e, k, as_stream(stream), &plain) : shape_launch(e, k, as_stream(stream), nullptr);
}

extern "C" int goc_ensemble_tile_shape_count(void) { return kNumEnsembleShapes; }

extern "C" int goc_ensemble_tile_shape(int index, int* tx, int* ty) {
    if (index < 0 || index >= kNumEnsembleShapes || !tx || !ty)
        return set_error(GOC_ERR_ARG, "goc_ensemble_tile_shape: index %d out of range", index);
    *tx = kEnsembleShapes[index].tx;
    *ty = kEnsembleShapes[index].ty;
    return GOC_OK;
}

extern "C" int goc_ensemble_set_tile_shape(void* ensemble, int index) {
    if (!ensemble) return set_error(GOC_ERR_ARG, "goc_ensemble_set_tile_shape: null handle");
    if (index < 0 || index >= kNumEnsembleShapes)
        return set_error(GOC_ERR_ARG, "goc_ensemble_set_tile_shape: index %d out of range", index);
    Ensemble* e = static_cast<Ensemble*>(ensemble);
    if (e->shape == index) return GOC_OK;
    cudaError_t err = cudaDeviceSynchronize();   // the old queue may be in use
    if (err != cudaSuccess) return set_error(GOC_ERR_CUDA, "goc_ensemble_set_tile_shape: %s", cudaGetErrorString(err));
    e->shape = index;
    return build_tiles(e);
}

extern "C" int goc_ensemble_get_tile_shape(void* ensemble, int* index) {
    if (!ensemble || !index) return set_error(GOC_ERR_ARG, "goc_ensemble_get_tile_shape: null argument");
    *index = static_cast<Ensemble*>(ensemble)->shape;
    return GOC_OK;
}

extern "C" int goc_ensemble_end_block(void* ensemble, int n_launched, void* stream) {
    if (!ensemble) return set_error(GOC_ERR_ARG, "goc_ensemble_end_block: null handle");
    Ensemble* e = static_cast<Ensemble*>(ensemble);
    if (n_launched < 0 || n_launched > e->max_substeps)
        return set_error(GOC_ERR_ARG, "goc_ensemble_end_block: %d steps launched, max %d", n_launched, e->max_substeps);
    if (e->n_drift_chunks > 0 && n_launched > 0) {
        const int rc = launch_drift(e, n_launched - 1, 1, 0, e->d_drift_chunks, e->n_drift_chunks,
                                    e->block_noise == kNoiseLastStep ? e->d_spare : nullptr, stream);
        if (rc) return rc;
    }
    ensemble_end_block_kernel<<<(e->n_members + 127) / 128, 128, 0, as_stream(stream)>>>(e->d_members, e->d_nsub,
                                                                                      e->n_members);
    count_launch();
    int rc = check_launch("ensemble_end_block_kernel");
    if (rc) return rc;
    // the staging error flag, for goc_ensemble_staging_errors
    const cudaError_t err = cudaMemcpyAsync(const_cast<int*>(e->h_tma_err), e->d_tma_err, sizeof(int),
                                            cudaMemcpyDeviceToHost, as_stream(stream));
    if (err != cudaSuccess) return set_error(GOC_ERR_CUDA, "goc_ensemble_end_block: %s", cudaGetErrorString(err));
    return GOC_OK;
}

extern "C" int goc_ensemble_staging_errors(void* ensemble, int* errors) {
    if (!ensemble || !errors) return set_error(GOC_ERR_ARG, "goc_ensemble_staging_errors: null argument");
    *errors = *static_cast<Ensemble*>(ensemble)->h_tma_err;
    return GOC_OK;
}

extern "C" int goc_ensemble_get_member(void* ensemble, int m, GocMemberDesc* out, void* stream) {
    if (!ensemble || !out) return set_error(GOC_ERR_ARG, "goc_ensemble_get_member: null argument");
    Ensemble* e = static_cast<Ensemble*>(ensemble);
    if (m < 0 || m >= e->n_members) return set_error(GOC_ERR_ARG, "goc_ensemble_get_member: member %d out of range", m);
    cudaStream_t st = as_stream(stream);
    cudaError_t err = cudaMemcpyAsync(out, e->d_members + m, sizeof(GocMemberDesc), cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    if (err != cudaSuccess) return set_error(GOC_ERR_CUDA, "goc_ensemble_get_member: %s", cudaGetErrorString(err));
    return GOC_OK;
}

extern "C" int goc_ensemble_max_dt(void* ensemble, float* dt_out, void* stream) {
    if (!ensemble || !dt_out) return set_error(GOC_ERR_ARG, "goc_ensemble_max_dt: null argument");
    Ensemble* e = static_cast<Ensemble*>(ensemble);
    cudaStream_t st = as_stream(stream);
    ensemble_dt_partials_kernel<<<e->n_dt_items, dim3(kDtBX, kDtBY), 0, st>>>(e->d_members, e->d_dt_items,
                                                                             e->d_partials);
    count_launch();
    int rc = check_launch("ensemble_dt_partials_kernel");
    if (rc) return rc;
    ensemble_dt_final_kernel<<<e->n_members, 256, 0, st>>>(e->d_partials, e->d_dt_ranges, dt_out);
    count_launch();
    return check_launch("ensemble_dt_final_kernel");
}

static int split_chunks(Ensemble* e);

extern "C" int goc_ensemble_set_drifters(void* ensemble, float* const* positions, const int* num_drifters,
                                         float sensitivity, void* stream) {
    if (!ensemble || !positions || !num_drifters) return set_error(GOC_ERR_ARG, "goc_ensemble_set_drifters: null argument");
    Ensemble* e = static_cast<Ensemble*>(ensemble);
    std::vector<int4> chunks;
    std::vector<int> nd(e->n_members, 0);
    long long packed = 0;
    e->has_drifters.assign(e->n_members, 0);
    for (int m = 0; m < e->n_members; ++m) {
        if (!positions[m]) continue;
        e->has_drifters[m] = 1;
        if (num_drifters[m] < 0) return set_error(GOC_ERR_ARG, "goc_ensemble_set_drifters: negative count");
        nd[m] = num_drifters[m];
        const int n = num_drifters[m] + 1;  // with the observation row
        if (packed + n > INT_MAX) return set_error(GOC_ERR_ARG, "goc_ensemble_set_drifters: too many drifters");
        for (int f = 0; f < n; f += kDriftChunk)
            chunks.push_back(make_int4(m, f, std::min(kDriftChunk, n - f), (int)(packed + f)));
        packed += n;
    }
    cudaStream_t st = as_stream(stream);
    cudaError_t err = cudaStreamSynchronize(st);
    // the unperturbed copies follow the members with drifters: made anew
    cudaFree(e->d_spare_pool);
    cudaFree(e->d_spare);
    e->d_spare_pool = nullptr;
    e->d_spare = nullptr;
    if (e->block_noise == kNoiseLastStep && err == cudaSuccess) {
        const int rc = ensure_spares(e);
        if (rc) return rc;
    }
    if (e->d_step_chunks != e->d_drift_chunks) cudaFree(e->d_step_chunks);
    cudaFree(e->d_wind_chunks);
    e->d_step_chunks = nullptr;
    e->d_wind_chunks = nullptr;
    e->n_step_chunks = e->n_wind_chunks = 0;
    cudaFree(e->d_drift_pos);
    cudaFree(e->d_drift_chunks);
    cudaFree(e->d_drift_n);
    e->d_drift_pos = nullptr;
    e->d_drift_chunks = nullptr;
    e->d_drift_n = nullptr;
    e->n_drift_chunks = 0;
    e->drift_rows = 0;
    if (err == cudaSuccess) err = cudaMalloc(&e->d_drift_pos, sizeof(float*) * e->n_members);
    if (err == cudaSuccess) err = cudaMemcpy(e->d_drift_pos, positions, sizeof(float*) * e->n_members, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMalloc(&e->d_drift_n, sizeof(int) * e->n_members);
    if (err == cudaSuccess) err = cudaMemcpy(e->d_drift_n, nd.data(), sizeof(int) * e->n_members, cudaMemcpyHostToDevice);
    if (err == cudaSuccess && !chunks.empty()) {
        err = cudaMalloc(&e->d_drift_chunks, sizeof(int4) * chunks.size());
        if (err == cudaSuccess)
            err = cudaMemcpy(e->d_drift_chunks, chunks.data(), sizeof(int4) * chunks.size(), cudaMemcpyHostToDevice);
    }
    if (err != cudaSuccess) return set_error(GOC_ERR_CUDA, "goc_ensemble_set_drifters: %s", cudaGetErrorString(err));
    e->n_drift_chunks = (int)chunks.size();
    e->host_chunks = chunks;
    e->drift_rows = packed;
    e->drift_sensitivity = sensitivity;
    return split_chunks(e);
}

// The persistent step advects the drifters of members without wind drift;
// those with wind drift move in launches of their own (ensemble_drift_kernel).
static int split_chunks(Ensemble* e) {
    if (e->d_step_chunks != e->d_drift_chunks) cudaFree(e->d_step_chunks);
    cudaFree(e->d_wind_chunks);
    e->d_step_chunks = e->d_drift_chunks;
    e->n_step_chunks = e->n_drift_chunks;
    e->d_wind_chunks = nullptr;
    e->n_wind_chunks = 0;
    std::vector<int4> plain, windy;
    for (const int4& c : e->host_chunks)
        (c.x < (int)e->has_wind.size() && e->has_wind[c.x] ? windy : plain).push_back(c);
    if (windy.empty()) return GOC_OK;
    cudaError_t err = cudaMalloc(&e->d_wind_chunks, sizeof(int4) * windy.size());
    if (err == cudaSuccess)
        err = cudaMemcpy(e->d_wind_chunks, windy.data(), sizeof(int4) * windy.size(), cudaMemcpyHostToDevice);
    e->d_step_chunks = nullptr;
    if (err == cudaSuccess && !plain.empty()) {
        err = cudaMalloc(&e->d_step_chunks, sizeof(int4) * plain.size());
        if (err == cudaSuccess)
            err = cudaMemcpy(e->d_step_chunks, plain.data(), sizeof(int4) * plain.size(), cudaMemcpyHostToDevice);
    }
    if (err != cudaSuccess) return set_error(GOC_ERR_CUDA, "ensemble drifter chunks: %s", cudaGetErrorString(err));
    e->n_wind_chunks = (int)windy.size();
    e->n_step_chunks = (int)plain.size();
    return GOC_OK;
}

extern "C" int goc_ensemble_set_drift_wind(void* ensemble, const GocDriftWindDesc* wind, void* stream) {
    if (!ensemble) return set_error(GOC_ERR_ARG, "goc_ensemble_set_drift_wind: null handle");
    Ensemble* e = static_cast<Ensemble*>(ensemble);
    std::vector<DriftWind> table(e->n_members);
    e->has_wind.assign(e->n_members, 0);
    for (int m = 0; wind && m < e->n_members; ++m) {
        const GocDriftWindDesc& w = wind[m];
        if (w.wind_drift_factor == 0.0f) {
            table[m] = DriftWind{nullptr, nullptr, nullptr, nullptr, 1, 1, 0.0f, 0.0f};
            continue;
        }
        if (!w.x_current || !w.x_next || !w.y_current || !w.y_next || w.nx < 1 || w.ny < 1)
            return set_error(GOC_ERR_ARG, "goc_ensemble_set_drift_wind: member %d: wind textures missing", m);
        table[m] = DriftWind{w.x_current, w.x_next, w.y_current, w.y_next, w.nx, w.ny, 0.0f, w.wind_drift_factor};
        e->has_wind[m] = 1;
    }
    cudaError_t err = cudaStreamSynchronize(as_stream(stream));
    if (err == cudaSuccess && !e->d_wind) err = cudaMalloc(&e->d_wind, sizeof(DriftWind) * e->n_members);
    if (err == cudaSuccess && !e->d_wind_t)
        err = cudaMalloc(&e->d_wind_t, sizeof(float) * (size_t)e->n_members * e->max_substeps);
    if (err == cudaSuccess) err = cudaMemset(e->d_wind_t, 0, sizeof(float) * (size_t)e->n_members * e->max_substeps);
    if (err == cudaSuccess)
        err = cudaMemcpy(e->d_wind, table.data(), sizeof(DriftWind) * e->n_members, cudaMemcpyHostToDevice);
    if (err != cudaSuccess) return set_error(GOC_ERR_CUDA, "goc_ensemble_set_drift_wind: %s", cudaGetErrorString(err));
    return split_chunks(e);
}

extern "C" int goc_ensemble_set_wind_times(void* ensemble, const float* wind_t, void* stream) {
    if (!ensemble || !wind_t) return set_error(GOC_ERR_ARG, "goc_ensemble_set_wind_times: null argument");
    Ensemble* e = static_cast<Ensemble*>(ensemble);
    if (!e->d_wind_t) return set_error(GOC_ERR_ARG, "goc_ensemble_set_wind_times: call goc_ensemble_set_drift_wind first");
    cudaStream_t st = as_stream(stream);
    cudaError_t err = cudaMemcpyAsync(e->d_wind_t, wind_t, sizeof(float) * (size_t)e->n_members * e->max_substeps,
                                      cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);  // the host table may be reused on return
    if (err != cudaSuccess) return set_error(GOC_ERR_CUDA, "goc_ensemble_set_wind_times: %s", cudaGetErrorString(err));
    return GOC_OK;
}

namespace goc {
// every member's drifter rows (positions and observation row) into one
// packed array, in member order
__global__ void ensemble_gather_drifters_kernel(float* const* __restrict__ pos, const int4* __restrict__ chunks,
                                                float* __restrict__ dst) {
    const int4 c = chunks[blockIdx.x];
    const float* src = pos[c.x];
    for (int q = threadIdx.x; q < 2 * c.z; q += blockDim.x) dst[2 * (size_t)c.w + q] = src[2 * (size_t)c.y + q];
}

// observation row of every member with drifters from an (n_members x 2) array
__global__ void ensemble_scatter_observations_kernel(float* const* __restrict__ pos, const int* __restrict__ nd,
                                                     int n, const float* __restrict__ src) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n || !pos[m]) return;
    float* row = pos[m] + 2 * (size_t)nd[m];
    row[0] = src[2 * m];
    row[1] = src[2 * m + 1];
}
}  // namespace goc

extern "C" int goc_ensemble_drifter_rows(void* ensemble, long long* rows) {
    if (!ensemble || !rows) return set_error(GOC_ERR_ARG, "goc_ensemble_drifter_rows: null argument");
    *rows = static_cast<Ensemble*>(ensemble)->drift_rows;
    return GOC_OK;
}

extern "C" int goc_ensemble_gather_drifters(void* ensemble, float* dst, void* stream) {
    if (!ensemble) return set_error(GOC_ERR_ARG, "goc_ensemble_gather_drifters: null ensemble");
    Ensemble* e = static_cast<Ensemble*>(ensemble);
    if (e->n_drift_chunks == 0) return GOC_OK;
    if (!dst) return set_error(GOC_ERR_ARG, "goc_ensemble_gather_drifters: null destination");
    ensemble_gather_drifters_kernel<<<e->n_drift_chunks, 256, 0, as_stream(stream)>>>(e->d_drift_pos,
                                                                                     e->d_drift_chunks, dst);
    count_launch();
    return check_launch("ensemble_gather_drifters_kernel");
}

extern "C" int goc_ensemble_scatter_observations(void* ensemble, const float* src, void* stream) {
    if (!ensemble) return set_error(GOC_ERR_ARG, "goc_ensemble_scatter_observations: null ensemble");
    Ensemble* e = static_cast<Ensemble*>(ensemble);
    if (!e->d_drift_pos) return GOC_OK;
    if (!src) return set_error(GOC_ERR_ARG, "goc_ensemble_scatter_observations: null source");
    ensemble_scatter_observations_kernel<<<(e->n_members + 127) / 128, 128, 0, as_stream(stream)>>>(
        e->d_drift_pos, e->d_drift_n, e->n_members, src);
    count_launch();
    return check_launch("ensemble_scatter_observations_kernel");
}
