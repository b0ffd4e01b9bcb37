// Host entry points of the single-simulator CDKLM16 step kernels.
#include <cstdio>

#include "cdklm_tile.cuh"

namespace goc {

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// Launch constants and the texture specialisation flags.
static int make_const(const GocCdklmParams* p, StepConst* k, bool* const_f, bool* simple) {
    *k = make_step_const(*p);
    *const_f = (p->coriolis_nx == 1 && p->coriolis_ny == 1);
    *simple = (p->wind_x_nx == 1 && p->wind_x_ny == 1 && p->wind_y_nx == 1 && p->wind_y_ny == 1 &&
               p->atm_p_nx == 1 && p->atm_p_ny == 1);
    return GOC_OK;
}

// Members that share parameters and bathymetry but not their state: member
// z of the launch (blockIdx.z) reads and writes its buffers at offset
// z * member_stride floats, and its uniform wind stress at z * wind_stride.
template <int TX, int TY, int NT, bool CONST_F, bool SIMPLE_FORCING>
__global__ void __launch_bounds__(NT, 3)
cdklm_members_kernel(const GocCdklmParams p, const StepConst k, float dt, const float* __restrict__ e_in,
                     const float* __restrict__ hu_in, const float* __restrict__ hv_in, float* e_out, float* hu_out,
                     float* hv_out, float* e_st, float* hu_st, float* hv_st, int pitch, long long member_stride,
                     int wind_stride, const float* __restrict__ Hi_g, int hi_pitch, const float* __restrict__ Hm_g,
                     int hm_pitch) {
    extern __shared__ __align__(16) float smem_raw[];
    const size_t off = (size_t)blockIdx.z * (size_t)member_stride;
    GocCdklmParams pm = p;
    if (wind_stride) {
        const size_t wo = (size_t)blockIdx.z * wind_stride;
        pm.wind_x_cur += wo; pm.wind_x_next += wo; pm.wind_y_cur += wo; pm.wind_y_next += wo;
    }
    cdklm_tile<TX, TY, 2, NT, CONST_F, SIMPLE_FORCING>(pm, k, dt, 1, blockIdx.x, blockIdx.y, e_in + off, hu_in + off,
                                                       hv_in + off, e_out + off, hu_out + off, hv_out + off,
                                                       e_st ? e_st + off : nullptr, e_st ? hu_st + off : nullptr,
                                                       e_st ? hv_st + off : nullptr, pitch, Hi_g, hi_pitch, Hm_g,
                                                       hm_pitch, smem_raw);
}

template <bool CF, bool SF>
static int launch_members(const GocCdklmParams* p, const StepConst& k, float dt, const float* e0, const float* hu0,
                          const float* hv0, float* e1, float* hu1, float* hv1, float* es, float* hus, float* hvs,
                          int pitch_f, long long stride, int n, int wind_stride, const float* Hi, int hip,
                          const float* Hm, int hmp, cudaStream_t st) {
    constexpr int W = kTX + 8, H = kTY + 8;
    constexpr size_t smem = sizeof(TileSmem<W, H>);
    auto kern = cdklm_members_kernel<kTX, kTY, kNT, CF, SF>;
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return set_error(GOC_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(e));
        configured = true;
    }
    dim3 grid((p->nx + kTX - 1) / kTX, (p->ny + kTY - 1) / kTY, n);
    kern<<<grid, kNT, smem, st>>>(*p, k, dt, e0, hu0, hv0, e1, hu1, hv1, es, hus, hvs, pitch_f, stride, wind_stride,
                                  Hi, hip, Hm, hmp);
    count_launch();
    return check_launch("cdklm_members_kernel");
}

template <int NSTAGE, bool CF, bool SF, bool ANGLE = false>
static int launch_tile(const GocCdklmParams* p, const StepConst& k, float dt, int rk_step,
                       const float* e0, const float* hu0, const float* hv0, float* e1, float* hu1, float* hv1,
                       float* ea, float* hua, float* hva, int pitch_f, const float* Hi, int hi_pitch_f,
                       const float* Hm, int hm_pitch_f, cudaStream_t st) {
    constexpr int HALO = 2 * NSTAGE;
    constexpr int W = kTX + 2 * HALO, H = kTY + 2 * HALO;
    constexpr size_t smem = ANGLE ? sizeof(TileSmemAngle<W, H>) : sizeof(TileSmem<W, H>);
    auto kern = cdklm_tile_kernel<kTX, kTY, NSTAGE, kNT, CF, SF, ANGLE>;
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return set_error(GOC_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(e));
        configured = true;
    }
    dim3 grid((p->nx + kTX - 1) / kTX, (p->ny + kTY - 1) / kTY);
    kern<<<grid, kNT, smem, st>>>(*p, k, dt, rk_step, e0, hu0, hv0, e1, hu1, hv1, ea, hua, hva, pitch_f, Hi,
                                  hi_pitch_f, Hm, hm_pitch_f);
    count_launch();
    return check_launch("cdklm_tile_kernel");
}

template <int NSTAGE>
static int dispatch(const GocCdklmParams* p, const StepConst& k, bool cf, bool sf, float dt, int rk_step,
                    const float* e0, const float* hu0, const float* hv0, float* e1, float* hu1, float* hv1,
                    float* ea, float* hua, float* hva, int pitch_f, const float* Hi, int hi_pitch_f,
                    const float* Hm, int hm_pitch_f, cudaStream_t st) {
    if (cf && sf)
        return launch_tile<NSTAGE, true, true>(p, k, dt, rk_step, e0, hu0, hv0, e1, hu1, hv1, ea, hua, hva, pitch_f, Hi, hi_pitch_f, Hm, hm_pitch_f, st);
    if (cf)
        return launch_tile<NSTAGE, true, false>(p, k, dt, rk_step, e0, hu0, hv0, e1, hu1, hv1, ea, hua, hva, pitch_f, Hi, hi_pitch_f, Hm, hm_pitch_f, st);
    if (sf)
        return launch_tile<NSTAGE, false, true>(p, k, dt, rk_step, e0, hu0, hv0, e1, hu1, hv1, ea, hua, hva, pitch_f, Hi, hi_pitch_f, Hm, hm_pitch_f, st);
    return launch_tile<NSTAGE, false, false>(p, k, dt, rk_step, e0, hu0, hv0, e1, hu1, hv1, ea, hua, hva, pitch_f, Hi, hi_pitch_f, Hm, hm_pitch_f, st);
}

static int check_pitch(const GocCdklmParams* p, int pitch, int Hi_pitch, int Hm_pitch, const char* who) {
    if (pitch < (p->nx + 4) * 4 || pitch % 4)
        return set_error(GOC_ERR_ARG, "%s: pitch %d too small for nx+4=%d floats", who, pitch, p->nx + 4);
    if (Hm_pitch < (p->nx + 4) * 4 || Hm_pitch % 4)
        return set_error(GOC_ERR_ARG, "%s: Hm pitch %d too small for nx+4=%d floats", who, Hm_pitch, p->nx + 4);
    if (Hi_pitch < (p->nx + 5) * 4 || Hi_pitch % 4)
        return set_error(GOC_ERR_ARG, "%s: Hi pitch %d too small for nx+5=%d floats", who, Hi_pitch, p->nx + 5);
    return GOC_OK;
}

}  // namespace goc

using namespace goc;

extern "C" int goc_cdklm_rk2_step(const GocCdklmParams* p, float dt, const float* eta0, const float* hu0,
                                  const float* hv0, float* eta1, float* hu1, float* hv1, int pitch,
                                  const float* Hi, int Hi_pitch, const float* Hm, int Hm_pitch, void* stream) {
    int rc = validate_params(p, "goc_cdklm_rk2_step");
    if (rc) return rc;
    if ((rc = check_pitch(p, pitch, Hi_pitch, Hm_pitch, "goc_cdklm_rk2_step"))) return rc;
    if (!eta0 || !hu0 || !hv0 || !eta1 || !hu1 || !hv1 || !Hi || !Hm)
        return set_error(GOC_ERR_ARG, "goc_cdklm_rk2_step: null buffer");
    if (eta0 == eta1 || hu0 == hu1 || hv0 == hv1)
        return set_error(GOC_ERR_ARG, "goc_cdklm_rk2_step: input and output buffers must differ");
    if (p->rk_order != 2) return set_error(GOC_ERR_ARG, "goc_cdklm_rk2_step: params.rk_order must be 2");
    if (!(dt >= 0.0f)) return set_error(GOC_ERR_ARG, "goc_cdklm_rk2_step: dt must be >= 0");
    StepConst k;
    bool cf, sf;
    cudaStream_t st = as_stream(stream);
    if ((rc = make_const(p, &k, &cf, &sf))) return rc;
    return dispatch<2>(p, k, cf, sf, dt, 1, eta0, hu0, hv0, eta1, hu1, hv1, nullptr, nullptr, nullptr, pitch / 4,
                       Hi, Hi_pitch / 4, Hm, Hm_pitch / 4, st);
}

// n_steps fused RK2 steps with the time steps dts[0..n_steps) (host
// memory), alternating between buffer set 0 and set 1 from set 0: the state
// ends in set n_steps % 2.  One launch per step, issued from this loop, so a
// long run of steps is not bound by the caller's per-step overhead.
extern "C" int goc_cdklm_rk2_steps(const GocCdklmParams* p, const float* dts, int n_steps, float* eta0, float* hu0,
                                   float* hv0, float* eta1, float* hu1, float* hv1, int pitch, const float* Hi,
                                   int Hi_pitch, const float* Hm, int Hm_pitch, void* stream) {
    int rc = validate_params(p, "goc_cdklm_rk2_steps");
    if (rc) return rc;
    if ((rc = check_pitch(p, pitch, Hi_pitch, Hm_pitch, "goc_cdklm_rk2_steps"))) return rc;
    if (n_steps < 0 || (n_steps > 0 && !dts)) return set_error(GOC_ERR_ARG, "goc_cdklm_rk2_steps: bad step list");
    if (!eta0 || !hu0 || !hv0 || !eta1 || !hu1 || !hv1 || !Hi || !Hm)
        return set_error(GOC_ERR_ARG, "goc_cdklm_rk2_steps: null buffer");
    if (eta0 == eta1 || hu0 == hu1 || hv0 == hv1)
        return set_error(GOC_ERR_ARG, "goc_cdklm_rk2_steps: the two buffer sets must differ");
    if (p->rk_order != 2) return set_error(GOC_ERR_ARG, "goc_cdklm_rk2_steps: params.rk_order must be 2");
    for (int s = 0; s < n_steps; ++s)
        if (!(dts[s] >= 0.0f)) return set_error(GOC_ERR_ARG, "goc_cdklm_rk2_steps: dt %d must be >= 0", s);
    StepConst k;
    bool cf, sf;
    cudaStream_t st = as_stream(stream);
    if ((rc = make_const(p, &k, &cf, &sf))) return rc;
    float* e[2] = {eta0, eta1};
    float* u[2] = {hu0, hu1};
    float* v[2] = {hv0, hv1};
    for (int s = 0; s < n_steps; ++s) {
        const int a = s & 1, b = a ^ 1;
        if ((rc = dispatch<2>(p, k, cf, sf, dts[s], 1, e[a], u[a], v[a], e[b], u[b], v[b], nullptr, nullptr, nullptr,
                              pitch / 4, Hi, Hi_pitch / 4, Hm, Hm_pitch / 4, st)))
            return rc;
    }
    return GOC_OK;
}

extern "C" int goc_cdklm_rk2_step_stage(const GocCdklmParams* p, float dt, const float* eta0, const float* hu0,
                                        const float* hv0, float* eta1, float* hu1, float* hv1, float* eta_s,
                                        float* hu_s, float* hv_s, int pitch, const float* Hi, int Hi_pitch,
                                        const float* Hm, int Hm_pitch, void* stream) {
    int rc = validate_params(p, "goc_cdklm_rk2_step_stage");
    if (rc) return rc;
    if ((rc = check_pitch(p, pitch, Hi_pitch, Hm_pitch, "goc_cdklm_rk2_step_stage"))) return rc;
    if (!eta0 || !hu0 || !hv0 || !eta1 || !hu1 || !hv1 || !eta_s || !hu_s || !hv_s || !Hi || !Hm)
        return set_error(GOC_ERR_ARG, "goc_cdklm_rk2_step_stage: null buffer");
    if (eta0 == eta1 || eta_s == eta0 || eta_s == eta1)
        return set_error(GOC_ERR_ARG, "goc_cdklm_rk2_step_stage: the three buffer sets must differ");
    if (p->rk_order != 2) return set_error(GOC_ERR_ARG, "goc_cdklm_rk2_step_stage: params.rk_order must be 2");
    StepConst k;
    bool cf, sf;
    cudaStream_t st = as_stream(stream);
    if ((rc = make_const(p, &k, &cf, &sf))) return rc;
    return dispatch<2>(p, k, cf, sf, dt, 1, eta0, hu0, hv0, eta1, hu1, hv1, eta_s, hu_s, hv_s, pitch / 4, Hi,
                       Hi_pitch / 4, Hm, Hm_pitch / 4, st);
}

extern "C" int goc_cdklm_rk2_step_members(const GocCdklmParams* p, float dt, const float* eta0, const float* hu0,
                                          const float* hv0, float* eta1, float* hu1, float* hv1, float* eta_s,
                                          float* hu_s, float* hv_s, int pitch, long long member_stride,
                                          int n_members, int wind_stride, const float* Hi, int Hi_pitch,
                                          const float* Hm, int Hm_pitch, void* stream) {
    int rc = validate_params(p, "goc_cdklm_rk2_step_members");
    if (rc) return rc;
    if ((rc = check_pitch(p, pitch, Hi_pitch, Hm_pitch, "goc_cdklm_rk2_step_members"))) return rc;
    if (!eta0 || !hu0 || !hv0 || !eta1 || !hu1 || !hv1 || !Hi || !Hm)
        return set_error(GOC_ERR_ARG, "goc_cdklm_rk2_step_members: null buffer");
    if ((eta_s || hu_s || hv_s) && !(eta_s && hu_s && hv_s))
        return set_error(GOC_ERR_ARG, "goc_cdklm_rk2_step_members: the first-stage set must be all or none");
    if (n_members < 1 || n_members > 65535 || member_stride < (long long)(p->ny + 4) * (pitch / 4) || wind_stride < 0)
        return set_error(GOC_ERR_ARG, "goc_cdklm_rk2_step_members: bad member count or stride");
    if (p->rk_order != 2) return set_error(GOC_ERR_ARG, "goc_cdklm_rk2_step_members: params.rk_order must be 2");
    StepConst k;
    bool cf, sf;
    cudaStream_t st = as_stream(stream);
    if ((rc = make_const(p, &k, &cf, &sf))) return rc;
    if (!sf) return set_error(GOC_ERR_UNSUPPORTED, "goc_cdklm_rk2_step_members: needs uniform forcing textures");
    if (cf)
        return launch_members<true, true>(p, k, dt, eta0, hu0, hv0, eta1, hu1, hv1, eta_s, hu_s, hv_s, pitch / 4,
                                          member_stride, n_members, wind_stride, Hi, Hi_pitch / 4, Hm, Hm_pitch / 4, st);
    return launch_members<false, true>(p, k, dt, eta0, hu0, hv0, eta1, hu1, hv1, eta_s, hu_s, hv_s, pitch / 4,
                                       member_stride, n_members, wind_stride, Hi, Hi_pitch / 4, Hm, Hm_pitch / 4, st);
}

extern "C" int goc_cdklm_stage(const GocCdklmParams* p, float dt, int rk_step, const float* eta_in,
                               const float* hu_in, const float* hv_in, float* eta_out, float* hu_out,
                               float* hv_out, float* eta_alt, float* hu_alt, float* hv_alt, int pitch,
                               const float* Hi, int Hi_pitch, const float* Hm, int Hm_pitch, void* stream) {
    int rc = validate_params(p, "goc_cdklm_stage", true, true);
    if (rc) return rc;
    if ((rc = check_pitch(p, pitch, Hi_pitch, Hm_pitch, "goc_cdklm_stage"))) return rc;
    if (!eta_in || !hu_in || !hv_in || !eta_out || !hu_out || !hv_out || !Hi || !Hm)
        return set_error(GOC_ERR_ARG, "goc_cdklm_stage: null buffer");
    if (rk_step < 0 || rk_step >= p->rk_order)
        return set_error(GOC_ERR_ARG, "goc_cdklm_stage: rk_step %d out of range for rk_order %d", rk_step, p->rk_order);
    if (p->rk_order == 3 && rk_step == 1 && (!eta_alt || !hu_alt || !hv_alt))
        return set_error(GOC_ERR_ARG, "goc_cdklm_stage: RK3 stage 1 needs the alternate output set");
    if (eta_in == eta_out) return set_error(GOC_ERR_ARG, "goc_cdklm_stage: input and output buffers must differ");
    StepConst k;
    bool cf, sf;
    cudaStream_t st = as_stream(stream);
    if ((rc = make_const(p, &k, &cf, &sf))) return rc;
    if (p->angle_nx * p->angle_ny > 1) {
        // a north vector per cell (angle texture): its own kernel, general
        // Coriolis and forcing lookups
        return launch_tile<1, false, false, true>(p, k, dt, rk_step, eta_in, hu_in, hv_in, eta_out, hu_out, hv_out,
                                                  eta_alt, hu_alt, hv_alt, pitch / 4, Hi, Hi_pitch / 4, Hm,
                                                  Hm_pitch / 4, st);
    }
    return dispatch<1>(p, k, cf, sf, dt, rk_step, eta_in, hu_in, hv_in, eta_out, hu_out, hv_out, eta_alt, hu_alt,
                       hv_alt, pitch / 4, Hi, Hi_pitch / 4, Hm, Hm_pitch / 4, st);
}

namespace goc {
__global__ void cell_texture_kernel(const float* __restrict__ tex, int tnx, int tny, int nx, int ny,
                                    float* __restrict__ out, int pitch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= nx + 4 || j >= ny + 4) return;
    const float s = (i + 0.5f) / (nx + 4.0f);
    const float t = (j + 0.5f) / (ny + 4.0f);
    out[(size_t)j * pitch + i] = tex_bilinear(tex, tnx, tny, s, t);
}
}  // namespace goc

extern "C" int goc_cell_texture(const float* tex, int tex_nx, int tex_ny, int nx, int ny, float* out, int out_pitch,
                                void* stream) {
    if (!tex || !out || tex_nx < 1 || tex_ny < 1 || nx < 1 || ny < 1 || out_pitch < (nx + 4) * 4 || out_pitch % 4)
        return set_error(GOC_ERR_ARG, "goc_cell_texture: bad arguments");
    dim3 blk(32, 8), grd((nx + 4 + 31) / 32, (ny + 4 + 7) / 8);
    cell_texture_kernel<<<grd, blk, 0, as_stream(stream)>>>(tex, tex_nx, tex_ny, nx, ny, out, out_pitch / 4);
    count_launch();
    return check_launch("cell_texture_kernel");
}
