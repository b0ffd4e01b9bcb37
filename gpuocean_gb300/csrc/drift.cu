// Drifter kernels of a single drifter collection.
#include "drift.cuh"

namespace goc {

__global__ void drift_kernel(DriftGrid g, DriftWind w, int use_wind, float dt, float sensitivity, int n,
                             float* __restrict__ pos, int pos_pitch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float* d = pos + (size_t)i * pos_pitch;
    float px = d[0], py = d[1];
    drift_one(g, use_wind ? &w : nullptr, dt, sensitivity, px, py);
    d[0] = px;
    d[1] = py;
}

__global__ void drift_wrap_kernel(float Lx, float Ly, int periodic_ns, int periodic_ew, int n, float* pos,
                                  int pos_pitch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float* d = pos + (size_t)i * pos_pitch;
    float px = d[0], py = d[1];
    if (periodic_ew && px < 0) px += Lx;
    if (periodic_ew && px > Lx) px -= Lx;
    if (periodic_ns && py < 0) py += Ly;
    if (periodic_ns && py > Ly) py -= Ly;
    d[0] = px;
    d[1] = py;
}

}  // namespace goc

using namespace goc;

extern "C" int goc_drift(int nx, int ny, float dx, float dy, float dt, int x_zero_ref, int y_zero_ref,
                         const float* eta, const float* hu, const float* hv, int pitch, const float* Hm, int Hm_pitch,
                         int periodic_north_south, int periodic_east_west, int num_drifters, float* positions,
                         int positions_pitch, float sensitivity, const float* wind_x_cur, const float* wind_x_next,
                         const float* wind_y_cur, const float* wind_y_next, int wind_nx, int wind_ny, float wind_t,
                         float wind_drift_factor, void* stream) {
    if (nx < 1 || ny < 1 || !(dx > 0.0f) || !(dy > 0.0f)) return set_error(GOC_ERR_ARG, "goc_drift: bad grid");
    if (num_drifters < 0) return set_error(GOC_ERR_ARG, "goc_drift: negative drifter count");
    if (!eta || !hu || !hv || !Hm || !positions) return set_error(GOC_ERR_ARG, "goc_drift: null buffer");
    if (pitch < (nx + 4) * 4 || Hm_pitch < (nx + 4) * 4 || positions_pitch < 8 || pitch % 4 || Hm_pitch % 4 ||
        positions_pitch % 4)
        return set_error(GOC_ERR_ARG, "goc_drift: pitch too small");
    const int use_wind = wind_drift_factor != 0.0f;
    if (use_wind && (!wind_x_cur || !wind_x_next || !wind_y_cur || !wind_y_next || wind_nx < 1 || wind_ny < 1))
        return set_error(GOC_ERR_ARG, "goc_drift: wind drift needs the wind textures");
    DriftGrid g{nx, ny, dx, dy, x_zero_ref, y_zero_ref, eta, hu, hv, pitch / 4, Hm, Hm_pitch / 4,
                periodic_north_south, periodic_east_west};
    DriftWind w{wind_x_cur, wind_x_next, wind_y_cur, wind_y_next, wind_nx, wind_ny, wind_t, wind_drift_factor};
    const int n = num_drifters + 1;  // the last row is the observation position
    drift_kernel<<<(n + 127) / 128, 128, 0, as_stream(stream)>>>(g, w, use_wind, dt, sensitivity, n, positions,
                                                                  positions_pitch / 4);
    count_launch();
    return check_launch("drift_kernel");
}

extern "C" int goc_drift_enforce_boundary(float domain_size_x, float domain_size_y, int periodic_north_south,
                                          int periodic_east_west, int num_drifters, float* positions,
                                          int positions_pitch, void* stream) {
    if (num_drifters < 0 || !positions || positions_pitch < 8 || positions_pitch % 4)
        return set_error(GOC_ERR_ARG, "goc_drift_enforce_boundary: bad arguments");
    const int n = num_drifters + 1;
    drift_wrap_kernel<<<(n + 127) / 128, 128, 0, as_stream(stream)>>>(domain_size_x, domain_size_y,
                                                                       periodic_north_south, periodic_east_west, n,
                                                                       positions, positions_pitch / 4);
    count_launch();
    return check_launch("drift_wrap_kernel");
}

// ---------------------------------------------------------------------------
// adjoint of one drift step (no counterpart in the reference)
// ---------------------------------------------------------------------------

namespace goc {

// Interior cell that memory cell (i, j) holds, or -1 when it holds a wall
// ghost (a value the step never writes, hence no adjoint).
__device__ __forceinline__ int drift_adj_col(const DriftGrid& g, int i) {
    i = clampi(i, 0, g.nx + 3);
    if (i >= 2 && i < g.nx + 2) return i;
    return g.periodic_ew ? wrap_interior(i, g.nx) : -1;
}
__device__ __forceinline__ int drift_adj_row(const DriftGrid& g, int j) {
    j = clampi(j, 0, g.ny + 3);
    if (j >= 2 && j < g.ny + 2) return j;
    return g.periodic_ns ? wrap_interior(j, g.ny) : -1;
}

// Reverse of drift_one without wind drift: pb (2 per drifter) holds the
// adjoint of the new position on entry and of the old one on exit; the
// state adjoint of the four cells each drifter read is accumulated
// atomically into (eb, hub, hvb).
__global__ void drift_vjp_kernel(DriftGrid g, float dt, float sensitivity, int n, const float* __restrict__ pos,
                                 int pos_pitch, float* pb, int pb_pitch, float* eb, float* hub, float* hvb) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const float px = pos[(size_t)q * pos_pitch], py = pos[(size_t)q * pos_pitch + 1];
    float* b = pb + (size_t)q * pb_pitch;
    const float pxb = b[0], pyb = b[1];
    const float fx = floorf(px / g.dx), fy = floorf(py / g.dy);
    const int cx = (int)(fx + g.x0ref), cy = (int)(fy + g.y0ref);
    const float frac_x = px / g.dx - fx, frac_y = py / g.dy - fy;
    const int x0 = frac_x < 0.5f ? cx - 1 : cx;
    const float xf = frac_x < 0.5f ? frac_x + 0.5f : frac_x - 0.5f;
    const int y0 = frac_y < 0.5f ? cy - 1 : cy;
    const float yf = frac_y < 0.5f ? frac_y + 0.5f : frac_y - 0.5f;
    const int xs[2] = {x0, x0 + 1}, ys[2] = {y0, y0 + 1};
    float uc[2][2], vc[2][2], hc[2][2];
    for (int a = 0; a < 2; ++a)
        for (int c = 0; c < 2; ++c) {
            const int i = clampi(xs[c], 0, g.nx + 3), j = clampi(ys[a], 0, g.ny + 3);
            hc[a][c] = g.Hm[(size_t)j * g.hm_pitch + i] + g.eta[(size_t)j * g.pitch + i];
            uc[a][c] = g.hu[(size_t)j * g.pitch + i] / hc[a][c];
            vc[a][c] = g.hv[(size_t)j * g.pitch + i] / hc[a][c];
        }
    const float ub = sensitivity * dt * pxb, vb = sensitivity * dt * pyb;
    // weights of corner (a, c): wy[a] * wx[c]
    const float wx[2] = {1.0f - xf, xf}, wy[2] = {1.0f - yf, yf};
    const float uy0 = wx[0] * uc[0][0] + wx[1] * uc[0][1], uy1 = wx[0] * uc[1][0] + wx[1] * uc[1][1];
    const float vy0 = wx[0] * vc[0][0] + wx[1] * vc[0][1], vy1 = wx[0] * vc[1][0] + wx[1] * vc[1][1];
    float xfb = ub * (wy[0] * (uc[0][1] - uc[0][0]) + wy[1] * (uc[1][1] - uc[1][0])) +
                vb * (wy[0] * (vc[0][1] - vc[0][0]) + wy[1] * (vc[1][1] - vc[1][0]));
    float yfb = ub * (uy1 - uy0) + vb * (vy1 - vy0);
    b[0] = pxb + xfb / g.dx;
    b[1] = pyb + yfb / g.dy;
    for (int a = 0; a < 2; ++a) {
        const int j = drift_adj_row(g, ys[a]);
        if (j < 0) continue;
        for (int c = 0; c < 2; ++c) {
            const int i = drift_adj_col(g, xs[c]);
            if (i < 0) continue;
            const float w = wy[a] * wx[c];
            const float ucb = ub * w, vcb = vb * w;
            const size_t o = (size_t)j * g.pitch + i;
            atomicAdd(hub + o, ucb / hc[a][c]);
            atomicAdd(hvb + o, vcb / hc[a][c]);
            atomicAdd(eb + o, -(ucb * uc[a][c] + vcb * vc[a][c]) / hc[a][c]);
        }
    }
}

}  // namespace goc

extern "C" int goc_drift_vjp(int nx, int ny, float dx, float dy, float dt, int x_zero_ref, int y_zero_ref,
                             const float* eta, const float* hu, const float* hv, int pitch, const float* Hm,
                             int Hm_pitch, int periodic_north_south, int periodic_east_west, int num_positions,
                             const float* positions, int positions_pitch, float* positions_bar,
                             int positions_bar_pitch, float sensitivity, float* eta_bar, float* hu_bar,
                             float* hv_bar, void* stream) {
    if (nx < 1 || ny < 1 || !(dx > 0.0f) || !(dy > 0.0f)) return set_error(GOC_ERR_ARG, "goc_drift_vjp: bad grid");
    if (num_positions < 0) return set_error(GOC_ERR_ARG, "goc_drift_vjp: negative count");
    if (!eta || !hu || !hv || !Hm || !positions || !positions_bar || !eta_bar || !hu_bar || !hv_bar)
        return set_error(GOC_ERR_ARG, "goc_drift_vjp: null buffer");
    if (pitch < (nx + 4) * 4 || pitch % 4 || Hm_pitch < (nx + 4) * 4 || Hm_pitch % 4 || positions_pitch < 8 ||
        positions_pitch % 4 || positions_bar_pitch < 8 || positions_bar_pitch % 4)
        return set_error(GOC_ERR_ARG, "goc_drift_vjp: bad pitch");
    if (num_positions == 0) return GOC_OK;
    DriftGrid g{nx, ny, dx, dy, x_zero_ref, y_zero_ref, eta, hu, hv, pitch / 4, Hm, Hm_pitch / 4,
                periodic_north_south, periodic_east_west};
    drift_vjp_kernel<<<(num_positions + 127) / 128, 128, 0, as_stream(stream)>>>(
        g, dt, sensitivity, num_positions, positions, positions_pitch / 4, positions_bar, positions_bar_pitch / 4,
        eta_bar, hu_bar, hv_bar);
    count_launch();
    return check_launch("drift_vjp_kernel");
}
