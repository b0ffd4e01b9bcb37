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
