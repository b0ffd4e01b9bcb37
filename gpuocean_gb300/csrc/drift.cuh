// Lagrangian drifter advection (device side), shared by the single-collection
// kernel and the batched ensemble kernel.
#pragma once

#include "common.cuh"

namespace goc {

struct DriftGrid {
    int nx, ny;
    float dx, dy;
    int x0ref, y0ref;             // cell column/row of x = 0 / y = 0 (2 = first interior)
    const float* eta; const float* hu; const float* hv; int pitch;   // floats
    const float* Hm; int hm_pitch;                                   // floats
    int periodic_ns, periodic_ew;
};

struct DriftWind {
    const float* x_cur; const float* x_next;
    const float* y_cur; const float* y_next;
    int nx, ny;                   // texture size (the x texture's, for both)
    float t, factor;
};

// Velocity hu/(Hm + eta) of one cell (K/driftKernels.cu:54-71).  Indices are
// clamped to the array; the reference reads whatever lies there.
__device__ __forceinline__ float cell_velocity(const DriftGrid& g, const float* mom, int i, int j) {
    i = clampi(i, 0, g.nx + 3);
    j = clampi(j, 0, g.ny + 3);
    const float h = g.Hm[(size_t)j * g.hm_pitch + i] + g.eta[(size_t)j * g.pitch + i];
    return mom[(size_t)j * g.pitch + i] / h;
}

// Cell velocities read from the grid's own arrays.
struct GridVelocity {
    const DriftGrid& g;
    __device__ __forceinline__ float operator()(int v, int i, int j) const {
        return cell_velocity(g, v ? g.hv : g.hu, i, j);
    }
};

// Cell velocities of a state whose interior cells and periodic images are
// read from a copy (eta, hu, hv with the grid's pitch) and whose other ghost
// cells (behind walls, which no step writes) from the grid's arrays; the
// arithmetic is cell_velocity's.
struct CopyVelocity {
    const DriftGrid& g;
    const float* eta; const float* hu; const float* hv;
    __device__ __forceinline__ float operator()(int v, int i, int j) const {
        i = clampi(i, 0, g.nx + 3);
        j = clampi(j, 0, g.ny + 3);
        const bool copied = (g.periodic_ew || (i >= 2 && i < g.nx + 2)) && (g.periodic_ns || (j >= 2 && j < g.ny + 2));
        const float* e = copied ? eta : g.eta;
        const float* mom = copied ? (v ? hv : hu) : (v ? g.hv : g.hu);
        const float h = g.Hm[(size_t)j * g.hm_pitch + i] + e[(size_t)j * g.pitch + i];
        return mom[(size_t)j * g.pitch + i] / h;
    }
};

// One forward-Euler drifter step with cell-centred bilinear velocities,
// optional wind drift and periodic wrap (K/driftKernels.cu:74-183);
// vel(0 | 1, i, j) gives u | v of cell (i, j).
template <class VEL>
__device__ __forceinline__ void drift_one_with(const DriftGrid& g, const VEL& vel, const DriftWind* w, float dt,
                                               float sensitivity, float& px, float& py) {
    const float fx = floorf(px / g.dx), fy = floorf(py / g.dy);
    const int cx = (int)(fx + g.x0ref);
    const int cy = (int)(fy + g.y0ref);
    const float frac_x = px / g.dx - fx;
    const float frac_y = py / g.dy - fy;
    const int x0 = frac_x < 0.5f ? cx - 1 : cx;
    const float xf = frac_x < 0.5f ? frac_x + 0.5f : frac_x - 0.5f;
    const int y0 = frac_y < 0.5f ? cy - 1 : cy;
    const float yf = frac_y < 0.5f ? frac_y + 0.5f : frac_y - 0.5f;
    const int x1 = x0 + 1, y1 = y0 + 1;
    const float u00 = vel(0, x0, y0), u10 = vel(0, x1, y0);
    const float u01 = vel(0, x0, y1), u11 = vel(0, x1, y1);
    const float v00 = vel(1, x0, y0), v10 = vel(1, x1, y0);
    const float v01 = vel(1, x0, y1), v11 = vel(1, x1, y1);
    const float uy0 = (1 - xf) * u00 + xf * u10;
    const float uy1 = (1 - xf) * u01 + xf * u11;
    const float vy0 = (1 - xf) * v00 + xf * v10;
    const float vy1 = (1 - xf) * v01 + xf * v11;
    float u = (1 - yf) * uy0 + yf * uy1;
    float v = (1 - yf) * vy0 + yf * vy1;
    if (w && w->factor != 0.0f) {
        const float Hmc = g.Hm[(size_t)clampi(cy, 0, g.ny + 3) * g.hm_pitch + clampi(cx, 0, g.nx + 3)];
        if (Hmc < 1e20f) {
            const float s = px / (g.nx * g.dx), t = py / (g.ny * g.dy);
            const float wxc = tex_bilinear(w->x_cur, w->nx, w->ny, s, t);
            const float wxn = tex_bilinear(w->x_next, w->nx, w->ny, s, t);
            const float wyc = tex_bilinear(w->y_cur, w->nx, w->ny, s, t);
            const float wyn = tex_bilinear(w->y_next, w->nx, w->ny, s, t);
            u = u + ((w->t * wxn + (1.0f - w->t) * wxc) - u) * w->factor;
            v = v + ((w->t * wyn + (1.0f - w->t) * wyc) - v) * w->factor;
        }
    }
    px += sensitivity * u * dt;
    py += sensitivity * v * dt;
    const float Lx = g.nx * g.dx, Ly = g.ny * g.dy;
    if (g.periodic_ew && px < 0) px += Lx;
    if (g.periodic_ew && px > Lx) px -= Lx;
    if (g.periodic_ns && py < 0) py += Ly;
    if (g.periodic_ns && py > Ly) py -= Ly;
}

__device__ __forceinline__ void drift_one(const DriftGrid& g, const DriftWind* w, float dt, float sensitivity,
                                          float& px, float& py) {
    drift_one_with(g, GridVelocity{g}, w, dt, sensitivity, px, py);
}

}  // namespace goc
