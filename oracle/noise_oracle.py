"""FP64 NumPy restatement of GPU Ocean's stochastic model error and drifters.

TEST INFRASTRUCTURE ONLY: the checker for the CUDA noise and drift kernels.
No product code imports it.

Follows the reference GPU kernels (K/ = src/gpuocean/gpu_kernels):

* ``soar_coarse``          SOAR kernel, K/ocean_noise.cu:126-247
* ``geostrophic_balance``  geostrophicBalance, K/ocean_noise.cu:256-397
* ``bicubic_perturbation`` bicubicInterpolation, K/ocean_noise.cu:404-666
                           with K/interpolation.cu (coefficients + evaluation)
* ``lcg_uniform`` / ``lcg_normal``  K/random_number_generators.cu:1-134
* ``drift``                passiveDrifterKernel, K/driftKernels.cu:74-183

Pinned against vectors produced by the reference's own CPU twins
(``tests/golden/noise_drift_reference.npz``).  Deliberate differences, each a
reference defect: the non-periodic SOAR read is clamped to the last row/column
of the random field (the reference clamps one past it, :194-206); the north
vector of the noise kernels is the angle texture's first value (the reference
calls the texture lookup with its arguments swapped, :68, which reads
element 0 for any texture); the odd-width LCG field fills its last column
(the reference's test `2*ti == random_nx_` never holds, :127).
"""
from __future__ import annotations

import math

import numpy as np

CUTOFF = 2  # utils/config.py soar_cutoff


def soar_weights(cdx, cdy, q0, L):
    """5x5 SOAR covariance q0 (1 + d/L) exp(-d/L) of the stencil offsets."""
    oy, ox = np.mgrid[-CUTOFF:CUTOFF + 1, -CUTOFF:CUTOFF + 1]
    d = np.sqrt(cdx * cdx * ox * ox + cdy * cdy * oy * oy)
    return q0 * (1.0 + d / L) * np.exp(-d / L)


def soar_coarse(xi, cnx, cny, cdx, cdy, q0, L, periodic_ns, periodic_ew, scale=1.0):
    """(cny+4, cnx+4) coarse field scale * sum_{5x5} Q xi.

    The random field is (cny, cnx) when periodic in a direction, otherwise
    (cny+8, cnx+8); coarse cell (j, i) reads xi rows j..j+4 (mod cny when
    periodic, shifted by 4)."""
    xi = np.asarray(xi, dtype=np.float64)
    w = soar_weights(cdx, cdy, q0, L)
    jj = np.arange(cny + 8)
    ii = np.arange(cnx + 8)
    rows = (jj - 4) % cny if periodic_ns else np.minimum(jj, xi.shape[0] - 1)
    cols = (ii - 4) % cnx if periodic_ew else np.minimum(ii, xi.shape[1] - 1)
    local = xi[np.ix_(rows, cols)]
    out = np.zeros((cny + 4, cnx + 4))
    for a in range(5):
        for b in range(5):
            out += w[a, b] * local[a:a + cny + 4, b:b + cnx + 4]
    return scale * out


def _coriolis(nx, ny, dx, dy, f, beta, north, ftex):
    """Coriolis f at the interior cells (ny, nx): f + beta((i+0.5)dx n_x +
    (j+0.5)dy n_y) with ghost-inclusive indices, or the Coriolis texture when
    f == 0 (K/ocean_noise.cu:365-368)."""
    j = np.arange(2, ny + 2)[:, None]
    i = np.arange(2, nx + 2)[None, :]
    if f == 0 and ftex is not None:
        from oracle.cdklm16_oracle import cell_texture
        return cell_texture(ftex, nx, ny)[2:ny + 2, 2:nx + 2]
    return f + beta * ((i + 0.5) * dx * north[0] + (j + 0.5) * dy * north[1])


def geostrophic_balance(eta, hu, hv, coarse, Hi, nx, ny, dx, dy, f, beta, g, land=1e20,
                        north=(0.0, 1.0), ftex=None):
    """Add the SOAR field (same grid) and its balanced momentum to the
    interior; land cells are set to zero (K/ocean_noise.cu:256-397)."""
    I, J = slice(2, nx + 2), slice(2, ny + 2)
    c = np.asarray(coarse, dtype=np.float64)
    Hd = np.asarray(Hi, dtype=np.float64)
    a, b2, cc, d = Hd[J, I], Hd[J, 3:nx + 3], Hd[3:ny + 3, I], Hd[3:ny + 3, 3:nx + 3]
    dry = (a == land) | (b2 == land) | (cc == land) | (d == land)
    H_mid = 0.25 * (a + b2 + cc + d)
    cor = _coriolis(nx, ny, dx, dy, f, beta, north, ftex)
    de = c[J, I]
    h_mid = de + H_mid + eta[J, I]
    ex = (c[J, 3:nx + 3] - c[J, 1:nx + 1]) / (2.0 * dx)
    ey = (c[3:ny + 3, I] - c[1:ny + 1, I]) / (2.0 * dy)
    eta[J, I] += de
    hu[J, I] += -(g / cor) * h_mid * ey
    hv[J, I] += (g / cor) * h_mid * ex
    for arr in (eta, hu, hv):
        arr[J, I] = np.where(dry, 0.0, arr[J, I])


_B = np.array([[1., 0., 0., 0.], [0., 0., 1., 0.], [-3., 3., -2., -1.], [2., -2., 1., 1.]])


def bicubic_eta(coarse, nx, ny, dx, dy, cnx, cny, cdx, cdy, offset_i=0, offset_j=0):
    """d_eta on the fine cells [1, nx+3) x [1, ny+3) (interior + one ring) by
    bicubic interpolation of the coarse field (K/ocean_noise.cu:497-586).
    Every fine cell at once: its coarse cell (cj, ci) and fractions (ry, rx)
    per row and column, the 4x4 table of values, x / y differences and the
    cross difference gathered from the clamped coarse field, then
    [1 rx rx^2 rx^3] B F B^T [1 ry ry^2 ry^3]^T."""
    c = np.asarray(coarse, dtype=np.float64)
    out = np.zeros((ny + 4, nx + 4))
    j = np.arange(1, ny + 3, dtype=np.float64)
    i = np.arange(1, nx + 3, dtype=np.float64)
    y = (j - 2 + 0.5 + offset_j) * dy
    x = (i - 2 + 0.5 + offset_i) * dx
    cj = np.floor(y / cdy + 2 - 0.5).astype(np.int64)
    ci = np.floor(x / cdx + 2 - 0.5).astype(np.int64)
    cj = np.where(cj > cny + 1, cj - 1, cj)
    ci = np.where(ci > cnx + 1, ci - 1, ci)
    ry = (y - (cj - 2 + 0.5) * cdy) / cdy
    rx = (x - (ci - 2 + 0.5) * cdx) / cdx

    def C(dj, di):
        rows = np.clip(cj + dj, 0, cny + 3)[:, None]
        cols = np.clip(ci + di, 0, cnx + 3)[None, :]
        return c[rows, cols]
    f00, f01, f10, f11 = C(0, 0), C(1, 0), C(0, 1), C(1, 1)
    fx00 = (C(0, 1) - C(0, -1)) / 2
    fx01 = (C(1, 1) - C(1, -1)) / 2
    fx10 = (C(0, 2) - C(0, 0)) / 2
    fx11 = (C(1, 2) - C(1, 0)) / 2
    fy00 = (C(1, 0) - C(-1, 0)) / 2
    fy01 = (C(2, 0) - C(0, 0)) / 2
    fy10 = (C(1, 1) - C(-1, 1)) / 2
    fy11 = (C(2, 1) - C(0, 1)) / 2
    fy_10 = (C(1, -1) - C(-1, -1)) / 2
    fy_11 = (C(2, -1) - C(0, -1)) / 2
    fy20 = (C(1, 2) - C(-1, 2)) / 2
    fy21 = (C(2, 2) - C(0, 2)) / 2
    F = np.stack([np.stack([f00, f01, fy00, fy01], -1), np.stack([f10, f11, fy10, fy11], -1),
                  np.stack([fx00, fx01, (fy10 - fy_10) / 2, (fy11 - fy_11) / 2], -1),
                  np.stack([fx10, fx11, (fy20 - fy00) / 2, (fy21 - fy01) / 2], -1)], -2)
    A = _B @ F @ _B.T
    px = np.stack([np.ones_like(rx), rx, rx * rx, rx ** 3], -1)      # (nx+2, 4)
    py = np.stack([np.ones_like(ry), ry, ry * ry, ry ** 3], -1)      # (ny+2, 4)
    out[1:ny + 3, 1:nx + 3] = np.einsum("xa,yxab,yb->yx", px, A, py)
    return out


def bicubic_perturbation(eta, hu, hv, coarse, Hi, nx, ny, dx, dy, cnx, cny, cdx, cdy, f, beta, g,
                         offset_i=0, offset_j=0, land=1e20, north=(0.0, 1.0), ftex=None):
    """Bicubic up-sampling + geostrophic balance; land cells get no
    perturbation (K/ocean_noise.cu:404-666)."""
    I, J = slice(2, nx + 2), slice(2, ny + 2)
    de = bicubic_eta(coarse, nx, ny, dx, dy, cnx, cny, cdx, cdy, offset_i, offset_j)
    Hd = np.asarray(Hi, dtype=np.float64)
    a, b2, cc, d = Hd[J, I], Hd[J, 3:nx + 3], Hd[3:ny + 3, I], Hd[3:ny + 3, 3:nx + 3]
    dry = (a == land) | (b2 == land) | (cc == land) | (d == land)
    H_mid = 0.25 * (a + b2 + cc + d)
    cor = _coriolis(nx, ny, dx, dy, f, beta, north, ftex)
    ex = (de[J, 3:nx + 3] - de[J, 1:nx + 1]) / (2.0 * dx)
    ey = (de[3:ny + 3, I] - de[1:ny + 1, I]) / (2.0 * dy)
    dhu = -(g / cor) * (H_mid + de[J, I]) * ey
    dhv = (g / cor) * (H_mid + de[J, I]) * ex
    eta[J, I] += np.where(dry, 0.0, de[J, I])
    hu[J, I] += np.where(dry, 0.0, dhu)
    hv[J, I] += np.where(dry, 0.0, dhv)
    return de


# ---------------------------------------------------------------------------
# LCG random numbers (K/random_number_generators.cu)
# ---------------------------------------------------------------------------

MOD = 2147483647


def _lcg_step(seed):
    return (seed * 1103515245 + 12345) % MOD


def lcg_uniform(seeds, random_nx):
    """Two uniforms per uint64 seed: u = seed_k / 2^31.  Returns (field, seeds)."""
    s = np.asarray(seeds, dtype=object)
    ny, snx = s.shape
    out = np.zeros((ny, random_nx))
    new = np.empty_like(s)
    for j in range(ny):
        for i in range(snx):
            a = _lcg_step(int(s[j, i]))
            b = _lcg_step(a)
            new[j, i] = b
            if 2 * i < random_nx:
                out[j, 2 * i] = a / 2147483648.0
            if 2 * i + 1 < random_nx:
                out[j, 2 * i + 1] = b / 2147483648.0
    return out, new.astype(np.uint64)


def lcg_normal(seeds, random_nx, redraw_zero=True):
    """Box-Muller normals from LCG uniform pairs; a zero first uniform is
    redrawn (K/random_number_generators.cu:44-52)."""
    s = np.asarray(seeds, dtype=object)
    ny, snx = s.shape
    out = np.zeros((ny, random_nx))
    new = np.empty_like(s)
    for j in range(ny):
        for i in range(snx):
            a = _lcg_step(int(s[j, i]))
            b = _lcg_step(a)
            u1, u2 = a / 2147483648.0, b / 2147483648.0
            if redraw_zero and float(np.float32(u1)) == 0.0:
                a = _lcg_step(b)
                b = _lcg_step(a)
                u1, u2 = a / 2147483648.0, b / 2147483648.0
            new[j, i] = b
            r = math.sqrt(-2.0 * math.log(u1))
            n1, n2 = r * math.cos(2 * math.pi * u2), r * math.sin(2 * math.pi * u2)
            if 2 * i < random_nx:
                out[j, 2 * i] = n1
            if 2 * i + 1 < random_nx:
                out[j, 2 * i + 1] = n2
    return out, new.astype(np.uint64)


# ---------------------------------------------------------------------------
# drifters (K/driftKernels.cu:74-183)
# ---------------------------------------------------------------------------

def drift(positions, eta, hu, hv, Hm, nx, ny, dx, dy, dt, periodic_ns, periodic_ew, x0ref=2, y0ref=2,
          sensitivity=1.0):
    """One forward-Euler step of every row of `positions` (N+1, 2)."""
    pos = np.array(positions, dtype=np.float64, copy=True)
    u_f = np.asarray(hu, np.float64) / (np.asarray(Hm, np.float64) + np.asarray(eta, np.float64))
    v_f = np.asarray(hv, np.float64) / (np.asarray(Hm, np.float64) + np.asarray(eta, np.float64))
    x, y = pos[:, 0], pos[:, 1]
    fx, fy = np.floor(x / dx), np.floor(y / dy)
    cx = (fx + x0ref).astype(int)
    cy = (fy + y0ref).astype(int)
    frx, fry = x / dx - fx, y / dy - fy
    x0 = np.where(frx < 0.5, cx - 1, cx)
    xf = np.where(frx < 0.5, frx + 0.5, frx - 0.5)
    y0 = np.where(fry < 0.5, cy - 1, cy)
    yf = np.where(fry < 0.5, fry + 0.5, fry - 0.5)
    x0c, x1c = np.clip(x0, 0, nx + 3), np.clip(x0 + 1, 0, nx + 3)
    y0c, y1c = np.clip(y0, 0, ny + 3), np.clip(y0 + 1, 0, ny + 3)

    def interp(fld):
        a = (1 - xf) * fld[y0c, x0c] + xf * fld[y0c, x1c]
        b = (1 - xf) * fld[y1c, x0c] + xf * fld[y1c, x1c]
        return (1 - yf) * a + yf * b
    x = x + sensitivity * interp(u_f) * dt
    y = y + sensitivity * interp(v_f) * dt
    Lx, Ly = nx * dx, ny * dy
    if periodic_ew:
        x = np.where(x < 0, x + Lx, x)
        x = np.where(x > Lx, x - Lx, x)
    if periodic_ns:
        y = np.where(y < 0, y + Ly, y)
        y = np.where(y > Ly, y - Ly, y)
    pos[:, 0], pos[:, 1] = x, y
    return pos
