"""numpy restatement of the reference erosion path (test infrastructure only).

Every function follows the reference file:line named in its docstring
(paths inside the SVIErosion project).  Arithmetic is float32 wherever the
reference computes in float32 (torch float32 tensors, Python scalars rounded
to float32 as torch does), float64 where it uses float64.  numpy's float32
FFT (pocketfft) stands in for torch.fft.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

F32 = np.float32
C64 = np.complex64   # spectrum type (complex128 in the float64 variant, oracle/fp64.py)
I64 = np.int64
MARGIN = 4
KEY_EMPTY = np.iinfo(np.int64).max

__all__ = [
    "next_fast_size", "grid_around", "godunov_inward", "cell_fractions", "cube_plane_fraction",
    "closest_points", "tricubic", "tricubic_with_gradient", "trilinear", "principal_curvatures",
    "interface_mask", "reinit_geometry", "reinit_rhs", "point_triangle_distance2", "rebuild_band",
    "band_volume", "dense_fractions", "ball_cell_weights", "kernel_hat", "exterior_fraction",
    "SVILaw", "CurvatureLaw", "make_law", "Simulation", "reinitialize", "dilate", "strides_of", "check_margin",
    "split_long_triangles", "mesh_to_sdf", "inside_mask", "edge_topology", "StepRecord",
]


# ------------------------------------------------------------------- grid
def next_fast_size(n: int) -> int:
    """grid.py:18-28: smallest m >= n with prime factors in {2, 3, 5, 7}."""
    m = max(int(n), 1)
    while True:
        k = m
        for p in (2, 3, 5, 7):
            while k % p == 0:
                k //= p
        if k == 1:
            return m
        m += 1


def grid_around(lo, hi, spacing, padding, fast=True):
    """grid.py:44-56: (origin, spacing, shape) of the padded grid."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    need = np.ceil((hi - lo + 2 * padding) / spacing).astype(int) + 1
    shape = tuple(next_fast_size(n) if fast else int(n) for n in need)
    center = 0.5 * (lo + hi)
    origin = center - 0.5 * (np.asarray(shape) - 1) * spacing
    return tuple(float(o) for o in origin), float(spacing), tuple(int(s) for s in shape)


def strides_of(shape):
    nx, ny, nz = shape
    return (ny * nz, nz, 1)


# ---------------------------------------------------------------- kernels
def _weno5(v1, v2, v3, v4, v5):
    """kernels.py:83-97."""
    p1 = v1 / 3 - 7 * v2 / 6 + 11 * v3 / 6
    p2 = -v2 / 6 + 5 * v3 / 6 + v4 / 3
    p3 = v3 / 3 + 5 * v4 / 6 - v5 / 6
    s1 = 13.0 / 12 * (v1 - 2 * v2 + v3) ** 2 + 0.25 * (v1 - 4 * v2 + 3 * v3) ** 2
    s2 = 13.0 / 12 * (v2 - 2 * v3 + v4) ** 2 + 0.25 * (v2 - v4) ** 2
    s3 = 13.0 / 12 * (v3 - 2 * v4 + v5) ** 2 + 0.25 * (3 * v3 - 4 * v4 + v5) ** 2
    vmax = np.maximum(np.maximum(np.maximum(v1 * v1, v2 * v2), np.maximum(v3 * v3, v4 * v4)), v5 * v5)
    eps = 1e-6 * vmax + 1e-10
    a1 = 0.1 / (s1 + eps) ** 2
    a2 = 0.6 / (s2 + eps) ** 2
    a3 = 0.3 / (s3 + eps) ** 2
    return (a1 * p1 + a2 * p2 + a3 * p3) / (a1 + a2 + a3)


def _minmod(a, b):
    """kernels.py:100-101."""
    return np.where(a * b > 0, np.where(np.abs(a) < np.abs(b), a, b), np.zeros_like(a))


def cube_plane_fraction(s, a, b, c):
    """kernels.py:104-122 (float32)."""
    s, a, b, c = (np.asarray(v, dtype=F32) for v in (s, a, b, c))
    M = 0.5 * (a + b + c)
    y = M - s
    flip = y > M
    y = np.maximum(np.where(flip, 2 * M - y, y), F32(0))
    tiny = F32(1e-12)
    bs = np.maximum(b, tiny)
    cs = np.maximum(c, tiny)
    q = 3 * y * y - 3 * y * c + c * c
    H1 = (y * y * y) / (bs * cs)
    H2 = q / bs
    u = np.maximum(y - b, F32(0))
    H3 = (q - (u * u * u) / cs) / bs
    H4 = 3 * (2 * y - b - c)
    H = np.where(y <= c, H1, np.where(y <= b, H2, np.where(y <= b + c, H3, H4)))
    ua = np.maximum(y - a, F32(0))
    F = H / (6 * a) - (ua * ua * ua) / (6 * a * bs * cs)
    F = np.where(flip, 1 - F, F)
    return np.clip(F, F32(0), F32(1)).astype(F32)


def _sort3_abs(gx, gy, gz):
    """kernels.py:125-131."""
    x, y, z = np.abs(gx), np.abs(gy), np.abs(gz)
    hi = np.maximum(np.maximum(x, y), z)
    lo = np.minimum(np.minimum(x, y), z)
    mid = x + y + z - hi - lo
    return hi, mid, lo


def _cubic_w(t):
    """kernels.py:134-136."""
    return (-t * (t - 1) * (t - 2) / 6, (t + 1) * (t - 1) * (t - 2) / 2,
            -(t + 1) * t * (t - 2) / 2, (t + 1) * t * (t - 1) / 6)


def _cubic_dw(t):
    """kernels.py:139-141."""
    return (-(3 * t * t - 6 * t + 2) / 6, (3 * t * t - 4 * t - 1) / 2,
            -(3 * t * t - 2 * t - 2) / 2, (3 * t * t - 1) / 6)


def godunov_inward(flat, idx, sx, sy, sz, inv_h):
    """kernels.py:146-169."""
    inv_h = F32(inv_h)
    c = flat[idx]
    g2 = np.zeros_like(c)
    for s in (sx, sy, sz):
        m3, m2, m1 = flat[idx - 3 * s], flat[idx - 2 * s], flat[idx - s]
        p1, p2, p3 = flat[idx + s], flat[idx + 2 * s], flat[idx + 3 * s]
        d0 = (m2 - m3) * inv_h
        d1 = (m1 - m2) * inv_h
        d2 = (c - m1) * inv_h
        d3 = (p1 - c) * inv_h
        d4 = (p2 - p1) * inv_h
        d5 = (p3 - p2) * inv_h
        dm = _weno5(d0, d1, d2, d3, d4)
        dp = _weno5(d5, d4, d3, d2, d1)
        g2 = g2 + np.maximum(np.minimum(dm, F32(0)) ** 2, np.maximum(dp, F32(0)) ** 2)
    return np.sqrt(g2)


def cell_fractions(flat, idx, sx, sy, sz):
    """kernels.py:173-181."""
    c = flat[idx]
    gx = 0.5 * (flat[idx + sx] - flat[idx - sx])
    gy = 0.5 * (flat[idx + sy] - flat[idx - sy])
    gz = 0.5 * (flat[idx + sz] - flat[idx - sz])
    gn = np.maximum(np.sqrt(gx * gx + gy * gy + gz * gz), F32(1e-30))
    a, b, cc = _sort3_abs(gx / gn, gy / gn, gz / gn)
    return cube_plane_fraction(c / gn, a, b, cc)


def closest_points(flat, idx, ny, nz, hi_x, hi_y, hi_z, h):
    """kernels.py:185-208."""
    h = F32(h)
    sx, sy = ny * nz, nz
    c = flat[idx]
    gx = 0.5 * (flat[idx + sx] - flat[idx - sx])
    gy = 0.5 * (flat[idx + sy] - flat[idx - sy])
    gz = 0.5 * (flat[idx + 1] - flat[idx - 1])
    g2 = np.maximum(gx * gx + gy * gy + gz * gz, F32(1e-30))
    length = np.abs(c) / np.sqrt(g2)
    cap = 1.25 * np.abs(c) / h + 0.25
    scale = (c / g2) * np.minimum(cap / np.maximum(length, F32(1e-30)), F32(1.0))
    i = (idx // sx).astype(F32)
    j = ((idx // sy) % ny).astype(F32)
    k = (idx % nz).astype(F32)
    px = np.minimum(np.maximum(i - scale * gx, F32(1.0)), F32(hi_x))
    py = np.minimum(np.maximum(j - scale * gy, F32(1.0)), F32(hi_y))
    pz = np.minimum(np.maximum(k - scale * gz, F32(1.0)), F32(hi_z))
    return np.stack([px, py, pz], 1)


def tricubic(flat, ny, nz, p):
    """kernels.py:212-228."""
    fl = np.floor(p)
    t = p - fl
    base = fl.astype(I64) - 1
    b0 = base[:, 0] * (ny * nz) + base[:, 1] * nz + base[:, 2]
    wx, wy, wz = _cubic_w(t[:, 0]), _cubic_w(t[:, 1]), _cubic_w(t[:, 2])
    out = np.zeros_like(t[:, 0])
    for a in range(4):
        for b in range(4):
            wab = wx[a] * wy[b]
            off = a * ny * nz + b * nz
            for c in range(4):
                out = out + (wab * wz[c]) * flat[b0 + (off + c)]
    return out


def tricubic_with_gradient(flat, ny, nz, p):
    """kernels.py:232-253."""
    fl = np.floor(p)
    t = p - fl
    base = fl.astype(I64) - 1
    b0 = base[:, 0] * (ny * nz) + base[:, 1] * nz + base[:, 2]
    wx, wy, wz = _cubic_w(t[:, 0]), _cubic_w(t[:, 1]), _cubic_w(t[:, 2])
    dx, dy, dz = _cubic_dw(t[:, 0]), _cubic_dw(t[:, 1]), _cubic_dw(t[:, 2])
    val = np.zeros_like(t[:, 0])
    gx, gy, gz = np.zeros_like(val), np.zeros_like(val), np.zeros_like(val)
    for a in range(4):
        for b in range(4):
            off = a * ny * nz + b * nz
            for c in range(4):
                v = flat[b0 + (off + c)]
                val = val + wx[a] * wy[b] * wz[c] * v
                gx = gx + dx[a] * wy[b] * wz[c] * v
                gy = gy + wx[a] * dy[b] * wz[c] * v
                gz = gz + wx[a] * wy[b] * dz[c] * v
    return val, np.stack([gx, gy, gz], 1)


def trilinear(flat, ny, nz, p):
    """kernels.py:257-270."""
    fl = np.floor(p)
    t = p - fl
    base = fl.astype(I64)
    b0 = base[:, 0] * (ny * nz) + base[:, 1] * nz + base[:, 2]
    out = np.zeros_like(t[:, 0])
    for a in range(2):
        wa = t[:, 0] if a else 1 - t[:, 0]
        for b in range(2):
            wb = wa * (t[:, 1] if b else 1 - t[:, 1])
            for c in range(2):
                out = out + wb * (t[:, 2] if c else 1 - t[:, 2]) * flat[b0 + (a * ny * nz + b * nz + c)]
    return out


def principal_curvatures(flat, idx, sx, sy, sz, h):
    """kernels.py:274-299."""
    h = F32(h)
    c = flat[idx]
    xp, xm = flat[idx + sx], flat[idx - sx]
    yp, ym = flat[idx + sy], flat[idx - sy]
    zp, zm = flat[idx + sz], flat[idx - sz]
    px, py, pz = (xp - xm) / (2 * h), (yp - ym) / (2 * h), (zp - zm) / (2 * h)
    pxx = (xp - 2 * c + xm) / (h * h)
    pyy = (yp - 2 * c + ym) / (h * h)
    pzz = (zp - 2 * c + zm) / (h * h)

    def mixed(a, b):
        return (flat[idx + a + b] - flat[idx + a - b] - flat[idx - a + b] + flat[idx - a - b]) / (4 * h * h)

    pxy, pxz, pyz = mixed(sx, sy), mixed(sx, sz), mixed(sy, sz)
    g2 = np.maximum(px * px + py * py + pz * pz, F32(1e-30))
    gn = np.sqrt(g2)
    ksum = ((pyy + pzz) * px * px + (pxx + pzz) * py * py + (pxx + pyy) * pz * pz
            - 2 * (px * py * pxy + px * pz * pxz + py * pz * pyz)) / (g2 * gn)
    K = (px * px * (pyy * pzz - pyz * pyz) + py * py * (pxx * pzz - pxz * pxz)
         + pz * pz * (pxx * pyy - pxy * pxy)
         + 2 * px * py * (pxz * pyz - pxy * pzz) + 2 * py * pz * (pxy * pxz - pyz * pxx)
         + 2 * px * pz * (pxy * pyz - pxz * pyy)) / (g2 * g2)
    H = 0.5 * ksum
    r = np.sqrt(np.maximum(H * H - K, F32(0)))
    return H + r, H - r


def interface_mask(flat, idx, sx, sy, sz):
    """kernels.py:303-309."""
    c = flat[idx]
    hit = np.zeros(c.shape, dtype=bool)
    for s in (sx, sy, sz):
        hit = hit | (flat[idx + s] * c <= 0) | (flat[idx - s] * c <= 0)
    return hit


def _interface_distance(p0, p1, dd, h):
    """kernels.py:312-331."""
    den = p0 - p1
    lin = h * p0 / np.where(den != 0, den, F32(1e-30))
    c2 = 0.5 * dd / (h * h)
    c1 = (p1 - p0) / h
    c0 = 0.5 * (p0 + p1) - c2 * h * h / 4
    disc = c1 * c1 - 4 * c2 * c0
    sq = np.sqrt(np.maximum(disc, F32(0)))
    q = -0.5 * (c1 + np.where(c1 >= 0, sq, -sq))
    xi = c0 / np.where(q != 0, q, F32(1e-30))
    quad = h / 2 + xi
    ok = (disc >= 0) & (np.abs(dd) > 1e-10 * h * h) & (quad >= 0) & (quad <= h)
    return np.minimum(np.maximum(np.where(ok, quad, lin), F32(0)), h)


def reinit_geometry(flat, idx, sx, sy, sz, h, cfl):
    """kernels.py:335-359: (sgn, dtau, cp_x, cm_x, xp_x, xm_x, ..., xm_z)."""
    h, cfl = F32(h), F32(cfl)
    c = flat[idx]
    sgn = np.sign(c)
    hmin = np.zeros_like(c) + h
    out = []
    for s in (sx, sy, sz):
        m2, m1, p1, p2 = flat[idx - 2 * s], flat[idx - s], flat[idx + s], flat[idx + 2 * s]
        d_m1 = c - 2 * m1 + m2
        d_0 = p1 - 2 * c + m1
        d_p1 = p2 - 2 * p1 + c
        cp = (c * p1) < 0
        cm = (c * m1) < 0
        xp = _interface_distance(c, p1, _minmod(d_0, d_p1), h)
        xm = _interface_distance(c, m1, _minmod(d_0, d_m1), h)
        hmin = np.minimum(hmin, np.where(cp, xp, hmin))
        hmin = np.minimum(hmin, np.where(cm, xm, hmin))
        out += [cp, cm, np.maximum(xp, 1e-6 * h), np.maximum(xm, 1e-6 * h)]
    dtau = cfl * np.maximum(hmin, 1e-3 * h)
    return (sgn, dtau, *out)


def reinit_rhs(flat, idx, sx, sy, sz, h, sgn, cpx, cmx, xpx, xmx, cpy, cmy, xpy, xmy, cpz, cmz, xpz, xmz):
    """kernels.py:363-379."""
    h = F32(h)
    c = flat[idx]
    g2 = np.zeros_like(c)
    outside = sgn > 0
    for s, cp, cm, xp, xm in ((sx, cpx, cmx, xpx, xmx), (sy, cpy, cmy, xpy, xmy), (sz, cpz, cmz, xpz, xmz)):
        m2, m1, p1, p2 = flat[idx - 2 * s], flat[idx - s], flat[idx + s], flat[idx + 2 * s]
        mm_p = _minmod(p1 - 2 * c + m1, p2 - 2 * p1 + c)
        mm_m = _minmod(p1 - 2 * c + m1, c - 2 * m1 + m2)
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            Dp = np.where(cp, -c / xp - 0.5 * xp * mm_p / (h * h), (p1 - c - 0.5 * mm_p) / h)
            Dm = np.where(cm, c / xm + 0.5 * xm * mm_m / (h * h), (c - m1 + 0.5 * mm_m) / h)
        pos = np.maximum(np.maximum(Dm, F32(0)) ** 2, np.minimum(Dp, F32(0)) ** 2)
        neg = np.maximum(np.minimum(Dm, F32(0)) ** 2, np.maximum(Dp, F32(0)) ** 2)
        g2 = g2 + np.where(outside, pos, neg)
    return -sgn * (np.sqrt(g2) - 1.0)


def point_triangle_distance2(p, a, b, c):
    """kernels.py:382-427 (Ericson region classification, float32)."""
    ab, ac = b - a, c - a
    ap, bp, cp = p - a, p - b, p - c
    d1 = (ab * ap).sum(-1)
    d2 = (ac * ap).sum(-1)
    d3 = (ab * bp).sum(-1)
    d4 = (ac * bp).sum(-1)
    d5 = (ab * cp).sum(-1)
    d6 = (ac * cp).sum(-1)
    va = d3 * d6 - d5 * d4
    vb = d5 * d2 - d1 * d6
    vc = d1 * d4 - d3 * d2
    tiny = F32(1e-30)
    denom = va + vb + vc
    denom = np.where(np.abs(denom) > tiny, denom, tiny)
    with np.errstate(divide="ignore", invalid="ignore"):
        v = vb / denom
        w = vc / denom
        e1 = d4 - d3
        e2 = d5 - d6
        in_bc = (va <= 0) & (e1 >= 0) & (e2 >= 0)
        wbc = e1 / np.maximum(e1 + e2, tiny)
        v = np.where(in_bc, 1 - wbc, v)
        w = np.where(in_bc, wbc, w)
        in_ac = (vb <= 0) & (d2 >= 0) & (d6 <= 0)
        wac = d2 / np.maximum(d2 - d6, tiny)
        v = np.where(in_ac, F32(0), v)
        w = np.where(in_ac, wac, w)
        in_c = (d6 >= 0) & (d5 <= d6)
        v = np.where(in_c, F32(0), v)
        w = np.where(in_c, F32(1), w)
        in_ab = (vc <= 0) & (d1 >= 0) & (d3 <= 0)
        vab = d1 / np.maximum(d1 - d3, tiny)
        v = np.where(in_ab, vab, v)
        w = np.where(in_ab, F32(0), w)
        in_b = (d3 >= 0) & (d4 <= d3)
        v = np.where(in_b, F32(1), v)
        w = np.where(in_b, F32(0), w)
        in_a = (d1 <= 0) & (d2 <= 0)
        v = np.where(in_a, F32(0), v)
        w = np.where(in_a, F32(0), w)
    q = a + v[..., None].astype(F32) * ab + w[..., None].astype(F32) * ac
    return ((p - q) ** 2).sum(-1).astype(F32)


# ------------------------------------------------------------- level set
def rebuild_band(phi_flat, width, h):
    """levelset.py:70-77 (in place clamp, returns sorted int64 band)."""
    cap = width * h
    np.clip(phi_flat, F32(-cap), F32(cap), out=phi_flat)
    return np.nonzero(np.abs(phi_flat) < F32(cap * (1 - 1e-5)))[0].astype(I64)


def check_margin(band, shape):
    """levelset.py:79-86."""
    if band.size == 0:
        return
    for ax, s in enumerate(strides_of(shape)):
        coord = (band // s) % shape[ax]
        if int(coord.min()) < MARGIN or int(coord.max()) > shape[ax] - 1 - MARGIN:
            raise RuntimeError("narrow band reaches the grid boundary; enlarge the padding")


def dense_fractions(phi_flat, band, shape):
    """levelset.py:117-121."""
    f = (phi_flat < 0).astype(F32)
    f[band] = cell_fractions(phi_flat, band, *strides_of(shape))
    return f


def band_volume(phi_flat, band, shape, h):
    """levelset.py:123-126."""
    outside_band_inside = int((phi_flat < 0).sum()) - int((phi_flat[band] < 0).sum())
    fr = cell_fractions(phi_flat, band, *strides_of(shape)).astype(np.float64)
    return (outside_band_inside + float(fr.sum())) * h ** 3


def dilate(mask, steps=1):
    """levelset.py:25-34."""
    out = mask.copy()
    for ax in range(3):
        n = out.shape[ax]
        for _ in range(steps):
            src = out.copy()
            sl = [slice(None)] * 3
            a, b = list(sl), list(sl)
            a[ax], b[ax] = slice(1, n), slice(0, n - 1)
            out[tuple(a)] |= src[tuple(b)]
            out[tuple(b)] |= src[tuple(a)]
    return out


def reinitialize(phi3, band, h, iterations=12, cfl=0.45, dilation=3, width=6.0):
    """levelset.py:154-183; returns the rebuilt band."""
    shape = phi3.shape
    mask = np.zeros(shape, dtype=bool)
    mask.reshape(-1)[band] = True
    mask = dilate(mask, dilation)
    for ax in range(3):
        n = mask.shape[ax]
        sl = [slice(None)] * 3
        sl[ax] = slice(0, MARGIN)
        mask[tuple(sl)] = False
        sl[ax] = slice(n - MARGIN, n)
        mask[tuple(sl)] = False
    idx = np.nonzero(mask.reshape(-1))[0].astype(I64)
    f = phi3.reshape(-1)
    st = strides_of(shape)
    geo = reinit_geometry(f, idx, *st, h, cfl)
    sgn, dtau, rest = geo[0], geo[1], geo[2:]
    for _ in range(iterations):
        u0 = f[idx].copy()
        f[idx] = u0 + dtau * reinit_rhs(f, idx, *st, h, sgn, *rest)
        u1 = f[idx].copy()
        f[idx] = 0.5 * (u0 + u1 + dtau * reinit_rhs(f, idx, *st, h, sgn, *rest))
    b = rebuild_band(f, width, h)
    check_margin(b, shape)
    return b


# ------------------------------------------------------------------ svi
def ball_cell_weights(radius, spacing, quad=32):
    """svi.py:24-55 (float64)."""
    R = radius / spacing
    m = int(math.floor(R + 0.5)) + 1
    ax = np.arange(-m, m + 1, dtype=np.float64)
    I, J, K = np.meshgrid(ax, ax, ax, indexing="ij")
    c = np.stack([I, J, K], -1)
    near = np.sqrt((np.maximum(np.abs(c) - 0.5, 0) ** 2).sum(-1))
    far = np.sqrt(((np.abs(c) + 0.5) ** 2).sum(-1))
    w = np.zeros(I.shape)
    w[far <= R] = 1.0
    cut = (near < R) & (far > R)
    g, gw = np.polynomial.legendre.leggauss(quad)
    g, gw = 0.5 * g, 0.5 * gw
    cc = c[cut]
    vols = np.empty(len(cc))
    for s in range(0, len(cc), 4096):
        cs = cc[s:s + 4096]
        X = cs[:, 0, None, None] + g[None, :, None]
        Y = cs[:, 1, None, None] + g[None, None, :]
        zr = np.sqrt(np.maximum(R * R - X * X - Y * Y, 0.0))
        lo = cs[:, 2, None, None] - 0.5
        hi = cs[:, 2, None, None] + 0.5
        L = np.maximum(np.minimum(hi, zr) - np.maximum(lo, -zr), 0.0)
        vols[s:s + 4096] = (L * gw[None, :, None] * gw[None, None, :]).sum((1, 2))
    w[cut] = vols
    return w


def kernel_hat(shape, radius, spacing, quad=32):
    """svi.py:66-81: rfftn of the float32 wrapped weights; returns (khat, m)."""
    w = ball_cell_weights(radius, spacing, quad)
    m = (w.shape[0] - 1) // 2
    if any(2 * m + 1 > n for n in shape):
        raise ValueError("ball kernel larger than the grid")
    kern = np.zeros(shape, dtype=F32)
    r = np.arange(-m, m + 1)
    ii, jj, kk = r % shape[0], r % shape[1], r % shape[2]
    kern[ii[:, None, None], jj[None, :, None], kk[None, None, :]] = w.astype(F32)
    return np.fft.rfftn(kern).astype(C64), m


def exterior_fraction(fractions3, khat, radius, spacing):
    """svi.py:84-93."""
    fh = np.fft.rfftn(fractions3.astype(F32)).astype(C64)
    fh *= khat
    g = np.fft.irfftn(fh, s=fractions3.shape, axes=(0, 1, 2)).astype(F32) * F32(spacing ** 3)
    ball_volume = 4.0 / 3.0 * math.pi * radius ** 3
    return (g * F32(-1.0 / ball_volume) + F32(1.0)).astype(F32)


# ----------------------------------------------------------------- laws
class SVILaw:
    """flows.py:51-108."""
    requires_svi, requires_curvature = True, False

    def __init__(self, radius, k=1, s=0, t=None, max_speed_ratio=100.0, eps=0.0):
        if radius <= 0:
            raise ValueError("radius must be positive")
        if int(k) != k or k < 0:
            raise ValueError("k must be a nonnegative integer")
        if s not in (0, 1):
            raise ValueError("s must be 0 or 1")
        if s == 1 and (t is None or not (0.5 < t < 1.0)):
            raise ValueError("s = 1 requires 1/2 < t < 1")
        if eps < 0:
            raise ValueError("eps must be >= 0")
        self.radius, self.k, self.s = float(radius), int(k), int(s)
        self.t = None if t is None else float(t)
        self.eps, self.max_speed_ratio = float(eps), float(max_speed_ratio)
        self.n_cap = 1.0
        if self.s == 1:
            target = self.max_speed_ratio * self._raw(0.5)
            lo, hi = 0.5, self.t
            for _ in range(200):
                mid = 0.5 * (lo + hi)
                if self._raw(mid) < target:
                    lo = mid
                else:
                    hi = mid
            self.n_cap = lo

    def _raw(self, n):
        v = n ** self.k
        if self.s:
            v /= (self.t - n)
        return v + self.eps

    def speed(self, N):
        N = np.clip(N, F32(0), F32(1))
        if self.s:
            N = np.minimum(N, F32(self.n_cap))
            V = N ** self.k / (F32(self.t) - N)
        else:
            V = N ** self.k if self.k else np.ones_like(N)
        return (V + F32(self.eps) if self.eps else V).astype(F32)

    def dspeed(self, N):
        N = np.clip(N, F32(1e-12), F32(1.0))
        if self.s:
            N = np.minimum(N, F32(self.n_cap))
            d = F32(self.t) - N
            V = N ** self.k / d
            return V * (self.k / N + 1.0 / d)
        if self.k == 0:
            return np.zeros_like(N)
        return self.k * N ** (self.k - 1)


class CurvatureLaw:
    """flows.py:111-206 (kind 'mean' or 'gauss')."""
    requires_svi, requires_curvature = False, True

    def __init__(self, kind, alpha=1.0, eps=0.0, delta=0.0):
        if alpha <= 0:
            raise ValueError("alpha must be positive")
        if delta < 0:
            raise ValueError("delta must be >= 0")
        self.kind, self.alpha, self.eps, self.delta = kind, float(alpha), float(eps), float(delta)
        if self.alpha < 1 and self.delta == 0:
            raise ValueError("alpha < 1 needs a regularisation delta > 0")

    def _power(self, x):
        if self.alpha == 1.0:
            return x
        if self.alpha < 1:
            return x * (x + F32(self.delta)) ** F32(self.alpha - 1)
        return x ** F32(self.alpha)

    def _dpower(self, x):
        a = self.alpha
        if a == 1.0:
            return np.ones_like(x)
        if a < 1:
            y = x + F32(self.delta)
            return y ** F32(a - 2) * (F32(a) * x + F32(self.delta))
        return F32(a) * np.maximum(x, F32(0)) ** F32(a - 1)

    def speed_and_diffusivity(self, k1, k2):
        if self.kind == "mean":
            H = 0.5 * (k1 + k2)
            Hp = np.maximum(H, F32(0))
            V = self._power(Hp) + F32(self.eps)
            D = np.where(H > 0, self._dpower(Hp), np.zeros_like(H))
            return V.astype(F32), D.astype(F32)
        a = np.maximum(k1, F32(0))
        b = np.maximum(k2, F32(0))
        Kc = a * b
        V = self._power(Kc) + F32(self.eps)
        dF = self._dpower(Kc)
        D = np.where(Kc > 0, dF * (a + b), dF * 0)
        return V.astype(F32), D.astype(F32)


def make_law(kind, radius=None, k=1, s=0, t=None, eps=0.0, max_speed_ratio=100.0, alpha=1.0, delta=None,
             length_scale=1.0):
    """api.py:54-66."""
    if kind == "svi":
        return SVILaw(radius, k, s, t, max_speed_ratio, eps)
    if kind in ("mean", "mean_curvature"):
        d = delta if delta is not None else (1.0 / length_scale if alpha < 1 else 0.0)
        return CurvatureLaw("mean", alpha, eps, d)
    if kind in ("gauss", "gauss_curvature"):
        d = delta if delta is not None else (length_scale ** -2 if alpha < 1 else 0.0)
        return CurvatureLaw("gauss", alpha, eps, d)
    raise ValueError(f"unknown law {kind!r}")


# ----------------------------------------------------------- simulation
@dataclass
class StepRecord:
    """evolve.py:43-55."""
    step: int
    time: float
    dt: float
    volume: float
    fraction: float
    vmax: float
    vmean: float
    qmin: float = float("nan")
    qmax: float = float("nan")
    capped: int = 0
    reinit: bool = False


class Simulation:
    """evolve.py:67-250 restated on a dense float32 numpy grid."""

    def __init__(self, phi3, h, law, width=6.0, cfl=0.5, feedback_cfl=1.0, parabolic_cfl=0.25,
                 reinit_distance=1.5, reinit_iterations=20, cutoff=(4.0, 5.5)):
        self.phi = np.ascontiguousarray(phi3, dtype=F32).copy()
        self.shape = self.phi.shape
        self.h, self.width, self.law = float(h), float(width), law
        self.cfl, self.feedback_cfl, self.parabolic_cfl = float(cfl), float(feedback_cfl), float(parabolic_cfl)
        self.reinit_distance, self.reinit_iterations = float(reinit_distance), int(reinit_iterations)
        self.cutoff = tuple(float(c) for c in cutoff)
        self.st = strides_of(self.shape)
        self.band = rebuild_band(self.flat, self.width, self.h)
        check_margin(self.band, self.shape)
        if law.requires_svi:
            self.khat, self.m = kernel_hat(self.shape, law.radius, self.h)
        self.initial_volume = self.volume()
        self.time, self.steps, self.history, self._displacement = 0.0, 0, [], 0.0
        self.band_updates = 0   # band nodes x accepted steps (the benchmark's work unit)

    @property
    def flat(self):
        return self.phi.reshape(-1)

    def volume(self):
        return band_volume(self.flat, self.band, self.shape, self.h)

    def svi_field(self):
        f = dense_fractions(self.flat, self.band, self.shape).reshape(self.shape)
        return exterior_fraction(f, self.khat, self.law.radius, self.h)

    def closest_points(self, idx):
        nx, ny, nz = self.shape
        return closest_points(self.flat, idx, ny, nz, nx - 3.001, ny - 3.001, nz - 3.001, self.h)

    def _cutoff_factor(self, phi_b):
        a, b = self.cutoff[0] * self.h, self.cutoff[1] * self.h
        x = np.abs(phi_b)
        t = np.clip((F32(b) - x) / F32(b - a), F32(0), F32(1))
        return t * t * (3 - 2 * t)

    def _velocity(self, stats=False):
        idx = self.band
        phi_b = self.flat[idx]
        cp = self.closest_points(idx)
        info = {}
        near = np.abs(phi_b) < F32(self.h)
        nx, ny, nz = self.shape
        if self.law.requires_svi:
            Nd = self.svi_field()
            N = tricubic(Nd.reshape(-1), ny, nz, cp)
            V = self.law.speed(N)
            if stats:
                Nn = N[near] if near.any() else N
                info["qmin"] = float(Nn.min())
                info["qmax"] = float(Nn.max())
                info["dvmax"] = float(self.law.dspeed(Nn).max())
                info["capped"] = int((Nn > F32(self.law.n_cap)).sum())
        else:
            k1, k2 = principal_curvatures(self.flat, idx, *self.st, self.h)
            dense = np.zeros(self.phi.size, dtype=F32)
            dense[idx] = k1
            k1c = trilinear(dense, ny, nz, cp)
            dense[idx] = k2
            k2c = trilinear(dense, ny, nz, cp)
            V, D = self.law.speed_and_diffusivity(k1c, k2c)
            if stats:
                sel = near if near.any() else np.ones_like(near)
                Hn = (0.5 * (k1c + k2c))[sel]
                info["qmin"] = float(Hn.min())
                info["qmax"] = float(Hn.max())
                info["dmax"] = float(D[sel].max())
        if stats:
            info["vmean"] = float(V[near].astype(np.float64).mean()) if near.any() else float(V.mean())
        V = V * self._cutoff_factor(phi_b)
        return V.astype(F32), info

    def _reinitialize(self):
        """levelset.py:154-183 on this level set; returns the rebuilt band."""
        return reinitialize(self.phi, self.band, self.h, self.reinit_iterations, width=self.width)

    def _rhs(self, stats=False):
        V, info = self._velocity(stats)
        G = godunov_inward(self.flat, self.band, *self.st, 1.0 / self.h)
        return V * G, V, info

    def stable_dt(self, V, info):
        h = self.h
        vmax = float(V.max()) if V.size else 0.0
        dt = self.cfl * h / vmax if vmax > 0 else math.inf
        if self.law.requires_svi and info.get("dvmax", 0) > 0:
            dt = min(dt, self.feedback_cfl * (4.0 * self.law.radius / 3.0) / info["dvmax"])
        if self.law.requires_curvature and info.get("dmax", 0) > 0:
            dt = min(dt, self.parabolic_cfl * h * h / info["dmax"])
        return dt

    def _rk3(self, u0, L0, dt):
        f, idx = self.flat, self.band
        dtf = F32(dt)
        f[idx] = u0 + dtf * L0
        L1, _, _ = self._rhs()
        f[idx] = 0.75 * u0 + 0.25 * (f[idx] + dtf * L1)
        L2, _, _ = self._rhs()
        f[idx] = u0 / F32(3.0) + F32(2.0 / 3.0) * (f[idx] + dtf * L2)

    def run(self, target_fraction=0.9, max_steps=100000, max_time=None, tol=1e-6):
        """evolve.py:182-250; returns (reason, steps, time, fraction)."""
        V0 = self.initial_volume
        target = None if target_fraction is None else target_fraction * V0
        vol = self.volume()
        reason = "max_steps"
        n_start = self.steps
        while self.steps - n_start < max_steps:
            if target is not None and vol <= target * (1 + tol):
                reason = "target_volume"
                break
            if max_time is not None and self.time >= max_time * (1 - 1e-12):
                reason = "max_time"
                break
            b = self.flat[self.band]
            if not ((b < 0).any() and (b > 0).any()):
                reason = "vanished"
                break
            idx = self.band
            u0 = self.flat[idx].copy()
            L0, Vb, info = self._rhs(stats=True)
            dt = self.stable_dt(Vb, info)
            if max_time is not None:
                dt = min(dt, max_time - self.time)
            if not math.isfinite(dt) or dt <= 0:
                reason = "stalled"
                break
            self._rk3(u0, L0, dt)
            vnew = self.volume()
            if target is not None and vnew < target:
                lo_t, lo_v, hi_t, hi_v = 0.0, vol, dt, vnew
                for _ in range(8):
                    if hi_v >= lo_v:
                        break
                    dts = lo_t + (target - lo_v) * (hi_t - lo_t) / (hi_v - lo_v)
                    self.flat[idx] = u0
                    self._rk3(u0, L0, dts)
                    v = self.volume()
                    if abs(v - target) <= tol * V0:
                        break
                    if v > target:
                        lo_t, lo_v = dts, v
                    else:
                        hi_t, hi_v = dts, v
                dt, vnew = dts, v
            vmax = float(Vb.max())
            self.time += dt
            self.steps += 1
            self.band_updates += idx.size
            self._displacement += dt * vmax
            did_reinit = False
            reached = target is not None and vnew <= target * (1 + tol)
            if self._displacement >= self.reinit_distance * self.h and not reached:
                self.band = self._reinitialize()
                self._displacement = 0.0
                did_reinit = True
                vnew = self.volume()
            self.history.append(StepRecord(self.steps, self.time, dt, vnew, vnew / V0, vmax,
                                           info.get("vmean", vmax), info.get("qmin", float("nan")),
                                           info.get("qmax", float("nan")), info.get("capped", 0), did_reinit))
            vol = vnew
        return reason, self.steps, self.time, vol / V0


# ------------------------------------------------------------------ SDF
def split_long_triangles(tri, max_edge):
    """sdf.py:54-70."""
    out = []
    while len(tri):
        e = np.stack([np.linalg.norm(tri[:, 1] - tri[:, 0], axis=1),
                      np.linalg.norm(tri[:, 2] - tri[:, 1], axis=1),
                      np.linalg.norm(tri[:, 0] - tri[:, 2], axis=1)], 1).max(1)
        small = e <= max_edge
        out.append(tri[small])
        big = tri[~small]
        if not len(big):
            break
        a, b, c = big[:, 0], big[:, 1], big[:, 2]
        ab, bc, ca = (a + b) / 2, (b + c) / 2, (c + a) / 2
        tri = np.concatenate([np.stack([a, ab, ca], 1), np.stack([ab, b, bc], 1),
                              np.stack([ca, bc, c], 1), np.stack([ab, bc, ca], 1)])
    return np.concatenate(out) if out else np.zeros((0, 3, 3))


def edge_topology(faces, nverts):
    """meshio.py:88-105."""
    e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
    ks = np.sort(e, axis=1)
    n = max(int(nverts), 1)
    keys = ks[:, 0] * n + ks[:, 1]
    uniq, inv, counts = np.unique(keys, return_inverse=True, return_counts=True)
    direction = np.where(e[:, 0] < e[:, 1], 1, -1)
    dir_sum = np.bincount(inv.reshape(-1), weights=direction, minlength=len(uniq))
    manifold = counts == 2
    return {"edges": int(len(uniq)), "boundary_edges": int(np.sum(counts == 1)),
            "nonmanifold_edges": int(np.sum(counts > 2)),
            "misoriented_edges": int(np.sum(manifold & (dir_sum != 0)))}


def _near_field(tri_idx, shape, exact_band, max_pairs=1 << 20):
    """sdf.py:100-145."""
    shape_a = np.asarray(shape)
    size = int(np.prod(shape))
    keys = np.full(size, KEY_EMPTY, dtype=np.int64)
    lo = np.clip(np.ceil(tri_idx.min(1) - exact_band).astype(np.int64), 0, shape_a - 1)
    hi = np.clip(np.floor(tri_idx.max(1) + exact_band).astype(np.int64), 0, shape_a - 1)
    dims = np.maximum(hi - lo + 1, 0)
    counts = dims.prod(1)
    tri32 = tri_idx.astype(F32)
    st = strides_of(shape)
    eb = F32(float(exact_band) * (1 + 1e-6))
    order = np.argsort(counts, kind="stable")
    csum = np.cumsum(counts[order])
    start = 0
    while start < len(order):
        base = csum[start - 1] if start else 0
        stop = max(int(np.searchsorted(csum, base + max_pairs, side="right")), start + 1)
        sel = order[start:stop]
        start = stop
        cnt = counts[sel]
        if int(cnt.sum()) == 0:
            continue
        local = np.repeat(np.arange(len(sel)), cnt)
        first = np.cumsum(cnt) - cnt
        q = np.arange(int(cnt.sum())) - first[local]
        d_l = dims[sel][local]
        nyz = d_l[:, 1] * d_l[:, 2]
        ii = lo[sel][local, 0] + q // nyz
        rem = q % nyz
        jj = lo[sel][local, 1] + rem // d_l[:, 2]
        kk = lo[sel][local, 2] + rem % d_l[:, 2]
        p = np.stack([ii, jj, kk], 1).astype(F32)
        t = tri32[sel[local]]
        d = np.sqrt(point_triangle_distance2(p, t[:, 0], t[:, 1], t[:, 2]))
        keep = d <= eb
        flat = (ii * st[0] + jj * st[1] + kk)[keep]
        key = (d[keep].view(np.int32).astype(np.int64) << 32) | sel[local][keep].astype(np.int64)
        np.minimum.at(keys, flat, key)
    return keys


def _dilate26(mask):
    """sdf.py:148-156."""
    return dilate(mask, 1)


_OFFSETS26 = [(i, j, k) for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1) if (i, j, k) != (0, 0, 0)]


def _unravel(u, shape):
    nx, ny, nz = shape
    return np.stack([u // (ny * nz), (u // nz) % ny, u % nz], 1)


def _propagate(dist, tid, tri32, shape, rings, chunk=1 << 22):
    """sdf.py:163-202."""
    known = (tid >= 0).reshape(shape)
    st = strides_of(shape)
    offs = [o[0] * st[0] + o[1] * st[1] + o[2] * st[2] for o in _OFFSETS26]
    n = dist.size
    prev = None
    for _ in range(rings):
        ring = _dilate26(known) & ~known
        for ax in range(3):
            sl = [slice(None)] * 3
            sl[ax] = slice(0, 1)
            ring[tuple(sl)] = False
            sl[ax] = slice(shape[ax] - 1, shape[ax])
            ring[tuple(sl)] = False
        upd = np.nonzero(ring.reshape(-1))[0]
        if prev is not None:
            upd = np.concatenate([upd, prev])
        if upd.size == 0:
            break
        for c0 in range(0, upd.size, chunk):
            u = upd[c0:c0 + chunk]
            p = _unravel(u, shape).astype(F32)
            best = dist[u].copy()
            best_t = tid[u].copy()
            for o in offs:
                nb = np.clip(u + o, 0, n - 1)
                t = tid[nb]
                ok = t >= 0
                if not ok.any():
                    continue
                tt = tri32[np.maximum(t, 0)]
                d = np.sqrt(point_triangle_distance2(p, tt[:, 0], tt[:, 1], tt[:, 2]))
                better = ok & (d < best)
                best = np.where(better, d, best)
                best_t = np.where(better, t, best_t)
            dist[u] = best
            tid[u] = best_t
        known |= ring
        prev = np.nonzero(ring.reshape(-1))[0]


def _refine_with_stars(dist, tid, tri32, tri_vid, shape, nodes, passes=2):
    """sdf.py:211-265."""
    flat_v = tri_vid.reshape(-1)
    order = np.argsort(flat_v, kind="stable")
    star = order // 3
    deg = np.bincount(flat_v, minlength=int(flat_v.max()) + 1)
    first = np.cumsum(deg) - deg
    for _ in range(passes):
        changed = 0
        u = nodes[tid[nodes] >= 0]
        if u.size == 0:
            break
        t = tid[u]
        v = tri_vid[t].reshape(-1)
        d = deg[v]
        pair_node = np.repeat(np.repeat(np.arange(u.size), 3), d)
        start = np.repeat(first[v], d)
        offs = np.arange(int(d.sum())) - np.repeat(np.cumsum(d) - d, d)
        cand = star[start + offs]
        p = _unravel(u, shape).astype(F32)[pair_node]
        tt = tri32[cand]
        dd = np.sqrt(point_triangle_distance2(p, tt[:, 0], tt[:, 1], tt[:, 2]))
        key = (dd.view(np.int32).astype(np.int64) << 32) | cand.astype(np.int64)
        best = np.full(u.size, KEY_EMPTY, dtype=np.int64)
        np.minimum.at(best, pair_node, key)
        bd = (best >> 32).astype(np.int32).view(F32)
        bt = best & 0xFFFFFFFF
        better = bd < dist[u]
        changed += int(better.sum())
        dist[u[better]] = bd[better]
        tid[u[better]] = bt[better]
        if changed == 0:
            break


def _orient_sos(x1, y1, x2, y2):
    """sdf.py:269-282."""
    a = x1 * y2 - y1 * x2
    s = np.sign(a).astype(np.int8)
    zero = s == 0
    if zero.any():
        tie = np.where(y2 > y1, -1, np.where(y2 < y1, 1, np.where(x1 > x2, -1, np.where(x1 < x2, 1, 0)))).astype(np.int8)
        s = np.where(zero, tie, s)
    return s, a


def _crossings_along_axis(tri_idx, shape, axis, signed):
    """sdf.py:285-340."""
    a, b, c = axis, (axis + 1) % 3, (axis + 2) % 3
    na, nb, nc = shape[a], shape[b], shape[c]
    U, W, Z = tri_idx[:, :, b], tri_idx[:, :, c], tri_idx[:, :, a]
    j0 = np.clip(np.ceil(U.min(1)), 0, nb).astype(np.int64)
    j1 = np.clip(np.floor(U.max(1)), -1, nb - 1).astype(np.int64)
    k0 = np.clip(np.ceil(W.min(1)), 0, nc).astype(np.int64)
    k1 = np.clip(np.floor(W.max(1)), -1, nc - 1).astype(np.int64)
    dj = np.maximum(j1 - j0 + 1, 0)
    dk = np.maximum(k1 - k0 + 1, 0)
    cnt = dj * dk
    t = np.nonzero(cnt)[0]
    acc = np.zeros((na + 1) * nb * nc, dtype=np.int64)
    if len(t):
        n_t = cnt[t]
        rep = np.repeat(np.arange(len(t)), n_t)
        q = np.arange(int(n_t.sum())) - np.repeat(np.cumsum(n_t) - n_t, n_t)
        jj = j0[t][rep] + q // dk[t][rep]
        kk = k0[t][rep] + q % dk[t][rep]
        tt = t[rep]
        x1, x2, x3 = U[tt, 0] - jj, U[tt, 1] - jj, U[tt, 2] - jj
        y1, y2, y3 = W[tt, 0] - kk, W[tt, 1] - kk, W[tt, 2] - kk
        sa, A = _orient_sos(x2, y2, x3, y3)
        sb, B = _orient_sos(x3, y3, x1, y1)
        sc, C = _orient_sos(x1, y1, x2, y2)
        hit = (sa != 0) & (sb == sa) & (sc == sa)
        A, B, C, sa = A[hit], B[hit], C[hit], sa[hit]
        tt, jj, kk = tt[hit], jj[hit], kk[hit]
        S = A + B + C
        good = S != 0
        z = (A * Z[tt, 0] + B * Z[tt, 1] + C * Z[tt, 2])[good] / S[good]
        i0 = np.clip(np.floor(z).astype(np.int64) + 1, 0, na)
        flat = (i0 * nb + jj[good]) * nc + kk[good]
        w = -sa[good].astype(np.int64) if signed else np.ones(len(flat), dtype=np.int64)
        np.add.at(acc, flat, w)
    acc = acc.reshape(na + 1, nb, nc)
    cs = np.cumsum(acc, axis=0)[:na]
    inside = (cs != 0) if signed else ((cs & 1) != 0)
    inv = np.argsort([a, b, c])
    return np.ascontiguousarray(np.transpose(inside, inv))


def inside_mask(vertices, faces, origin, spacing, shape, axes=None, signed=None):
    """sdf.py:343-361."""
    topo = edge_topology(faces, len(vertices))
    closed = topo["boundary_edges"] == 0 and topo["nonmanifold_edges"] == 0
    if signed is None:
        signed = topo["misoriented_edges"] == 0
    if axes is None:
        axes = (0,) if closed else (0, 1, 2)
    tri_idx = (vertices[faces] - np.asarray(origin)) / spacing
    votes = None
    for ax in axes:
        m = _crossings_along_axis(tri_idx, shape, ax, signed).astype(np.uint8)
        votes = m if votes is None else votes + m
    return votes * 2 > len(axes)


def mesh_to_sdf(vertices, faces, origin, spacing, shape, band=6.0, exact_band=2.0, sign_axes=None):
    """sdf.py:365-415 (returns the dense float32 grid)."""
    h = spacing
    tri_idx = (vertices[faces] - np.asarray(origin)) / h
    tri_split = split_long_triangles(tri_idx, max_edge=8.0)
    keys = _near_field(tri_split, shape, exact_band)
    found = keys != KEY_EMPTY
    dist = np.where(found, (keys >> 32).astype(np.int32).view(F32), F32(np.inf)).astype(F32)
    tid = np.where(found, keys & 0xFFFFFFFF, -1).astype(np.int64)
    tri32 = tri_split.astype(F32)
    rings = max(int(math.ceil(band - exact_band)) + 1, 0)
    _propagate(dist, tid, tri32, shape, rings)
    if len(tri_split) == len(faces):
        _, inv = np.unique(vertices, axis=0, return_inverse=True)
        tri_vid = inv.reshape(-1)[faces]
    else:
        _, inv = np.unique(tri_split.reshape(-1, 3), axis=0, return_inverse=True)
        tri_vid = inv.reshape(-1)[: 3 * len(tri_split)].reshape(-1, 3)
    outer = np.nonzero((dist > exact_band) & (dist <= band + 1.0))[0]
    _refine_with_stars(dist, tid, tri32, tri_vid, shape, outer)
    inside = inside_mask(vertices, faces, origin, spacing, shape, axes=sign_axes).reshape(-1)
    d = np.minimum(dist, F32(band)) * F32(h)
    return np.where(inside, -d, d).reshape(shape).astype(F32)
