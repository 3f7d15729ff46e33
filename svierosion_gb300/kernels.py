"""Numerical kernels on flattened grids (reference svierosion/kernels.py).

Same names and argument orders as the reference's compiled kernels; each one is
a hand-written sm_103a CUDA kernel in libsvie.so.  ``flat`` is the C-ordered
flattened float32 grid on a CUDA device, ``idx`` flat node indices (int64 or
int32), ``(sx, sy, sz)`` the axis strides, points ``p`` in index coordinates.
There is no torch.compile here, so ``set_compile`` / ``compile_enabled`` only
keep the reference's switches callable.
"""

from __future__ import annotations

import torch

from . import _native as nat

_COMPILE = True


def set_compile(flag: bool) -> None:
    """Kept for API compatibility (kernels.py:26-29): the kernels are native."""
    global _COMPILE
    _COMPILE = bool(flag)


def compile_enabled() -> bool:
    return _COMPILE


class Kernel:
    """The reference's compile wrapper (kernels.py:35-66), kept for callers that
    decorate their own torch functions with ``kernel``: here the function runs
    as written, because nothing in this package is compiled at run time."""

    def __init__(self, fn):
        self.fn = fn
        self.__doc__ = fn.__doc__
        self.__name__ = fn.__name__

    def __call__(self, *args):
        return self.fn(*args)


def kernel(fn) -> Kernel:
    """Decorator form of Kernel (kernels.py:77-78)."""
    return Kernel(fn)


def _flat(flat: torch.Tensor) -> torch.Tensor:
    if flat.dtype != torch.float32 or not flat.is_contiguous():
        raise ValueError("flat must be a contiguous float32 tensor")
    nat.ptr(flat)
    return flat


def _i32(idx: torch.Tensor) -> torch.Tensor:
    if idx.dtype == torch.int32 and idx.is_contiguous():
        return idx
    return idx.to(torch.int32).contiguous()


def _pts(p: torch.Tensor) -> torch.Tensor:
    p = p.to(torch.float32).contiguous()
    if p.ndim != 2 or p.shape[1] != 3:
        raise ValueError("points must have shape (m, 3)")
    return p


def godunov_inward(flat, idx, sx, sy, sz, inv_h):
    """Godunov |grad phi| for inward motion with WENO5 derivatives (kernels.py:146-169)."""
    i = _i32(idx)
    out = torch.empty(i.numel(), dtype=torch.float32, device=flat.device)
    nat.call("svie_godunov_inward", nat.ptr(_flat(flat)), nat.ptr(i), i.numel(), int(sx), int(sy), int(sz),
             float(inv_h), nat.ptr(out), nat.stream())
    return out


def cell_fractions(flat, idx, sx, sy, sz):
    """Cell volume fraction below the tangent plane (kernels.py:173-181)."""
    i = _i32(idx)
    out = torch.empty(i.numel(), dtype=torch.float32, device=flat.device)
    nat.call("svie_cell_fractions", nat.ptr(_flat(flat)), nat.ptr(i), i.numel(), int(sx), int(sy), int(sz),
             nat.ptr(out), nat.stream())
    return out


def closest_points(flat, idx, ny, nz, hi_x, hi_y, hi_z, h):
    """First Newton projection to the zero set, (m, 3) (kernels.py:185-208)."""
    i = _i32(idx)
    out = torch.empty((i.numel(), 3), dtype=torch.float32, device=flat.device)
    nat.call("svie_closest_points", nat.ptr(_flat(flat)), nat.ptr(i), i.numel(), int(ny), int(nz), float(hi_x),
             float(hi_y), float(hi_z), float(h), nat.ptr(out), nat.stream())
    return out


def tricubic(flat, ny, nz, p):
    """Tricubic Lagrange interpolation at index coordinates (kernels.py:212-228)."""
    p = _pts(p)
    out = torch.empty(p.shape[0], dtype=torch.float32, device=flat.device)
    nat.call("svie_tricubic", nat.ptr(_flat(flat)), int(ny), int(nz), nat.ptr(p), p.shape[0], nat.ptr(out),
             nat.stream())
    return out


def tricubic_with_gradient(flat, ny, nz, p):
    """Tricubic value and gradient (kernels.py:232-253)."""
    p = _pts(p)
    val = torch.empty(p.shape[0], dtype=torch.float32, device=flat.device)
    grad = torch.empty((p.shape[0], 3), dtype=torch.float32, device=flat.device)
    nat.call("svie_tricubic_with_gradient", nat.ptr(_flat(flat)), int(ny), int(nz), nat.ptr(p), p.shape[0],
             nat.ptr(val), nat.ptr(grad), nat.stream())
    return val, grad


def trilinear(flat, ny, nz, p):
    """Trilinear interpolation (kernels.py:257-270)."""
    p = _pts(p)
    out = torch.empty(p.shape[0], dtype=torch.float32, device=flat.device)
    nat.call("svie_trilinear", nat.ptr(_flat(flat)), int(ny), int(nz), nat.ptr(p), p.shape[0], nat.ptr(out),
             nat.stream())
    return out


def principal_curvatures(flat, idx, sx, sy, sz, h):
    """Principal curvatures k1 >= k2 (kernels.py:274-299)."""
    i = _i32(idx)
    k1 = torch.empty(i.numel(), dtype=torch.float32, device=flat.device)
    k2 = torch.empty_like(k1)
    nat.call("svie_principal_curvatures", nat.ptr(_flat(flat)), nat.ptr(i), i.numel(), int(sx), int(sy), int(sz),
             float(h), nat.ptr(k1), nat.ptr(k2), nat.stream())
    return k1, k2


def interface_mask(flat, idx, sx, sy, sz):
    """Nodes with a 6-neighbour of opposite (or zero) sign (kernels.py:303-309)."""
    i = _i32(idx)
    out = torch.empty(i.numel(), dtype=torch.uint8, device=flat.device)
    nat.call("svie_interface_mask", nat.ptr(_flat(flat)), nat.ptr(i), i.numel(), int(sx), int(sy), int(sz),
             nat.ptr(out), nat.stream())
    return out.view(torch.bool)


def reinit_geometry(flat, idx, sx, sy, sz, h, cfl):
    """Per-axis crossings and subcell distances (kernels.py:335-359).

    Returns (sgn, dtau, cp_x, cm_x, xp_x, xm_x, cp_y, ..., xm_z) like the
    reference; the packed device form the fused reinitialisation uses rides
    along as ``.packed``."""
    i = _i32(idx)
    m = i.numel()
    f = _flat(flat)
    geo = torch.empty(nat.lib().svie_reinit_geometry_bytes(m), dtype=torch.uint8, device=flat.device)
    nat.call("svie_reinit_geometry", nat.ptr(f), nat.ptr(i), m, int(sx), int(sy), int(sz), float(h),
             float(cfl), nat.ptr(geo), nat.stream())
    sgn = torch.empty(m, dtype=torch.float32, device=flat.device)
    dtau = torch.empty_like(sgn)
    flags = torch.empty((6, m), dtype=torch.uint8, device=flat.device)
    dist = torch.empty((6, m), dtype=torch.float32, device=flat.device)
    nat.call("svie_reinit_geometry_arrays", nat.ptr(f), nat.ptr(i), m, int(sx), int(sy), int(sz), float(h),
             float(cfl), nat.ptr(sgn), nat.ptr(dtau), nat.ptr(flags), nat.ptr(dist), nat.stream())
    fl = flags.view(torch.bool)
    out = [sgn, dtau]
    for a in range(3):
        out += [fl[2 * a], fl[2 * a + 1], dist[2 * a], dist[2 * a + 1]]
    out = tuple(out)
    return _GeoTuple(out, geo)


class _GeoTuple(tuple):
    """Tuple of the 14 reinit_geometry arrays that also carries the packed
    device form for reinit_rhs."""

    def __new__(cls, items, packed):
        obj = super().__new__(cls, items)
        obj.packed = packed
        return obj


def reinit_rhs(flat, idx, sx, sy, sz, h, sgn, cpx, cmx, xpx, xmx, cpy, cmy, xpy, xmy, cpz, cmz, xpz, xmz):
    """-sgn(phi0) (|grad phi| - 1) with ENO2 + subcell fix (kernels.py:363-379)."""
    i = _i32(idx)
    m = i.numel()
    geo = _pack_geometry(sgn, (cpx, cmx, cpy, cmy, cpz, cmz), (xpx, xmx, xpy, xmy, xpz, xmz), m, flat.device)
    out = torch.empty(m, dtype=torch.float32, device=flat.device)
    nat.call("svie_reinit_rhs", nat.ptr(_flat(flat)), nat.ptr(i), m, int(sx), int(sy), int(sz), float(h),
             nat.ptr(geo), nat.ptr(out), nat.stream())
    return out


def _pack_geometry(sgn, flags6, dist6, m, device):
    """The packed device form of svie_reinit_geometry from the reference's arrays."""
    geo = torch.empty(nat.lib().svie_reinit_geometry_bytes(m), dtype=torch.uint8, device=device)
    s = sgn.to(torch.float32).contiguous()
    fl = torch.stack([f.to(torch.uint8) for f in flags6]).contiguous()
    di = torch.stack([d.to(torch.float32) for d in dist6]).contiguous()
    nat.call("svie_reinit_geometry_pack", nat.ptr(s), None, nat.ptr(fl), nat.ptr(di), m, nat.ptr(geo),
             nat.stream())
    return geo


def point_triangle_distance2(p, a, b, c):
    """Squared point-triangle distance, Ericson regions (kernels.py:382-427).
    Inputs broadcast to (m, 3)."""
    p, a, b, c = torch.broadcast_tensors(p, a, b, c)
    shape = p.shape[:-1]
    flat = [x.reshape(-1, 3).to(torch.float32).contiguous() for x in (p, a, b, c)]
    m = flat[0].shape[0]
    out = torch.empty(m, dtype=torch.float32, device=flat[0].device)
    nat.call("svie_point_triangle_distance2", *(nat.ptr(x) for x in flat), m, nat.ptr(out), nat.stream())
    return out.reshape(shape)


point_triangle_distance2_compiled = point_triangle_distance2
_point_triangle_distance2 = point_triangle_distance2


def cube_plane_fraction(s, a, b, c):
    """Cube volume fraction below a plane (kernels.py:104-122)."""
    s, a, b, c = (x.to(torch.float32).contiguous() for x in torch.broadcast_tensors(s, a, b, c))
    out = torch.empty_like(s)
    nat.call("svie_cube_plane_fraction", nat.ptr(s), nat.ptr(a), nat.ptr(b), nat.ptr(c), s.numel(), nat.ptr(out),
             nat.stream())
    return out
