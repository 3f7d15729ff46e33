"""Zero-level-set extraction as a triangle mesh (reference svierosion/surface.py).

Marching cubes over the band cells on the GPU (csrc/surface.cu; the case table
is generated from the method's definition), one limited Newton step of every
vertex on the tricubic interpolant of phi, and orientation by the signed
volume.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _native as nat
from .grid import Grid
from .levelset import LevelSet, tricubic
from .meshio import TriMesh


def extract_surface(ls: LevelSet, project: bool = True, max_shift: float = 0.5) -> TriMesh:
    """Marching cubes on the band, followed by an optional Newton projection (surface.py:16-56)."""
    grid = ls.grid
    band = ls.band32
    if band.numel() == 0 or not ls.has_interface():
        return TriMesh(np.zeros((0, 3)), np.zeros((0, 3), dtype=np.int64))
    nx, ny, nz = grid.shape
    m = band.numel()
    sc = ls.scratch
    lib = nat.lib()
    ws = sc.get("surface", lib.svie_surface_workspace_bytes(m))
    totals = sc.get("surface_totals", 16)
    nat.call("svie_surface_scan", nat.ptr(ls.flat), nat.ptr(band), m, nx, ny, nz, nat.ptr(ws), ws.numel(),
             nat.ptr(totals), nat.stream())
    nv, nt = (int(v) for v in totals[:16].cpu().view(torch.int64))
    vinfo = sc.get("surface_vinfo", 4 * grid.size)
    verts = torch.empty((nv, 3), dtype=torch.float32, device=ls.device)
    faces = torch.empty((nt, 3), dtype=torch.int32, device=ls.device)
    nat.call("svie_surface_write", nat.ptr(ls.flat), nat.ptr(band), m, nx, ny, nz, nat.ptr(ws), ws.numel(),
             nat.ptr(vinfo), nat.ptr(verts), nv, nat.ptr(faces), nt, nat.stream())
    if project and nv:
        nat.call("svie_surface_project", nat.ptr(ls.flat), ny, nz, nat.ptr(verts), nv, float(max_shift),
                 nat.stream())
    # orientation test on the device; world coordinates (float64) on the host
    vol = torch.empty(1, dtype=torch.float64, device=ls.device)
    centre = [0.5 * (n - 1) for n in grid.shape]
    nat.call("svie_surface_signed_volume", nat.ptr(verts), nat.ptr(faces), nt, *centre, nat.ptr(vol), nat.stream())
    v = nat.d2h(verts).astype(np.float64)
    f = nat.d2h(faces).astype(np.int64)
    if len(f) and f.min() < 0:
        raise RuntimeError("surface extraction met a crossing outside the band (phi is not distance-like)")
    if float(vol.item()) < 0:
        f = f[:, ::-1].copy()
    return TriMesh(np.asarray(grid.origin) + grid.spacing * v, f)


def sample_field(field: torch.Tensor, grid: Grid, points_world: np.ndarray) -> np.ndarray:
    """Tricubic interpolation of a dense grid field at world coordinates (surface.py:59-67)."""
    if len(points_world) == 0:
        return np.zeros(0)
    p = torch.as_tensor(grid.to_index(points_world), dtype=torch.float32, device=field.device)
    out = []
    for s in range(0, len(p), 1 << 20):
        out.append(tricubic(field.reshape(-1), grid.shape, p[s:s + (1 << 20)]))
    return torch.cat(out).double().cpu().numpy()
