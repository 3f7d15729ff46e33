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
    return extract_surface_device(ls, project, max_shift)[0]


def extract_surface_device(ls: LevelSet, project: bool = True, max_shift: float = 0.5):
    """extract_surface, also returning the float64 world vertices (n, 3) still on the device
    (None for an empty surface), for per-vertex sampling without another upload.

    The host mesh is assembled on the device: world coordinates origin + h * v in float64,
    int64 faces reversed when the signed volume is negative, and a count of faces that met a
    crossing outside the band."""
    grid = ls.grid
    band = ls.band32
    if band.numel() == 0 or not ls.has_interface():
        return TriMesh(np.zeros((0, 3)), np.zeros((0, 3), dtype=np.int64)), None
    nx, ny, nz = grid.shape
    m = band.numel()
    sc = ls.scratch
    lib = nat.lib()
    ws = sc.get("surface", lib.svie_surface_workspace_bytes(m))
    totals = sc.get("surface_totals", 16)
    nat.call("svie_surface_scan", nat.ptr(ls.flat), nat.ptr(band), m, nx, ny, nz, nat.ptr(ws), ws.numel(),
             nat.ptr(totals), nat.stream())
    nv, nt = (int(v) for v in totals[:16].cpu().view(torch.int64))
    # a grid-sized int32 scratch: the buffer of the reinitialisation's grid copy, which is
    # rewritten in full by every reinitialisation and holds nothing between calls
    vinfo = sc.get("reinit_phi", 4 * grid.size)
    verts = torch.empty((nv, 3), dtype=torch.float32, device=ls.device)
    faces = torch.empty((nt, 3), dtype=torch.int32, device=ls.device)
    nat.call("svie_surface_write", nat.ptr(ls.flat), nat.ptr(band), m, nx, ny, nz, nat.ptr(ws), ws.numel(),
             nat.ptr(vinfo), nat.ptr(verts), nv, nat.ptr(faces), nt, nat.stream())
    if project and nv:
        nat.call("svie_surface_project", nat.ptr(ls.flat), ny, nz, nat.ptr(verts), nv, float(max_shift),
                 nat.stream())
    # orientation test and the host arrays, on the device
    vol = sc.get("surface_volume", 8)
    centre = [0.5 * (n - 1) for n in grid.shape]
    nat.call("svie_surface_signed_volume", nat.ptr(verts), nat.ptr(faces), nt, *centre, nat.ptr(vol), nat.stream())
    world = torch.empty((nv, 3), dtype=torch.float64, device=ls.device)
    faces64 = torch.empty((nt, 3), dtype=torch.int64, device=ls.device)
    bad = sc.get("surface_bad", 4)
    nat.call("svie_surface_finish", nat.ptr(verts), nv, nat.ptr(faces), nt, nat.ptr(vol), *grid.origin,
             float(grid.spacing), nat.ptr(world), nat.ptr(faces64), nat.ptr(bad), nat.stream())
    v = nat.d2h(world)
    f = nat.d2h(faces64)
    if int(bad[:4].cpu().view(torch.int32)[0]):
        raise RuntimeError("surface extraction met a crossing outside the band (phi is not distance-like)")
    return TriMesh(v, f), world


def sample_field_device(field: torch.Tensor, grid: Grid, points_world) -> torch.Tensor:
    """Tricubic interpolation of a dense grid field at world coordinates (surface.py:59-67), as a
    float32 tensor on the field's device.

    `points_world` is a host array or a float64 device tensor (n, 3); either way the index
    coordinates are (p - origin) / h in float64, rounded to float32."""
    if len(points_world) == 0:
        return torch.zeros(0, dtype=torch.float32, device=field.device)
    if isinstance(points_world, torch.Tensor):
        n = points_world.shape[0]
        p = torch.empty((n, 3), dtype=torch.float32, device=field.device)
        nat.call("svie_points_f32", nat.ptr(points_world), n, *grid.origin, float(grid.spacing), nat.ptr(p),
                 nat.stream())
    else:
        p = torch.as_tensor(grid.to_index(points_world), dtype=torch.float32, device=field.device)
    return tricubic(field.reshape(-1), grid.shape, p)


def sample_field(field: torch.Tensor, grid: Grid, points_world) -> np.ndarray:
    """sample_field_device read back as a float64 host array."""
    if len(points_world) == 0:
        return np.zeros(0)
    return nat.d2h(sample_field_device(field, grid, points_world)).astype(np.float64)
