"""Compact forms of full-size results, shared by tests/golden/make_config_golden.py and the tests.

A grid of 13-37M nodes does not fit a fixture, so the fixtures of the precision and scan
configurations keep: sha256 digests, packed inside bits (phi < 0), seeded samples, and the zero level
set as a "shell" -- the field's inside bits plus its values, quantised to h/64 as int8, at the corners of
every cell whose corners are not all on one side (the only values marching cubes reads).  The
surface distance here is test infrastructure: vertex-to-surface distances between two marching-cubes
meshes of the oracle's extraction (oracle/marching.py).
"""

from __future__ import annotations

import hashlib

import numpy as np

SAMPLES = 40000
# the four laws of the precision configuration (fragment subdivided 6x, resolution 256, r = 0.08 L)
PRECISION_LAWS = {
    "svi_k0s0": dict(law="svi", k=0, s=0, target=0.9),
    "svi_k1s1": dict(law="svi", k=1, s=1, t=0.93, target=0.9),
    "svi_k2s1": dict(law="svi", k=2, s=1, t=0.95, target=0.9),
    "mean_a1": dict(law="mean", alpha=1.0, target=0.9, max_steps=40),
}


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def mesh_digest(vertices: np.ndarray, faces: np.ndarray) -> str:
    return digest(np.asarray(vertices, dtype=np.float64)) + digest(np.asarray(faces, dtype=np.int64))


def shell_nodes(inside: np.ndarray) -> np.ndarray:
    """Ascending flat indices of the corners of the cells whose 8 corners are not all inside or all
    outside (inside: bool grid)."""
    a = inside
    lo = a[:-1, :-1, :-1]
    mixed = np.zeros(lo.shape, dtype=bool)
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                mixed |= a[dx:a.shape[0] - 1 + dx, dy:a.shape[1] - 1 + dy, dz:a.shape[2] - 1 + dz] != lo
    corner = np.zeros(a.shape, dtype=bool)
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                corner[dx:a.shape[0] - 1 + dx, dy:a.shape[1] - 1 + dy, dz:a.shape[2] - 1 + dz] |= mixed
    return np.flatnonzero(corner.reshape(-1))


def shell_encode(phi3: np.ndarray, h: float) -> dict:
    inside = phi3 < 0
    nodes = shell_nodes(inside)
    q = np.clip(np.rint(phi3.reshape(-1)[nodes] / h * 64.0), -127, 127).astype(np.int8)
    return {"shell_inside": np.packbits(inside.reshape(-1)), "shell_q": q}


def shell_decode(d: dict, prefix: str, shape, h: float, far: float) -> np.ndarray:
    """The field the shell describes: the stored values at the shell nodes (their sign taken from the
    inside bits), -far / +far elsewhere."""
    n = int(np.prod(shape))
    inside = np.unpackbits(d[prefix + "shell_inside"], count=n).astype(bool)
    nodes = shell_nodes(inside.reshape(shape))
    phi = np.where(inside, -far, far).astype(np.float32)
    v = d[prefix + "shell_q"].astype(np.float32) * np.float32(h / 64.0)
    tiny = np.float32(h / 4096.0)
    ins = inside[nodes]
    phi[nodes] = np.where(ins, np.minimum(v, -tiny), np.maximum(v, 0.0))
    return phi.reshape(shape)


def sample_of(n: int, k: int, seed: int) -> np.ndarray:
    """k sorted positions of range(n), seeded."""
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n, size=min(k, n), replace=False))


def _to_surface(pts, verts, faces, k=16):
    """Distance from each point to the mesh (verts, faces), exact over the k triangles with the
    nearest centroids: an upper bound of the true distance, equal to it wherever the nearest
    triangle is among those k."""
    from scipy.spatial import cKDTree

    from oracle.reference_np import point_triangle_distance2

    tri = verts[faces].astype(np.float64)
    _, cand = cKDTree(tri.mean(1)).query(pts, k=min(k, len(tri)))
    cand = cand.reshape(len(pts), -1)
    best = np.full(len(pts), np.inf)
    for j in range(cand.shape[1]):
        t = tri[cand[:, j]]
        best = np.minimum(best, point_triangle_distance2(pts, t[:, 0], t[:, 1], t[:, 2]))
    return np.sqrt(best)


def surface_of(phi3: np.ndarray):
    """Marching-cubes vertices (index coordinates, float64) and faces of the zero set of phi3, over
    the cells whose lower corner is a shell node."""
    from oracle import marching as M

    nodes = shell_nodes(phi3 < 0).astype(np.int64)
    v, f = M.extract(np.ascontiguousarray(phi3, dtype=np.float32), nodes)
    return v.astype(np.float64), f


def hausdorff_cells(phi_a: np.ndarray, phi_b: np.ndarray) -> float:
    """Symmetric Hausdorff distance, in grid cells, between the zero sets of two fields on one grid
    (vertex-to-surface distances both ways; an upper bound, see _to_surface)."""
    va, fa = surface_of(phi_a)
    vb, fb = surface_of(phi_b)
    if len(fa) == 0 or len(fb) == 0:
        return 0.0 if len(fa) == len(fb) else float("inf")
    return float(max(_to_surface(va, vb, fb).max(), _to_surface(vb, va, fa).max()))
