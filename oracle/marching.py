"""Marching cubes on the narrow band (test infrastructure only): the restatement the GPU surface
extraction (svierosion_gb300/csrc/surface.cu) is checked against.

The reference extracts the zero level set with scikit-image's marching cubes (Lewiner et al.) on
the band, then moves every vertex by one limited Newton step on the tricubic interpolant and
orients the mesh by its signed volume (svierosion/surface.py:16-56).  scikit-image is not part of
this project, so its case table is not used: the triangulation table below is generated from the
definition of the method (Lorensen and Cline 1987).  For each of the 256 inside/outside patterns of
a cell's corners (inside = phi < 0), the zero set crosses every cell edge whose ends differ; on
each cell face the crossings are joined in pairs, and on a face with four crossings (an ambiguous
face) the pairs cut off the two inside corners, a choice made from the face alone, so two cells
sharing a face agree and the mesh is closed.  The face segments form closed loops, and each loop is
fanned into triangles oriented from the inside to the outside.  Vertices sit on grid edges at the
linear-interpolation crossing, one vertex per crossed edge (owned by the edge's lower node), so
neighbouring cells share them.
"""

from __future__ import annotations

import numpy as np

F32 = np.float32

# corner v of a cell: offset (v & 1, (v >> 1) & 1, (v >> 2) & 1) along (x, y, z)
CORNERS = [(v & 1, (v >> 1) & 1, (v >> 2) & 1) for v in range(8)]


def _edges():
    """Edge e = 4 a + u + 2 w along axis a; (u, w) are the other two coordinates in axis order."""
    out = []
    for a in range(3):
        o = [b for b in range(3) if b != a]
        for w in range(2):
            for u in range(2):
                c0 = [0, 0, 0]
                c0[o[0]], c0[o[1]] = u, w
                c1 = list(c0)
                c1[a] = 1
                v0 = c0[0] | (c0[1] << 1) | (c0[2] << 2)
                v1 = c1[0] | (c1[1] << 1) | (c1[2] << 2)
                out.append((a, v0, v1))
    return out


EDGES = _edges()


def _faces():
    """The six faces as (corner cycle, edge cycle): edge k joins corners k and k + 1 of the cycle."""
    edge_of = {frozenset((v0, v1)): e for e, (_, v0, v1) in enumerate(EDGES)}
    faces = []
    for a in range(3):
        o = [b for b in range(3) if b != a]
        for s in range(2):
            cyc = []
            for u, w in ((0, 0), (1, 0), (1, 1), (0, 1)):
                c = [0, 0, 0]
                c[a], c[o[0]], c[o[1]] = s, u, w
                cyc.append(c[0] | (c[1] << 1) | (c[2] << 2))
            faces.append((cyc, [edge_of[frozenset((cyc[k], cyc[(k + 1) % 4]))] for k in range(4)]))
    return faces


FACES = _faces()


def _case_triangles(case: int):
    inside = [(case >> v) & 1 for v in range(8)]
    crossing = [e for e, (_, v0, v1) in enumerate(EDGES) if inside[v0] != inside[v1]]
    if not crossing:
        return []
    adj = {e: [] for e in crossing}
    for cyc, fe in FACES:
        cut = [k for k in range(4) if inside[cyc[k]] != inside[cyc[(k + 1) % 4]]]
        if len(cut) == 2:
            pairs = [(fe[cut[0]], fe[cut[1]])]
        elif len(cut) == 4:
            # ambiguous face: cut off each inside corner (its two face edges are joined)
            pairs = []
            for k in range(4):
                if inside[cyc[k]]:
                    pairs.append((fe[(k - 1) % 4], fe[k]))
        else:
            pairs = []
        for p, q in pairs:
            adj[p].append(q)
            adj[q].append(p)
    # edge midpoints and the inside -> outside direction of each crossing
    mid = {e: np.add(CORNERS[v0], CORNERS[v1]) * 0.5 for e, (_, v0, v1) in enumerate(EDGES)}
    out_dir = {}
    for e in crossing:
        _, v0, v1 = EDGES[e]
        vi, vo = (v0, v1) if inside[v0] else (v1, v0)
        out_dir[e] = np.subtract(CORNERS[vo], CORNERS[vi])
    tris, seen = [], set()
    for start in crossing:
        if start in seen:
            continue
        loop, prev, cur = [start], None, start
        seen.add(start)
        while True:
            nxt = [q for q in adj[cur] if q != prev]
            if len(adj[cur]) == 2 and adj[cur][0] == adj[cur][1]:
                nxt = [adj[cur][0]]
            q = nxt[0]
            if q == start:
                break
            loop.append(q)
            seen.add(q)
            prev, cur = cur, q
        area = np.zeros(3)
        for k in range(1, len(loop) - 1):
            area += np.cross(mid[loop[k]] - mid[loop[0]], mid[loop[k + 1]] - mid[loop[0]])
        if float(np.dot(area, sum(out_dir[e] for e in loop))) < 0:
            loop = loop[::-1]
        for k in range(1, len(loop) - 1):
            tris.append((loop[0], loop[k], loop[k + 1]))
    return tris


def triangle_table():
    """(256, 16) int8: the cell-edge triples of each case, -1 after the last triangle."""
    tab = np.full((256, 16), -1, dtype=np.int8)
    for c in range(256):
        t = _case_triangles(c)
        assert 3 * len(t) <= 15, (c, len(t))
        for i, tri in enumerate(t):
            tab[c, 3 * i: 3 * i + 3] = tri
    return tab


TABLE = triangle_table()


def extract(phi3: np.ndarray, band: np.ndarray):
    """Zero-level-set mesh of phi over the cells whose lower corner is a band node.

    Returns (vertices (n, 3) float32 in index coordinates, faces (m, 3) int64).  Vertices are
    numbered by their owner's position in the ascending band, then by axis; faces by cell (band
    order), then by the table order.  Matches svie_surface_* bit for bit."""
    shape = phi3.shape
    nx, ny, nz = shape
    f = phi3.reshape(-1)
    st = (ny * nz, nz, 1)
    band = np.asarray(band, dtype=np.int64)
    ins = f < 0
    # vertices owned by band nodes: one per crossed edge towards +axis
    cross = np.zeros((band.size, 3), dtype=bool)
    for a in range(3):
        nb = band + st[a]
        cross[:, a] = ins[band] != ins[nb]
    nvert = cross.sum(1)
    vbase = np.zeros(f.size, dtype=np.int64)
    vstart = np.concatenate([[0], np.cumsum(nvert)[:-1]])
    vbase[band] = vstart
    x, r = np.divmod(band, ny * nz)
    y, z = np.divmod(r, nz)
    coords = np.stack([x, y, z], 1).astype(F32)
    verts = []
    for i in range(band.size):
        for a in range(3):
            if cross[i, a]:
                p0, p1 = f[band[i]], f[band[i] + st[a]]
                t = F32(p0 / (p0 - p1))
                v = coords[i].copy()
                v[a] = F32(v[a] + t)
                verts.append(v)
    verts = np.array(verts, dtype=F32).reshape(-1, 3)
    faces = []
    for i in range(band.size):
        n = band[i]
        case = 0
        for v, (dx, dy, dz) in enumerate(CORNERS):
            if ins[n + dx * st[0] + dy * st[1] + dz * st[2]]:
                case |= 1 << v
        row = TABLE[case]
        for k in range(0, 15, 3):
            if row[k] < 0:
                break
            tri = []
            for e in row[k:k + 3]:
                a, v0, _ = EDGES[e]
                dx, dy, dz = CORNERS[v0]
                owner = n + dx * st[0] + dy * st[1] + dz * st[2]
                rank = int(sum(ins[owner] != ins[owner + st[b]] for b in range(a)))
                tri.append(vbase[owner] + rank)
            faces.append(tri)
    return verts, np.array(faces, dtype=np.int64).reshape(-1, 3)


def project(phi_flat: np.ndarray, shape, verts: np.ndarray, max_shift: float = 0.5) -> np.ndarray:
    """One Newton step of every vertex on the tricubic interpolant, limited to max_shift cells
    (svierosion/surface.py:44-51); float32 as the reference."""
    from .reference_np import tricubic_with_gradient

    p = np.asarray(verts, dtype=F32)
    val, grad = tricubic_with_gradient(phi_flat, shape[1], shape[2], p)
    g2 = np.maximum((grad * grad).sum(1), F32(1e-30))
    step = (val / g2)[:, None] * grad
    n = np.sqrt((step * step).sum(1, keepdims=True))
    step = step * np.minimum(F32(max_shift) / np.maximum(n, F32(max_shift)), F32(1.0))
    return (p - step).astype(F32)
