"""Precision study at full size: the float32 GPU path against a full-float64 run (not a pytest module).

Workload: the seeded fragment (icosphere subdivided 6x, 81,920 triangles, seed 0), resolution 256,
r = 0.08 L, four laws: svi k0 s0, svi k1 s1 t0.93, svi k2 s1 t0.95 (to 90% of the volume) and mean
curvature alpha 1 (capped at 40 steps).  Two phases, so that the float64 oracle (CPU, minutes per law)
does not hold a GPU:

    python tests/precision_study.py gpu precision.npz      # with a GPU: the GPU runs and their inputs
    python tests/precision_study.py compare precision.npz  # anywhere: the float64 runs and the report

The report (one JSON line per law) gives max |N_r(fp32) - N_r(fp64)| on the initial grid, the largest
volume-fraction difference along the trajectory, both stopping steps, max |phi(fp32) - phi(fp64)|
over the final band in cells, and the symmetric Hausdorff distance in cells between the two final
zero level sets, each extracted by the CPU marching cubes of oracle/marching.py (vertex-to-surface
distances, exact over the triangles with the 16 nearest centroids).
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

LAWS = {
    "svi_k0s0": ("svi", dict(k=0, s=0), 0.9),
    "svi_k1s1_t0.93": ("svi", dict(k=1, s=1, t=0.93), 0.9),
    "svi_k2s1_t0.95": ("svi", dict(k=2, s=1, t=0.95), 0.9),
    "mean_a1": ("mean", dict(alpha=1.0), None),
}
MEAN_STEPS = 40


def _setup():
    from svierosion_gb300 import shapes
    from svierosion_gb300.api import ErosionParams, make_grid

    mesh = shapes.fragment(6, seed=0)
    lo, hi = mesh.bounds
    length = float((hi - lo).max())
    out = {}
    for name, (kind, kw, target) in LAWS.items():
        kw = dict(kw)
        if kind == "svi":
            kw["radius"] = 0.08 * length
        params = ErosionParams(law=kind, resolution=256, target_fraction=target or 0.9, **kw)
        out[name] = (kind, kw, target, params)
    return mesh, length, out


def run_gpu(path: str) -> None:
    import torch
    import svierosion_gb300 as S

    mesh, length, laws = _setup()
    save = {}
    for name, (kind, kw, target, params) in laws.items():
        grid = S.make_grid(mesh, params)
        phi0 = S.mesh_to_sdf(mesh, grid, band=params.band)
        key = "phi0_%dx%dx%d" % grid.shape
        if key not in save:
            save[key] = phi0.cpu().numpy()
        save[name + "/grid"] = np.array([*grid.origin, grid.spacing, *grid.shape], dtype=np.float64)
        ls = S.LevelSet(phi0.clone(), grid, width=params.band)
        sim = S.ErosionSimulation(ls, params.make_law(length_scale=length))
        if sim.law.requires_svi:
            n = sim.svi_field().cpu().numpy().reshape(-1)
            idx = np.random.default_rng(0).choice(n.size, size=200000, replace=False)
            save[name + "/n_idx"] = idx
            save[name + "/n"] = n[idx]
        res = sim.run(target_fraction=target, max_steps=200 if target is not None else MEAN_STEPS)
        torch.cuda.synchronize()
        save[name + "/fractions"] = np.array([r.fraction for r in res.history])
        save[name + "/steps"] = np.array([res.steps])
        save[name + "/reason"] = np.array([res.stop_reason])
        band = ls.band.cpu().numpy()
        save[name + "/band"] = band
        save[name + "/phi_band"] = ls.flat[ls.band].cpu().numpy()
    np.savez_compressed(path, **save)
    print("saved", path)


def _to_surface(pts, verts, faces, k=16):
    """Distance from each point to the mesh, exact over the k triangles with the nearest centroids."""
    from scipy.spatial import cKDTree

    from oracle.reference_np import point_triangle_distance2

    tri = verts[faces].astype(np.float64)
    _, cand = cKDTree(tri.mean(1)).query(pts, k=k)
    best = np.full(len(pts), np.inf)
    for j in range(k):
        t = tri[cand[:, j]]
        best = np.minimum(best, point_triangle_distance2(pts, t[:, 0], t[:, 1], t[:, 2]))
    return np.sqrt(best)


def _hausdorff_cells(phi32, band32, phi64, band64) -> float:
    """Symmetric Hausdorff distance (grid cells) between the zero sets of two fields."""
    from oracle import marching as M

    va, fa = M.extract(phi32, band32)
    vb, fb = M.extract(phi64, band64)
    va, vb = va.astype(np.float64), vb.astype(np.float64)
    return float(max(_to_surface(va, vb, fb).max(), _to_surface(vb, va, fa).max()))


def compare(path: str) -> None:
    from oracle.fp64 import fp64

    d = np.load(path, allow_pickle=False)
    mesh, length, laws = _setup()
    for name, (kind, kw, target, params) in laws.items():
        g = d[name + "/grid"]
        shape = tuple(int(v) for v in g[4:7])
        h = float(g[3])
        phi0 = d["phi0_%dx%dx%d" % shape].astype(np.float64).reshape(shape)
        law = fp64.make_law(kind, length_scale=length, **kw)
        ref = fp64.Simulation(phi0, h, law)
        rep = {"law": name, "grid": list(shape)}
        if law.requires_svi:
            n64 = ref.svi_field().reshape(-1)[d[name + "/n_idx"]]
            rep["max_abs_dN"] = float(np.abs(d[name + "/n"] - n64).max())
        reason, steps, _, _ = ref.run(target_fraction=target, max_steps=200 if target is not None else MEAN_STEPS)
        f32 = d[name + "/fractions"]
        f64 = np.array([r.fraction for r in ref.history])
        k = min(len(f32), len(f64))
        rep.update({"steps_fp32": int(d[name + "/steps"][0]), "steps_fp64": int(steps),
                    "reason_fp32": str(d[name + "/reason"][0]), "reason_fp64": reason,
                    "max_abs_dfraction": float(np.abs(f32[:k] - f64[:k]).max()) if k else None})
        band32 = d[name + "/band"]
        if int(d[name + "/steps"][0]) == steps:
            common = np.intersect1d(band32, ref.band)
            pos = np.searchsorted(band32, common)
            rep["max_abs_dphi_cells"] = float(np.abs(d[name + "/phi_band"][pos] - ref.flat[common]).max() / h)
            # the float32 field: band values on the band, the clamped value (sign of the float64 field,
            # the same far from the interface) elsewhere
            cap = np.float32(params.band * h)
            f64 = ref.flat.reshape(shape)
            phi32 = np.where(f64 < 0, -cap, cap).astype(np.float32).reshape(-1)
            phi32[band32] = d[name + "/phi_band"]
            rep["hausdorff_cells"] = _hausdorff_cells(phi32.reshape(shape), band32.astype(np.int64),
                                                      f64.astype(np.float32), np.asarray(ref.band, dtype=np.int64))
        print(json.dumps(rep), flush=True)


if __name__ == "__main__":
    mode, path = sys.argv[1], sys.argv[2]
    (run_gpu if mode == "gpu" else compare)(path)
