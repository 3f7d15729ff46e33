"""Several erosion laws on one solid, each to the same remaining volume (reference svierosion/compare.py).

``run_comparison`` erodes the solid once per law through :func:`~svierosion_gb300.api.erode` (the GPU
path end to end: SDF, evolution, meshing and annotation) and writes, into one directory, the initial
mesh, every final mesh (vertex quality = depth below the initial surface), a CSV table of the runs and
the mean distances between the final surfaces.  The reference also renders a figure of all meshes with
matplotlib; no plotting library is part of this build, so that figure is not written.
"""

from __future__ import annotations

import csv
import json
import re
import time
from pathlib import Path

import numpy as np

from .api import ErosionParams, erode, point_mesh_distance
from .meshio import TriMesh, write_ply


def default_comparison_laws(radius: float, t: float = 0.93) -> list:
    """(label, ErosionParams keywords) of the standard comparison (compare.py:19-30): grassfire,
    V = N, V = N^4, V = N/(t - N), mean curvature and Gauss curvature (alpha 1)."""
    svi = [("grassfire V=1", 0, 0), ("SVI V=N", 1, 0), ("SVI V=N^4", 4, 0), (f"SVI V=N/({t:g}-N)", 1, 1)]
    laws = [(label, dict(law="svi", radius=radius, k=k, s=s, **({"t": t} if s else {}))) for label, k, s in svi]
    laws.append(("mean curv. V=H+", dict(law="mean", alpha=1.0)))
    laws.append(("Gauss curv. V=K+", dict(law="gauss", alpha=1.0)))
    return laws


def slug(label: str) -> str:
    """File-name form of a law label: runs of other characters become one underscore, lower case."""
    return re.sub(r"[^A-Za-z0-9]+", "_", label).strip("_").lower()


def mesh_distance_stats(a: TriMesh, b: TriMesh, device=None) -> dict:
    """Symmetric surface distances between two meshes: the mean and rms of the vertex-to-surface
    distances taken both ways, and the Hausdorff distance (their maximum)."""
    ab = point_mesh_distance(a.vertices, b, device=device)
    ba = point_mesh_distance(b.vertices, a, device=device)
    return {"mean": 0.5 * (float(ab.mean()) + float(ba.mean())),
            "rms": float(np.sqrt(0.5 * (float((ab ** 2).mean()) + float((ba ** 2).mean())))),
            "hausdorff": float(max(ab.max(), ba.max()))}


def run_comparison(mesh: TriMesh, laws: list, outdir, target: float = 0.9, resolution: int = 160,
                   spacing: float | None = None, device=None, verbose: bool = True, max_steps: int = 200_000,
                   title: str | None = None) -> list:
    """Erode ``mesh`` with every law of ``laws`` ((label, ErosionParams keywords) pairs) to ``target``
    and write the results into ``outdir`` (compare.py:33-85).  Returns [(label, ErosionResult)]."""
    out = Path(outdir)
    out.mkdir(parents=True, exist_ok=True)
    write_ply(out / "initial.ply", mesh)
    results, table = [], []
    for label, kw in laws:
        params = ErosionParams(**kw, target_fraction=target, resolution=resolution, spacing=spacing, device=device,
                               max_steps=max_steps)
        clock = time.time()
        res = erode(mesh, params)
        wall = time.time() - clock
        depth = res.mesh.vertex_data.get("depth", np.zeros(len(res.mesh.vertices)))
        write_ply(out / f"{slug(label)}.ply", res.mesh, vertex_data={"quality": depth})
        d = depth if depth.size else np.zeros(1)
        row = {"label": label, "stop": res.stop_reason, "steps": len(res.history), "model_time": res.time,
               "volume_fraction": res.fraction,
               "mesh_volume_fraction": res.mesh.volume() / mesh.volume() if len(res.mesh.faces) else 0.0,
               "depth_mean": float(d.mean()), "depth_max": float(d.max()), "wall_seconds": wall,
               "grid": "x".join(str(n) for n in res.grid.shape)}
        table.append(row)
        results.append((label, res))
        if verbose:
            print(f"[compare] {label:24s} {res.stop_reason:13s} steps {row['steps']:6d}  "
                  f"V/V0 {row['volume_fraction']:.4f}  depth mean {row['depth_mean']:.4g} "
                  f"max {row['depth_max']:.4g}  ({wall:.1f}s)", flush=True)
    with open(out / "summary.csv", "w", newline="") as fh:
        writer = csv.DictWriter(fh, fieldnames=list(table[0]))
        writer.writeheader()
        writer.writerows(table)
    finals = [r.mesh for _, r in results]
    dist = np.zeros((len(finals), len(finals)))
    for i, j in ((i, j) for i in range(len(finals)) for j in range(i + 1, len(finals))):
        if len(finals[i].faces) and len(finals[j].faces):
            dist[i, j] = dist[j, i] = mesh_distance_stats(finals[i], finals[j], device=device)["mean"]
    (out / "pairwise_mean_distance.json").write_text(
        json.dumps({"labels": [lab for lab, _ in results], "mean_distance": dist.tolist()}, indent=2) + "\n")
    return results
