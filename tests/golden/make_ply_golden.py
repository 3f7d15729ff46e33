"""Golden PLY and result files written by the reference's own code (run here, on the CPU, once).

    python tests/golden/make_ply_golden.py /path/to/reference

Imports the reference package read-only from its source tree and writes into tests/golden/ply/:
- a small torus with a per-vertex scalar in the three encodings its tests use (binary float,
  binary double, ASCII double), with the mesh itself;
- the result files of a synthetic erosion result (`synthetic_result`) through the reference's
  result writer (cli.py:101-126): snapshot and final meshes, history CSV and JSON summary.
tests/test_ply.py checks this package's reader against the files and its writers byte for byte.
"""

from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def main(ref_root: str) -> None:
    os.environ["PYTHONDONTWRITEBYTECODE"] = "1"
    sys.dont_write_bytecode = True
    sys.path.insert(0, ref_root)
    from svierosion import shapes
    from svierosion.meshio import write_ply

    out = HERE / "ply"
    out.mkdir(exist_ok=True)
    mesh = shapes.torus(1.0, 0.3, 16, 8)
    q = mesh.vertices[:, 2].copy()
    np.savez_compressed(out / "torus.npz", vertices=mesh.vertices, faces=mesh.faces, quality=q)
    for binary, prec in ((True, "float"), (True, "double"), (False, "double")):
        name = f"torus_{'binary' if binary else 'ascii'}_{prec}.ply"
        write_ply(out / name, mesh, binary=binary, precision=prec, vertex_data={"quality": q},
                  comments=["written by the reference"])
        print("wrote", out / name)

    # the result files of a synthetic result (no erosion is run)
    from svierosion.api import ErosionResult
    from svierosion.cli import _write_result
    from svierosion.evolve import StepRecord
    from svierosion.grid import Grid
    from svierosion.meshio import TriMesh

    res = synthetic_result(ErosionResult, StepRecord, Grid, TriMesh, shapes.cube(1.0))
    for p in _write_result(res, out / "result.ply", "depth"):
        print("wrote", p)


def synthetic_result(ErosionResult, StepRecord, Grid, TriMesh, cube):
    """A fixed ErosionResult built from the given classes (the reference's or this package's)."""
    v = cube.vertices
    depth = np.linalg.norm(v, axis=1)
    final = TriMesh(0.9 * v, cube.faces, {"depth": depth, "N": np.full(len(v), 0.25)})
    snap = TriMesh(0.95 * v, cube.faces, {"depth": 0.5 * depth})
    hist = [StepRecord(step=i + 1, time=0.01 * (i + 1), dt=0.01, volume=1.0 - 0.02 * i, fraction=1.0 - 0.02 * i,
                       vmax=1.5, vmean=0.75, qmin=0.1, qmax=0.6, capped=i % 2, reinit=i == 1, wall=0.001 * i)
            for i in range(3)]
    return ErosionResult(mesh=final, snapshots=[(0.95, 0.02, snap)], history=hist,
                         grid=Grid((-0.75, -0.75, -0.75), 0.03125, (48, 48, 48)), stop_reason="target_volume",
                         time=0.03, fraction=0.9, initial_volume_grid=1.0, initial_volume_mesh=1.0,
                         timings={"sdf": 0.5, "evolve": 2.0, "mesh": 0.25},
                         params={"law": "svi", "radius": 0.1, "k": 1, "s": 1, "t": 0.93})


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
