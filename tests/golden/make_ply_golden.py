"""Golden PLY files written by the reference's own meshio (run here, on the CPU, once).

    python tests/golden/make_ply_golden.py /path/to/reference

Imports the reference package read-only from its source tree, writes a small torus with a
per-vertex scalar in the three encodings its tests use (binary float, binary double, ASCII
double), and stores the files with the mesh itself in tests/golden/ply/.  tests/test_ply.py
checks this package's reader against the files and its writer byte for byte against them.
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


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
