"""How fast the oracle port runs the reference's step loop, against the reference itself (test
infrastructure only; it reads the reference's source tree and runs on the CPU):

    PYTHONDONTWRITEBYTECODE=1 python oracle/calibrate_port.py /path/to/SVIErosion [threads]

On the scan workload (seeded fragment subdivided 8x, resolution 400, svi k1 s1 t0.93, r = 0.05 L;
grid 448 x 336 x 245) both start from the reference's own SDF and run, on the same number of host
threads: one RHS stage (the reference's ErosionSimulation._rhs with torch.compile warm, and eager; the
port's ThreadedStage.rhs) and whole steps of the run loop (evolve.py:182-250, reinitialisations
included).  The benchmark's reference arm times the port; this ratio says how it compares with
timing the reference itself on the same cores.
"""

from __future__ import annotations

import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def _time(fn, reps=3):
    out = []
    for _ in range(reps):
        t0 = time.time()
        fn()
        out.append(time.time() - t0)
    return min(out)


def main(ref_root: str, threads: int) -> None:
    sys.dont_write_bytecode = True
    sys.path.insert(0, ref_root)
    import torch
    torch.set_num_threads(threads)
    from svierosion import kernels as K
    from svierosion.api import ErosionParams, make_grid
    from svierosion.evolve import ErosionSimulation
    from svierosion.levelset import LevelSet
    from svierosion.meshio import TriMesh
    from svierosion.sdf import mesh_to_sdf

    from svierosion_gb300 import shapes
    from oracle.threaded_np import ThreadedSimulation
    import oracle as O

    frag = shapes.fragment(8, seed=0)
    lo, hi = frag.bounds
    L = float((hi - lo).max())
    params = ErosionParams(law="svi", radius=0.05 * L, k=1, s=1, t=0.93, resolution=400, target_fraction=0.9,
                           device="cpu")
    mesh = TriMesh(frag.vertices, frag.faces)
    grid = make_grid(mesh, params)
    phi0 = mesh_to_sdf(mesh, grid, band=params.band, device="cpu").numpy().copy()
    law = params.make_law(length_scale=L)
    print(f"grid {grid.shape}, threads {threads}", flush=True)

    report = {}
    for compiled in (True, False):
        K.set_compile(compiled)
        ls = LevelSet(__import__("torch").from_numpy(phi0.copy()), grid, width=params.band)
        sim = ErosionSimulation(ls, law)
        sim._rhs(stats=True)                       # warm-up (compiles when enabled)
        report[f"reference rhs ({'compiled' if compiled else 'eager'})"] = _time(lambda: sim._rhs(stats=True))
        if compiled:
            sim.run(target_fraction=None, max_steps=1)   # warm the step loop's other kernels
            t0 = time.time()
            sim.run(target_fraction=None, max_steps=6)
            report["reference 6 whole steps (compiled)"] = time.time() - t0
            report["reference reinitialisations in them"] = sum(r.reinit for r in sim.history[1:])
    port = ThreadedSimulation(phi0.copy(), grid.spacing, O.make_law("svi", radius=law.radius, k=1, s=1, t=0.93),
                              workers=threads)
    try:
        port.stage.rhs()
        report["port rhs"] = _time(lambda: port.stage.rhs())
        port.run(target_fraction=None, max_steps=1)
        t0 = time.time()
        port.run(target_fraction=None, max_steps=6)
        report["port 6 whole steps"] = time.time() - t0
        report["port reinitialisations in them"] = sum(r.reinit for r in port.history[1:])
    finally:
        port.close()
    for k, v in report.items():
        print(f"{k}: {v:.3f}" if isinstance(v, float) else f"{k}: {v}", flush=True)
    print("ratio port/reference: rhs %.2f, whole steps %.2f"
          % (report["port rhs"] / report["reference rhs (compiled)"],
             report["port 6 whole steps"] / report["reference 6 whole steps (compiled)"]), flush=True)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference",
         int(sys.argv[2]) if len(sys.argv) > 2 else (os.cpu_count() or 1))
