"""Fixtures at the full sizes of the precision and scan configurations, made by running the reference.

    PYTHONDONTWRITEBYTECODE=1 SVIEROSION_COMPILE=0 \
        python tests/golden/make_config_golden.py /path/to/SVIErosion [precision] [scan] [fp64]

* ``precision``: the seeded fragment subdivided 6x (81,920 triangles, seed 0) at resolution 256, for the
  four laws of the precision study -- svi k0 s0, svi k1 s1 t0.93, svi k2 s1 t0.95 (to 90% of the volume,
  r = 0.08 L) and mean curvature alpha 1 (40 steps).  The reference's own make_grid, mesh_to_sdf,
  LevelSet and ErosionSimulation.run (svierosion/api.py:94-101, sdf.py:365-415, levelset.py:54-86,
  evolve.py:182-250) run on the CPU in float32, as the reference always computes.
* ``scan``: the fragment subdivided 8x (1,310,720 triangles) at resolution 400, svi k1 s1 t0.93,
  r = 0.05 L: the SDF, the band, N_r and one RHS stage with its statistics (evolve.py:118-170).
* ``fp64``: the precision configuration's four laws once more with the float64 variant of the oracle
  (oracle/fp64.py) from the same float32 SDF: the full-FP64 run the float32 path's error is stated against.

A full grid does not fit a fixture, so each file keeps what the tests compare, in compact form:
sha256 digests (band lists, the mesh), the grid's inside bits (phi < 0) packed, seeded samples of the
SDF, N_r and the stage values, the step history, and the final zero level set as a "shell": the inside
bits of the final field plus its values, quantised to h/64 as int8, at the corners of every cell whose
corners change sign (the only values marching cubes reads).  The tests rebuild the final field from the
shell and compare surfaces.  Meshes come from svierosion_gb300.shapes.fragment, which is bit-identical
across machines; the fixture stores the mesh digest, and the tests check it first.
"""

from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent
ROOT = OUT.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(OUT.parent))


from config_fixtures import (SAMPLES, PRECISION_LAWS, digest, mesh_digest, sample_of,  # noqa: E402
                             shell_encode)


def history_arrays(hist) -> dict:
    keys = ["step", "time", "dt", "volume", "fraction", "vmax", "vmean", "qmin", "qmax", "capped", "reinit"]
    return {"hist_" + k: np.array([getattr(r, k) for r in hist], dtype=np.float64) for k in keys}


def fragment(sub: int, seed: int = 0):
    from svierosion_gb300 import shapes
    m = shapes.fragment(sub, seed=seed)
    lo, hi = m.bounds
    return m, float((hi - lo).max())


# ---------------------------------------------------------------------------- the reference
def _reference(ref_root: str):
    os.environ.setdefault("SVIEROSION_COMPILE", "0")
    sys.dont_write_bytecode = True
    sys.path.insert(0, ref_root)
    import torch
    from svierosion import kernels as K
    torch.set_num_threads(os.cpu_count() or 1)
    K.set_compile(False)


def _ref_params(spec: dict, length: float, resolution: int, radius_rel: float):
    from svierosion.api import ErosionParams
    kw = {k: v for k, v in spec.items() if k in ("law", "k", "s", "t", "alpha")}
    if kw["law"] == "svi":
        kw["radius"] = radius_rel * length
    return ErosionParams(resolution=resolution, target_fraction=spec["target"], device="cpu",
                         max_steps=spec.get("max_steps", 100000), **kw)


def _state(mesh_np, params, length):
    """Reference grid, SDF, level set and simulation (what api.py:210-233 builds before the run)."""
    from svierosion.api import make_grid
    from svierosion.evolve import ErosionSimulation
    from svierosion.levelset import LevelSet
    from svierosion.meshio import TriMesh
    from svierosion.sdf import mesh_to_sdf

    mesh = TriMesh(mesh_np.vertices, mesh_np.faces)
    grid = make_grid(mesh, params)
    phi = mesh_to_sdf(mesh, grid, band=params.band, device="cpu")
    phi0 = phi.numpy().copy()
    ls = LevelSet(phi, grid, width=params.band)
    law = params.make_law(length_scale=length)
    sim = ErosionSimulation(ls, law, cfl=params.cfl, feedback_cfl=params.feedback_cfl,
                            parabolic_cfl=params.parabolic_cfl, reinit_distance=params.reinit_distance,
                            reinit_iterations=params.reinit_iterations)
    return grid, phi0, ls, sim


def _initial(out: dict, grid, phi0: np.ndarray, ls, sim, seed: int) -> np.ndarray:
    """Grid, SDF, band and (SVI) N_r of the initial state; returns the sampled band positions."""
    band = ls.band.numpy()
    pos = sample_of(band.size, SAMPLES, seed)
    out.update(origin=np.array(grid.origin), shape=np.array(grid.shape), h=grid.spacing,
               sdf_inside=np.packbits((phi0 < 0).reshape(-1)), sdf_digest=digest(phi0),
               sample_idx=band[pos].astype(np.int64), sdf_sample=phi0.reshape(-1)[band[pos]],
               band_count=band.size, band_digest=digest(band.astype(np.int64)),
               band_head=band[:1000].astype(np.int64), band_tail=band[-1000:].astype(np.int64),
               initial_volume=sim.initial_volume)
    if sim.law.requires_svi:
        out["n_sample"] = sim.svi_field().numpy().reshape(-1)[band[pos]]
    return pos


def precision(ref_root: str) -> None:
    _reference(ref_root)
    mesh, length = fragment(6)
    for name, spec in PRECISION_LAWS.items():
        t0 = time.time()
        params = _ref_params(spec, length, 256, 0.08)
        grid, phi0, ls, sim = _state(mesh, params, length)
        np.save(_phi0_cache(name), phi0)
        out = {"mesh_digest": mesh_digest(mesh.vertices, mesh.faces), "length": length,
               "spec": json.dumps(spec)}
        _initial(out, grid, phi0, ls, sim, seed=1)
        res = sim.run(target_fraction=spec["target"], max_steps=spec.get("max_steps", 100000))
        final = ls.phi.numpy()
        band = ls.band.numpy()
        probe = band[sample_of(band.size, 4000, 2)]
        out.update(stop_reason=res.stop_reason, steps=res.steps, fraction=res.fraction,
                   band_final_count=band.size, probe_idx=probe.astype(np.int64),
                   probe_phi=final.reshape(-1)[probe], **shell_encode(final, grid.spacing),
                   **history_arrays(sim.history))
        np.savez_compressed(OUT / f"cfg_precision_{name}.npz", **out)
        print(name, grid.shape, res.stop_reason, res.steps, round(res.fraction, 7),
              f"{time.time() - t0:.0f}s", flush=True)


def scan(ref_root: str) -> None:
    _reference(ref_root)
    import torch
    mesh, length = fragment(8)
    spec = dict(law="svi", k=1, s=1, t=0.93, target=0.9)
    t0 = time.time()
    params = _ref_params(spec, length, 400, 0.05)
    grid, phi0, ls, sim = _state(mesh, params, length)
    out = {"mesh_digest": mesh_digest(mesh.vertices, mesh.faces), "length": length, "spec": json.dumps(spec)}
    pos = _initial(out, grid, phi0, ls, sim, seed=1)
    # one RHS stage with statistics, and the time step it gives (evolve.py:118-170, 193-196)
    L, V, info = sim._rhs(stats=True)
    dt = sim.stable_dt(V, info)
    out.update(stage_L=L.numpy()[pos], stage_V=V.numpy()[pos], stage_dt=dt, stage_vmax=float(V.max()),
               stage_info=json.dumps(info))
    np.savez_compressed(OUT / "cfg_scan.npz", **out)
    print("scan", grid.shape, "band", ls.band.numel(), "dt", dt, f"{time.time() - t0:.0f}s", flush=True)


def fp64_runs() -> None:
    """The float64 oracle on the precision configuration, from the reference's float32 SDF."""
    from oracle.fp64 import fp64 as O

    for name, spec in PRECISION_LAWS.items():
        t0 = time.time()
        src = np.load(OUT / f"cfg_precision_{name}.npz")
        shape = tuple(int(v) for v in src["shape"])
        h = float(src["h"])
        phi0 = _sdf_from(name, src)
        kw = {k: v for k, v in spec.items() if k in ("k", "s", "t", "alpha")}
        if spec["law"] == "svi":
            kw["radius"] = 0.08 * float(src["length"])
        law = O.make_law(spec["law"], length_scale=float(src["length"]), **kw)
        sim = O.Simulation(phi0.astype(np.float64).reshape(shape), h, law)
        out = {}
        if law.requires_svi:
            out["n_sample"] = sim.svi_field().reshape(-1)[src["sample_idx"]]
        reason, steps, _, frac = sim.run(target_fraction=spec["target"], max_steps=spec.get("max_steps", 100000))
        final = sim.flat.reshape(shape)
        out.update(stop_reason=reason, steps=steps, fraction=frac, **shell_encode(final, h),
                   hist_fraction=np.array([r.fraction for r in sim.history]),
                   probe_phi=sim.flat[src["probe_idx"]])
        np.savez_compressed(OUT / f"cfg_precision_{name}_fp64.npz", **out)
        print(name, "fp64", reason, steps, round(frac, 7), f"{time.time() - t0:.0f}s", flush=True)


def _phi0_cache(name: str) -> Path:
    return Path(tempfile.gettempdir()) / f"svie_cfg_precision_{name}_phi0.npy"


def _sdf_from(name: str, src) -> np.ndarray:
    """The reference's float32 SDF of this law's grid: kept from the precision pass, else recomputed
    with the oracle restatement; either way checked against the fixture's digest."""
    shape = tuple(int(v) for v in src["shape"])
    if _phi0_cache(name).exists():
        phi = np.load(_phi0_cache(name))
    else:
        import oracle as OR
        mesh, _ = fragment(6)
        phi = OR.mesh_to_sdf(mesh.vertices, mesh.faces, src["origin"], float(src["h"]), shape)
    phi = np.asarray(phi, dtype=np.float32).reshape(shape)
    if digest(phi) != str(src["sdf_digest"]):
        raise SystemExit(f"{name}: the oracle SDF differs from the reference's")
    return phi


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    parts = sys.argv[2:] or ["precision", "scan", "fp64"]
    if "precision" in parts:
        precision(root)
    if "scan" in parts:
        scan(root)
    if "fp64" in parts:
        fp64_runs()
