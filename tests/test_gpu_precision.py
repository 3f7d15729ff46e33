"""Error of the float32 GPU path against a full-float64 run of the same algorithm, for the four laws of
the precision study (svi k0 s0; svi k1 s1 t0.93; svi k2 s1 t0.95; mean curvature alpha 1) on a small
seeded fragment (icosphere subdivided 4x, resolution 64, eroded to 75% of its volume).

The float64 run is ``oracle.fp64`` (the oracle with every float32 quantity in float64, spectra in
complex128) started from the same level set (the float32 SDF, which equals the reference's, cast to
float64).  Stated bounds: max |N_r(fp32) - N_r(fp64)| <= 1e-4 over the grid; the volume-fraction
trajectory within 2e-5 per step; the stopping step equal within one step; max |phi(fp32) - phi(fp64)|
over the final band below 0.05 h, so the zero level sets lie well within half a cell of each other.
"""

import numpy as np
import pytest
import torch

from oracle.fp64 import fp64

pytestmark = pytest.mark.gpu

if torch.cuda.is_available():
    import svierosion_gb300 as S
    from svierosion_gb300 import shapes

LAWS = [
    ("svi", dict(radius_rel=0.08, k=0, s=0), 0.75),
    ("svi", dict(radius_rel=0.08, k=1, s=1, t=0.93), 0.75),
    ("svi", dict(radius_rel=0.08, k=2, s=1, t=0.95), 0.75),
    ("mean", dict(alpha=1.0), None),
]


@pytest.mark.parametrize("kind,kw,target", LAWS, ids=["svi_k0s0", "svi_k1s1", "svi_k2s1", "mean"])
def test_fp32_path_against_fp64(kind, kw, target):
    mesh = shapes.fragment(4, seed=0)
    lo, hi = mesh.bounds
    length = float((hi - lo).max())
    kw = dict(kw)
    if "radius_rel" in kw:
        kw["radius"] = kw.pop("radius_rel") * length
    params = S.ErosionParams(law=kind, resolution=64, target_fraction=target or 0.9, **kw)
    grid = S.make_grid(mesh, params)
    phi = S.mesh_to_sdf(mesh, grid, band=params.band)
    law = params.make_law(length_scale=length)
    max_steps = 60 if target is not None else 25

    ls = S.LevelSet(phi.clone(), grid, width=params.band)
    sim = S.ErosionSimulation(ls, law)
    law64 = fp64.make_law(kind, length_scale=length, **{k: v for k, v in kw.items()})
    ref = fp64.Simulation(phi.cpu().numpy().astype(np.float64), grid.spacing, law64)
    if law.requires_svi:
        n32 = sim.svi_field().cpu().numpy()
        n64 = ref.svi_field()
        assert float(np.abs(n32 - n64).max()) <= 1e-4

    res = sim.run(target_fraction=target, max_steps=max_steps)
    reason64, steps64, _, frac64 = ref.run(target_fraction=target, max_steps=max_steps)
    assert res.stop_reason == reason64
    assert abs(res.steps - steps64) <= 1
    f32 = np.array([r.fraction for r in res.history])
    f64 = np.array([r.fraction for r in ref.history])
    k = min(len(f32), len(f64))
    assert k > 0
    assert float(np.abs(f32[:k] - f64[:k]).max()) <= 2e-5
    if res.steps == steps64:
        band = np.union1d(ls.band.cpu().numpy(), ref.band)
        dphi = np.abs(ls.flat.cpu().numpy()[band].astype(np.float64) - ref.flat[band])
        assert float(dphi.max()) <= 0.05 * grid.spacing
