"""Parity at the full sizes of the precision and scan configurations, against fixtures made by running
the reference itself (tests/golden/make_config_golden.py), and against the full-FP64 oracle run.

Precision configuration: the seeded fragment subdivided 6x (81,920 triangles) at resolution 256, four
laws (svi k0 s0; svi k1 s1 t0.93; svi k2 s1 t0.95, to 90% of the volume with r = 0.08 L; mean
curvature alpha 1 for 40 steps), grid 315 x 240 x 175 (13.2M nodes) for the SVI laws.  Stated bounds,
against the reference:
  * SDF: inside bits (phi < 0) bit-exact over the whole grid; distances within 1e-6 h at 40,000 band
    nodes;
  * the initial band: the same nodes in the same order (sha256 of the int64 list);
  * N_r at 40,000 band nodes within 1e-5 relative (1e-7 absolute near 0);
  * the same stopping step and reason, the volume-fraction history within 1e-6, dt within 1e-3
    relative, reinitialisations at the same steps;
  * the final zero level sets within 0.5 cells (symmetric Hausdorff distance, marching cubes of
    oracle/marching.py on both fields; the reference's field rebuilt from its shell).
Against the full-FP64 oracle run (oracle/fp64.py from the same SDF): max |dN_r| <= 1e-4 at the same
nodes, the stopping step within one step, fractions within 2e-5, final surfaces within 0.5 cells.

Scan configuration: the fragment subdivided 8x (1,310,720 triangles) at resolution 400 (grid
448 x 336 x 245, 36.9M nodes), svi k1 s1 t0.93 with r = 0.05 L: the SDF, the band and N_r as above,
and one RHS stage: L and V at 40,000 band nodes within 1e-5 relative of their scale, the stage
statistics and the time step within 1e-5 relative.
"""

import json

import numpy as np
import pytest
import torch

from config_fixtures import PRECISION_LAWS, digest, hausdorff_cells, mesh_digest, shell_decode

pytestmark = pytest.mark.gpu

if torch.cuda.is_available():
    import svierosion_gb300 as S
    from svierosion_gb300 import shapes


def _params(spec, length, resolution, radius_rel):
    kw = {k: v for k, v in spec.items() if k in ("law", "k", "s", "t", "alpha")}
    if kw["law"] == "svi":
        kw["radius"] = radius_rel * length
    return S.ErosionParams(resolution=resolution, target_fraction=spec["target"],
                           max_steps=spec.get("max_steps", 100000), **kw)


def _initial_state(d, sub, resolution, radius_rel):
    """Mesh, grid, SDF and level set of a fixture's configuration, each checked against the fixture."""
    spec = json.loads(str(d["spec"]))
    mesh = shapes.fragment(sub, seed=0)
    assert mesh_digest(mesh.vertices, mesh.faces) == str(d["mesh_digest"]), "fragment generator differs"
    length = float(d["length"])
    params = _params(spec, length, resolution, radius_rel)
    grid = S.make_grid(mesh, params)
    assert tuple(grid.shape) == tuple(int(v) for v in d["shape"])
    assert grid.spacing == float(d["h"]) and np.array_equal(np.array(grid.origin), d["origin"])
    h = grid.spacing
    phi = S.mesh_to_sdf(mesh, grid, band=params.band)
    ph = phi.cpu().numpy().reshape(-1)
    assert np.array_equal(np.packbits(ph < 0), d["sdf_inside"]), "SDF signs differ"
    err = float(np.abs(ph[d["sample_idx"]] - d["sdf_sample"]).max())
    assert err <= 1e-6 * h, err
    ls = S.LevelSet(phi, grid, width=params.band)
    band = ls.band.cpu().numpy().astype(np.int64)
    assert band.size == int(d["band_count"])
    assert digest(band) == str(d["band_digest"]), "initial band differs"
    law = params.make_law(length_scale=length)
    sim = S.ErosionSimulation(ls, law, cfl=params.cfl, feedback_cfl=params.feedback_cfl,
                              parabolic_cfl=params.parabolic_cfl, reinit_distance=params.reinit_distance,
                              reinit_iterations=params.reinit_iterations)
    assert abs(sim.initial_volume - float(d["initial_volume"])) <= 1e-9 * float(d["initial_volume"])
    return spec, grid, ls, sim


def _n_close(n, ref):
    err = np.abs(n.astype(np.float64) - ref.astype(np.float64))
    return bool(np.all(err <= 1e-5 * np.abs(ref) + 1e-7)), float(err.max())


@pytest.mark.parametrize("name", list(PRECISION_LAWS))
def test_precision_config_matches_reference_and_fp64(golden, name):
    d = golden(f"cfg_precision_{name}")
    spec, grid, ls, sim = _initial_state(d, 6, 256, 0.08)
    h = grid.spacing
    n_gpu = None
    if sim.law.requires_svi:
        n_gpu = sim.svi_field().reshape(-1)[torch.from_numpy(d["sample_idx"]).cuda()].cpu().numpy()
        ok, err = _n_close(n_gpu, d["n_sample"])
        assert ok, err
    res = sim.run(target_fraction=spec["target"], max_steps=spec.get("max_steps", 100000))
    assert res.stop_reason == str(d["stop_reason"])
    assert res.steps == int(d["steps"])
    fr = np.array([r.fraction for r in res.history])
    np.testing.assert_allclose(fr, d["hist_fraction"], atol=1e-6)
    np.testing.assert_allclose([r.dt for r in res.history], d["hist_dt"], rtol=1e-3)
    assert [int(r.reinit) for r in res.history] == d["hist_reinit"].astype(int).tolist()
    cnt = ls.band.numel()
    assert abs(cnt - int(d["band_final_count"])) <= max(2, cnt // 20000)
    final = ls.phi.cpu().numpy()
    shape = final.shape
    far = np.float32(6 * h)
    hd = hausdorff_cells(final, shell_decode(d, "", shape, h, far))
    assert hd <= 0.5, hd

    # the full-FP64 oracle run of the same configuration
    d64 = golden(f"cfg_precision_{name}_fp64")
    if n_gpu is not None:
        assert float(np.abs(n_gpu.astype(np.float64) - d64["n_sample"]).max()) <= 1e-4
    assert abs(res.steps - int(d64["steps"])) <= 1
    f64 = d64["hist_fraction"]
    k = min(len(fr), len(f64))
    assert float(np.abs(fr[:k] - f64[:k]).max()) <= 2e-5
    hd64 = hausdorff_cells(final, shell_decode(d64, "", shape, h, far))
    assert hd64 <= 0.5, hd64
    dn64 = float(np.abs(n_gpu.astype(np.float64) - d64["n_sample"]).max()) if n_gpu is not None else float("nan")
    # the measured figures (shown with pytest -s)
    print(f"\n[{name}] grid {shape}: steps {res.steps} (reference {int(d['steps'])}, fp64 {int(d64['steps'])}); "
          f"max |dN_r| vs fp64 {dn64:.2e}; max |d fraction| vs reference "
          f"{float(np.abs(fr - d['hist_fraction']).max()):.1e}, vs fp64 {float(np.abs(fr[:k] - f64[:k]).max()):.1e}; "
          f"Hausdorff vs reference {hd:.4f} cells, vs fp64 {hd64:.4f} cells")


def test_scan_config_first_stage_matches_reference(golden):
    d = golden("cfg_scan")
    spec, grid, ls, sim = _initial_state(d, 8, 400, 0.05)
    idx = torch.from_numpy(d["sample_idx"]).cuda()
    n = sim.svi_field().reshape(-1)[idx].cpu().numpy()
    ok, err = _n_close(n, d["n_sample"])
    assert ok, err
    L, V, info = sim._rhs(stats=True)
    pos = np.searchsorted(ls.band.cpu().numpy(), d["sample_idx"])
    for got, ref in ((L, d["stage_L"]), (V, d["stage_V"])):
        g = got.cpu().numpy()[pos].astype(np.float64)
        scale = float(np.abs(ref).max())
        assert float(np.abs(g - ref).max()) <= 1e-5 * scale
    ref_info = json.loads(str(d["stage_info"]))
    for key in ("qmin", "qmax", "dvmax", "vmean"):
        assert abs(info[key] - ref_info[key]) <= 1e-5 * abs(ref_info[key]) + 1e-7, key
    assert abs(info["capped"] - ref_info["capped"]) <= 2
    vmax = float(V.max())
    assert abs(vmax - float(d["stage_vmax"])) <= 1e-5 * float(d["stage_vmax"])
    for dt in (sim.stable_dt(V, info), sim.last_stage_dt):
        assert abs(dt - float(d["stage_dt"])) <= 1e-5 * float(d["stage_dt"])
