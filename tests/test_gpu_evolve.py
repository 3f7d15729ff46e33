"""Reinitialisation, SDF and full erosion runs against the reference fixtures."""

import math

import numpy as np
import pytest
import torch

import oracle as O

pytestmark = pytest.mark.gpu

if torch.cuda.is_available():
    import svierosion_gb300 as S
    from svierosion_gb300 import shapes
    from svierosion_gb300.grid import Grid
    from svierosion_gb300.meshio import TriMesh


def test_reinitialize(golden):
    r = golden("reinit_sphere")
    shape = tuple(int(v) for v in r["shape"])
    g = Grid((0.0, 0.0, 0.0), float(r["h"]), shape)
    ls = S.LevelSet(torch.from_numpy(r["phi0"]).cuda(), g, width=6)
    assert np.array_equal(ls.band.cpu().numpy(), r["band0"])
    ls.reinitialize(20)
    assert float(np.abs(ls.phi.cpu().numpy() - r["phi"]).max()) < 5e-6
    # band sets agree except where phi sits within rounding of the threshold
    got, ref = set(ls.band.cpu().numpy().tolist()), set(r["band"].tolist())
    assert len(got ^ ref) <= 2


def test_sdf_cube_and_torus(golden):
    sd = golden("sdf")
    for key in ("cube", "torus"):
        mesh = TriMesh(sd[f"{key}_v"], sd[f"{key}_f"])
        shape = tuple(int(v) for v in sd[f"{key}_shape"])
        g = Grid(tuple(float(v) for v in sd[f"{key}_origin"]), float(sd[f"{key}_h"]), shape)
        phi = S.mesh_to_sdf(mesh, g, band=6).cpu().numpy()
        ref = sd[f"{key}_phi"]
        assert np.array_equal(np.sign(phi), np.sign(ref)), key
        assert float(np.abs(phi - ref).max()) < 1e-6 * g.spacing * 10, key


def test_sdf_fragment_vs_oracle():
    mesh = shapes.fragment(4, seed=3)
    params = S.ErosionParams(law="svi", radius=0.1 * 2.08, k=1, s=1, t=0.93, resolution=48)
    g = S.make_grid(mesh, params)
    phi = S.mesh_to_sdf(mesh, g, band=6).cpu().numpy()
    ref = O.mesh_to_sdf(mesh.vertices, mesh.faces, g.origin, g.spacing, g.shape)
    assert np.array_equal(np.sign(phi), np.sign(ref))
    assert float(np.abs(phi - ref).max()) < 1e-5 * g.spacing


def _run(golden, name):
    d = golden(f"run_{name}")
    P = d["params"]
    mesh = TriMesh(d["vertices"], d["faces"])
    shape = tuple(int(v) for v in d["shape"])
    g = Grid(tuple(float(v) for v in d["origin"]), float(d["h"]), shape)
    phi = S.mesh_to_sdf(mesh, g, band=6)
    assert float(np.abs(phi.cpu().numpy() - d["phi_init"]).max()) < 1e-6
    ls = S.LevelSet(phi, g, width=6)
    assert np.array_equal(ls.band.cpu().numpy(), d["band_init"])
    lo, hi = mesh.bounds
    params = S.ErosionParams(law=str(d["law"]), radius=float(P[0]) or None, k=int(P[1]), s=int(P[2]),
                             t=float(P[3]) or None, alpha=float(P[4]))
    law = params.make_law(length_scale=float((hi - lo).max()))
    sim = S.ErosionSimulation(ls, law)
    assert abs(sim.initial_volume - float(d["initial_volume"])) < 1e-9
    res = sim.run(float(P[6]), max_steps=int(d.get("max_steps", 100000)))
    return d, res, ls


@pytest.mark.parametrize("name", ["cube64", "cube32_k0s0", "cube32_mean", "cube32_gauss"])
def test_full_run_matches_reference(golden, name):
    d, res, ls = _run(golden, name)
    assert res.stop_reason == str(d["stop_reason"])
    assert res.steps == int(d["steps"])
    assert abs(res.fraction - float(d["fraction"])) < 1e-6
    fr = np.array([r.fraction for r in res.history])
    np.testing.assert_allclose(fr, d["hist_fraction"], atol=1e-6)
    dts = np.array([r.dt for r in res.history])
    # the Gauss law's step is the parabolic limit h^2 / (4 max D), and D = F'(K)(k1+ + k2+) peaks at the
    # cube's edges and corners, where k1,2 = H +- sqrt(H^2 - K) turns rounding-level differences of phi
    # into percent-level differences of max D: the oracle, which follows the reference's operation
    # order in numpy, differs from the reference there by up to 1.3% as well (fractions: 5e-7)
    np.testing.assert_allclose(dts, d["hist_dt"], rtol=3e-2 if name == "cube32_gauss" else 1e-3)
    np.testing.assert_allclose([r.vmax for r in res.history], d["hist_vmax"], rtol=1e-3)
    assert [int(r.reinit) for r in res.history] == d["hist_reinit"].astype(int).tolist()
    cnt = ls.band.numel()
    assert abs(cnt - int(d["band_final_count"])) <= max(2, cnt // 20000)
    # final phi at the probe nodes
    probe = torch.from_numpy(d["probe_idx"]).cuda()
    err = float(np.abs(ls.flat[probe].cpu().numpy() - d["probe_phi"]).max())
    assert err < 1e-3 * float(d["h"]), err


def test_rejects_t_below_max_n():
    with pytest.raises(ValueError):
        S.erode(shapes.cube(1.0), S.ErosionParams(law="svi", radius=0.2, k=1, s=1, t=0.8, resolution=40),
                extract_meshes=False)


def test_erode_stops_at_target():
    res = S.erode(shapes.cube(1.0), S.ErosionParams(law="svi", radius=0.2, k=1, s=1, t=0.9, resolution=40,
                                                    target_fraction=0.93), extract_meshes=False, keep_state=True)
    assert res.stop_reason == "target_volume"
    assert abs(res.fraction - 0.93) < 1e-5


def test_work_set_rebuild_equals_full_rebuild():
    """After evolution steps (phi changed on the band only), reinitialisation with the band rebuilt
    over the work set gives exactly the state of a full-grid rebuild: phi, band list and order,
    occupancy, static inside count and band box; the inside box contains the exact one."""
    mesh = shapes.fragment(3, seed=1)
    params = S.ErosionParams(law="svi", radius=0.2, k=1, s=1, t=0.93, resolution=56)
    L = float((mesh.bounds[1] - mesh.bounds[0]).max())
    states = []
    for fast in (False, True):
        g = S.make_grid(mesh, params)
        ls = S.LevelSet(S.mesh_to_sdf(mesh, g, band=6), g, width=6)
        sim = S.ErosionSimulation(ls, params.make_law(length_scale=L), reinit_distance=1e9)  # no reinit in run
        sim.run(target_fraction=None, max_steps=4)
        ls.reinitialize(20, work_set_rebuild=fast)
        states.append((ls.flat.cpu().numpy(), ls.work32.cpu().numpy(), ls.occ.cpu().numpy(), ls.static_inside,
                       ls.band_lo, ls.band_hi, ls.inside_lo, ls.inside_hi, ls.volume()))
    full, fast = states
    for k in range(6):
        assert np.array_equal(np.asarray(full[k]), np.asarray(fast[k])), k
    assert all(a <= b for a, b in zip(fast[6], full[6])) and all(a >= b for a, b in zip(fast[7], full[7]))
    assert fast[8] == full[8]
