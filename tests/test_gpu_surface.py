"""GPU surface extraction (svie_surface_*) against the oracle's marching cubes, and the meshes that
erode() returns (the reference's stopping test, tests/test_flows.py:120-127: closed mesh whose volume
ratio is the target within 2e-3)."""

import numpy as np
import pytest
import torch

from oracle import marching as M

pytestmark = pytest.mark.gpu

if torch.cuda.is_available():
    import svierosion_gb300 as S
    from svierosion_gb300 import _native as nat
    from svierosion_gb300 import shapes
    from svierosion_gb300.grid import Grid
    from svierosion_gb300.surface import extract_surface


def _levelset(shape=(64, 56, 48), h=0.05):
    ax = [(np.arange(n) - 0.5 * (n - 1)) * h for n in shape]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    phi = (np.sqrt(X ** 2 + (Y / 0.8) ** 2 + (Z / 0.6) ** 2) - 0.75).astype(np.float32)
    return phi, Grid(tuple(float(a[0]) for a in ax), h, phi.shape)


def _raw_mesh(ls):
    nx, ny, nz = ls.grid.shape
    band = ls.band32
    m = band.numel()
    lib = nat.lib()
    ws = torch.empty(lib.svie_surface_workspace_bytes(m), dtype=torch.uint8, device="cuda")
    totals = torch.zeros(2, dtype=torch.int64, device="cuda")
    nat.call("svie_surface_scan", nat.ptr(ls.flat), nat.ptr(band), m, nx, ny, nz, nat.ptr(ws), ws.numel(),
             nat.ptr(totals), nat.stream())
    nv, nt = (int(v) for v in totals.cpu())
    vinfo = torch.empty(ls.grid.size, dtype=torch.int32, device="cuda")
    verts = torch.empty((nv, 3), dtype=torch.float32, device="cuda")
    faces = torch.empty((nt, 3), dtype=torch.int32, device="cuda")
    nat.call("svie_surface_write", nat.ptr(ls.flat), nat.ptr(band), m, nx, ny, nz, nat.ptr(ws), ws.numel(),
             nat.ptr(vinfo), nat.ptr(verts), nv, nat.ptr(faces), nt, nat.stream())
    return verts, faces


def test_marching_cubes_bit_exact_vs_oracle():
    phi, grid = _levelset()
    ls = S.LevelSet(torch.from_numpy(phi).cuda(), grid, width=6)
    verts, faces = _raw_mesh(ls)
    ref_v, ref_f = M.extract(ls.phi.cpu().numpy(), ls.band.cpu().numpy())
    assert np.array_equal(verts.cpu().numpy(), ref_v)
    assert np.array_equal(faces.cpu().numpy().astype(np.int64), ref_f)
    # the Newton projection (float32, FMA contraction aside)
    nx, ny, nz = grid.shape
    nat.call("svie_surface_project", nat.ptr(ls.flat), ny, nz, nat.ptr(verts), verts.shape[0], 0.5, nat.stream())
    ref_p = M.project(ls.flat.cpu().numpy(), grid.shape, ref_v, 0.5)
    assert float(np.abs(verts.cpu().numpy() - ref_p).max()) < 2e-5


def test_extract_surface_mesh_properties():
    phi, grid = _levelset()
    ls = S.LevelSet(torch.from_numpy(phi).cuda(), grid, width=6)
    mesh = extract_surface(ls)
    assert mesh.is_watertight() and mesh.is_consistently_oriented()
    assert mesh.signed_volume() > 0
    # a coarse ellipsoid (9-15 cells across, phi not a distance): the two volume estimates agree to 1%
    assert abs(mesh.volume() / ls.volume() - 1) < 1e-2
    # projected vertices sit on the zero set of the tricubic interpolant
    from svierosion_gb300.surface import sample_field
    vals = sample_field(ls.phi, grid, mesh.vertices)
    assert float(np.abs(vals).max()) < 2e-3 * grid.spacing


def test_erode_returns_closed_mesh_at_target():
    m = shapes.cube(1.0)
    res = S.erode(m, S.ErosionParams(law="svi", radius=0.2, k=1, s=1, t=0.9, resolution=60, target_fraction=0.93,
                                     snapshots=(0.97,)))
    assert res.stop_reason == "target_volume"
    assert abs(res.fraction - 0.93) < 1e-5
    assert res.mesh is not None and res.mesh.is_watertight()
    assert abs(res.mesh.volume() / m.volume() - 0.93) < 2e-3
    assert len(res.snapshots) == 1 and res.snapshots[0][2] is not None
    assert res.snapshots[0][2].is_watertight()
    assert "mesh" in res.timings


def test_point_mesh_distance_is_exact():
    """GPU shell search against brute force over all pieces (float64 numpy)."""
    from svierosion_gb300.api import point_mesh_distance
    from svierosion_gb300.sdf import bisect_long_triangles

    mesh = shapes.icosphere(3)
    rng = np.random.default_rng(5)
    pts = np.concatenate([rng.uniform(-1.3, 1.3, (400, 3)), rng.standard_normal((200, 3)) * 0.02,
                          mesh.vertices[:50] * 0.97])
    got = point_mesh_distance(pts, mesh, max_edge=0.05)
    tri = bisect_long_triangles(mesh.triangles(), max(0.05, 2 * float(np.median(
        np.linalg.norm(mesh.triangles()[:, 1] - mesh.triangles()[:, 0], axis=1)))))
    a, b, c = tri[:, 0], tri[:, 1], tri[:, 2]
    from oracle.reference_np import point_triangle_distance2
    ref = np.array([np.sqrt(point_triangle_distance2(np.broadcast_to(p, a.shape).astype(np.float32),
                                                     a.astype(np.float32), b.astype(np.float32),
                                                     c.astype(np.float32)).min()) for p in pts])
    assert np.allclose(got, ref, rtol=1e-5, atol=2e-6)


def test_erode_meshes_carry_vertex_data():
    m = shapes.cube(1.0)
    res = S.erode(m, S.ErosionParams(law="svi", radius=0.2, k=1, s=1, t=0.9, resolution=48, target_fraction=0.95))
    vd = res.mesh.vertex_data
    for key in ("depth", "N", "speed"):
        assert key in vd and len(vd[key]) == len(res.mesh.vertices)
    assert float(vd["depth"].max()) > 0
    assert np.all((vd["N"] > 0) & (vd["N"] < 1))
    res2 = S.erode(m, S.ErosionParams(law="mean", alpha=1.0, resolution=40, target_fraction=0.99, max_steps=30))
    for key in ("depth", "H", "K", "speed"):
        assert key in res2.mesh.vertex_data


def test_result_files_of_an_erosion(tmp_path):
    """An erode() result with a snapshot goes to disk in the reference's result format
    (cli.py:101-126) and reads back: meshes with their vertex fields, history, summary."""
    import csv
    import json

    res = S.erode(shapes.cube(1.0), S.ErosionParams(law="svi", radius=0.2, k=1, s=1, t=0.9, resolution=48,
                                                    target_fraction=0.95, snapshots=(0.97,)))
    written = S.write_result(res, tmp_path / "cube.ply")
    assert [p.name for p in written] == ["cube_v0.970.ply", "cube.ply"]
    m = S.read_ply(tmp_path / "cube.ply")
    assert np.array_equal(m.faces, res.mesh.faces)
    assert np.allclose(m.vertices, res.mesh.vertices, atol=1e-6)
    assert np.allclose(m.vertex_data["quality"], res.mesh.vertex_data["depth"], atol=1e-6)
    assert m.is_watertight()
    rows = list(csv.DictReader(open(tmp_path / "cube_history.csv")))
    assert len(rows) == len(res.history) and float(rows[-1]["fraction"]) == pytest.approx(res.fraction)
    meta = json.loads((tmp_path / "cube.json").read_text())
    assert meta["stop_reason"] == res.stop_reason
    # the snapshot records the fraction reached, within the tolerance of the request
    assert meta["snapshots"][0]["fraction"] == pytest.approx(0.97, abs=1e-3)
