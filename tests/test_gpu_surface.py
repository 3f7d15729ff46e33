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


def test_device_assembled_mesh_equals_host_assembly():
    """extract_surface assembles the host mesh on the device: the same arrays as origin + h * v
    in float64 and int64 faces on the host (surface.py:52-56), reversed for a negative volume."""
    from svierosion_gb300.meshio import TriMesh
    from svierosion_gb300.surface import extract_surface_device

    phi, grid = _levelset()
    for sign in (1.0, -1.0):   # outward and inward orientation of the raw triangles
        ls = S.LevelSet(torch.from_numpy((sign * phi).astype(np.float32)).cuda(), grid, width=6)
        verts, faces = _raw_mesh(ls)
        nx, ny, nz = grid.shape
        nat.call("svie_surface_project", nat.ptr(ls.flat), ny, nz, nat.ptr(verts), verts.shape[0], 0.5,
                 nat.stream())
        world = np.asarray(grid.origin) + grid.spacing * verts.cpu().numpy().astype(np.float64)
        f = faces.cpu().numpy().astype(np.int64)
        if TriMesh(world, f).signed_volume() < 0:
            f = f[:, ::-1]
        mesh, dev_world = extract_surface_device(ls)
        assert np.array_equal(mesh.vertices, world)
        assert np.array_equal(mesh.faces, f)
        assert np.array_equal(dev_world.cpu().numpy(), world)
        assert mesh.signed_volume() > 0


def test_device_point_conversions_round_like_numpy():
    """svie_points_f32: float32((p - shift) / h) as numpy computes it (no contraction)."""
    rng = np.random.default_rng(11)
    pts = rng.uniform(-3.0, 3.0, (20000, 3)) * 1.2345
    grid = Grid((-1.1, -2.3, 0.7), 0.0123, (10, 10, 10))
    p = torch.from_numpy(pts).cuda()
    out = torch.empty((len(pts), 3), dtype=torch.float32, device="cuda")
    nat.call("svie_points_f32", nat.ptr(p), len(pts), *grid.origin, grid.spacing, nat.ptr(out), nat.stream())
    assert np.array_equal(out.cpu().numpy(), grid.to_index(pts).astype(np.float32))
    shift = np.array([0.3, -0.2, 0.1])
    nat.call("svie_points_f32", nat.ptr(p), len(pts), *shift, 1.0, nat.ptr(out), nat.stream())
    assert np.array_equal(out.cpu().numpy(), (pts - shift).astype(np.float32))


def test_annotation_from_device_points_equals_host_points():
    """erode() annotates from the device copy of the vertices: the same depth, N and speed as
    from the host vertices."""
    from svierosion_gb300.api import _annotate, _PieceGrid
    from svierosion_gb300.meshio import TriMesh
    from svierosion_gb300.sdf import device_mesh
    from svierosion_gb300.surface import extract_surface_device

    m = shapes.cube(1.0)
    p = S.ErosionParams(law="svi", radius=0.2, k=1, s=1, t=0.9, resolution=48, target_fraction=0.95)
    res = S.erode(m, p, keep_state=True, extract_meshes=False)
    surf, world = extract_surface_device(res.level_set)
    dev = res.level_set.device
    pieces = _PieceGrid(m, 4 * res.grid.spacing, dev, device_mesh(m, dev))
    law = p.make_law(length_scale=1.0)
    a = TriMesh(surf.vertices, surf.faces)
    b = TriMesh(surf.vertices, surf.faces)
    _annotate(res.simulation, a, pieces, law)
    _annotate(res.simulation, b, pieces, law, world)
    assert set(a.vertex_data) == {"depth", "N", "speed"}
    for key in a.vertex_data:
        assert np.array_equal(a.vertex_data[key], b.vertex_data[key]), key


def test_order_statistics_and_bounds_are_exact():
    """svie_order_stats_f32 against np.partition, svie_mesh_bounds against TriMesh.bounds."""
    rng = np.random.default_rng(3)
    cases = [rng.random(1), rng.random(2), rng.random(1001), np.round(rng.standard_normal(100000) * 10, 1),
             np.concatenate([np.zeros(40), -np.zeros(3), np.full(7, np.inf), -rng.random(20)]),
             rng.random(1 << 20) * 1e-3 + 0.5]
    ws = torch.empty(nat.lib().svie_order_stats_bytes(), dtype=torch.uint8, device="cuda")
    out = torch.empty(2, dtype=torch.float32, device="cuda")
    for x in cases:
        x = x.astype(np.float32)
        n = len(x)
        xd = torch.from_numpy(x).cuda()
        for k0, k1 in {(0, n - 1), (max(n // 2 - 1, 0), n // 2), (n - 1, n - 1), (n // 3, 0)}:
            nat.call("svie_order_stats_f32", nat.ptr(xd), n, k0, k1, nat.ptr(ws), ws.numel(), nat.ptr(out),
                     nat.stream())
            got = out.cpu().numpy()
            ref = np.partition(x, sorted({k0, k1}))
            assert got[0] == ref[k0] and got[1] == ref[k1], (n, k0, k1)
    with pytest.raises(nat.SvieError):
        nat.call("svie_order_stats_f32", nat.ptr(xd), n, n, 0, nat.ptr(ws), ws.numel(), nat.ptr(out), nat.stream())

    from svierosion_gb300.meshio import TriMesh
    bws = torch.empty(64, dtype=torch.uint8, device="cuda")
    bout = torch.empty(6, dtype=torch.float64, device="cuda")
    for v in (rng.standard_normal((1, 3)), rng.standard_normal((70001, 3)) * 1e3 - 5.0,
              np.abs(rng.standard_normal((999, 3))) + 1.0):
        vd = torch.from_numpy(v).cuda()
        nat.call("svie_mesh_bounds", nat.ptr(vd), len(v), nat.ptr(bws), bws.numel(), nat.ptr(bout), nat.stream())
        assert np.array_equal(bout.cpu().numpy().reshape(2, 3), TriMesh(v, np.zeros((0, 3))).bounds)
