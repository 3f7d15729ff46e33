"""CUDA kernels against the reference fixtures and the numpy oracle.

Tolerances: integer / index / mask results bit-exact; float32 stencils within a
few float32 ulps of the values (the GPU contracts multiply-adds into FMAs, the
reference does not); float64 ball weights to 1e-12.
"""

import numpy as np
import pytest
import torch

import oracle as O

pytestmark = pytest.mark.gpu

if torch.cuda.is_available():
    import svierosion_gb300 as S
    from svierosion_gb300 import kernels as K
    from svierosion_gb300 import _native as nat
    from svierosion_gb300.grid import Grid


def _close(a, b, atol, rtol=0.0):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    err = np.abs(a - b)
    assert np.all(err <= atol + rtol * np.abs(b)), f"max err {float(err.max())}"


def _cuda(x, dtype=None):
    t = torch.as_tensor(np.ascontiguousarray(x)).cuda()
    return t if dtype is None else t.to(dtype)


@pytest.fixture(scope="module")
def sphere(golden):
    d = golden("kernels_sphere")
    shape = tuple(int(v) for v in d["shape"])
    grid = Grid(tuple(float(v) for v in d["origin"]), float(d["h"]), shape)
    return d, grid


def test_library_loaded_from_tree():
    lib = nat.load()
    assert lib.svie_version() == 1
    assert nat.LIB_PATH.parent.name == "svierosion_gb300"


def test_band_bit_exact(sphere):
    d, grid = sphere
    ls = S.LevelSet(_cuda(d["phi_in"]), grid, width=6)
    assert np.array_equal(ls.band.cpu().numpy(), d["band"])
    _close(ls.phi, d["phi"], 0)
    # static count of inside nodes off the band and the float64 volume
    assert abs(ls.volume() - float(d["volume"])) < 1e-7 * abs(float(d["volume"]))


def test_band_threshold_edge_cases():
    # float32(6h) can round below the float64 cap (test_geometry.py:98-107)
    h = 0.0075
    g = Grid((0.0, 0.0, 0.0), h, (24, 24, 24))
    phi = torch.full(g.shape, 6.0, dtype=torch.float32) * h
    phi[12, 12, 12] = -h
    ls = S.LevelSet(phi.cuda(), g, width=6.0)
    ref = O.rebuild_band((torch.full(g.shape, 6.0) * h).numpy().reshape(-1).copy(), 6.0, h)
    assert ls.band.numel() < 30
    # values exactly at the float32 threshold and one ulp either side
    t32 = np.float32(6 * h * (1 - 1e-5))
    vals = np.array([np.nextafter(t32, 0, dtype=np.float32), t32, np.nextafter(t32, 1, dtype=np.float32)])
    p = np.full(g.shape, np.float32(6 * h), dtype=np.float32)
    p[8, 8, 8:11] = vals
    p[16, 16, 8:11] = -vals
    p[12, 12, 12] = -h
    ls = S.LevelSet(torch.from_numpy(p).cuda(), g, width=6.0)
    assert np.array_equal(ls.band.cpu().numpy(), O.rebuild_band(p.reshape(-1).copy(), 6.0, h))


def test_margin_error():
    g = Grid((0.0, 0.0, 0.0), 0.1, (20, 20, 20))
    phi = torch.full(g.shape, 0.6)
    phi[2, 10, 10] = -0.05
    with pytest.raises(RuntimeError, match="grid boundary"):
        S.LevelSet(phi.cuda(), g, width=6.0)


def test_empty_band():
    g = Grid((0.0, 0.0, 0.0), 0.1, (16, 16, 16))
    ls = S.LevelSet(torch.full(g.shape, 0.6).cuda(), g, width=6.0)
    assert ls.band.numel() == 0
    assert ls.volume() == 0.0
    assert not ls.has_interface()


def test_stencil_kernels(sphere):
    d, grid = sphere
    flat = _cuda(d["phi"]).view(-1)
    idx = _cuda(d["band"])
    st = grid.strides
    nx, ny, nz = grid.shape
    h = float(d["h"])
    _close(K.godunov_inward(flat, idx, *st, 1.0 / h), d["godunov"], 2e-5, 2e-6)
    _close(K.cell_fractions(flat, idx, *st), d["fractions"], 2e-6)
    cp = K.closest_points(flat, idx, ny, nz, nx - 3.001, ny - 3.001, nz - 3.001, h)
    _close(cp, d["closest"], 2e-5)
    ref_cp = _cuda(d["closest"])
    _close(K.tricubic(flat, ny, nz, ref_cp), d["tricubic"], 2e-6)
    v, g = K.tricubic_with_gradient(flat, ny, nz, ref_cp)
    _close(v, d["tricubic_val"], 2e-6)
    _close(g, d["tricubic_grad"], 2e-6)
    _close(K.trilinear(flat, ny, nz, ref_cp), d["trilinear"], 2e-6)
    k1, k2 = K.principal_curvatures(flat, idx, *st, h)
    # H and K are well conditioned; k1,2 = H +- sqrt(H^2 - K) lose digits near
    # umbilic points (on this near-sphere), so they are checked against their scale
    H, Kg = 0.5 * (k1 + k2), k1 * k2
    _close(H, 0.5 * (d["k1"] + d["k2"]), 1e-4, 1e-5)
    _close(Kg, d["k1"] * d["k2"], 1e-3, 1e-5)
    kscale = float(np.abs(d["k1"]).max())
    _close(k1, d["k1"], 1e-4 * kscale)
    _close(k2, d["k2"], 1e-4 * kscale)
    assert np.array_equal(K.interface_mask(flat, idx, *st).cpu().numpy(), d["interface"])
    geo = K.reinit_geometry(flat, idx, *st, h, 0.45)
    _close(geo[0], d["geo_sgn"], 0)
    _close(geo[1], d["geo_dtau"], 1e-7)
    flags = np.stack([geo[2 + 4 * a + j].cpu().numpy() for j in (0, 1) for a in range(3)])
    assert np.array_equal(flags, d["geo_flags"])
    _close(K.reinit_rhs(flat, idx, *st, h, geo[0], *geo[2:]), d["reinit_rhs"], 2e-5)
    pts = _cuda(d["pts"])
    _close(K.tricubic(flat, ny, nz, pts), d["tricubic_pts"], 2e-6)
    _close(K.trilinear(flat, ny, nz, pts), d["trilinear_pts"], 2e-6)


def test_interface_nodes_and_dense_fractions(sphere):
    d, grid = sphere
    ls = S.LevelSet(_cuda(d["phi"]), grid, width=6)
    ref = d["band"][d["interface"]]
    assert np.array_equal(ls.interface_nodes().cpu().numpy(), ref)
    _close(ls.dense_fractions().view(-1), d["dense_fractions"].reshape(-1), 2e-6)


def test_cube_plane_fraction(golden):
    c = golden("cube_plane")
    a = _cuda(c["a"])
    f = K.cube_plane_fraction(_cuda(c["s"]), a[:, 0], a[:, 1], a[:, 2])
    _close(f, c["f"], 2e-6)
    # degenerate normals (test_geometry.py:130-138)
    s = torch.linspace(-1, 1, 101).cuda()
    one, zero = torch.ones_like(s), torch.zeros_like(s)
    _close(K.cube_plane_fraction(s, one, zero, zero), (0.5 - s).clamp(0, 1).cpu().numpy(), 1e-6)
    r = 2 ** -0.5 * one
    assert torch.isfinite(K.cube_plane_fraction(s, r, r, zero)).all()


def test_point_triangle_distance():
    rng = np.random.default_rng(5)
    p, a, b, c = (rng.normal(size=(4096, 3)).astype(np.float32) for _ in range(4))
    got = K.point_triangle_distance2(*(_cuda(x) for x in (p, a, b, c)))
    _close(got, O.point_triangle_distance2(p, a, b, c), 1e-5, 1e-5)


def test_laws_elementwise():
    N = torch.linspace(-0.1, 1.1, 4001).cuda()
    for law, ref in ((S.SVIPowerLaw(0.1, 1, 1, 0.93), O.SVILaw(0.1, 1, 1, 0.93)),
                     (S.SVIPowerLaw(0.1, 2, 1, 0.95), O.SVILaw(0.1, 2, 1, 0.95)),
                     (S.SVIPowerLaw(0.1, 0, 0), O.SVILaw(0.1, 0, 0))):
        assert law.n_cap == ref.n_cap
        n = N.cpu().numpy()
        _close(law.speed(N), ref.speed(n), 1e-6, 1e-5)
        _close(law.dspeed(N), ref.dspeed(n), 1e-5, 1e-4)
    k1 = torch.linspace(-5, 5, 1001).cuda()
    k2 = torch.flip(k1, [0]) * 0.5
    for law, ref in ((S.MeanCurvatureLaw(1.0), O.CurvatureLaw("mean", 1.0)),
                     (S.GaussCurvatureLaw(0.25, delta=1e-2), O.CurvatureLaw("gauss", 0.25, delta=1e-2))):
        V, D = law.speed_and_diffusivity(k1, k2)
        Vr, Dr = ref.speed_and_diffusivity(k1.cpu().numpy(), k2.cpu().numpy())
        _close(V, Vr, 1e-5, 1e-5)
        _close(D, Dr, 1e-5, 1e-4)


def test_sdf_slices_do_not_change_results():
    """svie_sdf_near_field and svie_sdf_crossings split a group of 32 triangles over `slices`
    warps; the node keys and crossing counters are the same for any split (coarse cube
    triangles, which cover many lines and nodes, and a fine fragment)."""
    from svierosion_gb300 import shapes
    from svierosion_gb300.sdf import device_mesh

    for mesh, res in ((shapes.cube(1.0), 40), (shapes.fragment(3, seed=1), 48)):
        params = S.ErosionParams(law="svi", radius=0.1, k=1, s=1, t=0.93, resolution=res)
        g = S.make_grid(mesh, params)
        nx, ny, nz = g.shape
        tri64, tri32, _ = device_mesh(mesh).tri_index(g)
        T = tri64.shape[0]
        keys, accs = [], []
        for slices in (1, 7, 32):
            k = torch.empty(g.size, dtype=torch.int64, device="cuda")
            nat.call("svie_sdf_keys_init", nat.ptr(k), g.size, nat.stream())
            nat.call("svie_sdf_near_field", nat.ptr(tri32), nat.ptr(tri64), T, nx, ny, nz, 2.0,
                     nat.f32(2.0 * (1 + 1e-6)), slices, nat.ptr(k), nat.stream())
            keys.append(k.cpu().numpy())
            acc = torch.zeros((nx + 1) * ny * nz, dtype=torch.int32, device="cuda")
            nat.call("svie_sdf_crossings", nat.ptr(tri64), T, nx, ny, nz, 0, 1, slices * 3, nat.ptr(acc),
                     nat.stream())
            accs.append(acc.cpu().numpy())
        assert (keys[0] != np.iinfo(np.int64).max).any() and accs[0].any()
        for k, a in zip(keys[1:], accs[1:]):
            assert np.array_equal(k, keys[0]) and np.array_equal(a, accs[0])


def test_reinit_sweep_lists_cover_every_entry():
    """One pseudo-time iteration of svie_reinit_iterate, whose sweeps walk the plain and general entry
    lists of the packed geometry, against the same iteration composed from reinit_rhs (the general
    formula at every entry) and the array form's dtau: every work-set entry is updated once, with its
    sign (entries with phi0 exactly 0 included), and nothing off the work set changes."""
    shape = (40, 36, 44)
    nx, ny, nz = shape
    h = 0.05
    ax = [np.arange(n) * h for n in shape]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    phi = (np.sqrt((X - 1.0) ** 2 + (Y - 0.9) ** 2 + (Z - 1.1) ** 2) - 0.62).astype(np.float32)
    coords = np.stack(np.meshgrid(*[np.arange(n) for n in shape], indexing="ij"))
    inner = np.all([(coords[a] >= 2) & (coords[a] <= shape[a] - 3) for a in range(3)], axis=0)
    work = np.flatnonzero((np.abs(phi) < 4 * h) & inner)
    planted = work[::97]
    phi.reshape(-1)[planted] = 0.0              # sign-less entries: the general path
    flat = _cuda(phi.reshape(-1))
    idx = _cuda(work.astype(np.int32))
    m, n = idx.numel(), flat.numel()
    sx, sy = ny * nz, nz
    geo = K.reinit_geometry(flat, idx, sx, sy, 1, h, 0.45)
    sgn, dtau = geo[0], geo[1]
    assert int((sgn == 0).sum()) >= len(planted)
    a = flat.clone()
    b = torch.empty_like(a)
    nat.call("svie_reinit_iterate", nat.ptr(a), nat.ptr(b), n, nat.ptr(idx), m, sx, sy, 1, h, nat.ptr(geo.packed),
             1, nat.stream())
    i = idx.long()
    a2, b2 = flat.clone(), flat.clone()
    b2[i] = a2[i] + dtau * K.reinit_rhs(a2, idx, sx, sy, 1, h, sgn, *geo[2:])
    a2[i] = 0.5 * (a2[i] + b2[i] + dtau * K.reinit_rhs(b2, idx, sx, sy, 1, h, sgn, *geo[2:]))
    off = torch.ones(n, dtype=torch.bool, device="cuda")
    off[i] = False
    assert torch.equal(a[off], flat[off])
    assert torch.equal(a[_cuda(planted)], flat[_cuda(planted)])
    _close(a[i], a2[i].cpu().numpy(), 2e-6 * float(flat[i].abs().max()))
    assert float((a[i] - flat[i]).abs().max()) > 1e-4   # the iteration moved the level set
