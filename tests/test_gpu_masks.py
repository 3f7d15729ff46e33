"""Dense-mask kernels through the C ABI: box dilation, the reinitialisation work mask and the
order-preserving compactions (flat order and brick order), bit-exact against numpy.

Shapes are odd and smaller or larger than one compaction tile (4096 nodes) and one dilation tile
(16 x 16 x 64), so partial tiles, partial warps and grid edges are all exercised.
"""

import numpy as np
import pytest
import torch

import oracle as O

pytestmark = pytest.mark.gpu

if torch.cuda.is_available():
    from svierosion_gb300 import _native as nat
    from svierosion_gb300.levelset import dilate

SHAPES = [(5, 7, 3), (37, 29, 83), (70, 50, 130), (19, 41, 245)]


def _mask(shape, density, seed):
    rng = np.random.default_rng(seed)
    return rng.random(shape) < density


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("steps", [0, 1, 3, 8, 9])
def test_dilate_matches_oracle(shape, steps):
    m = _mask(shape, 0.002, 1)
    m.reshape(-1)[0] = True  # a seed on the grid corner
    ref = O.dilate(m, steps)
    got = dilate(torch.from_numpy(m).cuda(), steps).cpu().numpy()
    assert np.array_equal(got, ref)
    # in place (mask == out)
    t = torch.from_numpy(m.astype(np.uint8)).cuda()
    tmp = torch.empty_like(t)
    nx, ny, nz = shape
    nat.call("svie_dilate", nat.ptr(t), nx, ny, nz, steps, nat.ptr(t), nat.ptr(tmp), nat.stream())
    assert np.array_equal(t.cpu().numpy().astype(bool), ref)


@pytest.mark.parametrize("shape", SHAPES[1:])
@pytest.mark.parametrize("dilation,margin", [(3, 4), (1, 0), (9, 4)])
def test_reinit_work_mask(shape, dilation, margin):
    n = int(np.prod(shape))
    rng = np.random.default_rng(2)
    band = np.sort(rng.choice(n, size=n // 50, replace=False)).astype(np.int32)
    m = np.zeros(n, bool)
    m[band] = True
    ref = O.dilate(m.reshape(shape), dilation)
    if margin:
        for ax in range(3):
            sl = [slice(None)] * 3
            sl[ax] = slice(0, margin)
            ref[tuple(sl)] = False
            sl[ax] = slice(shape[ax] - margin, shape[ax])
            ref[tuple(sl)] = False
    out = torch.empty(n, dtype=torch.uint8, device="cuda")
    tmp = torch.empty(n, dtype=torch.uint8, device="cuda")
    b = torch.from_numpy(band).cuda()
    nat.call("svie_reinit_mask", nat.ptr(b), band.size, *shape, dilation, margin, nat.ptr(out), nat.ptr(tmp),
             nat.stream())
    assert np.array_equal(out.cpu().numpy().reshape(shape).astype(bool), ref)


@pytest.mark.parametrize("shape", SHAPES[1:])
@pytest.mark.parametrize("dilation,margin", [(3, 4), (1, 0), (9, 4), (0, 0)])
def test_reinit_bits_match_byte_mask(shape, dilation, margin):
    """The bit-packed work mask lists the same nodes, in the same brick order, as the byte mask."""
    n = int(np.prod(shape))
    nx, ny, nz = shape
    rng = np.random.default_rng(4)
    band = torch.from_numpy(np.sort(rng.choice(n, size=n // 40, replace=False)).astype(np.int32)).cuda()
    lib = nat.lib()
    mask = torch.empty(n, dtype=torch.uint8, device="cuda")
    tmp = torch.empty(n, dtype=torch.uint8, device="cuda")
    nat.call("svie_reinit_mask", nat.ptr(band), band.numel(), nx, ny, nz, dilation, margin, nat.ptr(mask),
             nat.ptr(tmp), nat.stream())
    nb = lib.svie_reinit_bits_bytes(nx, ny, nz)
    bits = torch.empty(nb // 4, dtype=torch.int32, device="cuda")
    btmp = torch.empty_like(bits)
    marked = torch.empty_like(bits)
    nat.call("svie_reinit_bits", nat.ptr(band), band.numel(), nx, ny, nz, dilation, margin, nat.ptr(bits),
             nat.ptr(btmp), nat.ptr(marked), nat.stream())
    # the band's own bits, kept in `marked`
    mw = marked.cpu().numpy().view(np.uint32).reshape(nx, ny, -1)
    zz = np.arange(nz)
    own = ((mw[:, :, zz // 32] >> (zz % 32).astype(np.uint32)) & 1).astype(bool).reshape(-1)
    assert np.array_equal(np.flatnonzero(own), np.sort(band.cpu().numpy()))
    # unpack: bit z % 32 of word z // 32 of row (x, y)
    w = bits.cpu().numpy().view(np.uint32).reshape(nx, ny, -1)
    z = np.arange(nz)
    unpacked = (w[:, :, z // 32] >> (z % 32).astype(np.uint32)) & 1
    assert np.array_equal(unpacked.astype(bool), mask.cpu().numpy().reshape(shape).astype(bool))
    # no bits past nz
    if nz % 32:
        assert not (w[:, :, -1] >> np.uint32(nz % 32)).any()
    bws = torch.empty(lib.svie_brick_workspace_bytes(nx, ny, nz), dtype=torch.uint8, device="cuda")
    lists = []
    for kind, src in ((0, mask), (2, bits)):
        cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
        nat.call("svie_brick_scan", kind, nat.ptr(src), nx, ny, nz, 0.0, nat.ptr(bws), bws.numel(), nat.ptr(cnt),
                 nat.stream())
        k = int(cnt.item())
        out = torch.full((max(k, 1),), -1, dtype=torch.int32, device="cuda")
        nat.call("svie_brick_write", kind, nat.ptr(src), nx, ny, nz, 0.0, nat.ptr(bws), bws.numel(), nat.ptr(out), k,
                 nat.stream())
        lists.append(out[:k].cpu().numpy())
    assert np.array_equal(lists[0], lists[1])
    ref = np.flatnonzero(mask.cpu().numpy())
    assert np.array_equal(lists[1], _brick_order(ref, shape))


def _brick_order(idx, shape):
    nx, ny, nz = shape
    x, r = np.divmod(idx, ny * nz)
    y, z = np.divmod(r, nz)
    key = np.lexsort((z % 16, y % 4, x % 4, z // 16, y // 4, x // 4))
    return idx[key]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("density", [0.0, 0.01, 0.3, 1.0])
def test_mask_and_brick_compaction(shape, density):
    m = _mask(shape, density, 3)
    n = m.size
    nx, ny, nz = shape
    t = torch.from_numpy(m.astype(np.uint8)).cuda().view(-1)
    lib = nat.lib()
    ws = torch.empty(lib.svie_band_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    nat.call("svie_mask_scan", nat.ptr(t), n, nat.ptr(ws), ws.numel(), nat.ptr(cnt), nat.stream())
    k = int(cnt.item())
    ref = np.flatnonzero(m.reshape(-1))
    assert k == ref.size
    out = torch.full((max(k, 1),), -1, dtype=torch.int32, device="cuda")
    nat.call("svie_mask_write", nat.ptr(t), n, nat.ptr(ws), ws.numel(), nat.ptr(out), k, nat.stream())
    assert np.array_equal(out[:k].cpu().numpy(), ref)
    # selection of values in the same order
    vals = torch.arange(n, dtype=torch.int32, device="cuda") * 3 + 1
    sel = torch.full((max(k, 1),), -1, dtype=torch.int32, device="cuda")
    nat.call("svie_mask_select", nat.ptr(t), nat.ptr(vals), n, nat.ptr(ws), ws.numel(), nat.ptr(sel), k, nat.stream())
    assert np.array_equal(sel[:k].cpu().numpy(), ref * 3 + 1)
    # brick order, mask kind
    bws = torch.empty(lib.svie_brick_workspace_bytes(nx, ny, nz), dtype=torch.uint8, device="cuda")
    nat.call("svie_brick_scan", 0, nat.ptr(t), nx, ny, nz, 0.0, nat.ptr(bws), bws.numel(), nat.ptr(cnt), nat.stream())
    assert int(cnt.item()) == ref.size
    bout = torch.full((max(k, 1),), -1, dtype=torch.int32, device="cuda")
    nat.call("svie_brick_write", 0, nat.ptr(t), nx, ny, nz, 0.0, nat.ptr(bws), bws.numel(), nat.ptr(bout), k,
             nat.stream())
    assert np.array_equal(bout[:k].cpu().numpy(), _brick_order(ref, shape))


@pytest.mark.parametrize("shape", SHAPES[1:])
def test_band_scan_write_and_info(shape):
    rng = np.random.default_rng(4)
    h = np.float32(0.05)
    phi = (rng.standard_normal(shape) * 0.4).astype(np.float32)
    n = phi.size
    nx, ny, nz = shape
    width = 6.0
    cap = np.float32(width * h)
    thresh = np.float32(width * h * (1 - 1e-5))
    clamped = np.clip(phi, -cap, cap)
    sel = np.abs(clamped) < thresh
    ref = np.flatnonzero(sel.reshape(-1))
    neg = clamped < 0
    t = torch.from_numpy(phi).cuda().view(-1)
    lib = nat.lib()
    ws = torch.empty(lib.svie_band_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    info = torch.zeros(nat.BAND_INFO_BYTES, dtype=torch.uint8, device="cuda")
    nat.call("svie_band_scan", nat.ptr(t), n, float(cap), float(thresh), nat.ptr(ws), ws.numel(), nat.ptr(info),
             nat.stream())
    k = int(np.frombuffer(info.cpu().numpy().tobytes(), dtype=nat.BAND_INFO_DTYPE)[0]["count"])
    assert k == ref.size
    assert np.array_equal(t.cpu().numpy().reshape(shape), clamped)  # clamped in place
    band = torch.empty(k, dtype=torch.int32, device="cuda")
    occ = torch.empty(n, dtype=torch.float32, device="cuda")
    nat.call("svie_band_write", nat.ptr(t), nx, ny, nz, float(thresh), nat.ptr(ws), ws.numel(), nat.ptr(band), k,
             nat.ptr(occ), nat.ptr(info), nat.stream())
    assert np.array_equal(band.cpu().numpy(), ref)
    assert np.array_equal(occ.cpu().numpy().reshape(shape), neg.astype(np.float32))
    d = np.frombuffer(info.cpu().numpy().tobytes(), dtype=nat.BAND_INFO_DTYPE)[0]
    coords = np.argwhere(sel)
    icoords = np.argwhere(neg)
    assert int(d["static_inside"]) == int((neg & ~sel).sum())
    assert list(d["lo"]) == list(coords.min(0)) and list(d["hi"]) == list(coords.max(0))
    assert list(d["ilo"]) == list(icoords.min(0)) and list(d["ihi"]) == list(icoords.max(0))
    # brick-ordered band list (|phi| < thresh)
    bws = torch.empty(lib.svie_brick_workspace_bytes(nx, ny, nz), dtype=torch.uint8, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    nat.call("svie_brick_scan", 1, nat.ptr(t), nx, ny, nz, float(thresh), nat.ptr(bws), bws.numel(), nat.ptr(cnt),
             nat.stream())
    assert int(cnt.item()) == k
    bout = torch.empty(k, dtype=torch.int32, device="cuda")
    nat.call("svie_brick_write", 1, nat.ptr(t), nx, ny, nz, float(thresh), nat.ptr(bws), bws.numel(), nat.ptr(bout),
             k, nat.stream())
    assert np.array_equal(bout.cpu().numpy(), _brick_order(ref, shape))


@pytest.mark.parametrize("shape", SHAPES[1:])
def test_brick_band_scan_write(shape):
    """The brick-ordered rebuild (clamp, list, occupancy, info) equals the ascending one reordered."""
    rng = np.random.default_rng(5)
    h = np.float32(0.05)
    phi = (rng.standard_normal(shape) * 0.4).astype(np.float32)
    phi.reshape(-1)[7] = np.nan  # NaN stays NaN and is not in the band
    nx, ny, nz = shape
    cap = np.float32(6.0 * h)
    thresh = np.float32(6.0 * h * (1 - 1e-5))
    clamped = np.where(np.isnan(phi), phi, np.clip(phi, -cap, cap))
    with np.errstate(invalid="ignore"):
        sel = np.abs(clamped) < thresh
        neg = clamped < 0
    ref = _brick_order(np.flatnonzero(sel.reshape(-1)), shape)
    t = torch.from_numpy(phi).cuda().view(-1)
    lib = nat.lib()
    bws = torch.empty(lib.svie_brick_workspace_bytes(nx, ny, nz), dtype=torch.uint8, device="cuda")
    info = torch.zeros(nat.BAND_INFO_BYTES, dtype=torch.uint8, device="cuda")
    nat.call("svie_brick_band_scan", nat.ptr(t), nx, ny, nz, float(cap), float(thresh), nat.ptr(bws), bws.numel(),
             nat.ptr(info), nat.stream())
    k = int(np.frombuffer(info.cpu().numpy().tobytes(), dtype=nat.BAND_INFO_DTYPE)[0]["count"])
    assert k == ref.size
    got_phi = t.cpu().numpy().reshape(shape)
    assert np.array_equal(got_phi, clamped, equal_nan=True)
    out = torch.empty(k, dtype=torch.int32, device="cuda")
    occ = torch.empty(phi.size, dtype=torch.float32, device="cuda")
    nat.call("svie_brick_band_write", nat.ptr(t), nx, ny, nz, float(thresh), nat.ptr(bws), bws.numel(),
             nat.ptr(out), k, nat.ptr(occ), nat.ptr(info), nat.stream())
    assert np.array_equal(out.cpu().numpy(), ref)
    assert np.array_equal(occ.cpu().numpy().reshape(shape), neg.astype(np.float32))
    d = np.frombuffer(info.cpu().numpy().tobytes(), dtype=nat.BAND_INFO_DTYPE)[0]
    coords, icoords = np.argwhere(sel), np.argwhere(neg)
    assert int(d["static_inside"]) == int((neg & ~sel).sum())
    assert list(d["lo"]) == list(coords.min(0)) and list(d["hi"]) == list(coords.max(0))
    assert list(d["ilo"]) == list(icoords.min(0)) and list(d["ihi"]) == list(icoords.max(0))


def test_levelset_band_views_agree():
    """LevelSet keeps the brick-ordered work list; its ascending band is the same node set, sorted,
    and stays the band of the last rebuild while phi changes."""
    from svierosion_gb300.grid import Grid
    from svierosion_gb300.levelset import LevelSet

    n, h = 48, 0.05
    ax = (np.arange(n) - 0.5 * (n - 1)) * h
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    phi = (np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - 0.6).astype(np.float32)
    ls = LevelSet(torch.from_numpy(phi).cuda(), Grid((float(ax[0]),) * 3, h, (n, n, n)), width=6)
    work = ls.work32.cpu().numpy()
    ls.flat[ls.work32.long()] += 0.3 * h  # values move; the band set must not
    band = ls.band32.cpu().numpy()
    assert np.array_equal(band, np.sort(work))
    ref = np.flatnonzero(np.abs(np.clip(phi, -6 * h, 6 * h)) < np.float32(6 * h * (1 - 1e-5)))
    assert np.array_equal(band, ref)
    # band values through the library's gather equal phi at the band
    assert np.array_equal(ls.band_values().cpu().numpy(), ls.flat.cpu().numpy()[band])
