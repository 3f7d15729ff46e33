"""Ball weights, the hand-written 3-D FFT and the N_r convolution."""

import json
import math

import numpy as np
import pytest
import torch

import oracle as O

pytestmark = pytest.mark.gpu

if torch.cuda.is_available():
    import svierosion_gb300 as S
    from svierosion_gb300 import svi
    from svierosion_gb300.grid import Grid


def test_ball_weights(golden):
    s = golden("svi_conv")
    np.testing.assert_allclose(svi.ball_cell_weights(1.0, 1 / 3.3), s["w_r33"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(svi.ball_cell_weights(0.1, 1 / 64), s["w_r64"], rtol=0, atol=1e-12)
    for ratio in (3.3, 8.0, 12.7):  # test_flows.py:41-44
        w = svi.ball_cell_weights(1.0, 1.0 / ratio)
        assert abs(w.sum() / ratio ** 3 / (4 * math.pi / 3) - 1.0) < 1e-4


@pytest.mark.parametrize("shape", [(16, 18, 20), (20, 21, 25), (27, 28, 30), (90, 90, 90), (45, 60, 49),
                                   (64, 48, 35), (40, 42, 36)])
def test_rfft_matches_numpy(shape):
    rng = np.random.default_rng(sum(shape))
    f = rng.standard_normal(shape).astype(np.float32)
    g = Grid((0.0, 0.0, 0.0), 1.0, shape)
    conv = S.BallConvolution(g, 2.0)
    spec = svi.rfftn(torch.from_numpy(f).cuda(), conv)
    ref = np.fft.rfftn(f.astype(np.float64))
    scale = np.abs(ref).max()
    assert np.abs(spec.cpu().numpy() - ref).max() < 2e-6 * scale * math.log2(f.size)
    back = svi.irfftn(spec, conv)
    assert np.abs(back.cpu().numpy() - f).max() < 2e-6 * math.log2(f.size) * np.abs(f).max()


def test_kernel_hat_and_exterior_fraction(golden):
    s = golden("svi_conv")
    shape = tuple(int(v) for v in s["shape"])
    g = Grid((0.0, 0.0, 0.0), float(s["h"]), shape)
    conv = S.BallConvolution(g, float(s["radius"]))
    assert conv.m == int(s["m"])
    assert abs(conv.quadrature_volume - float(s["quadrature_volume"])) < 1e-10
    kh = conv.kernel_hat.cpu().numpy()
    np.testing.assert_allclose(kh.real, s["khat_re"], atol=1e-4 * np.abs(s["khat_re"]).max())
    N = conv.exterior_fraction(torch.from_numpy(s["fractions"]).cuda())
    assert float(np.abs(N.cpu().numpy() - s["N"]).max()) < 2e-6
    # interior volume + exterior fraction consistency
    iv = conv.interior_volume(torch.from_numpy(s["fractions"]).cuda())
    np.testing.assert_allclose(1 - iv.cpu().numpy() / conv.ball_volume, N.cpu().numpy(), atol=2e-6)


@pytest.mark.parametrize("ratio,tol", [(8, 3e-4), (16, 6e-5)])
def test_sphere_exterior_fraction(ratio, tol):
    # known answer N_r = 1/2 + 3r/(16R) on a sphere (test_flows.py:46-56)
    R, r = 1.0, 0.4
    h = r / ratio
    ctr = np.array([0.0123, -0.0311, 0.0217])
    g = Grid.around([-R] * 3, [R] * 3, h, padding=r + 10 * h)
    X, Y, Z = [torch.tensor(a, device="cuda") for a in np.meshgrid(*g.axes(), indexing="ij")]
    phi = torch.sqrt((X - ctr[0]) ** 2 + (Y - ctr[1]) ** 2 + (Z - ctr[2]) ** 2) - R
    ls = S.LevelSet(phi.float(), g, width=6)
    conv = S.BallConvolution(g, r)
    N = conv.exterior_fraction(ls.dense_fractions())
    pts = ls.closest_points(ls.interface_nodes())
    from svierosion_gb300.levelset import tricubic
    vals = tricubic(N.view(-1), g.shape, pts)
    err = (vals - svi.sphere_exterior_fraction(r, R)).abs().max().item()
    assert err < tol


def test_flat_plane_is_one_half():
    # test_flows.py:58-75
    h, r = 0.05, 0.3
    g = Grid.around([-1] * 3, [1] * 3, h, padding=r + 10 * h)
    X, Y, Z = [torch.tensor(a, device="cuda") for a in np.meshgrid(*g.axes(), indexing="ij")]
    n = torch.tensor([0.3, -0.5, 0.81], dtype=torch.float64)
    n /= n.norm()
    lin = n[0] * X + n[1] * Y + n[2] * Z - 0.0131
    phi = torch.maximum(lin, torch.sqrt(X * X + Y * Y + Z * Z) - 0.9).float()
    ls = S.LevelSet(phi, g)
    conv = S.BallConvolution(g, r)
    N = conv.exterior_fraction(ls.dense_fractions())
    idx = ls.interface_nodes()
    x = g.node_coords(idx).cpu()
    keep = ((x @ n - 0.0131).abs() < 2 * h) & (x.norm(dim=1) < 0.45)
    from svierosion_gb300.levelset import tricubic
    vals = tricubic(N.view(-1), g.shape, ls.closest_points(idx[keep.to(idx.device)]))
    assert (vals - 0.5).abs().max().item() < 2e-4


def test_convolution_vs_oracle_float64():
    """N_r error of the float32 path against a float64 evaluation of the same discrete convolution."""
    R, h, r = 1.0, 0.05, 0.4
    g = Grid.around([-R] * 3, [R] * 3, h, padding=r + 10 * h)
    X, Y, Z = np.meshgrid(*g.axes(), indexing="ij")
    phi = (np.sqrt(X ** 2 + Y ** 2 + (Z / 0.8) ** 2) - R).astype(np.float32)
    band = O.rebuild_band(phi.reshape(-1).copy(), 6.0, h)
    f = O.dense_fractions(np.clip(phi.reshape(-1), -6 * h, 6 * h).astype(np.float32), band, g.shape).reshape(g.shape)
    w = O.ball_cell_weights(r, h)
    m = (w.shape[0] - 1) // 2
    kern = np.zeros(g.shape)
    ii = np.arange(-m, m + 1)
    kern[(ii % g.shape[0])[:, None, None], (ii % g.shape[1])[None, :, None], (ii % g.shape[2])[None, None, :]] = w
    g64 = np.fft.irfftn(np.fft.rfftn(f.astype(np.float64)) * np.fft.rfftn(kern), s=g.shape, axes=(0, 1, 2)) * h ** 3
    N64 = 1 - g64 / (4 / 3 * np.pi * r ** 3)
    conv = S.BallConvolution(g, r)
    N = conv.exterior_fraction(torch.from_numpy(f).cuda()).cpu().numpy()
    assert np.abs(N - N64).max() < 1e-5


def test_masked_convolution_matches_on_needed_lines():
    """The convolution that skips empty and unread lines gives bit-identical N
    on every (x, y) line a closest-point stencil can read."""
    from svierosion_gb300 import _native as nat
    from svierosion_gb300.evolve import LINE_DILATION
    R, h, r = 0.8, 0.04, 0.2
    g = Grid.around([-R, -R * 0.6, -R * 0.5], [R, R * 0.6, R * 0.5], h, padding=r + 12 * h)
    X, Y, Z = [torch.tensor(a, device="cuda") for a in np.meshgrid(*g.axes(), indexing="ij")]
    phi = (torch.sqrt(X ** 2 + (Y / 0.6) ** 2 + (Z / 0.5) ** 2) - R).float()
    ls = S.LevelSet(phi, g, width=6)
    conv = S.BallConvolution(g, r)
    nx, ny, nz = g.shape
    lf = torch.empty(nx * ny, dtype=torch.uint8, device="cuda")
    sf = torch.empty(nx, dtype=torch.uint8, device="cuda")
    tmp = torch.empty(nx * ny, dtype=torch.uint8, device="cuda")
    nat.call("svie_conv_line_flags", nat.ptr(ls.work32), ls.work32.numel(), nx, ny, nz, LINE_DILATION, nat.ptr(lf),
             nat.ptr(sf), nat.ptr(tmp), nat.stream())
    f = ls.dense_fractions()
    full = conv.exterior_fraction(f)
    masked = torch.full(g.shape, float("nan"), device="cuda")
    conv.exterior_fraction_into(f, masked, flags=(lf, sf))
    need = (lf.view(nx, ny) & 2).bool()
    band_lines = (lf.view(nx, ny) & 1).bool()
    assert need.any() and (~need).any() and bool((need | ~band_lines).all())
    assert torch.equal(masked[need], full[need])
    # every line holding a band node's closest-point stencil is flagged
    cp = ls.closest_points(ls.band)
    base = torch.floor(cp).long() - 1
    for dx in range(4):
        for dy in range(4):
            assert bool(need[base[:, 0] + dx, base[:, 1] + dy].all())


@pytest.mark.parametrize("shape", [(40, 42, 36), (64, 48, 35), (45, 60, 49)])
def test_every_pass_form_gives_the_same_bits(shape):
    """The launch forms of each pass (lines per CTA, persistent or not) run the same radix stages.
    Within a code family (every z form; the 8-line y and x forms) the convolution, the masked
    convolution and rfftn / irfftn are bit-identical under every combination, and a tuned shape
    keeps the fixed rule's family.  The one-line y and x forms agree to rounding."""
    import itertools
    from svierosion_gb300 import _native as nat
    rng = np.random.default_rng(sum(shape))
    g = Grid((0.0, 0.0, 0.0), 1.0, shape)
    f = torch.from_numpy(rng.random(shape, dtype=np.float32)).cuda()
    conv = S.BallConvolution(g, 3.0)
    nx, ny, nz = shape
    lf = torch.from_numpy((rng.random(nx * ny) < 0.5).astype(np.uint8) * 3).cuda()
    sf = torch.from_numpy(np.full(nx, 3, dtype=np.uint8)).cuda()

    def run():
        full = conv.exterior_fraction(f)
        masked = torch.zeros(shape, device="cuda")
        conv.exterior_fraction_into(f, masked, flags=(lf, sf))
        spec = svi.rfftn(f, conv)
        return full, masked, spec.clone(), svi.irfftn(spec, conv)

    def same(a, b):
        return torch.equal(torch.view_as_real(a) if a.is_complex() else a,
                           torch.view_as_real(b) if b.is_complex() else b)

    try:
        for family in ((0, 1), (2,)):
            ref = None
            for z, y, x in itertools.product(range(3), family, family):
                svi.set_fft_choice(shape, z, y, x)
                assert svi.fft_choice(shape) == {"z": z, "y": y, "x": x, "tuned": True}
                got = run()
                if ref is None:
                    ref = got
                    continue
                assert all(same(a, b) for a, b in zip(ref, got)), (z, y, x)
            if family == (0, 1):
                ref8 = ref
        # the one-line family agrees with the 8-line one to float32 rounding
        for a, b in zip(ref8, ref):
            a, b = (torch.view_as_real(t) if t.is_complex() else t for t in (a, b))
            assert float((a - b).abs().max()) <= 1e-5 * max(float(a.abs().max()), 1.0)
        # a form that does not exist is refused
        with pytest.raises(RuntimeError):
            nat.call("svie_conv_set_choice", nx, ny, nz, 3, 0, 0)
        # the tuner keeps the fixed rule's family: the same bits
        svi.set_fft_choice(shape, -1, -1, -1)
        assert not svi.fft_choice(shape)["tuned"]
        ws = conv.scratch.get("conv", conv.workspace_bytes)
        scratch_out = torch.empty(shape, device="cuda")
        nat.call("svie_conv_tune", nat.ptr(conv.plan), nx, ny, nz, nat.ptr(f.reshape(-1)), nat.ptr(scratch_out),
                 nat.ptr(ws), ws.numel(), 2, nat.stream())
        c = svi.fft_choice(shape)
        assert c["tuned"] and c["y"] in (0, 1) and c["x"] in (0, 1) and 0 <= c["z"] < 3
        assert all(same(a, b) for a, b in zip(ref8, run()))
    finally:
        svi.set_fft_choice(shape, -1, -1, -1)


def test_tuned_forms_are_kept_in_the_cache_file(tmp_path, monkeypatch):
    """With SVIE_FFT_TUNE_CACHE set, a tuned shape's forms go to the file, and a later first use of
    the shape takes them from there instead of timing the forms again."""
    from svierosion_gb300 import _native as nat
    shape = (48, 40, 36)
    cache = tmp_path / "forms.json"
    monkeypatch.setenv("SVIE_FFT_TUNE", "all")
    monkeypatch.setenv("SVIE_FFT_TUNE_CACHE", str(cache))
    g = Grid((0.0, 0.0, 0.0), 1.0, shape)
    f = torch.rand(shape, device="cuda")
    conv = S.BallConvolution(g, 3.0)
    try:
        svi.set_fft_choice(shape, -1, -1, -1)
        conv.exterior_fraction(f)
        tuned = svi.fft_choice(shape)
        assert tuned["tuned"] and cache.exists()
        table = json.loads(cache.read_text())
        assert list(table.values()) == [{k: tuned[k] for k in "zyx"}]
        svi.set_fft_choice(shape, -1, -1, -1)
        n0 = nat.lib().svie_launch_count()
        conv.exterior_fraction(f)
        assert nat.lib().svie_launch_count() - n0 == 5     # the five passes only: no timing
        assert svi.fft_choice(shape) == tuned
    finally:
        svi.set_fft_choice(shape, -1, -1, -1)


@pytest.mark.parametrize("shape", [(40, 42, 36), (64, 48, 35), (90, 84, 60), (112, 98, 70)])
def test_passes_compiled_for_the_axis_lengths_give_the_same_bits(shape):
    """The y and x passes compiled at run time for the shape's axis lengths (svie_conv_jit) give the
    library's own passes' bits for the convolution, the masked convolution and rfftn / irfftn."""
    from svierosion_gb300 import _native as nat
    rng = np.random.default_rng(sum(shape) + 1)
    g = Grid((0.0, 0.0, 0.0), 1.0, shape)
    f = torch.from_numpy(rng.random(shape, dtype=np.float32)).cuda()
    conv = S.BallConvolution(g, 3.0)
    nx, ny, nz = shape
    lf = torch.from_numpy((rng.random(nx * ny) < 0.5).astype(np.uint8) * 3).cuda()
    sf = torch.from_numpy(np.full(nx, 3, dtype=np.uint8)).cuda()

    def run():
        full = conv.exterior_fraction(f)
        masked = torch.zeros(shape, device="cuda")
        conv.exterior_fraction_into(f, masked, flags=(lf, sf))
        spec = svi.rfftn(f, conv)
        return [full, masked, torch.view_as_real(spec).clone(), svi.irfftn(spec, conv)]

    lib = nat.lib()
    try:
        svi.set_fft_choice(shape, 0, 1, 0)
        assert not lib.svie_conv_jit_enabled(nx, ny, nz)
        ref = run()
        nat.call("svie_conv_jit", nx, ny, nz)
        assert lib.svie_conv_jit_enabled(nx, ny, nz)
        nat.call("svie_conv_jit_wait", 120000)
        assert lib.svie_conv_jit_ready(nx, ny, nz)
        got = run()
        for a, b in zip(ref, got):
            assert torch.equal(a, b)
        assert lib.svie_conv_tma_timeouts() == 0
    finally:
        svi.set_fft_choice(shape, -1, -1, -1)
