"""The allocation-free volume entry point, called through the C ABI.

svie_band_volume_noalloc serves callers that cannot allocate device memory
(a plugin inside a host framework that owns every device allocation, or a
loop that forbids cudaMalloc after start-up): its scratch is a static device
array instead of a caller workspace.  It must give the same result as
svie_band_volume with a workspace, on consecutive calls that reuse the
static array.  This file is collected last so that a failure here leaves
every other test already run.
"""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _stats_tensor():
    from svierosion_gb300 import _native as nat
    return torch.zeros(nat.STATS_BYTES, dtype=torch.uint8, device="cuda")


def _read(t):
    from svierosion_gb300 import _native as nat
    return np.frombuffer(t.cpu().numpy().tobytes(), dtype=nat.STATS_DTYPE)[0]


def _level_set(h=0.03):
    import svierosion_gb300 as S
    from svierosion_gb300.grid import Grid
    g = Grid.around([-1.0] * 3, [1.0] * 3, h, padding=12 * h)
    ax = [torch.tensor(a, device="cuda", dtype=torch.float32) for a in g.axes()]
    X, Y, Z = torch.meshgrid(*ax, indexing="ij")
    phi = torch.sqrt(X ** 2 + (Y / 0.8) ** 2 + (Z / 0.6) ** 2) - 0.9
    return S.LevelSet(phi, g, width=6)


def test_noalloc_volume_matches_workspace_version():
    from svierosion_gb300 import _native as nat
    lib = nat.load()
    ls = _level_set()
    band = ls.band32
    m = band.numel()
    assert 0 < m <= lib.svie_band_volume_noalloc_max()
    st = ls.strides
    ws = torch.empty(lib.svie_volume_workspace_bytes(m), dtype=torch.uint8, device="cuda")
    ref_stats = _stats_tensor()
    ref_occ = ls.dense_fractions().reshape(-1).clone()
    nat.check(lib.svie_band_volume(nat.ptr(ls.flat), nat.ptr(band), m, *st, nat.ptr(ref_occ), nat.ptr(ws),
                                   ws.numel(), nat.ptr(ref_stats), nat.stream()))
    ref = _read(ref_stats)
    for call in range(2):  # two calls in a row share the static scratch
        out_stats = _stats_tensor()
        occ = ls.dense_fractions().reshape(-1).clone()
        nat.check(lib.svie_band_volume_noalloc(nat.ptr(ls.flat), nat.ptr(band), m, *st, nat.ptr(occ),
                                               nat.ptr(out_stats), nat.stream()))
        got = _read(out_stats)
        assert got["fsum"] == ref["fsum"], (call, got["fsum"], ref["fsum"])
        assert (got["any_neg"], got["any_pos"], got["n_band"]) == (ref["any_neg"], ref["any_pos"], ref["n_band"])
        assert torch.equal(occ, ref_occ)
    # the volume through the level set agrees with the solid volume of the ellipsoid
    vol = (ls.static_inside + float(ref["fsum"])) * ls.h ** 3
    exact = 4.0 / 3.0 * np.pi * 0.9 * 0.72 * 0.54
    assert abs(vol - exact) < 2e-3 * exact


def test_noalloc_rejects_sizes_beyond_the_static_scratch():
    from svierosion_gb300 import _native as nat
    lib = nat.load()
    stats = _stats_tensor()
    too_many = lib.svie_band_volume_noalloc_max() + 1
    # no field or band is passed: the size check comes before any pointer is
    # used, so the call cannot reach device memory even if the check broke
    rc = lib.svie_band_volume_noalloc(None, None, too_many, 1 << 20, 1 << 10, 1, None, nat.ptr(stats), nat.stream())
    assert rc == 6  # SVIE_ERR_CAPACITY, before anything is launched
    assert b"static scratch limit" in lib.svie_last_error()
