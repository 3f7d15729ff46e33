"""One fused RHS stage (statistics and device time step included) against the oracle, for every law of the
precision study: svi k0 s0, svi k1 s1 t0.93, svi k2 s1 t0.95, mean curvature alpha 1, Gauss curvature
alpha 0.25 (automatic delta).

Tolerances: L = V |grad phi| within 2e-4 of max |L| (N_r from a different FFT summation order enters V
through V'(N) up to ~10 near t); statistics within 1e-4 relative; the device time step within 1e-4.
"""

import math

import numpy as np
import pytest
import torch

import oracle as O

pytestmark = pytest.mark.gpu

if torch.cuda.is_available():
    import svierosion_gb300 as S
    from svierosion_gb300 import _native as nat
    from svierosion_gb300.grid import Grid

LAWS = [
    ("svi", dict(radius=0.2, k=0, s=0)),
    ("svi", dict(radius=0.2, k=1, s=1, t=0.93)),
    ("svi", dict(radius=0.2, k=2, s=1, t=0.95)),
    ("mean", dict(alpha=1.0)),
    ("gauss", dict(alpha=0.25)),
]


def _ellipsoid(n=64, h=0.05):
    ax = (np.arange(n) - 0.5 * (n - 1)) * h
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    phi = ((np.sqrt(X ** 2 + (Y / 0.7) ** 2 + (Z / 0.5) ** 2) - 0.9) * 0.6).astype(np.float32)
    return phi, Grid(tuple(float(ax[0]) for _ in range(3)), h, (n, n, n))


@pytest.mark.parametrize("kind,kw", LAWS, ids=[f"{k}-{'-'.join(f'{a}{b}' for a, b in kw.items())}" for k, kw in LAWS])
def test_stage_matches_oracle(kind, kw):
    phi, grid = _ellipsoid()
    length = 1.8
    law_o = O.make_law(kind, length_scale=length, **kw)
    ref = O.Simulation(phi, grid.spacing, law_o)
    L_ref, V_ref, info_ref = ref._rhs(stats=True)
    dt_ref = ref.stable_dt(V_ref, info_ref)

    params = S.ErosionParams(law=kind, **kw)
    law = params.make_law(length_scale=length)
    ls = S.LevelSet(torch.from_numpy(phi).cuda(), grid, width=6)
    assert np.array_equal(ls.band.cpu().numpy(), ref.band)
    sim = S.ErosionSimulation(ls, law)
    sim._band_buffers()
    lib = nat.lib()
    m = ls.work32.numel()
    nat.call("svie_stats_reset", nat.ptr(sim._stats), 1e30, nat.stream())
    sim._stage(sim._L[0], sim._u0, stats=True)
    ws = ls.scratch.get("stage", lib.svie_stage_workspace_bytes(m))
    nat.call("svie_stats_finalize", nat.ptr(sim._stats), sim._law_c, nat.ptr(ws), ws.numel(), m, nat.stream())
    st, _ = sim._read_back()
    info, vmax = sim._info(st)

    # L per node (the GPU's work list is brick ordered)
    dense = torch.zeros(grid.size, dtype=torch.float32, device="cuda")
    dense[ls.work32.long()] = sim._L[0]
    L = dense[torch.from_numpy(ref.band).cuda()].cpu().numpy()
    scale = float(np.abs(L_ref).max())
    err = float(np.abs(L - L_ref).max())
    assert err <= 2e-4 * scale, (err, scale)
    # u0 holds phi on the work list
    assert torch.equal(sim._u0, ls.flat[ls.work32.long()])

    assert vmax == pytest.approx(float(V_ref.max()), rel=1e-4)
    for k in ("qmin", "qmax"):
        assert info[k] == pytest.approx(info_ref[k], rel=1e-4, abs=1e-5)
    assert info["vmean"] == pytest.approx(info_ref["vmean"], rel=1e-4)
    if law.requires_svi:
        assert info["dvmax"] == pytest.approx(info_ref["dvmax"], rel=1e-4)
        assert abs(info["capped"] - info_ref["capped"]) <= 2
    else:
        assert info["dmax"] == pytest.approx(info_ref["dmax"], rel=1e-4)
    dt = float(st["dt"])
    assert math.isfinite(dt_ref)
    assert dt == pytest.approx(dt_ref, rel=1e-4)


def test_stage_rejects_small_workspace():
    phi, grid = _ellipsoid()
    ls = S.LevelSet(torch.from_numpy(phi).cuda(), grid, width=6)
    sim = S.ErosionSimulation(ls, S.ErosionParams(law="svi", radius=0.2, k=1, s=1, t=0.93).make_law())
    sim._band_buffers()
    m = ls.work32.numel()
    need = nat.lib().svie_stage_workspace_bytes(m)
    ws = torch.empty(need // 2, dtype=torch.uint8, device="cuda")
    nx, ny, nz = grid.shape
    before = nat.lib().svie_launch_count()
    rc = nat.lib().svie_stage_svi(nat.ptr(ls.flat), nat.ptr(ls.work32), m, nx, ny, nz, nat.ptr(sim._field),
                                  sim._law_c, nat.ptr(sim._L[0]), nat.ptr(sim._u0), None, nat.ptr(sim._stats),
                                  nat.ptr(ws), ws.numel(), nat.stream())
    assert rc == nat.SVIE_ERR_WORKSPACE
    assert b"workspace" in nat.lib().svie_last_error()
    assert nat.lib().svie_launch_count() == before
