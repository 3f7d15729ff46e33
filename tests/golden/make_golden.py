"""Generate the golden fixtures by running the reference SVIErosion itself.

Run in a container that has the reference source tree (read-only is fine):

    PYTHONDONTWRITEBYTECODE=1 SVIEROSION_COMPILE=0 \
        python tests/golden/make_golden.py /path/to/SVIErosion

The reference is imported from that tree and run on the CPU (torch eager:
the kernels are the same functions torch.compile would fuse).  Every input is
generated here from fixed seeds; the outputs are stored as compressed .npz
files next to this script.  Nothing at test time reads the reference tree.
"""

from __future__ import annotations

import math
import os
import sys
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent


def history_arrays(hist) -> dict:
    keys = ["step", "time", "dt", "volume", "fraction", "vmax", "vmean", "qmin", "qmax", "capped", "reinit"]
    return {"hist_" + k: np.array([getattr(r, k) for r in hist], dtype=np.float64) for k in keys}


def run_case(name, mesh, params, phi_store=True) -> None:
    """One full run of the reference's ErosionSimulation.run, stored as run_<name>.npz."""
    from svierosion.api import make_grid
    from svierosion.evolve import ErosionSimulation
    from svierosion.levelset import LevelSet
    from svierosion.sdf import mesh_to_sdf

    grid = make_grid(mesh, params)
    lo, hi = mesh.bounds
    law = params.make_law(length_scale=float((hi - lo).max()))
    phi = mesh_to_sdf(mesh, grid, band=params.band, device="cpu")
    phi_init = phi.clone()
    ls = LevelSet(phi, grid, width=params.band)
    band_init = ls.band.clone()
    sim = ErosionSimulation(ls, law, cfl=params.cfl, feedback_cfl=params.feedback_cfl,
                            parabolic_cfl=params.parabolic_cfl, reinit_distance=params.reinit_distance,
                            reinit_iterations=params.reinit_iterations)
    res = sim.run(target_fraction=params.target_fraction, max_steps=params.max_steps)
    fb = ls.flat[ls.band].numpy()
    rng = np.random.default_rng(0)
    probe = np.sort(rng.choice(ls.band.numel(), size=min(4000, ls.band.numel()), replace=False))
    extra = {"phi_init": phi_init.numpy()} if phi_store else {}
    np.savez_compressed(
        OUT / f"run_{name}.npz", vertices=mesh.vertices, faces=mesh.faces, origin=np.array(grid.origin),
        shape=np.array(grid.shape), h=grid.spacing, band_init=band_init.numpy(),
        initial_volume=sim.initial_volume, stop_reason=res.stop_reason, steps=res.steps, time=res.time,
        fraction=res.fraction, band_final_count=ls.band.numel(),
        band_final_head=ls.band[:2000].numpy(), band_final_tail=ls.band[-2000:].numpy(),
        phi_band_sum=float(fb.astype(np.float64).sum()), phi_band_abs_sum=float(np.abs(fb).astype(np.float64).sum()),
        probe_idx=ls.band[probe].numpy(), probe_phi=ls.flat[ls.band[probe]].numpy(),
        params=np.array([params.radius or 0.0, params.k, params.s, params.t or 0.0, params.alpha,
                         params.resolution, params.target_fraction]),
        law=params.law, max_steps=params.max_steps, **extra, **history_arrays(sim.history))
    print(name, grid.shape, res.stop_reason, res.steps, res.fraction)


def full_runs(only=None) -> None:
    """The full-run fixtures: cube-64 svi k1 s1, cube-32 svi k0 s0, and cube-32 mean and Gauss curvature."""
    from svierosion import shapes
    from svierosion.api import ErosionParams

    cube = shapes.cube(1.0)
    cases = {
        "cube64": ErosionParams(law="svi", radius=0.1, k=1, s=1, t=0.93, resolution=64, target_fraction=0.9,
                                device="cpu"),
        "cube32_k0s0": ErosionParams(law="svi", radius=0.15, k=0, s=0, resolution=32, target_fraction=0.95,
                                     device="cpu"),
        "cube32_mean": ErosionParams(law="mean", alpha=1.0, resolution=32, target_fraction=0.97, device="cpu",
                                     max_steps=40),
        # GaussCurvatureLaw (flows.py:186-213) with the automatic delta = L^-2 (api.py:62-64)
        "cube32_gauss": ErosionParams(law="gauss", alpha=0.25, resolution=32, target_fraction=0.97,
                                      device="cpu", max_steps=40),
    }
    for name, params in cases.items():
        if only is None or name in only:
            run_case(name, cube, params)


def setup_reference(ref_root: str) -> None:
    os.environ.setdefault("SVIEROSION_COMPILE", "0")
    sys.dont_write_bytecode = True
    sys.path.insert(0, ref_root)
    import torch
    from svierosion import kernels as K
    torch.set_num_threads(os.cpu_count() or 1)
    K.set_compile(False)


def main(ref_root: str, only=None) -> None:
    setup_reference(ref_root)
    if only is not None:      # just the named full runs
        full_runs(only)
        return
    import torch
    from svierosion import kernels as K, shapes
    from svierosion.evolve import ErosionSimulation
    from svierosion.flows import GaussCurvatureLaw, MeanCurvatureLaw, SVIPowerLaw
    from svierosion.grid import Grid
    from svierosion.levelset import LevelSet, cube_plane_fraction, tricubic
    from svierosion.sdf import mesh_to_sdf
    from svierosion.svi import BallConvolution, ball_cell_weights
    from svierosion.api import ErosionParams, make_grid

    ctr = np.array([0.0123, -0.0311, 0.0217])

    def sphere_phi(R, h, pad, distort):
        g = Grid.around([-R] * 3, [R] * 3, h, padding=pad)
        X, Y, Z = [torch.tensor(a) for a in np.meshgrid(*g.axes(), indexing="ij")]
        phi = torch.sqrt((X - ctr[0]) ** 2 + (Y - ctr[1]) ** 2 + (Z - ctr[2]) ** 2) - R
        if distort:
            phi = phi * (1 + 0.4 * torch.sin(3 * X) * torch.cos(2 * Y)) + 0.3 * phi ** 2
        return phi.float(), g

    # ---- 1. stencil kernels on a distorted sphere (band of LevelSet)
    phi, g = sphere_phi(1.0, 0.1, 1.3, True)
    ls = LevelSet(phi.clone(), g, width=6)
    idx = ls.band
    st = ls.strides
    nx, ny, nz = g.shape
    hi = (nx - 3.001, ny - 3.001, nz - 3.001)
    cp = K.closest_points(ls.flat, idx, ny, nz, *hi, ls.h)
    k1, k2 = K.principal_curvatures(ls.flat, idx, *st, ls.h)
    tv, tg = K.tricubic_with_gradient(ls.flat, ny, nz, cp)
    geo = K.reinit_geometry(ls.flat, idx, *st, ls.h, 0.45)
    rhs = K.reinit_rhs(ls.flat, idx, *st, ls.h, geo[0], *geo[2:])
    pts = torch.tensor(np.random.default_rng(3).uniform(1.5, min(g.shape) - 3.5, size=(500, 3)), dtype=torch.float32)
    np.savez_compressed(
        OUT / "kernels_sphere.npz",
        phi_in=phi.numpy(), phi=ls.phi.numpy(), shape=np.array(g.shape), h=ls.h, origin=np.array(g.origin),
        band=idx.numpy(), godunov=K.godunov_inward(ls.flat, idx, *st, 1.0 / ls.h).numpy(),
        fractions=K.cell_fractions(ls.flat, idx, *st).numpy(), closest=cp.numpy(),
        tricubic=K.tricubic(ls.flat, ny, nz, cp).numpy(), tricubic_val=tv.numpy(), tricubic_grad=tg.numpy(),
        trilinear=K.trilinear(ls.flat, ny, nz, cp).numpy(), k1=k1.numpy(), k2=k2.numpy(),
        interface=K.interface_mask(ls.flat, idx, *st).numpy(),
        geo_sgn=geo[0].numpy(), geo_dtau=geo[1].numpy(),
        geo_flags=np.stack([t.numpy() for t in geo[2::4]] + [t.numpy() for t in geo[3::4]]),
        geo_dist=np.stack([t.numpy() for t in geo[4::4]] + [t.numpy() for t in geo[5::4]]),
        reinit_rhs=rhs.numpy(), volume=ls.volume(), dense_fractions=ls.dense_fractions().numpy(),
        pts=pts.numpy(), tricubic_pts=K.tricubic(ls.flat, ny, nz, pts).numpy(),
        trilinear_pts=K.trilinear(ls.flat, ny, nz, pts).numpy())

    # ---- 2. cube/plane fractions (test_geometry.py:111-138 inputs, seeded)
    gen = torch.Generator().manual_seed(1)
    n = torch.randn(2000, 3, generator=gen, dtype=torch.float64)
    n /= n.norm(dim=1, keepdim=True)
    s = (torch.rand(2000, generator=gen, dtype=torch.float64) - 0.5) * 2.0
    a = n.abs().sort(dim=1, descending=True).values.float()
    np.savez_compressed(OUT / "cube_plane.npz", s=s.float().numpy(), a=a.numpy(),
                        f=cube_plane_fraction(s.float(), a[:, 0], a[:, 1], a[:, 2]).numpy())

    # ---- 3. ball weights and the convolution
    w1 = ball_cell_weights(1.0, 1.0 / 3.3)
    w2 = ball_cell_weights(0.1, 1.0 / 64)
    phi, g = sphere_phi(1.0, 0.1, 1.3, False)
    ls = LevelSet(phi, g, width=6)
    conv = BallConvolution(g, 0.35)
    f = ls.dense_fractions()
    N = conv.exterior_fraction(f)
    np.savez_compressed(OUT / "svi_conv.npz", w_r33=w1, w_r64=w2, phi=ls.phi.numpy(), shape=np.array(g.shape),
                        h=ls.h, radius=0.35, fractions=f.numpy(), N=N.numpy(), m=conv.m,
                        khat_re=conv.kernel_hat.real.numpy(), khat_im=conv.kernel_hat.imag.numpy(),
                        quadrature_volume=conv.quadrature_volume, ball_volume=conv.ball_volume)

    # ---- 4. reinitialisation of the distorted sphere (test_flows.py:79-88 setup)
    phi, g = sphere_phi(1.0, 0.08, 12 * 0.08, True)
    ls = LevelSet(phi, g, width=6)
    phi0 = ls.phi.clone()
    band0 = ls.band.clone()
    ls.reinitialize(20)
    np.savez_compressed(OUT / "reinit_sphere.npz", phi0=phi0.numpy(), band0=band0.numpy(), phi=ls.phi.numpy(),
                        band=ls.band.numpy(), shape=np.array(g.shape), h=ls.h)

    # ---- 5. SDF of the cube and a torus
    m = shapes.cube(1.0)
    g = Grid.around(*m.bounds, spacing=0.05, padding=0.3)
    phi_c = mesh_to_sdf(m, g, band=6, device="cpu")
    t = shapes.torus(0.6, 0.25, 24, 12)
    gt = Grid.around(*t.bounds, spacing=0.06, padding=0.25)
    phi_t = mesh_to_sdf(t, gt, band=6, device="cpu")
    np.savez_compressed(OUT / "sdf.npz", cube_v=m.vertices, cube_f=m.faces, cube_origin=np.array(g.origin),
                        cube_shape=np.array(g.shape), cube_h=g.spacing, cube_phi=phi_c.numpy(),
                        torus_v=t.vertices, torus_f=t.faces, torus_origin=np.array(gt.origin),
                        torus_shape=np.array(gt.shape), torus_h=gt.spacing, torus_phi=phi_t.numpy())

    full_runs()
    print("fixtures written to", OUT)


if __name__ == "__main__":
    # make_golden.py [reference root] [run name ...]: with names, only those full runs are redone
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference", sys.argv[2:] or None)
