"""The numpy oracle against the fixtures produced by the reference itself."""

import numpy as np
import pytest

import oracle as O


def _close(a, b, atol, rtol=0.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape
    err = np.abs(a - b)
    assert np.all(err <= atol + rtol * np.abs(b)), float(err.max())


def test_band_bit_exact(golden):
    d = golden("kernels_sphere")
    band = O.rebuild_band(d["phi_in"].reshape(-1).copy(), 6.0, float(d["h"]))
    assert np.array_equal(band, d["band"])


def test_stencil_kernels(golden):
    d = golden("kernels_sphere")
    phi = d["phi"].reshape(-1)
    shape = tuple(int(v) for v in d["shape"])
    h = float(d["h"])
    st = O.strides_of(shape)
    nx, ny, nz = shape
    idx = d["band"]
    _close(O.godunov_inward(phi, idx, *st, 1.0 / h), d["godunov"], 1e-5)
    _close(O.cell_fractions(phi, idx, *st), d["fractions"], 1e-6)
    _close(O.closest_points(phi, idx, ny, nz, nx - 3.001, ny - 3.001, nz - 3.001, h), d["closest"], 1e-5)
    _close(O.tricubic(phi, ny, nz, d["closest"]), d["tricubic"], 1e-6)
    v, g = O.tricubic_with_gradient(phi, ny, nz, d["closest"])
    _close(v, d["tricubic_val"], 1e-6)
    _close(g, d["tricubic_grad"], 1e-6)
    _close(O.trilinear(phi, ny, nz, d["closest"]), d["trilinear"], 1e-6)
    k1, k2 = O.principal_curvatures(phi, idx, *st, h)
    _close(k1, d["k1"], 1e-5, 1e-4)
    _close(k2, d["k2"], 1e-5, 1e-4)
    assert np.array_equal(O.interface_mask(phi, idx, *st), d["interface"])
    geo = O.reinit_geometry(phi, idx, *st, h, 0.45)
    _close(geo[0], d["geo_sgn"], 0)
    _close(geo[1], d["geo_dtau"], 1e-7)
    _close(O.reinit_rhs(phi, idx, *st, h, geo[0], *geo[2:]), d["reinit_rhs"], 1e-5)
    assert abs(O.band_volume(phi, idx, shape, h) - float(d["volume"])) < 1e-8
    _close(O.tricubic(phi, ny, nz, d["pts"]), d["tricubic_pts"], 1e-6)
    _close(O.trilinear(phi, ny, nz, d["pts"]), d["trilinear_pts"], 1e-6)


def test_cube_plane_fraction(golden):
    c = golden("cube_plane")
    _close(O.cube_plane_fraction(c["s"], c["a"][:, 0], c["a"][:, 1], c["a"][:, 2]), c["f"], 1e-7)


def test_ball_weights_and_convolution(golden):
    s = golden("svi_conv")
    _close(O.ball_cell_weights(1.0, 1 / 3.3), s["w_r33"], 1e-12)
    _close(O.ball_cell_weights(0.1, 1 / 64), s["w_r64"], 1e-12)
    shape = tuple(int(v) for v in s["shape"])
    kh, m = O.kernel_hat(shape, float(s["radius"]), float(s["h"]))
    assert m == int(s["m"])
    _close(kh.real, s["khat_re"], 1e-4)
    N = O.exterior_fraction(s["fractions"], kh, float(s["radius"]), float(s["h"]))
    _close(N, s["N"], 2e-6)


def test_reinitialize(golden):
    r = golden("reinit_sphere")
    phi3 = r["phi0"].copy()
    band = O.reinitialize(phi3, r["band0"], float(r["h"]), 20)
    _close(phi3, r["phi"], 1e-6)
    assert np.array_equal(band, r["band"])


def test_sdf_cube_and_torus(golden):
    sd = golden("sdf")
    pc = O.mesh_to_sdf(sd["cube_v"], sd["cube_f"], sd["cube_origin"], float(sd["cube_h"]),
                       tuple(int(v) for v in sd["cube_shape"]))
    _close(pc, sd["cube_phi"], 1e-7)
    pt = O.mesh_to_sdf(sd["torus_v"], sd["torus_f"], sd["torus_origin"], float(sd["torus_h"]),
                       tuple(int(v) for v in sd["torus_shape"]))
    _close(pt, sd["torus_phi"], 1e-6)


@pytest.mark.parametrize("name", ["cube32_k0s0", "cube32_mean", "cube32_gauss"])
def test_full_run_small(golden, name):
    d = golden(f"run_{name}")
    P = d["params"]
    phi = d["phi_init"]
    lo, hi = d["vertices"].min(0), d["vertices"].max(0)
    law = O.make_law(str(d["law"]), radius=P[0], k=int(P[1]), s=int(P[2]), t=(P[3] or None), alpha=P[4],
                     length_scale=float((hi - lo).max()))
    sim = O.Simulation(phi, float(d["h"]), law)
    assert np.array_equal(sim.band, d["band_init"])
    reason, steps, _, frac = sim.run(float(P[6]), max_steps=int(d.get("max_steps", 100000)))
    assert reason == str(d["stop_reason"]) and steps == int(d["steps"])
    assert abs(frac - float(d["fraction"])) < 1e-6
    fr = np.array([r.fraction for r in sim.history])
    _close(fr, d["hist_fraction"], 1e-6)
    assert sim.band.size == int(d["band_final_count"])
