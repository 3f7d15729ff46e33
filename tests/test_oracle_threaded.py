"""The threaded oracle stage (the benchmark's CPU baseline) computes what the serial oracle computes."""

import numpy as np
import pytest

import oracle as O
from oracle.threaded_np import ThreadedStage


def _ellipsoid_sim(n=64, h=0.05):
    ax = (np.arange(n) - 0.5 * (n - 1)) * h
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    phi = ((np.sqrt(X ** 2 + (Y / 0.7) ** 2 + (Z / 0.5) ** 2) - 0.9) * 0.6).astype(np.float32)
    law = O.make_law("svi", radius=0.2, k=1, s=1, t=0.93)
    return O.Simulation(phi, h, law)


@pytest.mark.parametrize("workers", [1, 3])
def test_threaded_stage_matches_serial(workers):
    sim = _ellipsoid_sim()
    L0, V0, info0 = sim._rhs(stats=True)
    ts = ThreadedStage(sim, workers)
    try:
        L1, V1, info1 = ts.rhs()
        vol1 = ts.volume()
    finally:
        ts.close()
    np.testing.assert_allclose(V1, V0, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(L1, L0, rtol=1e-5, atol=1e-6)
    for k in ("qmin", "qmax", "dvmax", "vmean"):
        assert info1[k] == pytest.approx(info0[k], rel=1e-5)
    assert abs(info1["capped"] - info0["capped"]) <= 1
    assert vol1 == pytest.approx(sim.volume(), rel=1e-12)


def test_threaded_simulation_matches_serial():
    """Whole steps (three stages, RK combinations, volume, regula falsi at the target and
    reinitialisation at the reference's trigger) on threads give the serial oracle's results."""
    from oracle.threaded_np import ThreadedSimulation

    base = _ellipsoid_sim()
    phi0, law, h = base.phi.copy(), base.law, base.h
    # a short trigger distance, so that the steps include reinitialisations
    serial = O.Simulation(phi0, h, law, reinit_distance=0.3)
    out_s = serial.run(target_fraction=0.93, max_steps=12)
    threaded = ThreadedSimulation(phi0, h, law, workers=3, reinit_distance=0.3)
    try:
        out_t = threaded.run(target_fraction=0.93, max_steps=12)
    finally:
        threaded.close()
    assert out_t[0] == out_s[0] and out_t[1] == out_s[1]
    assert any(r.reinit for r in serial.history)
    np.testing.assert_allclose([r.fraction for r in threaded.history], [r.fraction for r in serial.history],
                               atol=1e-6)
    assert [r.reinit for r in threaded.history] == [r.reinit for r in serial.history]
    assert np.array_equal(threaded.band, serial.band)
    np.testing.assert_allclose(threaded.flat[serial.band], serial.flat[serial.band], atol=1e-5 * serial.h)
