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
