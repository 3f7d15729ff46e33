"""Batched and served forms: every job gives the same result alone and in the mix."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

if torch.cuda.is_available():
    import svierosion_gb300 as S
    from svierosion_gb300 import shapes
    from svierosion_gb300.batch import BatchedErosion, ErosionJob, ErosionServer, Request, run_plain


def _jobs():
    frag = shapes.fragment(3, seed=5)
    L = float((frag.bounds[1] - frag.bounds[0]).max())
    specs = [
        (shapes.cube(1.0), S.ErosionParams(law="svi", radius=0.15, k=1, s=1, t=0.93, resolution=24,
                                           target_fraction=0.9, snapshots=(0.95,))),
        (frag, S.ErosionParams(law="svi", radius=0.08 * L, k=0, s=0, resolution=32, target_fraction=0.93)),
        (shapes.cube(1.0), S.ErosionParams(law="mean", alpha=1.0, resolution=24, target_fraction=0.97,
                                           max_steps=25)),
        (frag, S.ErosionParams(law="gauss", alpha=0.25, resolution=28, target_fraction=0.98, max_steps=15)),
    ]
    return [ErosionJob(m, p, name=str(i)) for i, (m, p) in enumerate(specs)]


def _same(a, b):
    assert a.stop_reason == b.stop_reason and a.steps == b.steps
    fa = np.array([r.fraction for r in a.history])
    fb = np.array([r.fraction for r in b.history])
    np.testing.assert_array_equal(fa, fb)
    np.testing.assert_array_equal([r.dt for r in a.history], [r.dt for r in b.history])
    assert [s[:2] for s in a.snapshots] == [s[:2] for s in b.snapshots]


def test_batched_equals_plain():
    """The grouped launches (one per pass over the packed band tiles of all jobs, per-job time
    steps on the device, CUDA-graph replay for the curvature-law group) give every job the
    plain path's results bit for bit."""
    plain = run_plain(_jobs())
    runner = BatchedErosion(_jobs())
    batched = runner.run()
    assert runner.stepper.kernel_launches > 0   # the curvature group was replayed from a graph
    for a, b in zip(plain, batched):
        _same(a, b)
    assert plain[0].stop_reason == "target_volume" and len(plain[0].snapshots) == 1
    assert abs(plain[0].fraction - 0.9) < 1e-5


def test_served_equals_plain_and_reports_latency():
    plain = run_plain(_jobs())
    reqs = [Request(i, arr, j.mesh, j.params) for i, (arr, j) in enumerate(zip([0.0, 0.0, 0.02, 0.05], _jobs()))]
    srv = ErosionServer(hbm_budget_bytes=8 << 30, max_active=3)
    stats = srv.run(reqs)
    assert stats["requests"] == 4
    assert stats["latency_s"]["p99"] >= stats["latency_s"]["p50"] > 0
    by_id = {r.rid: r.result for r in srv.done}
    for i, a in enumerate(plain):
        _same(a, by_id[i])


def test_admission_respects_the_budget():
    jobs = _jobs()
    reqs = [Request(i, 0.0, j.mesh, j.params) for i, j in enumerate(jobs)]
    one = max(j.footprint() for j in jobs)
    srv = ErosionServer(hbm_budget_bytes=one, max_active=8)
    peak = []
    orig = srv._admit

    def admit(now):
        orig(now)
        peak.append(len(srv.active))

    srv._admit = admit
    stats = srv.run(reqs)
    assert stats["requests"] == 4 and max(peak) == 1


def test_cuda_graph_replay_matches_eager_launches():
    res = {}
    for graphs in (False, True):
        m = shapes.cube(1.0)
        p = S.ErosionParams(law="svi", radius=0.15, k=1, s=1, t=0.93, resolution=24)
        g = S.make_grid(m, p)
        ls = S.LevelSet(S.mesh_to_sdf(m, g), g)
        sim = S.ErosionSimulation(ls, p.make_law())
        sim.use_graphs = graphs
        res[graphs] = sim.run(target_fraction=0.85)
        if graphs:
            assert sim.graph_replays > 0
    a, b = res[False], res[True]
    assert a.stop_reason == b.stop_reason and a.steps == b.steps
    np.testing.assert_array_equal([r.fraction for r in a.history], [r.fraction for r in b.history])


def _many_jobs():
    """Twelve small jobs of uneven length, so that jobs finish while others are still being set up
    and lanes change members from step to step."""
    out = []
    for i in range(12):
        frag = shapes.fragment(2 + i % 2, seed=20 + i)
        L = float((frag.bounds[1] - frag.bounds[0]).max())
        if i % 3 == 0:
            p = S.ErosionParams(law="mean", alpha=1.0, resolution=20 + 2 * i, target_fraction=0.98, max_steps=6 + i)
        else:
            p = S.ErosionParams(law="svi", radius=0.1 * L, k=i % 2, s=0, resolution=20 + 2 * i,
                                target_fraction=0.97 - 0.005 * i)
        out.append(ErosionJob(frag, p, name=str(i)))
    return out


@pytest.mark.parametrize("serial", [False, True], ids=["packed", "serial"])
def test_lanes_with_turnover_equal_plain(serial):
    """Jobs set up while others step, lanes losing and gaining members: every job's history equals
    its plain solve bit for bit (a lane's cached launch table must never outlive its members)."""
    plain = run_plain(_many_jobs())
    batched = BatchedErosion(_many_jobs(), lanes_svi=2, lanes_curvature=2, serial_curvature=serial).run()
    for a, b in zip(plain, batched):
        _same(a, b)
