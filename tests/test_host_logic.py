"""Host-side logic that needs no GPU: grids, law parameters, workload generators."""

import numpy as np
import pytest

import oracle as O
from svierosion_gb300 import shapes
from svierosion_gb300.api import ErosionParams, make_grid
from svierosion_gb300.flows import GaussCurvatureLaw, MeanCurvatureLaw, SVIPowerLaw
from svierosion_gb300.grid import Grid, next_fast_size


def test_next_fast_size_and_grid():
    for n in range(1, 600):
        assert next_fast_size(n) == O.next_fast_size(n)
    g = Grid.around([-0.5] * 3, [0.5] * 3, 1 / 64, 12 / 64)
    assert g.shape == O.grid_around([-0.5] * 3, [0.5] * 3, 1 / 64, 12 / 64)[2] == (90, 90, 90)


def test_cube_matches_reference_fixture(golden):
    d = golden("sdf")
    c = shapes.cube(1.0)
    assert np.array_equal(c.faces, d["cube_f"]) and np.allclose(c.vertices, d["cube_v"])


def test_make_grid_configs():
    p = ErosionParams(law="svi", radius=0.1, k=1, s=1, t=0.93, resolution=64)
    assert make_grid(shapes.cube(1.0), p).shape == (90, 90, 90)
    m = shapes.fragment(4, seed=0)
    L = float((m.bounds[1] - m.bounds[0]).max())
    assert abs(L - 2.077) < 2e-3
    p = ErosionParams(law="svi", radius=0.05 * L, k=1, s=1, t=0.93, resolution=400)
    g = make_grid(m, p)
    assert all(next_fast_size(n) == n for n in g.shape)


def test_fragment_generator():
    m = shapes.fragment(6, seed=0)
    assert len(m.faces) == 81920 and m.is_watertight() and m.is_consistently_oriented()
    assert abs(m.volume() - 1.6556) < 1e-3
    L = float((m.bounds[1] - m.bounds[0]).max())
    assert abs(L - 2.078) < 1e-3


def test_law_parameters_match_oracle():
    for k, s, t in ((1, 1, 0.93), (2, 1, 0.95), (0, 0, None), (1, 0, None)):
        a = SVIPowerLaw(0.1, k, s, t)
        b = O.SVILaw(0.1, k, s, t)
        assert a.n_cap == b.n_cap
    with pytest.raises(ValueError):
        SVIPowerLaw(0.1, 1, 1, 0.4)
    with pytest.raises(ValueError):
        SVIPowerLaw(-1.0)
    with pytest.raises(ValueError):
        GaussCurvatureLaw(0.25)
    assert MeanCurvatureLaw(1.0).params()["law"] == "mean_curvature"


def test_params_make_law_auto_delta():
    p = ErosionParams(law="gauss", alpha=0.25)
    law = p.make_law(length_scale=2.0)
    assert law.delta == 0.25
    p = ErosionParams(law="mean", alpha=0.5)
    assert p.make_law(length_scale=2.0).delta == 0.5


def test_warp_slices_for_triangle_groups():
    """The number of warps that share a group of 32 triangles grows with the square of the
    longest edge (lines or nodes a triangle covers) and stays within [1, cap]."""
    from svierosion_gb300.sdf import _slices

    assert _slices(1.1, 64.0, 1024) == 1          # scan-size triangles: one warp per group
    assert _slices(1.1, 2.0, 32) == 1
    assert _slices(8.0, 2.0, 32) == 32            # split soup: edges up to 8 cells
    assert _slices(45.0, 64.0, 1024) == 32        # a coarse cube at resolution 32
    assert _slices(1e6, 64.0, 1024) == 1024
    assert _slices(0.0, 64.0, 1024) == 1


def test_mesh_bounds_without_a_device_copy():
    """mesh_bounds falls back to TriMesh.bounds when the mesh has no device copy."""
    from svierosion_gb300.sdf import mesh_bounds

    m = shapes.fragment(2, seed=4)
    assert np.array_equal(mesh_bounds(m), m.bounds)
    g = make_grid(m, ErosionParams(law="mean", resolution=48))
    lo, hi = m.bounds
    top = np.asarray(g.origin) + g.spacing * (np.asarray(g.shape) - 1)
    assert np.all(np.asarray(g.origin) < lo) and np.all(top > hi)


class _FakeConvLib:
    """Stand-in for the library's convolution entry points the per-shape set-up calls."""

    def __init__(self, jit_ok: bool):
        self.jit_ok = jit_ok
        self.jit_on = False
        self.kept = False
        self.calls = []

    def svie_conv_jit_enabled(self, nx, ny, nz):
        return int(self.jit_on)

    def svie_conv_jit(self, nx, ny, nz):
        self.calls.append("jit")
        self.jit_on = self.jit_ok
        return 0 if self.jit_ok else 5

    def svie_conv_get_choice(self, nx, ny, nz, z, y, x):
        return int(self.kept)


@pytest.mark.parametrize("jit_ok", [True, False])
def test_shape_setup_tunes_only_without_compiled_passes(monkeypatch, jit_ok):
    """At a large shape's first convolution the passes compiled for its axis lengths are requested;
    when that succeeds the fixed rule's forms stay (no timing of the library's passes while the
    compiled ones build), otherwise the pass forms are tuned."""
    import torch
    from svierosion_gb300 import svi

    fake = _FakeConvLib(jit_ok)
    tuned = []
    monkeypatch.setattr(svi.nat, "lib", lambda: fake)
    monkeypatch.setattr(svi.nat, "call", lambda name, *a: tuned.append(name))
    monkeypatch.setattr(svi.nat, "ptr", lambda t: None)
    monkeypatch.setattr(svi.nat, "stream", lambda: None)
    monkeypatch.setattr(torch.cuda, "is_current_stream_capturing", lambda: False)
    monkeypatch.setattr(svi, "save_tuned_forms", lambda device, shape: None)
    monkeypatch.setattr(svi, "load_tuned_forms", lambda device, shape: False)
    monkeypatch.delenv("SVIE_FFT_JIT", raising=False)
    monkeypatch.delenv("SVIE_FFT_TUNE", raising=False)
    conv = object.__new__(svi.BallConvolution)
    conv.device = torch.device("cuda", 0)
    conv.grid = Grid((0.0, 0.0, 0.0), 1.0, (448, 336, 245))
    conv.plan = None
    key = (0, (448, 336, 245))
    svi._TUNED.discard(key)
    try:
        conv._tune(torch.zeros(1), torch.zeros(1), torch.zeros(16, dtype=torch.uint8))
        assert fake.calls == ["jit"]
        assert tuned == ([] if jit_ok else ["svie_conv_tune"])
        assert key in svi._TUNED
    finally:
        svi._TUNED.discard(key)


class _FakeSampler:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0

    def kill(self):
        pass


def test_clock_samples_count_from_the_timed_region(tmp_path):
    """bench.py's nvidia-smi sampler starts during the warm-up; only the lines written after the timed
    region's mark count, and a line cut by the mark is dropped."""
    import bench
    path = tmp_path / "clocks.csv"
    warm = "0, 1800, 2070, 700.0, 0x0, Not Active, Not Active, Not Active, Not Active\n"
    timed = "0, 2070, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, Active\n"
    path.write_text(warm * 3 + warm[:10])
    s = object.__new__(bench.ClockSampler)
    s.file = open(path, "a+")
    s.proc = _FakeSampler()
    s.mark_at = 0
    s.mark()
    with open(path, "a") as fh:
        fh.write(warm[10:] + timed * 4)
    out = s.stop()
    assert out["samples"] == 4 and out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]
    assert not path.exists()
