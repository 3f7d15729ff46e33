"""The command line's GPU commands: `erode` writes the reference's result files, `compare` its table."""

import csv
import json

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

if torch.cuda.is_available():
    from svierosion_gb300 import cli, shapes
    from svierosion_gb300.compare import run_comparison
    from svierosion_gb300.meshio import read_ply, write_ply


def test_cli_erode_writes_the_result_files(tmp_path):
    src = tmp_path / "cube.ply"
    write_ply(src, shapes.cube(1.0))
    rc = cli.main(["erode", str(src), "--law", "svi", "-r", "0.15", "-k", "1", "-s", "1", "-t", "0.93",
                   "--resolution", "24", "--target", "0.9", "--snapshots", "0.95", "--quiet"])
    assert rc == 0
    stem = tmp_path / "cube_eroded"
    meta = json.loads((tmp_path / "cube_eroded.json").read_text())
    assert meta["stop_reason"] == "target_volume" and abs(meta["volume_fraction"] - 0.9) < 1e-5
    assert [s["fraction"] for s in meta["snapshots"]] == pytest.approx([0.95], abs=1e-5)
    final = read_ply(tmp_path / "cube_eroded.ply")
    snap = read_ply(tmp_path / "cube_eroded_v0.950.ply")
    assert final.is_watertight() and snap.is_watertight()
    assert np.array_equal(final.vertex_data["quality"], final.vertex_data["depth"])
    with open(f"{stem}_history.csv") as fh:
        rows = list(csv.DictReader(fh))
    assert len(rows) > 0
    assert float(rows[-1]["fraction"]) == pytest.approx(0.9, abs=1e-5)


def test_compare_runs_every_law_to_the_target(tmp_path):
    laws = [("grassfire V=1", dict(law="svi", radius=0.2, k=0, s=0)), ("mean curv. V=H+", dict(law="mean", alpha=1.0))]
    res = run_comparison(shapes.cube(1.0), laws, tmp_path, target=0.95, resolution=20, verbose=False)
    assert [r.stop_reason for _, r in res] == ["target_volume", "target_volume"]
    for name in ("initial.ply", "grassfire_v_1.ply", "mean_curv_v_h.ply", "summary.csv",
                 "pairwise_mean_distance.json"):
        assert (tmp_path / name).exists(), name
    with open(tmp_path / "summary.csv") as fh:
        rows = list(csv.DictReader(fh))
    assert [r["label"] for r in rows] == ["grassfire V=1", "mean curv. V=H+"]
    d = np.array(json.loads((tmp_path / "pairwise_mean_distance.json").read_text())["mean_distance"])
    assert d.shape == (2, 2) and d[0, 1] == d[1, 0] > 0 and d[0, 0] == 0
