"""The command line (reference svierosion/cli.py): parser, and the host-only commands `info` and `shapes`."""

import numpy as np
import pytest

from svierosion_gb300 import cli, shapes
from svierosion_gb300.meshio import read_ply, write_ply


def test_parser_takes_the_reference_options():
    a = cli.build_parser().parse_args(["erode", "m.ply", "-o", "out.ply", "--law", "svi", "-r", "0.1", "-k", "1",
                                       "-s", "1", "-t", "0.93", "--target", "0.85", "--snapshots", "0.95", "0.9",
                                       "--resolution", "64", "--band", "6", "--cfl", "0.5", "--no-compile",
                                       "--quality", "N", "--quiet"])
    assert (a.command, a.law, a.radius, a.k, a.s, a.t, a.target, a.snapshots, a.resolution) == \
        ("erode", "svi", 0.1, 1, 1, 0.93, 0.85, [0.95, 0.9], 64)
    p = cli._params(a, shapes.cube(1.0))
    assert (p.radius, p.snapshots, p.project_vertices) == (0.1, (0.95, 0.9), True)
    c = cli.build_parser().parse_args(["compare", "m.ply", "-o", "dir"])
    assert (c.t, c.target, c.resolution) == (0.93, 0.9, 160)
    b = cli.build_parser().parse_args(["erode", "m.ply", "--radius-rel", "0.05"])
    assert cli._params(b, shapes.cube(2.0)).radius == pytest.approx(0.1)
    with pytest.raises(SystemExit):
        cli._params(cli.build_parser().parse_args(["erode", "m.ply"]), shapes.cube(1.0))


def test_info_and_shapes(tmp_path, capsys):
    assert cli.main(["shapes", str(tmp_path)]) == 0
    for name in shapes.SHAPES:
        m = read_ply(tmp_path / f"{name}.ply")
        assert m.is_watertight() and m.signed_volume() > 0
    p = tmp_path / "t.ply"
    write_ply(p, shapes.torus(1.0, 0.3, 32, 16), vertex_data={"q": np.arange(512.0)})
    capsys.readouterr()
    assert cli.main(["info", str(p)]) == 0
    out = capsys.readouterr().out
    assert "vertices 512, triangles 1024" in out and "boundary 0" in out and "['q']" in out
