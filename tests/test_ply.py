"""PLY reading and writing (reference svierosion/meshio.py:136-362) on the CPU.

Pinned by files that the reference's own write_ply produced (tests/golden/make_ply_golden.py):
this package reads them back exactly and writes the same bytes.  The reference's own PLY tests
(tests/test_geometry.py:18-42) are restated beside them.
"""

import os
import struct
import tempfile
from pathlib import Path

import numpy as np
import pytest

from svierosion_gb300.meshio import TriMesh, read_ply, write_ply
from svierosion_gb300 import shapes

GOLD = Path(__file__).resolve().parent / "golden" / "ply"
CASES = [(True, "float"), (True, "double"), (False, "double")]


def _name(binary, prec):
    return f"torus_{'binary' if binary else 'ascii'}_{prec}.ply"


@pytest.fixture(scope="module")
def torus():
    d = np.load(GOLD / "torus.npz")
    return TriMesh(d["vertices"], d["faces"]), d["quality"]


@pytest.mark.parametrize("binary,prec", CASES)
def test_writer_matches_reference_bytes(tmp_path, torus, binary, prec):
    mesh, q = torus
    p = tmp_path / _name(binary, prec)
    write_ply(p, mesh, binary=binary, precision=prec, vertex_data={"quality": q},
              comments=["written by the reference"])
    assert p.read_bytes() == (GOLD / _name(binary, prec)).read_bytes()


@pytest.mark.parametrize("binary,prec", CASES)
def test_reader_reads_reference_files(torus, binary, prec):
    mesh, q = torus
    r = read_ply(GOLD / _name(binary, prec))
    if prec == "float":
        assert np.array_equal(r.vertices, mesh.vertices.astype(np.float32).astype(np.float64))
    else:
        assert np.array_equal(r.vertices, mesh.vertices)
    assert np.array_equal(r.faces, mesh.faces)
    assert np.array_equal(r.vertex_data["quality"], q.astype(np.float32))
    assert not read_ply(GOLD / _name(binary, prec), vertex_properties=False).vertex_data


def test_roundtrip_binary_and_ascii():
    """tests/test_geometry.py:18-31 of the reference."""
    m = shapes.torus(1.0, 0.3, 32, 16)
    q = m.vertices[:, 2].copy()
    with tempfile.TemporaryDirectory() as d:
        for binary, prec in CASES:
            p = os.path.join(d, f"t_{binary}_{prec}.ply")
            write_ply(p, m, binary=binary, precision=prec, vertex_data={"quality": q})
            r = read_ply(p)
            tol = 1e-6 if prec == "float" else 1e-12
            assert np.allclose(r.vertices, m.vertices, atol=tol)
            assert np.array_equal(r.faces, m.faces)
            assert np.allclose(r.vertex_data["quality"], q, atol=1e-6)


def test_quads_are_triangulated(tmp_path):
    """tests/test_geometry.py:33-42 of the reference."""
    txt = ("ply\nformat ascii 1.0\nelement vertex 4\nproperty float x\nproperty float y\n"
           "property float z\nelement face 1\nproperty list uchar int vertex_indices\nend_header\n"
           "0 0 0\n1 0 0\n1 1 0\n0 1 0\n4 0 1 2 3\n")
    p = tmp_path / "q.ply"
    p.write_text(txt)
    m = read_ply(p)
    assert m.faces.shape == (2, 3)
    assert np.array_equal(m.faces, [[0, 1, 2], [0, 2, 3]])


def test_big_endian_mixed_polygons(tmp_path):
    """Binary big-endian body with a triangle and a pentagon (the record-by-record path),
    an int16 vertex property, comments and obj_info lines."""
    verts = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [-1, 0.5, 0]], dtype=np.float64)
    head = ("ply\nformat binary_big_endian 1.0\ncomment a\nobj_info b\nelement vertex 5\n"
            "property double x\nproperty double y\nproperty double z\nproperty short label\n"
            "element face 2\nproperty list uchar int vertex_index\nend_header\n").encode("ascii")
    body = b"".join(struct.pack(">dddh", *v, i) for i, v in enumerate(verts))
    body += struct.pack(">B3i", 3, 0, 1, 2) + struct.pack(">B5i", 5, 0, 1, 2, 3, 4)
    p = tmp_path / "be.ply"
    p.write_bytes(head + body)
    m = read_ply(p)
    assert np.array_equal(m.vertices, verts)
    assert np.array_equal(m.faces, [[0, 1, 2], [0, 1, 2], [0, 2, 3], [0, 3, 4]])
    assert np.array_equal(m.vertex_data["label"], np.arange(5))


def test_bad_files(tmp_path):
    p = tmp_path / "x.ply"
    p.write_bytes(b"plx\nformat ascii 1.0\nend_header\n")
    with pytest.raises(ValueError, match="magic"):
        read_ply(p)
    p.write_bytes(b"ply\nformat ascii 1.0\nelement face 0\nproperty list uchar int vertex_indices\nend_header\n")
    with pytest.raises(ValueError, match="no vertex element"):
        read_ply(p)
    p.write_bytes(b"ply\nformat binary_middle_endian 1.0\nend_header\n")
    with pytest.raises(ValueError, match="unsupported PLY format"):
        read_ply(p)
    with pytest.raises(ValueError, match="shape"):
        write_ply(tmp_path / "y.ply", shapes.cube(1.0), vertex_data={"q": np.zeros(3)})


def test_mesh_cleanup():
    m = TriMesh(np.arange(15, dtype=float).reshape(5, 3), np.array([[0, 1, 1], [0, 2, 3]]),
                {"q": np.arange(5.0)})
    c = m.remove_degenerate_faces().remove_unreferenced_vertices()
    assert np.array_equal(c.faces, [[0, 1, 2]])
    assert np.array_equal(c.vertices, m.vertices[[0, 2, 3]])
    assert np.array_equal(c.vertex_data["q"], [0.0, 2.0, 3.0])


def test_result_files_match_reference(tmp_path):
    """write_result writes the files of the reference's result writer (cli.py:101-126), byte for
    byte, for the same synthetic result."""
    import importlib.util

    from svierosion_gb300.api import ErosionResult, write_result
    from svierosion_gb300.evolve import StepRecord
    from svierosion_gb300.grid import Grid

    spec = importlib.util.spec_from_file_location("make_ply_golden", GOLD.parent / "make_ply_golden.py")
    gold = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gold)
    res = gold.synthetic_result(ErosionResult, StepRecord, Grid, TriMesh, shapes.cube(1.0))
    written = write_result(res, tmp_path / "result.ply", "depth")
    assert [p.name for p in written] == ["result_v0.950.ply", "result.ply"]
    for name in ("result_v0.950.ply", "result.ply", "result_history.csv", "result.json"):
        assert (tmp_path / name).read_bytes() == (GOLD / name).read_bytes(), name
    m = read_ply(tmp_path / "result.ply")
    assert np.array_equal(m.vertex_data["quality"], m.vertex_data["depth"])
