"""The marching-cubes case table: the library's generator (host code, no GPU needed) against the
oracle's, and the properties that make the meshes closed and consistently oriented."""

import ctypes
from collections import Counter

import numpy as np

from oracle import marching as M


def _topology(faces):
    e = Counter()
    for a, b, c in faces:
        for u, v in ((a, b), (b, c), (c, a)):
            e[(int(u), int(v))] += 1
    repeated = sum(1 for c in e.values() if c != 1)
    unmatched = sum(1 for (u, v) in e if (v, u) not in e)
    return repeated, unmatched


def test_library_table_equals_oracle_table():
    from svierosion_gb300 import _native as nat

    tri = (ctypes.c_int8 * (256 * 16))()
    ntri = (ctypes.c_uint8 * 256)()
    assert nat.lib().svie_surface_table(tri, ntri) == 0
    tab = np.frombuffer(bytes(tri), dtype=np.int8).reshape(256, 16)
    assert np.array_equal(tab, M.TABLE)
    assert np.array_equal(np.frombuffer(bytes(ntri), dtype=np.uint8), (M.TABLE >= 0).sum(1) // 3)


def test_table_basic_cases():
    n = (M.TABLE >= 0).sum(1) // 3
    assert n[0] == 0 and n[255] == 0
    assert n.max() <= 5
    for v in range(8):          # one inside corner: one triangle on its three edges
        assert n[1 << v] == 1 and n[255 ^ (1 << v)] == 1


def test_random_fields_give_closed_oriented_meshes():
    rng = np.random.default_rng(0)
    shape = (12, 11, 10)
    idx = np.arange(int(np.prod(shape)))
    x, r = np.divmod(idx, shape[1] * shape[2])
    y, z = np.divmod(r, shape[2])
    band = idx[(x < shape[0] - 1) & (y < shape[1] - 1) & (z < shape[2] - 1)]
    for _ in range(3):
        phi = rng.standard_normal(shape).astype(np.float32)
        phi[0], phi[-1], phi[:, 0], phi[:, -1], phi[:, :, 0], phi[:, :, -1] = 1, 1, 1, 1, 1, 1
        _, faces = M.extract(phi, band)
        assert len(faces) > 0
        assert _topology(faces.tolist()) == (0, 0)


def test_sphere_volume_and_orientation():
    n = 32
    ax = np.arange(n) - (n - 1) / 2
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    phi = (np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - 9.3).astype(np.float32)
    band = np.flatnonzero(np.abs(phi) < 6)
    v, f = M.extract(phi, band)
    t = v[f].astype(np.float64)
    vol = np.einsum("ij,ij->i", t[:, 0], np.cross(t[:, 1], t[:, 2])).sum() / 6
    exact = 4 / 3 * np.pi * 9.3 ** 3
    assert vol > 0 and abs(vol / exact - 1) < 0.01
    assert _topology(f.tolist()) == (0, 0)
