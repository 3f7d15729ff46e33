"""Multi-threaded evaluation of the oracle's RK stage and volume (test infrastructure only).

The CPU baseline of the benchmark times the reference algorithm on all host
cores, as the reference itself runs on the CPU (torch with one intra-op
thread per core).  This module evaluates the same arithmetic as
``reference_np.Simulation._rhs`` (svierosion/evolve.py:118-160) and
``reference_np.band_volume`` (svierosion/levelset.py:123-126) with the band
split into contiguous chunks on a thread pool (numpy releases the GIL inside
its gather and ufunc loops) and the FFTs of svierosion/svi.py:84-93 on
scipy's multi-threaded pocketfft.  ``tests/test_oracle_golden.py`` checks it
against the serial oracle.
"""

from __future__ import annotations

import math
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import scipy.fft

from .reference_np import (F32, Simulation, cell_fractions, closest_points, godunov_inward, strides_of,
                           tricubic)


def _spans(n: int, parts: int):
    parts = max(1, min(parts, n)) if n else 1
    edges = np.linspace(0, n, parts + 1).astype(np.int64)
    return [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:]) if b > a]


class ThreadedStage:
    """One SVI-law RHS stage and one volume of a ``Simulation`` on ``workers`` threads."""

    def __init__(self, sim: Simulation, workers: int):
        if not sim.law.requires_svi:
            raise ValueError("the threaded stage covers the SVI laws")
        self.sim = sim
        self.workers = int(workers)
        self.pool = ThreadPoolExecutor(self.workers)

    def close(self) -> None:
        self.pool.shutdown()

    def _map(self, fn, spans):
        return list(self.pool.map(lambda ab: fn(*ab), spans))

    def svi_field(self) -> np.ndarray:
        """svi.py:84-93 on dense fractions (levelset.py:117-121)."""
        sim = self.sim
        flat, idx, st = sim.flat, sim.band, sim.st
        f = np.empty(flat.size, dtype=F32)

        def dense(a, b):
            f[a:b] = flat[a:b] < 0

        self._map(dense, _spans(flat.size, self.workers))
        fr = np.empty(idx.size, dtype=F32)

        def frac(a, b):
            fr[a:b] = cell_fractions(flat, idx[a:b], *st)

        self._map(frac, _spans(idx.size, self.workers))
        f[idx] = fr
        fh = scipy.fft.rfftn(f.reshape(sim.shape), workers=self.workers).astype(np.complex64)
        khat = sim.khat

        def mul(a, b):
            fh[a:b] *= khat[a:b]

        self._map(mul, _spans(fh.shape[0], self.workers))
        g = scipy.fft.irfftn(fh, s=sim.shape, workers=self.workers)
        out = np.empty(sim.shape, dtype=F32)
        scale = F32(sim.h ** 3)
        inv_ball = F32(-1.0 / (4.0 / 3.0 * math.pi * sim.law.radius ** 3))

        def fin(a, b):
            out[a:b] = (g[a:b].astype(F32) * scale) * inv_ball + F32(1.0)

        self._map(fin, _spans(sim.shape[0], self.workers))
        return out

    def rhs(self):
        """(L, V, info) as ``Simulation._rhs(stats=True)`` for an SVI law."""
        sim = self.sim
        flat, idx, st = sim.flat, sim.band, sim.st
        nx, ny, nz = sim.shape
        Nd = self.svi_field().reshape(-1)
        L = np.empty(idx.size, dtype=F32)
        V = np.empty(idx.size, dtype=F32)
        h = sim.h

        def band(a, b):
            i = idx[a:b]
            phi_b = flat[i]
            cp = closest_points(flat, i, ny, nz, nx - 3.001, ny - 3.001, nz - 3.001, h)
            N = tricubic(Nd, ny, nz, cp)
            v = sim.law.speed(N)
            near = np.abs(phi_b) < F32(h)
            part = None
            if near.any():
                Nn = N[near]
                part = (float(Nn.min()), float(Nn.max()), float(sim.law.dspeed(Nn).max()),
                        int((Nn > F32(sim.law.n_cap)).sum()), float(v[near].astype(np.float64).sum()),
                        int(near.sum()))
            v = (v * sim._cutoff_factor(phi_b)).astype(F32)
            V[a:b] = v
            L[a:b] = v * godunov_inward(flat, i, *st, 1.0 / h)
            return part

        parts = [p for p in self._map(band, _spans(idx.size, 4 * self.workers)) if p is not None]
        info = {}
        if parts:
            info["qmin"] = min(p[0] for p in parts)
            info["qmax"] = max(p[1] for p in parts)
            info["dvmax"] = max(p[2] for p in parts)
            info["capped"] = sum(p[3] for p in parts)
            info["vmean"] = sum(p[4] for p in parts) / sum(p[5] for p in parts)
        return L, V, info

    def volume(self) -> float:
        """levelset.py:123-126."""
        sim = self.sim
        flat, idx = sim.flat, sim.band
        st = strides_of(sim.shape)
        inside = sum(self._map(lambda a, b: int((flat[a:b] < 0).sum()), _spans(flat.size, self.workers)))
        parts = self._map(lambda a, b: (int((flat[idx[a:b]] < 0).sum()),
                                        float(cell_fractions(flat, idx[a:b], *st).astype(np.float64).sum())),
                          _spans(idx.size, self.workers))
        band_inside = sum(p[0] for p in parts)
        fsum = sum(p[1] for p in parts)
        return (inside - band_inside + fsum) * sim.h ** 3
