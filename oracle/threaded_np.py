"""Multi-threaded evaluation of the oracle's steps (test infrastructure only).

The CPU baseline of the benchmark times the reference algorithm on all host
cores, as the reference itself runs on the CPU (torch with one intra-op
thread per core).  This module evaluates the same arithmetic as
``reference_np.Simulation._rhs`` (svierosion/evolve.py:118-160) and
``reference_np.band_volume`` (svierosion/levelset.py:123-126) with the band
split into contiguous chunks on a thread pool (numpy releases the GIL inside
its gather and ufunc loops) and the FFTs of svierosion/svi.py:84-93 on
scipy's multi-threaded pocketfft.  ``tests/test_oracle_golden.py`` checks it
against the serial oracle.  ``ThreadedSimulation`` runs the reference's whole
step loop (svierosion/evolve.py:182-250: three stages, the RK combinations,
the volume, regula falsi and the reinitialisation of levelset.py:154-183 at the
reference's trigger) with these threaded pieces; every piece is elementwise
over the band or the work set, so its results equal the serial oracle's bit
for bit.
"""

from __future__ import annotations

import math
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import scipy.fft

from .reference_np import (F32, MARGIN, Simulation, cell_fractions, check_margin, closest_points, dilate,
                           godunov_inward, reinit_geometry, reinit_rhs, strides_of, tricubic)


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


def threaded_reinitialize(pool, workers: int, phi3, band, h, iterations=12, cfl=0.45, dilation=3, width=6.0):
    """reference_np.reinitialize (levelset.py:154-183) with the geometry, the pseudo-time sweeps and the
    band rebuild split over ``pool``; returns the rebuilt band.  Each sweep evaluates the right-hand
    side of every work node from the same field before any node is written, as the serial form does."""
    shape = phi3.shape
    mask = np.zeros(shape, dtype=bool)
    mask.reshape(-1)[band] = True
    mask = dilate(mask, dilation)
    for ax in range(3):
        sl = [slice(None)] * 3
        sl[ax] = slice(0, MARGIN)
        mask[tuple(sl)] = False
        sl[ax] = slice(shape[ax] - MARGIN, shape[ax])
        mask[tuple(sl)] = False
    idx = np.nonzero(mask.reshape(-1))[0].astype(np.int64)
    f = phi3.reshape(-1)
    st = strides_of(shape)
    spans = _spans(idx.size, 4 * workers)

    def each(fn):
        """fn(k, a, b) for every span k = [a, b) of the work list, on the pool."""
        list(pool.map(lambda k: fn(k, *spans[k]), range(len(spans))))

    geo = [None] * len(spans)

    def geometry(k, a, b):
        geo[k] = reinit_geometry(f, idx[a:b], *st, h, cfl)

    each(geometry)
    r = np.empty(idx.size, dtype=F32)
    u0 = np.empty(idx.size, dtype=F32)
    u1 = np.empty(idx.size, dtype=F32)

    def keep_u0(k, a, b):
        u0[a:b] = f[idx[a:b]]

    def keep_u1(k, a, b):
        u1[a:b] = f[idx[a:b]]

    def rhs(k, a, b):
        g = geo[k]
        r[a:b] = reinit_rhs(f, idx[a:b], *st, h, g[0], *g[2:])

    def first_half(k, a, b):
        f[idx[a:b]] = u0[a:b] + geo[k][1] * r[a:b]

    def second_half(k, a, b):
        f[idx[a:b]] = 0.5 * (u0[a:b] + u1[a:b] + geo[k][1] * r[a:b])

    # TVD-RK2 in pseudo time: every right-hand side of a half-step is evaluated before any node is written
    for _ in range(iterations):
        each(keep_u0)
        each(rhs)
        each(first_half)
        each(keep_u1)
        each(rhs)
        each(second_half)
    # levelset.py:70-77: clamp, then list |phi| < cap (1 - 1e-5), chunk by chunk of the grid
    cap = width * h
    gspans = _spans(f.size, workers)

    def rebuild(a, b):
        np.clip(f[a:b], F32(-cap), F32(cap), out=f[a:b])
        return np.nonzero(np.abs(f[a:b]) < F32(cap * (1 - 1e-5)))[0].astype(np.int64) + a

    out = np.concatenate(list(pool.map(lambda ab: rebuild(*ab), gspans)))
    check_margin(out, shape)
    return out


class ThreadedSimulation(Simulation):
    """reference_np.Simulation (evolve.py:67-250) whose stages, volume and reinitialisation run on
    ``workers`` threads (SVI laws)."""

    def __init__(self, phi3, h, law, workers: int, **kw):
        super().__init__(phi3, h, law, **kw)
        self.workers = int(workers)
        self.stage = ThreadedStage(self, self.workers)

    def close(self) -> None:
        self.stage.close()

    def _rhs(self, stats=False):
        return self.stage.rhs()

    def volume(self):
        if not hasattr(self, "stage"):   # the initial volume, taken in Simulation.__init__
            return super().volume()
        return self.stage.volume()

    def _reinitialize(self):
        return threaded_reinitialize(self.stage.pool, self.workers, self.phi, self.band, self.h,
                                     self.reinit_iterations, width=self.width)
