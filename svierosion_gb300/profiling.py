"""CUDA-event timing of individual kernels inside a timed region.

A pool of timing events is created up front (each recorded once so that the
driver object exists); kernels record events from the pool on the launching
stream, and ``summary()`` turns consecutive event pairs into per-kernel
durations after the region has been synchronised.
"""

from __future__ import annotations

import ctypes
from collections import defaultdict

import torch


class KernelTimer:
    """``only``: names of the sections to time (None = all); a section named
    "fft" stands for the five convolution passes."""

    def __init__(self, capacity: int = 8192, only=None):
        self.only = None if only is None else set(only)
        self.events = [torch.cuda.Event(enable_timing=True) for _ in range(capacity)]
        for e in self.events:
            e.record()
        torch.cuda.synchronize()
        self.next = 0
        self.groups = []  # (names, events, launches)
        self.notes = {}

    def wants(self, name: str) -> bool:
        return self.only is None or name in self.only

    def take(self, k: int) -> list:
        if self.next + k > len(self.events):
            raise RuntimeError("KernelTimer: event pool exhausted")
        evs = self.events[self.next:self.next + k]
        self.next += k
        return evs

    @staticmethod
    def handles(evs) -> ctypes.Array:
        return (ctypes.c_void_p * len(evs))(*[ctypes.c_void_p(e.cuda_event) for e in evs])

    def add(self, names, evs, launches=None) -> None:
        """Event pairs (evs[i], evs[i + 1]) for names[i]; ``launches[i]``: the
        kernel launches the pair brackets (default 1)."""
        self.groups.append((list(names), evs, list(launches) if launches is not None else [1] * len(names)))

    def note(self, key: str, value) -> None:
        """A value recorded beside the timings (e.g. the work-set size of a call)."""
        self.notes.setdefault(key, []).append(value)

    def reset(self) -> None:
        self.next = 0
        self.groups = []
        self.notes = {}

    def summary(self) -> dict:
        """name -> {"launches": n, "total_ms": t, "mean_ms": t / n}."""
        torch.cuda.synchronize()
        tot = defaultdict(float)
        cnt = defaultdict(int)
        for names, evs, launches in self.groups:
            for i, nm in enumerate(names):
                tot[nm] += evs[i].elapsed_time(evs[i + 1])
                cnt[nm] += launches[i]
        return {k: {"launches": cnt[k], "total_ms": float(tot[k]), "mean_ms": float(tot[k] / max(cnt[k], 1))}
                for k in tot}


def _synthetic_levelset(shape, h):
    """Analytic ellipsoid (semi-axes 1, 0.7, 0.5) level set on a grid of `shape`."""
    import svierosion_gb300 as S

    g = S.Grid(tuple(-0.5 * (n - 1) * h for n in shape), h, tuple(shape))
    ax = [torch.tensor(a, device="cuda", dtype=torch.float32) for a in g.axes()]
    X, Y, Z = torch.meshgrid(*ax, indexing="ij")
    phi = (torch.sqrt(X ** 2 + (Y / 0.7) ** 2 + (Z / 0.5) ** 2) - 1.0) * 0.6
    del X, Y, Z
    return S.LevelSet(phi.float(), g, width=6)


def main(argv=None) -> int:
    """Profiling driver for ncu captures of the step kernels on a synthetic level set.

        python -m svierosion_gb300.profiling --grid 448x336x245 --steps 2     # RK3 steps (FFT + stages)
        python -m svierosion_gb300.profiling --grid 448x336x245 --reinit 3    # reinitialisation sub-steps
    """
    import argparse
    import time

    import svierosion_gb300 as S
    from svierosion_gb300 import _native as nat

    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", default="448x336x245")
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--reinit", type=int, default=0)
    a = ap.parse_args(argv)
    shape = tuple(int(v) for v in a.grid.split("x"))
    h = 2.078 / 400
    ls = _synthetic_levelset(shape, h)
    print("grid", shape, "band", ls.band32.numel(), flush=True)
    if a.reinit:
        n = ls.grid.size
        nx, ny, nz = shape
        sc = ls.scratch
        for _ in range(a.reinit):
            # the steps of LevelSet.reinitialize, with events between them
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(7)]
            ev[0].record()
            nbits = nat.lib().svie_reinit_bits_bytes(nx, ny, nz)
            mask, tmp = sc.get("reinit_mask", nbits), sc.get("reinit_tmp", nbits)
            marked = sc.get("reinit_marked", nbits)
            nat.call("svie_reinit_bits", nat.ptr(ls.work32), ls.work32.numel(), nx, ny, nz, 3, 4, nat.ptr(mask),
                     nat.ptr(tmp), nat.ptr(marked), nat.stream())
            ev[1].record()
            ws = sc.get("brick", nat.lib().svie_brick_workspace_bytes(nx, ny, nz))
            cnt = sc.get("reinit_count", 8)
            nat.call("svie_brick_scan", 2, nat.ptr(mask), nx, ny, nz, 0.0, nat.ptr(ws), ws.numel(), nat.ptr(cnt),
                     nat.stream())
            m = int(cnt[:8].cpu().view(torch.int64)[0])
            idx = sc.get("reinit_idx", 4 * m)[:4 * m].view(torch.int32)
            nat.call("svie_brick_write", 2, nat.ptr(mask), nx, ny, nz, 0.0, nat.ptr(ws), ws.numel(), nat.ptr(idx), m,
                     nat.stream())
            ev[2].record()
            geo = sc.get("reinit_geo", nat.lib().svie_reinit_geometry_bytes(m))
            nat.call("svie_reinit_geometry", nat.ptr(ls.flat), nat.ptr(idx), m, *ls.strides, ls.h, 0.45, nat.ptr(geo),
                     nat.stream())
            off = sc.get("reinit_off_inside", 8)
            nat.call("svie_list_inside_off_mask", nat.ptr(ls.flat), nat.ptr(idx), m, nat.ptr(marked), nx, ny, nz,
                     nat.ptr(off), nat.stream())
            ev[3].record()
            pt = sc.get("reinit_phi", 4 * n)
            nat.call("svie_reinit_iterate", nat.ptr(ls.flat), nat.ptr(pt), n, nat.ptr(idx), m, *ls.strides, ls.h,
                     nat.ptr(geo), 20, nat.stream())
            ev[4].record()
            ls.rebuild_band_on(idx, off)
            ev[5].record()
            torch.cuda.synchronize()
            t = [ev[i].elapsed_time(ev[i + 1]) for i in range(5)]
            print("work set %d mask %.3f compact %.3f geometry %.3f copy+40 sweeps %.3f rebuild %.3f ms" % (m, *t),
                  flush=True)
        return 0
    law = S.SVIPowerLaw(0.05 * 2.078, 1, 1, 0.93)
    sim = S.ErosionSimulation(ls, law)
    t0 = time.time()
    res = sim.run(target_fraction=None, max_steps=a.steps)
    torch.cuda.synchronize()
    print("steps", len(res.history), "time", round(time.time() - t0, 4), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
