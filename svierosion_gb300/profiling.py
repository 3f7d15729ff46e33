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
        python -m svierosion_gb300.profiling --grid 448x336x245 --steps 2 --jit-wait   # ... after the
                                               # passes compiled for the axis lengths are loaded
        python -m svierosion_gb300.profiling --grid 448x336x245 --reinit 3    # reinitialisation calls
        python -m svierosion_gb300.profiling --job mean --resolution 160 --steps 30   # one served-mix job
    """
    import argparse
    import time

    import svierosion_gb300 as S
    from svierosion_gb300 import _native as nat

    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", default="448x336x245")
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--reinit", type=int, default=0)
    ap.add_argument("--job", choices=["svi", "mean", "gauss"], default=None,
                    help="erode one seeded fragment (subdivided 5x) with this law on the plain path, twice")
    ap.add_argument("--resolution", type=int, default=160)
    ap.add_argument("--jit-wait", action="store_true",
                    help="one untimed step first, then wait for the convolution passes compiled for the grid's "
                         "axis lengths, so that the --steps steps run them")
    a = ap.parse_args(argv)
    if a.job:
        # one request of the served mix's kind, solved alone (a mid-size curvature or SVI job)
        from svierosion_gb300 import shapes
        mesh = shapes.fragment(5, seed=3)
        L = float((mesh.bounds[1] - mesh.bounds[0]).max())
        kw = dict(radius=0.08 * L, k=1, s=1, t=0.93) if a.job == "svi" else dict(alpha=1.0 if a.job == "mean" else 0.25)
        params = S.ErosionParams(law=a.job, resolution=a.resolution, target_fraction=0.9, max_steps=a.steps, **kw)
        for _ in range(2):
            t0 = time.time()
            res = S.erode(mesh, params, extract_meshes=False, keep_state=True)
            torch.cuda.synchronize()
            print(a.job, res.grid.shape, "band", res.level_set.work32.numel(), len(res.history), "steps",
                  res.stop_reason, "%.1f us per step" % (1e6 * res.timings["evolve"] / max(len(res.history), 1)),
                  flush=True)
        return 0
    shape = tuple(int(v) for v in a.grid.split("x"))
    h = 2.078 / 400
    ls = _synthetic_levelset(shape, h)
    print("grid", shape, "band", ls.band32.numel(), flush=True)
    if a.reinit:
        # reinitialisation calls as the evolution loop makes them (work-set band rebuild): per call
        # the total and the 40 sweeps, by CUDA events
        for _ in range(a.reinit):
            timer = KernelTimer(capacity=16)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            ls.reinitialize(20, timer=timer, work_set_rebuild=True)
            e1.record()
            torch.cuda.synchronize()
            sw = timer.summary()["reinit_sweep"]
            print("work set %d, reinitialize %.3f ms, 40 sweeps %.3f ms (%.2f us each)"
                  % (timer.notes["reinit_work"][0], e0.elapsed_time(e1), sw["total_ms"], 1000 * sw["mean_ms"]),
                  flush=True)
        return 0
    law = S.SVIPowerLaw(0.05 * 2.078, 1, 1, 0.93)
    sim = S.ErosionSimulation(ls, law)
    if a.jit_wait:
        sim.run(target_fraction=None, max_steps=1)
        ready = nat.lib().svie_conv_jit_wait(120000)
        print("compiled passes ready" if ready == 0 else "compiled passes not ready (%d)" % ready, flush=True)
    t0 = time.time()
    res = sim.run(target_fraction=None, max_steps=a.steps)
    torch.cuda.synchronize()
    print("steps", len(res.history), "time", round(time.time() - t0, 4), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
