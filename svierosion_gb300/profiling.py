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
    def __init__(self, capacity: int = 8192):
        self.events = [torch.cuda.Event(enable_timing=True) for _ in range(capacity)]
        for e in self.events:
            e.record()
        torch.cuda.synchronize()
        self.next = 0
        self.groups = []  # (names, events)

    def take(self, k: int) -> list:
        if self.next + k > len(self.events):
            raise RuntimeError("KernelTimer: event pool exhausted")
        evs = self.events[self.next:self.next + k]
        self.next += k
        return evs

    @staticmethod
    def handles(evs) -> ctypes.Array:
        return (ctypes.c_void_p * len(evs))(*[ctypes.c_void_p(e.cuda_event) for e in evs])

    def add(self, names, evs) -> None:
        self.groups.append((list(names), evs))

    def reset(self) -> None:
        self.next = 0
        self.groups = []

    def summary(self) -> dict:
        """name -> {"launches": n, "total_ms": t, "mean_ms": t / n}."""
        torch.cuda.synchronize()
        acc = defaultdict(list)
        for names, evs in self.groups:
            for i, nm in enumerate(names):
                acc[nm].append(evs[i].elapsed_time(evs[i + 1]))
        return {k: {"launches": len(v), "total_ms": float(sum(v)), "mean_ms": float(sum(v) / len(v))}
                for k, v in acc.items()}
