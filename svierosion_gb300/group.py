"""Many level sets advanced in one launch per pass (the batched form of evolve.py:182-250).

The reference advances one solid at a time.  Here a ``GroupStep`` takes the
simulations whose next step is due and runs that step for all of them
together: every band kernel of the step (occupancy refresh, curvature
scatter, the fused stage right-hand side with its statistics, the time step,
the three RK combinations, the float64 volume) is one launch over the packed
(member, tile) list of all members (``svie_group_*`` in include/svie.h); only
the SVI members' FFT convolutions are launched per member, between the
batched occupancy refresh and the batched stage.  The members' statistics --
their time steps stay on the device -- are gathered into one block and read
back with one copy, after which each member finishes its step on the host
exactly as alone (``ErosionSimulation.step_finish``: regula falsi on the last
step, the reinitialisation trigger, history).  A member's arithmetic is the
one-level-set kernels' own, so its results equal a solve on its own bit for
bit.

The launch sequence is captured as a CUDA graph once the same members with
the same bands take two steps in a row, and replayed while that holds.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native as nat


class GroupStep:
    """One TVD-RK3 step for a list of ``ErosionSimulation``s, batched (see module docstring).

    Members need no time cap (``max_time`` None) and the one-Newton-step projection."""

    def __init__(self, device, use_graphs: bool = True):
        self.device = device
        self.use_graphs = use_graphs
        self.group = nat.Group()
        self._key = None
        self._table = None
        self._staging = None
        self._stats_dev = None
        self._stats_host = None
        self._sims = []
        self._graph = None
        self._graph_key = None
        self._warm_key = None
        self._event = None
        self.graph_replays = 0
        self.graph_kernels = 0
        self.steps = 0

    # ------------------------------------------------------------- table
    def _members(self, sims):
        members = (nat.GroupMember * len(sims))()
        lib = nat.lib()
        for k, sim in enumerate(sims):
            ls = sim.ls
            band = ls.work32
            m = band.numel()
            nx, ny, nz = ls.grid.shape
            sws = ls.scratch.get("stage", lib.svie_stage_workspace_bytes(m))
            vws = ls.scratch.get("volume", lib.svie_volume_workspace_bytes(m))
            g = members[k]
            g.phi, g.band, g.m = band_ptr(ls.flat), band_ptr(band), m
            g.nx, g.ny, g.nz = nx, ny, nz
            g.kind = 0 if sim.law.requires_svi else 1
            g.field, g.occ, g.u0 = band_ptr(sim._field), band_ptr(ls.occ), band_ptr(sim._u0)
            for j in range(3):
                g.L[j] = band_ptr(sim._L[j])
            g.stats, g.vstats = band_ptr(sim._stats), band_ptr(ls._vstats)
            g.stage_ws, g.stage_ws_bytes = band_ptr(sws), sws.numel()
            g.volume_ws, g.volume_ws_bytes = band_ptr(vws), vws.numel()
            g.law = sim._law_c
        return members

    def _build(self, sims, key) -> None:
        lib = nat.lib()
        members = self._members(sims)
        n = len(sims)
        tiles = lib.svie_group_tiles(members, n)
        nbytes = lib.svie_group_table_bytes(n, tiles)
        if self._table is None or self._table.numel() < nbytes:
            self._table = torch.empty(nbytes + (nbytes >> 2), dtype=torch.uint8, device=self.device)
            self._staging = torch.empty(self._table.numel(), dtype=torch.uint8, pin_memory=True)
        nat.call("svie_group_build", members, n, nat.ptr(self._table), self._table.numel(),
                 ctypes.c_void_p(self._staging.data_ptr()), ctypes.byref(self.group), nat.stream())
        # the staging buffer is reused by the next build: wait for this copy
        torch.cuda.current_stream().synchronize()
        sb = 2 * n * nat.STATS_BYTES
        if self._stats_dev is None or self._stats_dev.numel() < sb:
            self._stats_dev = torch.empty(sb, dtype=torch.uint8, device=self.device)
            self._stats_host = torch.empty(sb, dtype=torch.uint8, pin_memory=True)
        self._key = key
        self._graph = None

    @staticmethod
    def _key_of(sims):
        """What the table depends on: the members and their bands (a member's buffers and
        workspaces are sized by its band, so they change only with it)."""
        return tuple((sim.serial, sim._band_key) for sim in sims)

    # ------------------------------------------------------------ launch
    def _body(self, sims) -> None:
        g = ctypes.byref(self.group)
        s = nat.stream()
        svi = [sim for sim in sims if sim.law.requires_svi]
        curv = len(svi) < len(sims)
        nat.call("svie_group_stats_reset", g, s)
        for stage in range(3):
            if stage > 0:
                nat.call("svie_group_rk", g, stage, s)
            if svi:
                nat.call("svie_group_scatter_fractions", g, s)
                for sim in svi:
                    sim.conv.exterior_fraction_into(sim.ls.occ, sim._field, flags=(sim._lineflag, sim._slabflag))
            if curv:
                nat.call("svie_group_curvature_scatter", g, s)
            nat.call("svie_group_stage", g, stage, s)
            if stage == 0:
                nat.call("svie_group_stats_finalize", g, s)
        nat.call("svie_group_rk", g, 3, s)
        nat.call("svie_group_volume", g, s)
        n = len(sims)
        nat.call("svie_group_gather_stats", g, nat.ptr(self._stats_dev), s)
        sb = 2 * n * nat.STATS_BYTES
        self._stats_host[:sb].copy_(self._stats_dev[:sb], non_blocking=True)

    def launch(self, sims) -> None:
        """Enqueue one step of every simulation in ``sims`` (each one's ``step_begin`` returned True)
        on the current stream; ``finish`` completes it."""
        self._sims = list(sims)
        if not sims:
            return
        key = self._key_of(sims)
        if key != self._key:
            self._build(sims, key)
        graphable = self.use_graphs
        if graphable and self._graph is not None and self._graph_key == key:
            self._graph.replay()
            self.graph_replays += 1
        elif graphable and self._warm_key == key:
            lib = nat.lib()
            cur = torch.cuda.current_stream()
            side = torch.cuda.Stream(device=self.device)
            side.wait_stream(cur)
            graph = torch.cuda.CUDAGraph()
            n0 = lib.svie_launch_count()
            with torch.cuda.stream(side):
                graph.capture_begin(capture_error_mode="thread_local")
                try:
                    self._body(sims)
                finally:
                    graph.capture_end()
            cur.wait_stream(side)
            self.graph_kernels = int(lib.svie_launch_count() - n0)
            self._graph, self._graph_key = graph, key
            graph.replay()
            self.graph_replays += 1
        else:
            self._body(sims)
            self._warm_key = key
        for sim in sims:
            sim.ls.occ_current = True   # the volume pass wrote the band's fractions
        if self._event is None:
            self._event = torch.cuda.Event()
        self._event.record()
        self.steps += 1

    def ready(self) -> bool:
        return self._event is None or self._event.query()

    def finish(self) -> None:
        """Wait for the launched step, then finish it for every member on the host (on the current
        stream: regula falsi and reinitialisation run there)."""
        sims = self._sims
        self._sims = []
        if not sims:
            return
        self._event.synchronize()
        raw = self._stats_host[:2 * len(sims) * nat.STATS_BYTES].numpy().tobytes()
        rec = np.frombuffer(raw, dtype=nat.STATS_DTYPE).reshape(len(sims), 2)
        for k, sim in enumerate(sims):
            sim.step_finish(stats=(rec[k, 0], rec[k, 1]))

    @property
    def kernel_launches(self) -> int:
        """Kernels run by graph replays (direct launches are counted by the library)."""
        return self.graph_replays * self.graph_kernels


def band_ptr(t: torch.Tensor):
    return nat.ptr(t).value


class SerialStep:
    """The GroupStep interface over each member's own step: the members' launch sequences (the
    curvature laws' own CUDA graphs) go back to back on one stream, each with its statistics copy,
    and one event closes the step.  A member's kernels then run while its level set is the one in
    L2, where packed launches interleave all members' data."""

    def __init__(self, device):
        self.device = device
        self._sims = []
        self._event = None
        self.steps = 0
        self._replayed = 0   # kernels run by the members' graph replays so far

    def launch(self, sims) -> None:
        self._sims = list(sims)
        for sim in sims:
            before = sim.kernel_launches
            sim._launch_step()
            self._replayed += sim.kernel_launches - before
        if self._event is None:
            self._event = torch.cuda.Event()
        self._event.record()
        self.steps += 1

    def ready(self) -> bool:
        return self._event is None or self._event.query()

    def finish(self) -> None:
        sims = self._sims
        self._sims = []
        if not sims:
            return
        self._event.synchronize()
        for sim in sims:
            sim.step_finish()

    @property
    def kernel_launches(self) -> int:
        """Kernels run by the members' graph replays (direct launches are counted by the library)."""
        return self._replayed
