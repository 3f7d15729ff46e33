"""Batched and served erosion: many independent solids on one GPU.

Every solid (an :class:`ErosionJob`) owns its level set, simulation and
workspaces.  :class:`LaneScheduler` runs the jobs in a few lanes, each a
group of jobs of one law kind that advances a step at a time with a single
launch per pass over the packed band tiles of all its members
(:class:`~svierosion_gb300.group.GroupStep`), on its own stream.  The lanes
are not in lockstep: the host opens a lane's next steps (stop tests;
snapshot fractions and the next target when a run stops), finishes its
completed step (statistics, regula falsi on the last step,
reinitialisation) and relaunches it while the other lanes run on the GPU.
Each job's time step and stop test are its own and its arithmetic is the
plain path's, so its result is the same alone and in the mix.

:class:`ErosionServer` runs an open-loop request stream on top: requests are
admitted as slots and HBM (estimated footprint) free up, folded into the
running groups at step boundaries, and their latency (arrival to result) is
recorded.
"""

from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native as nat
from .api import ErosionParams, make_grid
from .evolve import ErosionSimulation
from .grid import get_device
from .group import GroupStep, SerialStep
from .levelset import LevelSet, tricubic
from .meshio import TriMesh
from .sdf import mesh_to_sdf

# Device bytes per grid node while a job runs: phi, occupancy, N field,
# padded half spectrum, the reinitialisation copy of phi and its two masks,
# the maintained (k1, k2) field of curvature laws, plus the transient SDF
# arrays (keys, distance, triangle ids, masks) during set-up.
BYTES_PER_NODE = 48
BYTES_PER_BAND_NODE = 40


def footprint_bytes(grid_nodes: int, band_nodes: int | None = None) -> int:
    """Estimated peak device memory of one job."""
    band = band_nodes if band_nodes is not None else grid_nodes // 8
    return int(BYTES_PER_NODE * grid_nodes + BYTES_PER_BAND_NODE * band + (64 << 20))


@dataclass
class JobResult:
    name: str
    stop_reason: str
    fraction: float
    time: float
    steps: int
    band_updates: int
    history: list = field(default_factory=list)
    snapshots: list = field(default_factory=list)      # [(fraction, time, band phi on the host)]
    grid_shape: tuple = ()
    setup_s: float = 0.0
    wall_s: float = 0.0


class ErosionJob:
    """One erosion solve that can be advanced a step at a time."""

    def __init__(self, mesh: TriMesh, params: ErosionParams, name: str = "", device=None, stream=None,
                 keep_snapshot_phi: bool = False):
        self.mesh = mesh
        self.params = params
        self.name = name
        self.device = get_device(device if device is not None else params.device)
        self.stream = stream if stream is not None else torch.cuda.Stream(device=self.device)
        self.keep_snapshot_phi = keep_snapshot_phi
        self.grid = make_grid(mesh, params)
        self.done = False
        self.result: JobResult | None = None
        self.sim: ErosionSimulation | None = None

    @property
    def grid_nodes(self) -> int:
        return self.grid.size

    def footprint(self) -> int:
        return footprint_bytes(self.grid.size)

    def setup(self) -> None:
        """SDF, narrow band and simulation on the job's stream (erode(), api.py:200-233)."""
        t0 = time.time()
        p = self.params
        lo, hi = self.mesh.bounds
        self.law = p.make_law(length_scale=float((hi - lo).max()))
        with torch.cuda.stream(self.stream):
            phi = mesh_to_sdf(self.mesh, self.grid, band=p.band, device=self.device)
            self.ls = LevelSet(phi, self.grid, width=p.band)
            self.sim = ErosionSimulation(self.ls, self.law, cfl=p.cfl, feedback_cfl=p.feedback_cfl,
                                         parabolic_cfl=p.parabolic_cfl, reinit_distance=p.reinit_distance,
                                         reinit_iterations=p.reinit_iterations)
            if self.law.requires_svi and self.law.s == 1:
                n0 = self.sim.svi_field()
                nmax = float(tricubic(n0.view(-1), self.grid.shape,
                                      self.ls.closest_points(self.ls.interface_nodes())).max())
                if nmax >= self.law.t:
                    raise ValueError(f"max N_r on the initial surface is {nmax:.4f} >= t = {self.law.t}")
            self.targets = sorted({float(f) for f in p.snapshots if f > p.target_fraction},
                                  reverse=True) + [p.target_fraction]
            self.snapshots = []
            self.sim.begin_run(self.targets[0], max_steps=p.max_steps)
        self.setup_s = time.time() - t0
        self.t_start = time.time()

    def launch(self) -> bool:
        """Enqueue the next step; False once the job has finished."""
        if self.done:
            return False
        with torch.cuda.stream(self.stream):
            while not self.sim.step_launch():
                if not self._next_target():
                    return False
        return True

    def begin_step(self) -> bool:
        """Open the job's next step (stop tests; at a stop, the snapshot and the next target);
        False once the job has finished.  The step itself is run by a :class:`LaneScheduler`."""
        if self.done:
            return False
        with torch.cuda.stream(self.stream):
            while not self.sim.step_begin():
                if not self._next_target():
                    return False
        return True

    def _next_target(self) -> bool:
        """The run stopped: keep the snapshot, then start the run to the next target fraction;
        False when the job is complete."""
        res = self.sim.end_run()
        snap_phi = None
        if self.keep_snapshot_phi:
            snap_phi = nat.d2h(self.ls.band_values())
        self.snapshots.append((res.fraction, self.sim.time, snap_phi))
        self.targets.pop(0)
        if res.stop_reason != "target_volume" or not self.targets:
            self._complete(res)
            return False
        self.sim.begin_run(self.targets[0], max_steps=self.params.max_steps)
        return True

    def finish(self) -> None:
        with torch.cuda.stream(self.stream):
            self.sim.step_finish()

    def ready(self) -> bool:
        """The launched step has completed on the GPU (non-blocking)."""
        return self.sim.step_ready()

    def wait(self) -> None:
        """Block until the launched step has completed."""
        ev = self.sim._done_event
        if ev is not None:
            ev.synchronize()

    def _complete(self, res) -> None:
        self.done = True
        self.result = JobResult(self.name, res.stop_reason, res.fraction, self.sim.time, self.sim.steps,
                                self.sim.band_updates, list(self.sim.history), self.snapshots[:-1],
                                tuple(self.grid.shape), self.setup_s, time.time() - self.t_start)

    def release(self) -> None:
        """Drop device state (the result stays)."""
        self.sim = None
        self.ls = None


class _Lane:
    """Jobs of one law kind advanced together on their own stream, by a :class:`GroupStep` (packed
    launches) or a :class:`SerialStep` (each job's own launch sequence, back to back)."""

    def __init__(self, device, svi: bool, serial: bool = False):
        self.svi = svi
        self.stream = torch.cuda.Stream(device=device)
        # an SVI job's band changes at every reinitialisation (every few steps), before a graph
        # capture pays off; curvature-law jobs keep theirs for hundreds of steps
        self.group = SerialStep(device) if serial else GroupStep(device, use_graphs=not svi)
        self.jobs: list[ErosionJob] = []
        self.busy = False


class LaneScheduler:
    """Runs many jobs as a few lanes: each lane a group of jobs of one law kind advanced a step
    at a time on its own stream.  SVI lanes use one launch per pass over all their jobs' band
    tiles (:class:`~svierosion_gb300.group.GroupStep`); curvature lanes by default replay each
    job's own step graph back to back (:class:`~svierosion_gb300.group.SerialStep`), which keeps
    one job's data in L2 while its kernels run (``serial_curvature=False``: packed launches).  The lanes are not in lockstep: while the GPU runs one lane's step, the host finishes
    another's (statistics, stop tests, regula falsi, reinitialisation) and relaunches it at once,
    so host work and GPU work overlap.  A job's arithmetic is its own throughout."""

    def __init__(self, device, lanes_svi: int = 2, lanes_curvature: int = 8, serial_curvature: bool = True):
        self.lanes = [_Lane(device, True) for _ in range(lanes_svi)] + \
                     [_Lane(device, False, serial_curvature) for _ in range(lanes_curvature)]

    def add(self, job: ErosionJob) -> None:
        """A set-up job joins the least loaded lane of its law kind (at that lane's next step)."""
        svi = job.sim.law.requires_svi
        lane = min((ln for ln in self.lanes if ln.svi == svi), key=lambda ln: len(ln.jobs))
        lane.jobs.append(job)

    @property
    def active(self) -> bool:
        return any(ln.jobs for ln in self.lanes)

    def _relaunch(self, lane: _Lane, on_done) -> None:
        """Open the next step of the lane's jobs (completed jobs leave it) and launch it."""
        with torch.cuda.stream(lane.stream):
            due = []
            for j in lane.jobs:
                if j.begin_step():
                    due.append(j)
                elif on_done is not None:
                    on_done(j)
            lane.jobs = due
            if due:
                lane.group.launch([j.sim for j in due])
        lane.busy = bool(due)

    def _finish(self, lane: _Lane) -> None:
        with torch.cuda.stream(lane.stream):
            lane.group.finish()
        lane.busy = False

    def poll(self, on_done=None, block: bool = True) -> None:
        """Advance: launch the idle lanes, finish (and relaunch) every lane whose step has completed;
        if none has and ``block``, wait for one.  ``on_done(job)`` is called for every job that
        completes."""
        progressed = False
        for lane in self.lanes:
            if not lane.busy and lane.jobs:
                self._relaunch(lane, on_done)
                progressed = True
        for lane in self.lanes:
            if lane.busy and lane.group.ready():
                self._finish(lane)
                self._relaunch(lane, on_done)
                progressed = True
        if not progressed and block:
            busy = [ln for ln in self.lanes if ln.busy]
            if busy:
                self._finish(busy[0])
                self._relaunch(busy[0], on_done)

    def drain(self, on_done=None) -> None:
        while self.active:
            self.poll(on_done)
        torch.cuda.synchronize()

    @property
    def kernel_launches(self) -> int:
        """Kernels run by graph replays (direct launches are counted by the library)."""
        return sum(ln.group.kernel_launches for ln in self.lanes)


class BatchedErosion:
    """Advance many solids together; each stops independently (spec batched form)."""

    def __init__(self, jobs: list[ErosionJob], lanes_svi: int = 2, lanes_curvature: int = 8,
                 serial_curvature: bool = True):
        self.jobs = list(jobs)
        self.lanes = (lanes_svi, lanes_curvature, serial_curvature)

    def run(self, release: bool = True) -> list[JobResult]:
        sched = self.stepper = LaneScheduler(self.jobs[0].device if self.jobs else get_device(None), *self.lanes)
        on_done = (lambda j: j.release()) if release else None
        for j in self.jobs:   # each job starts stepping as soon as it is set up
            j.setup()
            sched.add(j)
            sched.poll(on_done, block=False)
        sched.drain(on_done)
        return [j.result for j in self.jobs]


def run_plain(jobs: list[ErosionJob]) -> list[JobResult]:
    """The same jobs one at a time (the plain form)."""
    out = []
    for j in jobs:
        j.setup()
        while not j.done:
            if j.launch():
                j.finish()
        torch.cuda.synchronize()
        out.append(j.result)
        j.release()
    return out


@dataclass
class Request:
    rid: int
    arrival: float          # seconds after the start of the stream
    mesh: TriMesh
    params: ErosionParams
    admitted: float = math.nan
    completed: float = math.nan
    result: JobResult | None = None


class ErosionServer:
    """Continuous batching of erosion requests under an HBM budget."""

    def __init__(self, hbm_budget_bytes: int = 150 << 30, max_active: int = 64, device=None, lanes_svi: int = 2,
                 lanes_curvature: int = 8, serial_curvature: bool = True):
        self.lanes = (lanes_svi, lanes_curvature, serial_curvature)
        self.budget = int(hbm_budget_bytes)
        self.max_active = int(max_active)
        self.device = get_device(device)
        self.queue: deque[Request] = deque()
        self.active: list[tuple[Request, ErosionJob]] = []
        self.in_use = 0
        self.done: list[Request] = []

    def submit(self, req: Request) -> None:
        self.queue.append(req)

    def _admit(self, now: float) -> None:
        while self.queue and len(self.active) < self.max_active and self.queue[0].arrival <= now:
            req = self.queue[0]
            job = ErosionJob(req.mesh, req.params, name=str(req.rid), device=self.device)
            need = job.footprint()
            if self.active and self.in_use + need > self.budget:
                return  # wait for memory (first-come first-served)
            self.queue.popleft()
            job.setup()
            req.admitted = now
            self.in_use += need
            self.active.append((req, job))

    def run(self, requests: list[Request]) -> dict:
        """Open-loop: request i becomes visible at t0 + arrival_i; admitted requests join the
        running lanes at their next step boundary."""
        for r in sorted(requests, key=lambda r: r.arrival):
            self.submit(r)
        sched = LaneScheduler(self.device, *self.lanes)
        t0 = self._t0 = time.time()
        req_of = {}
        total = [0]

        def done(j):   # result, latency, memory back
            r = req_of.pop(id(j))
            r.completed = time.time() - t0
            r.result = j.result
            total[0] += j.result.band_updates
            self.in_use -= j.footprint()
            j.release()
            self.done.append(r)
            self.active = [(q, k) for q, k in self.active if k is not j]

        while self.queue or self.active:
            now = time.time() - t0
            n0 = len(self.active)
            self._admit(now)
            for r, j in self.active[n0:]:
                req_of[id(j)] = r
                sched.add(j)
            if not self.active:
                time.sleep(max(0.0, min(self.queue[0].arrival - now, 0.01)))
                continue
            sched.poll(on_done=done)
        torch.cuda.synchronize()
        updates = total[0]
        wall = time.time() - t0
        lat = np.array([r.completed - r.arrival for r in self.done])
        return {"requests": len(self.done), "wall_s": wall, "solves_per_s": len(self.done) / wall,
                "band_updates_per_s": updates / wall,
                "latency_s": {"p50": float(np.percentile(lat, 50)), "p95": float(np.percentile(lat, 95)),
                              "p99": float(np.percentile(lat, 99)), "max": float(lat.max())}}
