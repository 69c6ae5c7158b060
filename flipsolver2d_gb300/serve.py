"""Serving loop: continuous batching of FLIP frames and standalone pressure
solves on one GPU.

Requests arrive over time.  A *frame* request advances a resident scene by
one frame (FlipSolver::stepFrame); a *solve* request is one standalone
pressure system solved to a 1e-6 true relative residual.  The server keeps
every admitted scene's particles and grids on the device between requests
and drives the native batch (``fs_batch_*`` in include/fs_gpu.h) round by
round:

- a round advances every scene that is inside a frame by one substep and
  solves every submitted standalone system together with that round's
  pressure solves (one cluster launch per plan);
- between rounds, requests that have arrived are admitted: a frame request
  starts its scene's frame at once (it joins the next round while other
  scenes are mid-frame -- continuous batching, not a queue), a solve request
  is copied to the device and rides in the next round;
- admission is by device-memory footprint: a new scene or solve waits while
  the bytes held by resident scenes and in-flight solves plus its own would
  exceed the budget.  A scene already resident needs no new memory.

Every result is the same as when the request is served alone: each scene's
substeps and each system's solve are deterministic and independent of what
else shares the rounds.

Latency is measured from a request's arrival to the end of the round that
completes it.  Frame requests to a scene that is already inside a frame wait
for that frame to end.
"""
from __future__ import annotations

import collections
import dataclasses
import math
import time
from typing import Callable, Dict, List, Optional

import numpy as np

from . import gpu, scenes

# device bytes of a standalone system: material and operator bytes, FP64
# right-hand side and solution, plus the small per-system scalars
SOLVE_BYTES_PER_CELL = 18
SOLVE_BYTES_FIXED = 512
# above the on-chip limit of the cluster solve (about 512^2 cells) a system
# is solved by the chained cooperative kernel with five FP32 vectors
SOLVE_CHAIN_CELLS = 512 * 512
SOLVE_CHAIN_BYTES_PER_CELL = 20


def scene_bytes_estimate(scene) -> int:
    """An upper estimate of a scene's device footprint before it exists: the
    grids at about 180 B per cell, the PCG vectors at 48 B per cell (FP64 in
    spec mode) and particle storage for 2 x particlesPerCell per cell at
    80 B per particle slot.  Once created the exact figure replaces it."""
    p = scene.params
    _, ni, nj = p.grid()
    cells = ni * nj
    return int(cells * (180 + 48) + 2 * p.particlesPerCell * cells * 80)


@dataclasses.dataclass
class Request:
    kind: str                 # "frame" or "solve"
    arrival: float            # seconds from the start of the run
    scene: Optional[str] = None      # frame: the key of a registered scene
    problem: Optional[tuple] = None  # solve: (material, rhs, dt, density, dx)
    start: float = math.nan   # admitted
    done: float = math.nan    # completed
    result: object = None     # solve: (iterations, x, rel_residual)
    ticket: int = 0
    work: int = 0             # frame: particle-substeps; solve: cell-iterations


def _spec_solver(scene):
    return gpu.GpuFlipSolver(scene, precision=gpu.FS_PCG_SPEC)


class Server:
    """`make_batch` and `make_solver` build the native batch and the scene
    handles (gpu.Batch and FS_PCG_SPEC handles; tests pass stand-ins)."""

    def __init__(self, budget_bytes: float = 150e9, clock: Callable[[], float] = time.perf_counter,
                 make_batch: Callable = None, make_solver: Callable = None):
        self.batch = (make_batch or gpu.Batch)()
        self.make_solver = make_solver or _spec_solver
        self.budget = float(budget_bytes)
        self.clock = clock
        self.specs: Dict[str, object] = {}        # registered scenes (not yet resident)
        self.resident: Dict[str, gpu.GpuFlipSolver] = {}
        self.bytes: Dict[str, int] = {}
        self.solve_bytes: Dict[int, int] = {}
        self.pending: collections.deque = collections.deque()
        self.active_frames: Dict[str, Request] = {}
        self.active_solves: Dict[int, Request] = {}
        self.finished: List[Request] = []
        self.rounds = 0
        self.t0 = None

    # ---------------------------------------------------------------- setup
    def register_scene(self, key: str, scene) -> None:
        """Make a scene known; it becomes resident on its first frame request."""
        self.specs[key] = scene

    def used_bytes(self) -> int:
        return sum(self.bytes.values()) + sum(self.solve_bytes.values())

    # -------------------------------------------------------------- serving
    def _admit(self, now: float) -> None:
        keep = collections.deque()
        while self.pending:
            rq = self.pending.popleft()
            if rq.arrival > now:
                keep.append(rq)
                continue
            if rq.kind == "frame":
                if rq.scene in self.active_frames:
                    keep.append(rq)  # the scene's current frame ends first
                    continue
                if rq.scene not in self.resident:
                    need = scene_bytes_estimate(self.specs[rq.scene])
                    if self.used_bytes() + need > self.budget:
                        keep.append(rq)
                        continue
                    g = self.make_solver(self.specs[rq.scene])
                    self.batch.add(g)
                    self.resident[rq.scene] = g
                    self.bytes[rq.scene] = need
                g = self.resident[rq.scene]
                self.batch.begin_frame(g)  # seeds the particles at frame 0
                rq.work = g.particle_count()
                self.bytes[rq.scene] = g.device_bytes()
                rq.start = now
                self.active_frames[rq.scene] = rq
            else:
                mat = rq.problem[0]
                need = SOLVE_BYTES_PER_CELL * mat.size + SOLVE_BYTES_FIXED
                if mat.size > SOLVE_CHAIN_CELLS:
                    need += SOLVE_CHAIN_BYTES_PER_CELL * mat.size
                if self.used_bytes() + need > self.budget:
                    keep.append(rq)
                    continue
                rq.ticket = self.batch.submit_solve(*rq.problem)
                self.solve_bytes[rq.ticket] = need
                rq.start = now
                self.active_solves[rq.ticket] = rq
        self.pending = keep

    def _collect(self, now: float) -> None:
        for key in list(self.active_frames):
            g = self.resident[key]
            if not self.batch.in_frame(g):
                rq = self.active_frames.pop(key)
                rq.work *= g.stat(2)  # particles at the frame start x its substeps
                rq.done = now
                self.finished.append(rq)
        for t in list(self.active_solves):
            if self.batch.solve_done(t):
                rq = self.active_solves.pop(t)
                rq.result = self.batch.take_solve(t)
                rq.work = rq.problem[0].size * rq.result[0]
                del self.solve_bytes[t]
                rq.done = now
                self.finished.append(rq)

    def run(self, requests: List[Request], idle_sleep: float = 0.0) -> List[Request]:
        """Serves `requests` (arrival times relative to the start) until all
        are done; returns them with start and completion times set."""
        self.pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        self.t0 = self.clock()
        total = len(requests)
        while len(self.finished) < total:
            now = self.clock() - self.t0
            self._admit(now)
            if not (self.active_frames or self.active_solves) and self.pending and \
                    all(r.arrival <= now for r in self.pending):
                raise RuntimeError("a request cannot be admitted within the device-memory budget")
            if self.active_frames or self.active_solves:
                self.batch.round()
                self.rounds += 1
                self._collect(self.clock() - self.t0)
            elif self.pending:
                nxt = min(r.arrival for r in self.pending)
                if nxt > now and idle_sleep >= 0:
                    time.sleep(min(idle_sleep or (nxt - now), max(nxt - now, 0.0)))
        return self.finished

    def close(self) -> None:
        self.batch.close()
        for g in self.resident.values():
            g.close()
        self.resident.clear()


# ----------------------------------------------------------------- workload
def serving_workload(n_requests: int, rate: float = 2000.0, seed: int = 9, pool: int = 32,
                     frame_sides=(64, 1024), solve_sides=(256, 2048), solve_fraction: float = 0.2):
    """The serving workload: Poisson arrivals at `rate` per second from
    default_rng(seed); a fraction `solve_fraction` are standalone solves with
    a side log-uniform in `solve_sides` and the masks of scenes.poisson_case,
    the rest frame requests to one of `pool` resident scenes, each with a side
    log-uniform in `frame_sides` and the layout of scenes.random_scene.
    Returns (scene specs by key, requests)."""
    rng = np.random.default_rng(seed)
    specs = {}
    for k in range(pool):
        side = int(round(math.exp(rng.uniform(math.log(frame_sides[0]), math.log(frame_sides[1])))))
        side = max(frame_sides[0], min(frame_sides[1], 4 * (side // 4)))
        specs[f"scene{k}"] = scenes.random_scene(side, 5000 + k)
    t = 0.0
    reqs = []
    for k in range(n_requests):
        t += rng.exponential(1.0 / rate)
        if rng.random() < solve_fraction:
            side = int(round(math.exp(rng.uniform(math.log(solve_sides[0]), math.log(solve_sides[1])))))
            side = max(solve_sides[0], min(solve_sides[1], side))
            m, b, dx = scenes.poisson_case(side, seed=int(rng.integers(1 << 30)))
            reqs.append(Request("solve", t, problem=(m, b, 1.0 / 30, 1000.0, dx)))
        else:
            reqs.append(Request("frame", t, scene=f"scene{int(rng.integers(pool))}"))
    return specs, reqs


def latency_summary(done: List[Request]) -> dict:
    out = {}
    for kind in ("frame", "solve"):
        lat = [1e3 * (r.done - r.arrival) for r in done if r.kind == kind]
        if lat:
            out[kind] = {"n": len(lat), "p50_ms": float(np.percentile(lat, 50)),
                         "p99_ms": float(np.percentile(lat, 99))}
    lat = [1e3 * (r.done - r.arrival) for r in done]
    if lat:
        out["all"] = {"n": len(lat), "p50_ms": float(np.percentile(lat, 50)),
                      "p99_ms": float(np.percentile(lat, 99))}
    return out
