"""Host logic of the serving loop (flipsolver2d_gb300/serve.py) with
stand-ins for the native batch: admission by device-memory footprint,
continuous batching (a frame request joins the next round while other scenes
are mid-frame), per-scene ordering and latency accounting."""
import numpy as np
import pytest

from flipsolver2d_gb300 import scenes, serve


class FakeSolver:
    def __init__(self, scene, substeps=3):
        self.scene = scene
        self.substeps = substeps
        self.frames = 0

    def particle_count(self):
        return 100

    def stat(self, which):
        return self.substeps

    def device_bytes(self):
        return 1000


class FakeBatch:
    """Each frame takes `substeps` rounds; a solve completes in one round."""

    def __init__(self):
        self.left = {}
        self.solves = {}
        self.next = 1
        self.log = []

    def add(self, g):
        self.left[g] = 0

    def begin_frame(self, g):
        assert self.left[g] == 0
        self.left[g] = g.substeps

    def in_frame(self, g):
        return self.left[g] > 0

    def round(self):
        active = [g for g, n in self.left.items() if n > 0]
        self.log.append((len(active), sum(1 for v in self.solves.values() if not v)))
        for g in active:
            self.left[g] -= 1
            if self.left[g] == 0:
                g.frames += 1
        for t in self.solves:
            self.solves[t] = True
        return sum(1 for n in self.left.values() if n > 0)

    def submit_solve(self, m, b, dt, dens, dx):
        t = self.next
        self.next += 1
        self.solves[t] = False
        return t

    def solve_done(self, t):
        return self.solves[t]

    def take_solve(self, t):
        del self.solves[t]
        return (7, None, 1e-7)

    def close(self):
        pass


class Clock:
    def __init__(self, step=1e-3):
        self.t = 0.0
        self.step = step

    def __call__(self):
        self.t += self.step
        return self.t


def _server(budget=1e12):
    return serve.Server(budget, clock=Clock(), make_batch=FakeBatch, make_solver=FakeSolver)


def test_continuous_batching_and_per_scene_order():
    s = _server()
    s.register_scene("a", scenes.random_scene(64, 1))
    s.register_scene("b", scenes.random_scene(64, 2))
    reqs = [serve.Request("frame", 0.0, scene="a"), serve.Request("frame", 0.0015, scene="b"),
            serve.Request("frame", 0.0016, scene="a")]
    done = s.run(reqs, idle_sleep=-1)
    assert len(done) == 3
    a1, b1, a2 = reqs
    # b joined while a was mid-frame: their rounds overlap
    assert b1.start < a1.done
    # the second request to a waits for a's first frame
    assert a2.start >= a1.done
    assert max(n for n, _ in s.batch.log) == 2
    assert all(r.work == 300 for r in done)


def test_solves_ride_with_frames_and_admission_by_footprint():
    m, b, dx = scenes.poisson_case(64, seed=1)
    need = serve.SOLVE_BYTES_PER_CELL * m.size + serve.SOLVE_BYTES_FIXED
    s = _server(budget=1.5 * need)  # one solve at a time fits
    reqs = [serve.Request("solve", 0.0, problem=(m, b, 1 / 30, 1000.0, dx)) for _ in range(3)]
    done = s.run(reqs, idle_sleep=-1)
    assert len(done) == 3
    assert all(r.result[0] == 7 for r in done)
    starts = sorted(r.start for r in reqs)
    dones = sorted(r.done for r in reqs)
    assert starts[1] >= dones[0] and starts[2] >= dones[1]
    assert s.used_bytes() == 0


def test_request_over_budget_is_refused():
    s = _server(budget=10)
    s.register_scene("a", scenes.random_scene(64, 1))
    with pytest.raises(RuntimeError):
        s.run([serve.Request("frame", 0.0, scene="a")], idle_sleep=-1)


def test_workload_is_seeded():
    sp1, r1 = serve.serving_workload(50, pool=4, frame_sides=(64, 128), solve_sides=(64, 96))
    sp2, r2 = serve.serving_workload(50, pool=4, frame_sides=(64, 128), solve_sides=(64, 96))
    assert [r.arrival for r in r1] == [r.arrival for r in r2]
    assert [r.kind for r in r1] == [r.kind for r in r2]
    kinds = [r.kind for r in r1]
    assert 0 < kinds.count("solve") < len(kinds)
    assert np.all(np.diff([r.arrival for r in r1]) > 0)
