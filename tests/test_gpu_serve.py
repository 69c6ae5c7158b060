"""The serving loop on the GPU: a seeded Poisson stream of frame requests to
resident scenes and standalone solves, served with continuous batching.  Every
result must equal the one the same request gets alone: each scene's state
after its served frames equals stepping it alone (fs_step_frame, same mode)
bit for bit, and each solve equals fs_pcg_solve_batch on that system alone."""
import collections

import numpy as np
import pytest

from flipsolver2d_gb300 import gpu, serve

pytestmark = pytest.mark.gpu


def _state(g):
    p = g.get_particles()
    return [p["pos"], p["vel"], g.get_grid("u"), g.get_grid("v"), g.get_grid("material")]


def test_served_results_equal_alone(gpu_lib):
    specs, reqs = serve.serving_workload(40, rate=2000.0, pool=4, frame_sides=(64, 128),
                                         solve_sides=(64, 128))
    srv = serve.Server(budget_bytes=150e9)
    for k, sc in specs.items():
        srv.register_scene(k, sc)
    done = srv.run(reqs)
    assert len(done) == len(reqs)
    assert all(r.done >= r.start >= r.arrival for r in done)
    frames = collections.Counter(r.scene for r in done if r.kind == "frame")
    for key, nf in frames.items():
        g = gpu.GpuFlipSolver(specs[key], precision=gpu.FS_PCG_SPEC)
        for _ in range(nf):
            g.step_frame()
        for a, b in zip(_state(g), _state(srv.resident[key])):
            assert a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8)), key
        g.close()
    for r in done:
        if r.kind != "solve":
            continue
        it, x, rr = gpu.pcg_solve_batch([r.problem])[0]
        assert rr <= 1e-6
        assert it == r.result[0] and np.array_equal(x.view(np.uint64), r.result[1].view(np.uint64))
    summary = serve.latency_summary(done)
    assert summary["all"]["n"] == len(reqs)
    srv.close()
