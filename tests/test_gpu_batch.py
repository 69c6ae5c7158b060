"""FS_PCG_SPEC handles and the batch driver (fs_batch_*).

A handle in FS_PCG_SPEC mode solves its density and pressure systems to a
true relative residual of 1e-6 on one thread-block cluster; a batch steps
many such handles together.  The batch must give every handle the same bits
it gets when stepped alone, and the in-step solves must meet the residual
against the operator the substep assembled."""
import numpy as np
import pytest

from flipsolver2d_gb300 import gpu, scenes
from test_gpu_pcg import apply_a

pytestmark = pytest.mark.gpu

REL_TOL = 1e-6


def _scenes():
    return [scenes.random_scene(64, 1001), scenes.dam_break(96, seed=3, obstacle=True),
            scenes.random_scene(128, 1002), scenes.random_scene(192, 1003)]


def _state(g):
    p = g.get_particles()
    return (p["pos"], p["vel"], g.get_grid("u"), g.get_grid("v"), g.get_grid("material"),
            g.stat(2))


def test_batch_equals_alone(gpu_lib):
    alone = []
    for sc in _scenes():
        g = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_SPEC)
        for _ in range(2):
            g.step_frame()
        alone.append(_state(g))
        g.close()
    hs = [gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_SPEC) for sc in _scenes()]
    b = gpu.Batch(hs)
    for _ in range(2):
        b.step_frame()
    for k, g in enumerate(hs):
        got = _state(g)
        for a, c in zip(alone[k][:5], got[:5]):
            assert a.shape == c.shape and np.array_equal(a.view(np.uint8), c.view(np.uint8)), k
        assert alone[k][5] == got[5]
    # the handles stay usable on their own after the batch
    hs[0].step_frame()
    b.close()


def test_batch_run_frames_pipelined_equals_alone(gpu_lib):
    """Pipelined frames (a member starts its next frame while others are
    still in theirs) change nothing for any member."""
    alone = []
    for sc in _scenes()[:3]:
        g = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_SPEC)
        for _ in range(3):
            g.step_frame()
        alone.append((_state(g), g.stat(5)))
        g.close()
    hs = [gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_SPEC) for sc in _scenes()[:3]]
    b = gpu.Batch(hs)
    b.run_frames(3)
    for k, g in enumerate(hs):
        got = _state(g)
        for a, c in zip(alone[k][0][:5], got[:5]):
            assert a.shape == c.shape and np.array_equal(a.view(np.uint8), c.view(np.uint8)), k
        assert g.stat(3) == 3 and g.stat(5) == alone[k][1]
    b.close()


def test_spec_solves_in_step(gpu_lib):
    """Run one substep stage by stage and check both solves against the
    operator assembled at its start (DECOMPOSITION precedes P2G)."""
    g = gpu.GpuFlipSolver(scenes.dam_break(128, seed=42), precision=gpu.FS_PCG_SPEC)
    g.step_frame()
    g.set_dt(1.0 / 120)
    g.stage(gpu.ADVECT)
    g.stage(gpu.DECOMPOSITION)
    mat = g.get_grid("material")
    dt = g.dt
    dx = 1.0 / 128
    for st in (gpu.REBIN, gpu.DENSITY):
        g.stage(st)
    b, x = g.get_grid("density_rhs"), g.get_grid("density_pressure")
    if np.any(b):
        rr = np.linalg.norm(b - apply_a(mat, x, dt, 1000.0, dx)) / np.linalg.norm(b)
        assert rr <= 1.01 * REL_TOL, rr
    for st in (gpu.P2G, gpu.LEVELSET, gpu.VEL_EXTRAP, gpu.SAVE_GRID, gpu.BODY_FORCES, gpu.PROJECT):
        g.stage(st)
    b, x = g.get_grid("pressure_rhs"), g.get_grid("pressure")
    assert np.any(b)
    rr = np.linalg.norm(b - apply_a(mat, x, dt, 1000.0, dx)) / np.linalg.norm(b)
    assert rr <= 1.01 * REL_TOL, rr


def test_spec_above_on_chip_limit(gpu_lib):
    """A grid above the on-chip limit (640^2 > 512^2) solves with the
    chained cooperative solve: both in-step solves meet the residual, and the
    handle steps in a batch exactly as alone."""
    sc = scenes.dam_break(640, seed=11)
    g = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_SPEC)
    g.step_frame()
    g.set_dt(1.0 / 240)
    g.stage(gpu.ADVECT)
    g.stage(gpu.DECOMPOSITION)
    mat = g.get_grid("material")
    dt = g.dt
    for st in (gpu.REBIN, gpu.DENSITY, gpu.P2G, gpu.LEVELSET, gpu.VEL_EXTRAP, gpu.SAVE_GRID,
               gpu.BODY_FORCES, gpu.PROJECT):
        g.stage(st)
    b, x = g.get_grid("pressure_rhs"), g.get_grid("pressure")
    rr = np.linalg.norm(b - apply_a(mat, x, dt, 1000.0, 1.0 / 640)) / np.linalg.norm(b)
    assert rr <= 1.01 * REL_TOL, rr
    g.close()
    alone = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_SPEC)
    alone.step_frame()
    ref = _state(alone)
    alone.close()
    h = [gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_SPEC), gpu.GpuFlipSolver(scenes.random_scene(64, 7), precision=gpu.FS_PCG_SPEC)]
    bt = gpu.Batch(h)
    bt.step_frame()
    for a, c in zip(ref[:5], _state(h[0])[:5]):
        assert np.array_equal(a.view(np.uint8), c.view(np.uint8))
    bt.close()
