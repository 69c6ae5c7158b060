"""Failure detection on the device, without a fault (bounded waits and a
sentinel, never a trap, a bad address or an endless loop).

* A bounded wait that runs out: the PCG kernels' grid reductions, neighbour
  hand-offs and TMA completions poll a bounded number of times
  (fs_exec_params.wait_polls).  With a limit of a few polls a multi-block
  solve's waits give up before the other blocks arrive: every block returns,
  the call reports FS_ERR_TIMEOUT, and the context stays usable -- the same
  solve with the default limit then matches a fresh solve bit for bit.
* The non-finite sentinel: G2P checks every particle velocity a substep
  leaves.  A NaN placed in one uploaded particle velocity spreads through
  P2G, the solve and G2P within the substep (positions stay finite: the
  advection at its start samples the uploaded, finite grid), and fs_step
  reports FS_ERR_NONFINITE; a clean handle afterwards steps normally."""
import numpy as np
import pytest

from flipsolver2d_gb300 import gpu, scenes
from test_gpu_pcg import random_mask, rhs_for

from conftest import POOL_THREADS

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [512, 2048])
def test_wait_limit_times_out_and_context_survives(gpu_lib, n):
    # 512^2: the resident kernel (152 tiles); 2048^2: the TMA-tile kernel
    m = random_mask(n, 17)
    b = rhs_for(m, 17)
    args = (m, b, 1.0 / 30, 1000.0, 1.0 / n, 50, 1e-2)
    with pytest.raises(gpu.FsError) as e:
        gpu.pcg_solve(*args, precision=gpu.FS_PCG_FP32, pool_threads=POOL_THREADS, wait_polls=2)
    assert e.value.status == gpu.FS_ERR_TIMEOUT
    it1, x1 = gpu.pcg_solve(*args, precision=gpu.FS_PCG_FP32, pool_threads=POOL_THREADS)
    it2, x2 = gpu.pcg_solve(*args, precision=gpu.FS_PCG_FP32, pool_threads=POOL_THREADS)
    assert it1 == it2 and np.array_equal(x1, x2) and np.all(np.isfinite(x1))


def test_handle_wait_limit_times_out(gpu_lib):
    sc = scenes.dam_break(256, seed=7, obstacle=True)
    g = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_FP32, pool_threads=POOL_THREADS, wait_polls=2)
    with pytest.raises(gpu.FsError) as e:
        g.step_frame()
    assert e.value.status == gpu.FS_ERR_TIMEOUT
    g.close()


def test_nonfinite_sentinel(gpu_lib):
    sc = scenes.dam_break(64, seed=7, obstacle=True)
    g = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_FP32, pool_threads=POOL_THREADS)
    g.step_frame()
    p = g.get_particles()
    vel = p["vel"].copy()
    vel[len(vel) // 2, 0] = np.nan
    g.set_particles(dict(p, vel=vel))
    g.set_dt(1.0 / 240)
    with pytest.raises(gpu.FsError) as e:
        g.step()
    assert e.value.status == gpu.FS_ERR_NONFINITE
    g.close()
    # the context is fine: a clean handle steps and keeps finite velocities
    h = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_FP32, pool_threads=POOL_THREADS)
    h.step_frame()
    h.step_frame()
    assert np.all(np.isfinite(h.get_particles()["vel"]))
    h.close()
