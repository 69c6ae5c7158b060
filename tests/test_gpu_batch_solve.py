"""Batched spec-mode solve (fs_pcg_solve_batch): many pressure systems of
different sizes in one call, one thread-block cluster each.  Every system
must reach the 1e-6 true relative residual, stay within the stated error of
the full-FP64 PCG oracle (oracle/fsoracle.c fso_spec_solve), and give the
same bits alone as in the mix."""
import numpy as np
import pytest

from flipsolver2d_gb300 import gpu, scenes
import fsoracle as fo
from test_gpu_pcg import apply_a, random_mask, rhs_for

pytestmark = pytest.mark.gpu

DT, DENSITY = 1.0 / 30, 1000.0
REL_TOL = 1e-6
SOL_TOL = 1e-3  # solution error against the FP64 oracle solved to 1e-10


def _rect_case(ni, nj, seed):
    """A rectangular system: a random blob cut to ni x nj, solid border."""
    m = random_mask(max(ni, nj), seed)[:ni, :nj].copy()
    m[0, :] = m[-1, :] = m[:, 0] = m[:, -1] = 0x20
    return m, rhs_for(m, seed)


def _problems():
    out = []
    for n, seed in ((64, 11), (96, 12), (128, 13), (192, 14), (256, 15)):
        m, b, dx = scenes.poisson_case(n, seed=seed)
        out.append((m, b, DT, DENSITY, dx))
    for ni, nj, seed in ((150, 90, 16), (70, 230, 17), (33, 47, 18)):
        m, b = _rect_case(ni, nj, seed)
        out.append((m, b, DT, DENSITY, 1.0 / max(ni, nj)))
    return out


def _true_rel(m, b, x, dx):
    return np.linalg.norm(b - apply_a(m, x, DT, DENSITY, dx)) / np.linalg.norm(b)


def test_batch_reaches_residual_and_matches_fp64(port_lib, gpu_lib):
    probs = _problems()
    res = gpu.pcg_solve_batch(probs, REL_TOL)
    for (m, b, dt, dens, dx), (it, x, rr) in zip(probs, res):
        true_rr = _true_rel(m, b, x, dx)
        assert rr <= REL_TOL and true_rr <= 1.01 * REL_TOL, (m.shape, it, rr, true_rr)
        _, x64, _ = fo.spec_solve(m, b, dt, dens, dx, 1e-10)
        err = np.linalg.norm(x - x64) / np.linalg.norm(x64)
        assert err <= SOL_TOL, f"{m.shape}: error against the FP64 oracle {err}"


def test_batch_alone_equals_mixed(gpu_lib):
    probs = _problems()
    mixed = gpu.pcg_solve_batch(probs, REL_TOL)
    for k in (0, 3, 5, 7):
        alone = gpu.pcg_solve_batch([probs[k]], REL_TOL)[0]
        assert alone[0] == mixed[k][0]
        assert np.array_equal(alone[1].view(np.uint64), mixed[k][1].view(np.uint64))


def test_batch_largest_system(port_lib, gpu_lib):
    m, b, dx = scenes.poisson_case(512, seed=21)
    it, x, rr = gpu.pcg_solve_batch([(m, b, DT, DENSITY, dx)], REL_TOL)[0]
    assert rr <= REL_TOL and _true_rel(m, b, x, dx) <= 1.01 * REL_TOL


def test_batch_zero_rhs_and_limits(gpu_lib):
    m = random_mask(40, 3)
    it, x, rr = gpu.pcg_solve_batch([(m, np.zeros(m.shape), DT, DENSITY, 1.0 / 40)], REL_TOL)[0]
    assert it == 0 and rr == 0.0 and not np.any(x)
    big = np.full((600, 600), 0x20, np.int8)
    with pytest.raises(gpu.FsError):
        gpu.pcg_solve_batch([(big, np.zeros(big.shape), DT, DENSITY, 1.0 / 600)], REL_TOL)


def test_autotuned_plan_is_used(port_lib, gpu_lib):
    """The autotuner picks a cluster size that fits and later solves of that
    shape run with it and still meet the residual."""
    m, b, dx = scenes.poisson_case(192, seed=31)
    for objective in (1, 0):
        c, us = gpu.cluster_autotune(192, 192, objective)
        assert c in (4, 8, 16) and us > 0.0  # 192 rows of 192 need at least 4 CTAs
        it, x, rr = gpu.pcg_solve_batch([(m, b, DT, DENSITY, dx)], REL_TOL)[0]
        assert rr <= REL_TOL and _true_rel(m, b, x, dx) <= 1.01 * REL_TOL
    with pytest.raises(gpu.FsError):
        gpu.cluster_autotune(700, 700)


def test_batch_round_takes_a_large_system(port_lib, gpu_lib):
    """A standalone system above the on-chip limit rides in a batch round as
    a chained cooperative solve and equals the standalone spec solve."""
    m, b, dx = scenes.poisson_case(600, seed=41)
    it0, x0, rr0 = gpu.pcg_solve_spec(m, b, DT, DENSITY, dx, REL_TOL)
    bt = gpu.Batch()
    t = bt.submit_solve(m, b, DT, DENSITY, dx)
    bt.round()
    assert bt.solve_done(t)
    it, x, rr = bt.take_solve(t)
    assert rr <= REL_TOL and _true_rel(m, b, x, dx) <= 1.01 * REL_TOL
    assert it == it0 and np.array_equal(x.view(np.uint64), x0.view(np.uint64))
    bt.close()
