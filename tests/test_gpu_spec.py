"""Spec-mode solve: FP32 inner PCG with the textbook incomplete-Poisson
preconditioner and FP64 refinement, to a true relative residual of 1e-6,
checked against the full-FP64 PCG oracle (oracle/fsoracle.c fso_spec_solve)
on the same operator."""
import os

import numpy as np
import pytest

from flipsolver2d_gb300 import gpu, scenes
import fsoracle as fo
from test_gpu_pcg import apply_a, random_mask, rhs_for

DT, DENSITY = 1.0 / 30, 1000.0
REL_TOL = 1e-6
# the solution's error against the FP64 oracle's (solved to 1e-10) is
# bounded by the condition number times the residual; measured well below
SOL_TOL = 1e-3
SOL_TOL_2048 = 2e-2


def _true_rel_residual(m, b, x, dx):
    return np.linalg.norm(b - apply_a(m, x, DT, DENSITY, dx)) / np.linalg.norm(b)


def test_spec_oracle_converges(port_lib):
    m = random_mask(48, 2)
    b = rhs_for(m, 2)
    it, x, rr = fo.spec_solve(m, b, DT, DENSITY, 1.0 / 48, 1e-10)
    assert rr <= 1e-10
    assert _true_rel_residual(m, b, x, 1.0 / 48) <= 1.01e-10


@pytest.mark.gpu
@pytest.mark.parametrize("n,seed", [(64, 5), (128, 6), (256, 7)])
def test_spec_reaches_relative_residual(port_lib, gpu_lib, n, seed):
    m = random_mask(n, seed)
    b = rhs_for(m, seed)
    it, x, rr = gpu.pcg_solve_spec(m, b, DT, DENSITY, 1.0 / n, REL_TOL)
    true_rr = _true_rel_residual(m, b, x, 1.0 / n)
    assert rr <= REL_TOL and true_rr <= 1.01 * REL_TOL, (rr, true_rr)
    _, x64, _ = fo.spec_solve(m, b, DT, DENSITY, 1.0 / n, 1e-10)
    err = np.linalg.norm(x - x64) / np.linalg.norm(x64)
    assert err <= SOL_TOL, f"error against the FP64 oracle {err}"


@pytest.mark.gpu
def test_spec_poisson_case(port_lib, gpu_lib):
    m, b, dx = scenes.poisson_case(256, seed=3)
    frac = ((m & 0x40) != 0).mean()
    assert 0.53 <= frac <= 0.57
    it, x, rr = gpu.pcg_solve_spec(m, b, DT, DENSITY, dx, REL_TOL)
    assert rr <= REL_TOL and _true_rel_residual(m, b, x, dx) <= 1.01 * REL_TOL
    _, x64, _ = fo.spec_solve(m, b, DT, DENSITY, dx, 1e-10)
    assert np.linalg.norm(x - x64) / np.linalg.norm(x64) <= SOL_TOL


@pytest.mark.gpu
def test_spec_zero_rhs(gpu_lib):
    m = random_mask(32, 1)
    it, x, rr = gpu.pcg_solve_spec(m, np.zeros(m.shape), DT, DENSITY, 1.0 / 32, REL_TOL)
    assert it == 0 and rr == 0.0 and not np.any(x)


@pytest.mark.gpu
def test_spec_mixed_precision_configuration(port_lib, gpu_lib, monkeypatch):
    """The mixed-precision configuration itself: 2048^2 cells, a 55 % star
    mask, the divergence of N(0, 1) face velocities.  Both GPU forms of the
    solve -- fs_pcg_solve_spec (the cooperative solve, outer loop on the
    host) and a batch-submitted system (the chained cooperative solve, outer
    loop on the device) -- reach the 1e-6 true residual (recomputed here in
    FP64) and agree with the FP64 oracle solved to 1e-8.  At this size a
    residual of 1e-6 leaves a larger error than on the small grids: the FP64
    oracle itself, stopped at 1e-6, is 7.4e-3 relative-L2 from its 1e-8
    solution.  So the bar here is 2e-2, under three times that."""
    monkeypatch.setenv("FSO_HOST_THREADS", str(os.cpu_count() or 1))
    m, b, dx = scenes.poisson_case(2048, seed=0)
    _, x64, rr64 = fo.spec_solve(m, b, DT, DENSITY, dx, 1e-8)
    assert rr64 <= 1e-8
    it, x, rr = gpu.pcg_solve_spec(m, b, DT, DENSITY, dx, REL_TOL)
    true_rr = _true_rel_residual(m, b, x, dx)
    assert rr <= REL_TOL and true_rr <= 1.01 * REL_TOL, (rr, true_rr)
    assert np.linalg.norm(x - x64) / np.linalg.norm(x64) <= SOL_TOL_2048
    bt = gpu.Batch()
    t = bt.submit_solve(m, b, DT, DENSITY, dx)
    for _ in range(8):  # the chained solve completes within its round
        bt.round()
        if bt.solve_done(t):
            break
    assert bt.solve_done(t)
    it_c, x_c, rr_c = bt.take_solve(t)
    bt.close()
    true_rr = _true_rel_residual(m, b, x_c, dx)
    assert rr_c <= REL_TOL and true_rr <= 1.01 * REL_TOL, (rr_c, true_rr)
    assert np.linalg.norm(x_c - x64) / np.linalg.norm(x64) <= SOL_TOL_2048


def _apply_a_linear(m, x, dt, density, dx):
    """apply_a with the reference's linear-index neighbours: on a unit row
    at j = 0 or j = NJ - 1 the j neighbour is the previous or next row's end
    cell (linearindexable2d.h:103-106), which the 2-D form zero-pads."""
    ni, nj = m.shape
    n = ni * nj
    scale = np.float64(np.float32(dt)) / (density * dx * dx)
    fl = (m & 0x40) != 0
    pad_s = np.pad((m & 0x20) != 0, 1, mode="edge")
    pad_f = np.pad(fl, 1, mode="edge")
    xf = x.ravel()
    cnt = np.zeros(n)
    acc = np.zeros(n)
    for (di, dj), off in (((-1, 0), -nj), ((1, 0), nj), ((0, -1), -1), ((0, 1), 1)):
        ns = ~pad_s[1 + di:ni + 1 + di, 1 + dj:nj + 1 + dj]
        nf = pad_f[1 + di:ni + 1 + di, 1 + dj:nj + 1 + dj].ravel()
        cnt += ns.ravel()
        idx = np.arange(n) + off
        ok = nf & (idx >= 0) & (idx < n)
        acc[ok] += xf[idx[ok]]
    out = xf.copy()
    f = fl.ravel()
    out[f] = (scale * (cnt * xf - acc))[f]
    return out.reshape(ni, nj)


def _mask(ni, nj, seed):
    """random_mask cropped to ni x nj, with its solid border restored."""
    m = random_mask(max(ni, nj), seed)[:ni, :nj].copy()
    m[0, :] = m[-1, :] = m[:, 0] = m[:, -1] = 0x20
    return m


def _oracle_bar(m, b, dx):
    """3 x the FP64 oracle's own error at a 1e-6 stop (against its 1e-8
    solution), floor 1e-4: what a correct 1e-6 solve may differ by."""
    _, x8, rr8 = fo.spec_solve(m, b, DT, DENSITY, dx, 1e-8)
    assert rr8 <= 1e-8
    _, x6, _ = fo.spec_solve(m, b, DT, DENSITY, dx, REL_TOL)
    return x8, max(3.0 * np.linalg.norm(x6 - x8) / np.linalg.norm(x8), 1e-4)


@pytest.mark.gpu
@pytest.mark.parametrize("ni,nj,seed", [(600, 600, 11), (613, 797, 12), (1024, 1024, 13)])
def test_spec_resident_inner_solves(port_lib, gpu_lib, monkeypatch, ni, nj, seed):
    """Grids above the cluster solve's on-chip limit that fit one tile per
    SM: the chained solve's inner FP32 solves run on the resident kernel
    (K K^T preconditioner in shared memory, r.r stopping rule).  They reach
    the 1e-6 true residual, recomputed here in FP64, and agree with the FP64
    oracle."""
    monkeypatch.setenv("FSO_HOST_THREADS", str(os.cpu_count() or 1))
    m = _mask(ni, nj, seed)
    b = rhs_for(m, seed)
    dx = 1.0 / max(ni, nj)
    x8, bar = _oracle_bar(m, b, dx)
    it, x, rr = gpu.pcg_solve_spec(m, b, DT, DENSITY, dx, REL_TOL)
    true_rr = _true_rel_residual(m, b, x, dx)
    assert rr <= REL_TOL and true_rr <= 1.01 * REL_TOL, (rr, true_rr)
    err = np.linalg.norm(x - x8) / np.linalg.norm(x8)
    assert err <= bar, f"error against the FP64 oracle {err} (bar {bar})"


@pytest.mark.gpu
def test_spec_wrapping_grid_falls_back(port_lib, gpu_lib, monkeypatch):
    """Fluid on the j = 0 and j = NJ - 1 columns: the linear index wraps
    those rows' j neighbours into the next row, which the resident kernel's
    tiles do not, so the streaming inner solve runs instead -- and the solve
    still meets the residual and the oracle."""
    monkeypatch.setenv("FSO_HOST_THREADS", str(os.cpu_count() or 1))
    m = _mask(600, 600, 14)
    m[200:400, 0] = 0x40
    m[250:350, -1] = 0x40
    b = rhs_for(m, 14)
    dx = 1.0 / 600
    x8, bar = _oracle_bar(m, b, dx)
    it, x, rr = gpu.pcg_solve_spec(m, b, DT, DENSITY, dx, REL_TOL)
    true_rr = np.linalg.norm(b - _apply_a_linear(m, x, DT, DENSITY, dx)) / np.linalg.norm(b)
    assert rr <= REL_TOL and true_rr <= 1.01 * REL_TOL, (rr, true_rr)
    assert np.linalg.norm(x - x8) / np.linalg.norm(x8) <= bar
