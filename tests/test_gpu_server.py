"""The device-resident request loop (fs_server_*): one persistent launch of
the cluster solve whose clusters take spec-mode solve requests from a ring
in mapped pinned memory.  Every served result reaches the 1e-6 true residual
(recomputed here in FP64) and agrees with the FP64 oracle
(oracle/fsoracle.c fso_spec_solve); the same request gives the same bits
whenever it is served; slots, sizes and shutdown behave as documented."""
import time

import numpy as np
import pytest

import fsoracle as fo
from flipsolver2d_gb300 import gpu
from test_gpu_pcg import apply_a, random_mask, rhs_for

pytestmark = pytest.mark.gpu

DT, DENSITY = 1.0 / 30, 1000.0
REL_TOL = 1e-6
SOL_TOL = 1e-3  # error against the FP64 oracle solved to 1e-10 (as for the spec-mode solve)
FS_ERR_BAD_ARG, FS_ERR_STATE = 1, 6


def _mask(ni, nj, seed):
    m = random_mask(max(ni, nj), seed)[:ni, :nj].copy()
    m[0, :] = m[-1, :] = m[:, 0] = m[:, -1] = 0x20
    return m


def _serve_all(srv, tickets, limit_s=120.0):
    """polls until every ticket is done (bounded)"""
    t0 = time.time()
    pending = set(tickets)
    while pending:
        pending = {t for t in pending if not srv.poll(t)}
        assert time.time() - t0 < limit_s, f"{len(pending)} requests not served within {limit_s} s"
        if pending:
            time.sleep(0.0005)


def _true_rel(m, b, x, dx):
    return np.linalg.norm(b - apply_a(m, x, DT, DENSITY, dx)) / np.linalg.norm(b)


def test_server_solves_ragged_requests(port_lib, gpu_lib):
    srv = gpu.Server(512, 512, slots=16)
    shapes = [(64, 64, 1), (128, 96, 2), (200, 333, 3), (512, 512, 4), (37, 90, 5), (256, 256, 6),
              (511, 300, 7), (96, 512, 8), (300, 511, 9), (150, 150, 10)]
    reqs = {}
    for ni, nj, seed in shapes:
        m = _mask(ni, nj, seed)
        b = rhs_for(m, seed)
        dx = 1.0 / max(ni, nj)
        reqs[srv.submit(m, b, DT, DENSITY, dx)] = (m, b, dx)
    assert srv.clusters() >= 1
    _serve_all(srv, reqs)
    out = {}
    for t, (m, b, dx) in reqs.items():
        it, x, rr = srv.take(t)
        tr = _true_rel(m, b, x, dx)
        assert it > 0 and rr <= REL_TOL and tr <= 1.01 * REL_TOL, (m.shape, it, rr, tr)
        out[m.shape] = (x, m, b, dx)
    srv.close()
    for shape in ((64, 64), (128, 96), (37, 90)):
        x, m, b, dx = out[shape]
        _, x64, rr64 = fo.spec_solve(m, b, DT, DENSITY, dx, 1e-10)
        assert rr64 <= 1e-10
        err = np.linalg.norm(x - x64) / np.linalg.norm(x64)
        assert err <= SOL_TOL, f"{shape}: error against the FP64 oracle {err}"


def test_server_same_request_same_bits(gpu_lib):
    """In one launch, and again after the launch left for lack of requests."""
    srv = gpu.Server(256, 256, slots=4)
    m = _mask(200, 180, 11)
    b = rhs_for(m, 11)
    dx = 1.0 / 200
    t1 = srv.submit(m, b, DT, DENSITY, dx)
    t2 = srv.submit(m, b, DT, DENSITY, dx)
    _serve_all(srv, [t1, t2])
    i1, x1, r1 = srv.take(t1)
    i2, x2, r2 = srv.take(t2)
    assert i1 == i2 and r1 == r2 and np.array_equal(x1, x2)
    time.sleep(0.3)  # the launch leaves after about 50 ms of an empty ring
    t3 = srv.submit(m, b, DT, DENSITY, dx)
    _serve_all(srv, [t3])
    i3, x3, r3 = srv.take(t3)
    assert i3 == i1 and np.array_equal(x3, x1)
    srv.close()


def test_server_slots_sizes_and_zero_rhs(gpu_lib):
    srv = gpu.Server(128, 128, slots=2)
    m = _mask(100, 120, 12)
    b = rhs_for(m, 12)
    with pytest.raises(gpu.FsError) as e:
        srv.submit(_mask(129, 64, 12), rhs_for(_mask(129, 64, 12), 1), DT, DENSITY, 1.0 / 129)
    assert e.value.status == FS_ERR_BAD_ARG
    t1 = srv.submit(m, b, DT, DENSITY, 1.0 / 120)
    t2 = srv.submit(m, np.zeros_like(b), DT, DENSITY, 1.0 / 120)
    with pytest.raises(gpu.FsError) as e:
        srv.submit(m, b, DT, DENSITY, 1.0 / 120)
    assert e.value.status == FS_ERR_STATE
    _serve_all(srv, [t1, t2])
    it2, x2, rr2 = srv.take(t2)
    assert it2 == 0 and rr2 == 0.0 and not np.any(x2)
    srv.take(t1)
    t3 = srv.submit(m, b, DT, DENSITY, 1.0 / 120)  # the slots are free again
    _serve_all(srv, [t3])
    with pytest.raises(gpu.FsError):
        srv.take(t3 + 100)
    srv.close()


def test_server_destroy_with_requests_in_flight(gpu_lib):
    """Destroy returns once the clusters finish what they hold; requests not
    yet claimed are dropped."""
    srv = gpu.Server(512, 512, slots=8)
    for seed in range(8):
        m = _mask(512, 512, 20 + seed)
        srv.submit(m, rhs_for(m, 20 + seed), DT, DENSITY, 1.0 / 512)
    t0 = time.time()
    srv.close()
    assert time.time() - t0 < 60.0
