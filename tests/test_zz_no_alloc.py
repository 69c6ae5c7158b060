"""fs_pcg_solve_device_noalloc against fs_pcg_solve_device, through the C ABI.

The no-allocation entry point runs the same FP32 solve as the cached one, so
on the same device inputs both must give the same iteration count and the
same solution (relative L2 difference <= 1e-6).  Two calls in a row, the
second on a smaller grid, show that what the first call left in the shared
scratch array does not leak into the second.  Collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from flipsolver2d_gb300 import gpu
from conftest import POOL_THREADS
from test_gpu_pcg import random_mask, rhs_for

DT, DENSITY = 1.0 / 30, 1000.0
TOL_REL_L2 = 1e-6


def _exec():
    return gpu.ExecParams(gpu.FS_PCG_FP32, POOL_THREADS, 0)


@pytest.mark.gpu
def test_noalloc_matches_cached_solve_twice(gpu_lib):
    torch = pytest.importorskip("torch")
    lib = gpu.load()
    dev = torch.device("cuda:0")
    ex = _exec()
    for n, seed in [(96, 11), (64, 12)]:
        m = random_mask(n, seed)
        b = rhs_for(m, seed)
        mat = torch.from_numpy(np.ascontiguousarray(m, dtype=np.int8)).to(dev)
        rhs = torch.from_numpy(np.ascontiguousarray(b, dtype=np.float32)).to(dev)
        x_ref = torch.zeros_like(rhs)
        x_new = torch.full_like(rhs, float("nan"))
        torch.cuda.synchronize()
        it_ref, it_new = ctypes.c_int(-1), ctypes.c_int(-1)
        st = lib.fs_pcg_solve_device(n, n, mat.data_ptr(), DT, DENSITY, 1.0 / n, rhs.data_ptr(),
                                     x_ref.data_ptr(), 200, 1e-2, ctypes.byref(ex),
                                     ctypes.byref(it_ref))
        assert st == gpu.FS_OK, lib.fs_last_error()
        st = lib.fs_pcg_solve_device_noalloc(n, n, mat.data_ptr(), DT, DENSITY, 1.0 / n,
                                             rhs.data_ptr(), x_new.data_ptr(), 200, 1e-2,
                                             ctypes.byref(ex), ctypes.byref(it_new))
        assert st == gpu.FS_OK, lib.fs_last_error()
        assert it_new.value == it_ref.value
        a, r = x_new.cpu().numpy().astype(np.float64), x_ref.cpu().numpy().astype(np.float64)
        assert np.all(np.isfinite(a))
        err = np.linalg.norm(a - r) / max(np.linalg.norm(r), 1e-300)
        assert err <= TOL_REL_L2, f"n={n}: relative L2 {err}"


def narrow_mask(ni, nj, seed):
    """A 1-cell solid border around fluid, with about one interior cell in
    ten left empty (Dirichlet 0), so that the system is well posed."""
    rng = np.random.default_rng(seed)
    m = np.full((ni, nj), 0x40, np.int8)
    m[rng.random((ni, nj)) < 0.1] = 0x10
    m[0, :] = m[-1, :] = m[:, 0] = m[:, -1] = 0x20
    return m


# Shapes too wide for one resident tile per SM: 4 x 65536 takes the TMA-tile
# kernel (a row pitch of a multiple of 16 bytes), 3 x 87381 the tiled /
# linear-index pair.  Both entry points must choose the same kernel, so the
# solutions agree bit for bit.
@pytest.mark.gpu
@pytest.mark.parametrize("ni,nj,seed", [(4, 65536, 31), (3, 87381, 32)])
def test_noalloc_narrow_shapes_match_cached(gpu_lib, ni, nj, seed):
    torch = pytest.importorskip("torch")
    lib = gpu.load()
    dev = torch.device("cuda:0")
    ex = _exec()
    m = narrow_mask(ni, nj, seed)
    b = np.random.default_rng(seed).standard_normal((ni, nj)) * 100.0
    b[(m & 0x40) == 0] = 0.0
    mat = torch.from_numpy(m).to(dev)
    rhs = torch.from_numpy(b.astype(np.float32)).to(dev)
    x_ref = torch.zeros_like(rhs)
    x_new = torch.full_like(rhs, float("nan"))
    torch.cuda.synchronize()
    it_ref, it_new = ctypes.c_int(-1), ctypes.c_int(-1)
    dx = 1.0 / nj
    st = lib.fs_pcg_solve_device(ni, nj, mat.data_ptr(), DT, DENSITY, dx, rhs.data_ptr(),
                                 x_ref.data_ptr(), 200, 1e-2, ctypes.byref(ex), ctypes.byref(it_ref))
    assert st == gpu.FS_OK, lib.fs_last_error()
    st = lib.fs_pcg_solve_device_noalloc(ni, nj, mat.data_ptr(), DT, DENSITY, dx, rhs.data_ptr(),
                                         x_new.data_ptr(), 200, 1e-2, ctypes.byref(ex),
                                         ctypes.byref(it_new))
    assert st == gpu.FS_OK, lib.fs_last_error()
    assert it_new.value == it_ref.value
    a, r = x_new.cpu().numpy(), x_ref.cpu().numpy()
    assert np.all(np.isfinite(a))
    assert np.array_equal(a, r)


@pytest.mark.gpu
def test_noalloc_rejects_oversize(gpu_lib):
    lib = gpu.load()
    ex = _exec()
    it = ctypes.c_int(-1)
    # rejected before any pointer is touched or any device work is queued
    st = lib.fs_pcg_solve_device_noalloc(1024, 1024, 1, DT, DENSITY, 1.0 / 1024, 1, 1, 200, 1e-2,
                                         ctypes.byref(ex), ctypes.byref(it))
    assert st == gpu.FS_ERR_BAD_ARG
    assert b"exceeds" in lib.fs_last_error()
    assert it.value == -1
