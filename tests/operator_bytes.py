"""The pressure operator as one byte per cell, restated from a material grid
(test helper)."""
import numpy as np


def decomposition_bytes(mat):
    """The operator byte k_decomposition (csrc/fs_grid.cu) derives from a
    material grid, restated: non-solid neighbour count of every cell
    (out-of-grid neighbours clamp to the edge, materialgrid.cpp:5-8), and for
    fluid cells the unit bit and the fluid-neighbour mask of in-range linear
    neighbours (getPressureProjectionMatrix, flipsolver2d.cpp:797-887)."""
    ni, nj = mat.shape
    solid = np.pad((mat & 0x20) != 0, 1, mode="edge")
    fluid = np.pad((mat & 0x40) != 0, 1, mode="edge")
    nb = [(-1, 0, 1), (1, 0, 2), (0, -1, 4), (0, 1, 8)]
    cnt = np.zeros(mat.shape, np.int64)
    mask = np.zeros(mat.shape, np.int64)
    lin = np.arange(ni * nj).reshape(ni, nj)
    for di, dj, bit in nb:
        cnt += ~solid[1 + di:ni + 1 + di, 1 + dj:nj + 1 + dj]
        f = fluid[1 + di:ni + 1 + di, 1 + dj:nj + 1 + dj]
        off = lin + di * nj + dj
        mask |= np.where(f & (off >= 0) & (off < ni * nj), bit, 0)
    unit = (mat & 0x40) != 0
    b = (cnt << 4) | np.where(unit, 0x80 | mask, 0)
    return b.astype(np.uint8)
