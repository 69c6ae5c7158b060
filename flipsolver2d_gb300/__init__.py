"""GB300-native FLIP substep of FlipSolver2d (see include/fs_gpu.h).

    from flipsolver2d_gb300 import scenes, gpu
    s = gpu.GpuFlipSolver(scenes.dam_break(1024, seed=7, obstacle=True))
    s.step_frame()

The compute runs in the CUDA library flipsolver2d_gb300/_build/libfsgpu.so,
built by flipsolver2d_gb300.build; `gpu` raises when it is missing.
"""
from . import scenes  # noqa: F401

__all__ = ["scenes", "gpu", "build"]
