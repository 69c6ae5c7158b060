"""Per-frame solver statistics in the reference's AutoBench table layout.

The reference's AutoBench application (AutoBench/benchruntable.h:28-49,
benchruntable.cpp:50-100) writes one row per frame and scene: the frame
number, the substep count, the frame time, the time of every SolverStage
(flipsolver2d.h:58-72) in milliseconds and the pressure, density and
viscosity iteration counts.  This module produces the same columns, with the
same headers, as CSV (the reference writes XLSX through OpenXLSX, which is
not part of this path).

Stage times are device times from CUDA events (fs_get_stage_time); the
frame time is the host wall time of fs_step_frame.  For FLIP scenes the
reference's grid update includes particle-to-grid, which is fused into it
here, so "Particle to grid" is 0.  NB-FLIP scenes (simType "nbflip") end
their stages as NBFlipSolver::step does (nbflipsolver.cpp:26-64): particle to
grid on its own, no density correction, the level sets in after transfer.
Viscosity is not on this path, so its columns are 0.

    python -m flipsolver2d_gb300.autobench scene.json [more.json] --frames 60 --out stats.csv
"""
from __future__ import annotations

import argparse
import csv
import os
import time
from typing import Iterable, List

from . import gpu, scenes

COLUMNS = ["Step number", "Substeps", "Frame time", "Advection", "Decomposition",
           "Density correction", "Particle rebin", "Particle to grid", "Grid update",
           "After transfer", "Pressure", "Viscosity", "After-visc pressure", "Particle update",
           "Particle reseeding", "Pressure iterations", "Density iterations",
           "Viscosity iterations"]

# SolverStage indices in the column order above (flipsolver2d.h:58-72)
_STAGE_COLUMNS = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11]


def run_scene(scene, frames: int, precision: int = gpu.FS_PCG_FP32) -> List[list]:
    """`frames` frames of one scene; one row of COLUMNS per frame."""
    g = gpu.GpuFlipSolver(scene, precision=precision)
    g.enable_timers(True)
    rows = []
    try:
        for f in range(frames):
            g.reset_timers()
            t0 = time.perf_counter()
            g.step_frame()
            wall_ms = 1e3 * (time.perf_counter() - t0)
            st = g.stage_times()
            rows.append([f, g.stat(2), wall_ms] + [st[k] for k in _STAGE_COLUMNS] +
                        [g.stat(1), g.stat(0), 0])
    finally:
        g.close()
    return rows


def write_csv(path: str, tables: Iterable[tuple]) -> None:
    """tables: (scene name, rows).  One header; a leading "Scene" column
    stands in for the reference's one-sheet-per-scene workbook."""
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(["Scene"] + COLUMNS)
        for name, rows in tables:
            for r in rows:
                w.writerow([name] + r)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("scenes", nargs="+", help="scene files in the reference's JSON format")
    ap.add_argument("--frames", type=int, default=60)
    ap.add_argument("--out", default="autobench.csv")
    ap.add_argument("--precision", choices=["fp32", "fp64", "spec"], default="fp32")
    a = ap.parse_args(argv)
    prec = {"fp32": gpu.FS_PCG_FP32, "fp64": gpu.FS_PCG_FP64, "spec": gpu.FS_PCG_SPEC}[a.precision]
    tables = []
    for path in a.scenes:
        with open(path) as f:
            sc = scenes.scene_from_json(f.read(), os.path.splitext(os.path.basename(path))[0])
        tables.append((sc.name, run_scene(sc, a.frames, prec)))
    write_csv(a.out, tables)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
