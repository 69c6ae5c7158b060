"""Regenerate the golden fixtures in tests/golden/ from the reference itself.

    python tests/golden/make_golden.py [--reference <checkout of the reference project>]

Writes:
  * matviz.npz -- the reference's own known-answer system
    (devDocs/matviz/data.txt, vin.txt, vout.txt: a dumped 64x64 pressure
    operator with 402 unknowns, a right-hand side and the solver's result),
    with the material grid reconstructed from the operator coefficients.
  * frames_<scene>.npz -- states of small seeded scenes after frames 1..3,
    produced by the reference FlipSolver2d (oracle/_ref/libfsref.so, built
    from the reference sources in place by oracle/Makefile.ref with its
    single-threaded pool and -ffp-contract=off).  The reference's vector
    reductions depend on its thread-pool size; it is recorded as
    `pool_threads` and the CPU restatement must reproduce the fixtures bit
    for bit with that chunk count.
"""
from __future__ import annotations

import argparse
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

FRAME_SCENES = ["dam32", "random40", "nbdam40", "sink36", "ragged40"]
NB_FRAMES = 5  # NB-FLIP seeds its first particles at the end of frame 1
SCENE_FRAMES = {"sink36": 6}  # the front reaches the sink in frame 4
FLUID, SOLID, EMPTY = 0x40, 0x20, 0x10


def scene_by_name(name):
    from flipsolver2d_gb300 import scenes

    sys.path.insert(0, os.path.dirname(HERE))
    import edge_scenes

    return {"dam32": lambda: scenes.dam_break(32, seed=42),
            "random40": lambda: scenes.random_scene(40, 1001),
            "nbdam40": lambda: scenes.nb_dam_break(40, seed=3, obstacle=True),
            "sink36": edge_scenes.sink_dam,
            "ragged40": edge_scenes.ragged_dam}[name]()


def parse_matviz(ref: str):
    d = os.path.join(ref, "devDocs", "matviz")
    pat = re.compile(r"(\d+):(-?\d+\.*\d*) (-?\d+\.*\d*) (-?\d+\.*\d*) (-?\d+\.*\d*) (-?\d+\.*\d*)")
    units = {}
    h = w = None
    with open(os.path.join(d, "data.txt")) as f:
        for line in f:
            if "=" in line:
                continue
            m = pat.search(line)
            if not m:
                parts = line.strip().split(",")
                if len(parts) == 2:
                    h, w = int(parts[0]), int(parts[1])
                continue
            units[int(m.group(1))] = tuple(float(m.group(k)) for k in range(2, 7))

    def vec(name):
        vals = []
        with open(os.path.join(d, name)) as f:
            for line in f:
                if "=" in line or not line.strip():
                    continue
                vals.append(float(line))
        return np.array(vals, np.float64).reshape(h, w)

    return h, w, units, vec("vin.txt"), vec("vout.txt")


def reconstruct_material(h, w, units):
    """Fluid = listed unit rows.  A unit's diagonal / scale is its count of
    non-solid neighbours; neighbours with a zero coefficient are empty or
    solid.  Assign empty/solid so that every unit's count is reproduced."""
    scale = -min(v for u in units.values() for v in u[1:] if v != 0.0)
    mat = np.full(h * w, EMPTY, np.int8)
    for k in units:
        mat[k] = FLUID
    offs = [-w, w, -1, 1]  # iNeg, iPos, jNeg, jPos
    forced_empty = set()
    pending = []
    for k, (diag, *nb) in units.items():
        count = int(round(diag / scale))
        nonfluid = [k + o for o, c in zip(offs, nb) if c == 0.0 and 0 <= k + o < h * w]
        n_empty = count - (4 - len(nonfluid))
        pending.append((k, nonfluid, n_empty))
    # units whose non-fluid neighbours are all empty or all solid first
    for k, nonfluid, n_empty in pending:
        if n_empty == len(nonfluid):
            forced_empty.update(nonfluid)
    for k, nonfluid, n_empty in pending:
        if n_empty == 0:
            for c in nonfluid:
                if c not in forced_empty:
                    mat[c] = SOLID
    for k, nonfluid, n_empty in pending:  # ambiguous units: fill solids greedily
        cur = sum(1 for c in nonfluid if mat[c] != SOLID)
        for c in nonfluid:
            if cur <= n_empty:
                break
            if c not in forced_empty and mat[c] != SOLID:
                mat[c] = SOLID
                cur -= 1
    return mat.reshape(h, w), scale


def make_matviz(ref: str):
    h, w, units, vin, vout = parse_matviz(ref)
    mat, scale = reconstruct_material(h, w, units)
    np.savez_compressed(os.path.join(HERE, "matviz.npz"), material=mat, vin=vin, vout=vout,
                        scale=np.float64(scale), units=np.array(sorted(units), np.int64))
    return len(units)


def make_frames(frames: int = 3, names=FRAME_SCENES):
    """NB-FLIP scenes also record the advected grids and the engine state."""
    import fsoracle as fo

    for name in names:
        s = fo.OracleSolver(scene_by_name(name), "ref")
        out = {"pool_threads": np.int32(s.stat(4))}
        for f in range(1, (NB_FRAMES if s.nb else SCENE_FRAMES.get(name, frames)) + 1):
            s.step_frame()
            p = s.get_particles()
            for k, v in p.items():
                out[f"f{f}_{k}"] = v
            for g in ["material", "fluid_sdf", "u", "v", "u_valid", "v_valid", "density",
                      "particle_counts", "pressure"] + (fo.NB_GRIDS + ["viscosity"] if s.nb else []):
                out[f"f{f}_{g}"] = s.get_grid(g)
            if s.nb:
                out[f"f{f}_rng"] = s.get_rng()
            out[f"f{f}_stats"] = np.array([s.stat(0), s.stat(1), s.stat(2)], np.int32)
            out[f"f{f}_dt"] = np.float32(s.dt)
        np.savez_compressed(os.path.join(HERE, f"frames_{name}.npz"), **out)
        s.close()


def main():
    import build as oracle_build

    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=oracle_build.reference_dir())
    ap.add_argument("--only", nargs="*", default=None, help="frame scenes to regenerate")
    a = ap.parse_args()
    os.environ["FS_REFERENCE_DIR"] = a.reference

    oracle_build.build_ref()
    if a.only is None:
        print("matviz units:", make_matviz(a.reference))
    make_frames(names=a.only if a.only is not None else FRAME_SCENES)
    print("frames written")


if __name__ == "__main__":
    main()
