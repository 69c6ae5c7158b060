"""Pins the CPU oracle (oracle/fsoracle.c, the plain-C restatement) before it
is trusted as the checker of the CUDA path:
  * bit for bit against the reference FlipSolver2d built from its own sources
    (oracle/_ref, only where the reference tree exists);
  * bit for bit against the committed fixtures that the reference produced
    (tests/golden/frames_*.npz, tests/golden/make_golden.py);
  * against the reference's own known-answer system (devDocs/matviz).
"""
import os

import numpy as np
import pytest

import fsoracle as fo
from flipsolver2d_gb300 import scenes

from conftest import POOL_THREADS

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

from test_scenes_json import DAM_JSON  # noqa: E402
from edge_scenes import EDGE_SCENES  # noqa: E402

PIN_SCENES = {
    "dam32": lambda: scenes.dam_break(32, seed=42),
    "dam48_obstacle": lambda: scenes.dam_break(48, seed=7, obstacle=True),
    "random40": lambda: scenes.random_scene(40, 1001),
    "random33_literal_overlap": lambda: scenes.dam_break(33, seed=3, fluid_box=(0.0, 1.0, 0.0, 0.5)),
    "json_dam36": lambda: scenes.scene_from_json(DAM_JSON, "json_dam36"),
    "nb_dam48_obstacle": lambda: scenes.nb_dam_break(48, seed=7, obstacle=True),
    "nb_dam37_inviscid": lambda: scenes.nb_dam_break(37, seed=5, viscosity=0.0),
    # sources: FLIP reseeding and grid transfer, NB-FLIP's source branches
    "dam40_source": lambda: scenes.with_source(scenes.dam_break(40, seed=9), viscosity=3.0),
    "nb_dam44_source": lambda: scenes.with_source(scenes.nb_dam_break(44, seed=6), transfer=False,
                                                  box=(0.2, 0.35, 0.5, 0.7), viscosity=2.0),
    "nb_dam44_source_transfer": lambda: scenes.with_source(scenes.nb_dam_break(44, seed=6)),
    # viscosity: the light and heavy models (viscositymodel.cpp), FLIP and NB-FLIP
    "dam32_viscous": lambda: scenes.with_viscosity(scenes.dam_break(32, seed=42), 5.0),
    "dam32_viscous_heavy": lambda: scenes.with_viscosity(scenes.dam_break(32, seed=42), 5.0, heavy=True),
    "nb_dam40_viscous": lambda: scenes.with_viscosity(scenes.nb_dam_break(40, seed=7), 10.0),
    # a ragged grid, a sink that kills particles, a scene without fluid
    **EDGE_SCENES,
}


def same_state(a, b, with_pressure=True):
    pa, pb = a.get_particles(), b.get_particles()
    for k in pa:
        assert np.array_equal(pa[k], pb[k]), k
    for g in a.state_grids() + (["pressure", "pressure_rhs"] if with_pressure else []):
        x, y = a.get_grid(g), b.get_grid(g)
        assert np.array_equal(x, y, equal_nan=True), g
    assert np.array_equal(a.get_rng(), b.get_rng())


@pytest.mark.parametrize("name", sorted(PIN_SCENES))
def test_port_matches_reference_frames(port_lib, ref_lib, name):
    sc = PIN_SCENES[name]()
    r = fo.OracleSolver(sc, "ref")
    p = fo.OracleSolver(sc, "port")
    assert r.stat(4) == p.stat(4) == POOL_THREADS
    for _ in range(8 if r.nb else 5):
        r.step_frame()
        p.step_frame()
        same_state(r, p)
        for k in range(3):
            assert r.stat(k) == p.stat(k)


def test_port_matches_reference_stages(port_lib, ref_lib):
    """Each stage of step() on both oracles from one shared snapshot."""
    sc = PIN_SCENES["dam48_obstacle"]()
    r = fo.OracleSolver(sc, "ref")
    p = fo.OracleSolver(sc, "port")
    for _ in range(3):
        r.step_frame()
    p.restore(r.snapshot())
    p.set_dt(r.dt)
    projected = False
    for s in fo.STEP_STAGES:
        r.stage(s)
        p.stage(s)
        projected |= s == fo.PROJECT
        if s in (fo.ADVECT, fo.DECOMPOSITION):
            continue  # the rebin set exists only between these stages
        # the projection's vectors are not part of the restored snapshot
        same_state(r, p, with_pressure=projected)


def test_port_matches_reference_nbflip_stages(port_lib, ref_lib):
    """Each stage of NBFlipSolver::step on both oracles from one shared
    snapshot (advected grids and engine state included)."""
    sc = PIN_SCENES["nb_dam48_obstacle"]()
    r = fo.OracleSolver(sc, "ref")
    p = fo.OracleSolver(sc, "port")
    for _ in range(4):
        r.step_frame()
    assert r.particle_count() > 0
    p.restore(r.snapshot())
    p.set_dt(r.dt)
    projected = False
    for s in fo.NB_STEP_STAGES:
        r.stage(s)
        p.stage(s)
        projected |= s == fo.PROJECT
        if s == fo.ADVECT:
            continue  # the rebin set exists only between ADVECT and REBIN
        same_state(r, p, with_pressure=projected)


GOLDEN_SCENES = {"dam32": PIN_SCENES["dam32"], "random40": PIN_SCENES["random40"],
                 "nbdam40": lambda: scenes.nb_dam_break(40, seed=3, obstacle=True),
                 "sink36": EDGE_SCENES["sink_dam36"], "ragged40": EDGE_SCENES["ragged_dam40"]}


@pytest.mark.parametrize("name", sorted(GOLDEN_SCENES))
def test_port_matches_golden_fixture(port_lib, name):
    f = np.load(os.path.join(GOLDEN, f"frames_{name}.npz"))
    assert int(f["pool_threads"]) == POOL_THREADS
    p = fo.OracleSolver(GOLDEN_SCENES[name](), "port")
    nframes = sum(1 for k in f.files if k.endswith("_stats"))
    for fr in range(1, nframes + 1):
        p.step_frame()
        got = p.get_particles()
        for k in got:
            assert np.array_equal(got[k], f[f"f{fr}_{k}"]), (fr, k)
        grids = ["material", "fluid_sdf", "u", "v", "u_valid", "v_valid", "density",
                 "particle_counts", "pressure"] + (fo.NB_GRIDS + ["viscosity"] if p.nb else [])
        for g in grids:
            assert np.array_equal(p.get_grid(g), f[f"f{fr}_{g}"]), (fr, g)
        if p.nb:
            assert np.array_equal(p.get_rng(), f[f"f{fr}_rng"])
        assert [p.stat(0), p.stat(1), p.stat(2)] == f[f"f{fr}_stats"].tolist()
        assert np.float32(p.dt) == f[f"f{fr}_dt"]


def test_matviz_known_answer(port_lib):
    """The reference's dumped system: the oracle's operator, solved tightly,
    reproduces the reference's stored solution (vout)."""
    f = np.load(os.path.join(GOLDEN, "matviz.npz"))
    m, b, xr = f["material"], f["vin"], f["vout"]
    assert int(((m & 0x40) != 0).sum()) == len(f["units"]) == 402
    it, x = fo.pcg_solve(m, b, float(f["scale"]), 1.0, 1.0, 2000, 1e-9)
    fl = (m & 0x40) != 0
    err = np.linalg.norm(x[fl] - xr[fl]) / np.linalg.norm(xr[fl])
    assert it < 2000 and err < 1e-4


def test_pcg_reference_quirks(port_lib, ref_lib):
    """Iteration counts and results of LinearSolver::solve match the
    reference for a sweep of limits and tolerances (maxAbs chunking, return
    of the loop index, untouched non-fluid rows)."""
    rng = np.random.default_rng(0)
    n = 40
    m = np.full((n, n), 0x10, np.int8)
    m[8:32, 6:30] = 0x40
    m[0, :] = m[-1, :] = m[:, 0] = m[:, -1] = 0x20
    m[20:24, 10:14] = 0x20
    b = rng.standard_normal((n, n)) * 50
    b[(m & 0x40) == 0] = 0
    for limit, tol in [(1, 1e-2), (5, 1e-2), (200, 1e-2), (300, 1e-6), (50, 10.0)]:
        ir, xr = fo.pcg_solve(m, b, 1 / 30, 1000.0, 1 / n, limit, tol, kind="ref")
        ip, xp = fo.pcg_solve(m, b, 1 / 30, 1000.0, 1 / n, limit, tol, kind="port")
        assert ir == ip and np.array_equal(xr, xp), (limit, tol)
