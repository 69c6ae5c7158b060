"""The viscosity stage (FlipSolver::applyViscosity, flipsolver2d.cpp:128-136;
viscositymodel.cpp) on the GPU against the oracle port (oracle/fsoracle.c,
itself pinned bit for bit to the reference's own viscositymodel.cpp built
over a storage-only Eigen stand-in).

Both sides assemble the same matrix and right-hand side (the light model's
5-point rows with the reference's last-write rules, the heavy model's coupled
U+V rows with its += accumulation order) and solve them with the conjugate
gradient Eigen's ConjugateGradient<..., Upper> runs with the diagonal
preconditioner (x0 = 0, tolerance 1e-4, at most 2n iterations).  The GPU's
dot products are summed over fixed blocks, the oracle's left to right, so the
two recurrences round differently.  Bars:

* iteration counts within ITER_SLACK of each other;
* u and v within SAME_ITER_BAR relative-L2 of the oracle's when the counts
  agree (the recurrences differ by rounding only), within ONE_ITER_BAR when
  they differ by one (one CG step near the 1e-4 stop);
* everything else the stage touches is left bit-exact;
* the second projection that follows (FP64 parity mode) keeps the
  difference at the size the viscosity stage left.

Whole frames with viscosity on (FLIP and NB-FLIP, light and heavy, a scene
in the reference's file format) stay on the oracle's trajectory.
"""
import numpy as np
import pytest

import fsoracle as fo
from flipsolver2d_gb300 import gpu, scenes

import edge_scenes
from conftest import POOL_THREADS
from test_gpu_parity import assert_grid_equal, rel_l2

pytestmark = pytest.mark.gpu

ITER_SLACK = 1
PROJECT_STOP_BAR = 1e-4
SAME_ITER_BAR = 1e-8
ONE_ITER_BAR = 1e-3

# a viscous double dam break in the reference's scene format (units of the
# scene scale): two fluid columns of different viscosity and a friction
# obstacle
VISC_JSON = """
{
  "settings": {
    "simType": "flip", "domainSizeI": 10, "domainSizeJ": 10, "resolution": 40,
    "fps": 30, "density": 1000, "maxSubsteps": 10, "pcgIterLimit": 200, "seed": 11,
    "particlesPerCell": 4, "picRatio": 0.03, "cflNumber": 5, "scale": 0.1,
    "globalAcceleration": [9.81, 0], "viscosityEnabled": true
  },
  "solver": {
    "objects": [
      {"type": "solid", "verts": [[0, 0], [0, 10], [0.3, 10], [0.3, 0]]},
      {"type": "solid", "verts": [[9.7, 0], [9.7, 10], [10, 10], [10, 0]]},
      {"type": "solid", "verts": [[0, 0], [0, 0.3], [10, 0.3], [10, 0]]},
      {"type": "solid", "verts": [[0, 9.7], [0, 10], [10, 10], [10, 9.7]]},
      {"type": "solid", "friction": 0.2, "verts": [[4, 4.5], [4, 5.5], [5, 5.5], [5, 4.5]]},
      {"type": "fluid", "viscosity": 300, "verts": [[5.5, 0.3], [5.5, 3.5], [9.7, 3.5], [9.7, 0.3]]},
      {"type": "fluid", "viscosity": 20, "verts": [[5.5, 6.5], [5.5, 9.7], [9.7, 9.7], [9.7, 6.5]]}
    ]
  }
}
"""


def _json(heavy):
    sc = scenes.scene_from_json(VISC_JSON, "json_visc300_heavy" if heavy else "json_visc300")
    sc.params.useHeavyViscosity = heavy
    return sc


def _nb(heavy):
    return scenes.with_viscosity(scenes.nb_dam_break(40, seed=5), 50.0, heavy=heavy)


# viscosities high enough that the solves take tens of iterations
SCENES = {
    "dam40_light": lambda: scenes.with_viscosity(scenes.dam_break(40, seed=3), 60.0),
    "dam40_heavy": lambda: scenes.with_viscosity(scenes.dam_break(40, seed=3), 60.0, heavy=True),
    "dam48_obstacle_heavy": lambda: scenes.with_viscosity(
        scenes.dam_break(48, seed=7, obstacle=True), 150.0, heavy=True),
    "random44_light": lambda: scenes.with_viscosity(scenes.random_scene(44, 1007), 80.0),
    "ragged_light": lambda: scenes.with_viscosity(edge_scenes.ragged_dam(40, 13), 40.0),
    "ragged_heavy": lambda: scenes.with_viscosity(edge_scenes.ragged_dam(40, 13), 40.0, heavy=True),
    "nb_dam40_light": lambda: _nb(False),
    "nb_dam40_heavy": lambda: _nb(True),
    "json_visc300": lambda: _json(False),
    "json_visc300_heavy": lambda: _json(True),
}

# the stages of a substep before applyViscosity (flipsolver2d.cpp:412-447,
# nbflipsolver.cpp:26-48)
FLIP_ORDER = [fo.ADVECT, fo.DECOMPOSITION, fo.REBIN, fo.DENSITY, fo.P2G, fo.SDF, fo.MATERIALS,
              fo.AFTER_TRANSFER, fo.LEVELSET, fo.VEL_EXTRAP, fo.SAVE_GRID, fo.BODY_FORCES,
              fo.PROJECT, fo.FRICTION]
NB_ORDER = [fo.ADVECT, fo.REBIN, fo.P2G, fo.VEL_EXTRAP, fo.SAVE_GRID, fo.SDF,
            fo.LEVELSET_OUTSIDE, fo.AFTER_TRANSFER, fo.LEVELSET, fo.MATERIALS,
            fo.BODY_FORCES, fo.DECOMPOSITION, fo.PROJECT, fo.FRICTION]


@pytest.fixture(params=sorted(SCENES))
def scene(request, port_lib, gpu_lib):
    return SCENES[request.param]()


def oracle_before_viscosity(sc, frames):
    """The oracle after `frames` frames and the stages of one more substep up
    to the friction update (the state applyViscosity starts from), and its
    snapshot just before that substep's decomposition (the state the
    pressure operator is frozen from)."""
    o = fo.OracleSolver(sc, "port")
    for _ in range(frames):
        o.step_frame()
    nb = sc.sim_type == scenes.SIM_NBFLIP
    # FLIP decomposes right after advection, which moves particles only: the
    # substep's starting state has the same material (and no particle
    # marked for death, which only exists inside a substep)
    at_decomposition = None if nb else o.snapshot()
    for s in (NB_ORDER if nb else FLIP_ORDER):
        if s == fo.DECOMPOSITION and nb:
            at_decomposition = o.snapshot()
        o.stage(s)
    return o, at_decomposition


def gpu_at(sc, o, at_decomposition):
    """A GPU handle in the oracle's state, its pressure operator frozen from
    the same material as the oracle's."""
    g = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_FP64, pool_threads=POOL_THREADS)
    g.first_frame_init()
    g.restore(at_decomposition)
    g.stage(gpu.DECOMPOSITION)
    g.restore(o.snapshot())
    return g


def velocity_bar(it_o, it_g):
    return SAME_ITER_BAR if it_o == it_g else ONE_ITER_BAR


def test_viscosity_stage_from_identical_state(scene):
    o, at_dec = oracle_before_viscosity(scene, 3)
    g = gpu_at(scene, o, at_dec)
    u0 = o.get_grid("u")
    o.stage(fo.VISCOSITY)
    g.stage(gpu.VISCOSITY)
    it_o, it_g = o.stat(fo.S_VISCOSITY_ITERS), g.stat(gpu.FS_STAT_VISCOSITY_ITERS)
    du = max(rel_l2(g.get_grid("u"), o.get_grid("u")), rel_l2(g.get_grid("v"), o.get_grid("v")))
    moved = rel_l2(o.get_grid("u"), u0)
    print(f"\n{scene.name}: viscosity iterations {it_g} / oracle {it_o}, u,v rel-L2 {du:.3e}, "
          f"the stage moved u by {moved:.3e}")
    assert it_o > 0, "the scene must exercise the viscosity solve"
    assert abs(it_o - it_g) <= ITER_SLACK
    assert du <= velocity_bar(it_o, it_g)
    # the stage writes the face velocities only
    for name in ("u_valid", "v_valid", "material", "fluid_sdf", "viscosity", "saved_u", "saved_v"):
        assert_grid_equal(o, g, name, "viscosity stage")

    # the projection that follows (FP64 parity mode, tolerance 1e-6 with
    # viscosity on).  With identical inputs it keeps the oracle's iteration
    # count and the FP64 velocity bar of test_gpu_parity.py.  Near the 1e-6
    # absolute stop the chunked max-abs residual can hover at the tolerance
    # for several iterations, so the dot products' other summation order may
    # stop it elsewhere: then both solves must have met the tolerance and the
    # velocities stay within PROJECT_STOP_BAR.
    o.stage(fo.PROJECT)
    g.stage(gpu.PROJECT)
    po, pg = o.stat(fo.S_PRESSURE_ITERS), g.stat(gpu.FS_STAT_PRESSURE_ITERS)
    dv = max(rel_l2(g.get_grid(n), o.get_grid(n)) for n in ("u", "v"))
    print(f"  second projection: iterations {pg} / oracle {po}, u,v rel-L2 {dv:.3e}")
    limit = scene.params.pcgIterLimit
    assert po > 0
    if po == pg:
        assert dv <= max(10 * du, 1e-6)
    else:
        assert po < limit and pg < limit
        assert dv <= PROJECT_STOP_BAR
    g.close()
    o.close()


def test_viscosity_stage_is_deterministic(scene):
    """Two runs of the stage from one state give the same bits: the fixed-order
    block sums make the GPU solve reproducible run to run."""
    o, _ = oracle_before_viscosity(scene, 2)
    snap = o.snapshot()
    out = []
    for _ in range(2):
        g = gpu.GpuFlipSolver(scene, precision=gpu.FS_PCG_FP64, pool_threads=POOL_THREADS)
        g.first_frame_init()
        g.restore(snap)
        g.stage(gpu.VISCOSITY)
        out.append((g.get_grid("u"), g.get_grid("v"), g.stat(gpu.FS_STAT_VISCOSITY_ITERS)))
        g.close()
    o.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]


@pytest.mark.parametrize("name", ["dam40_light", "dam48_obstacle_heavy", "nb_dam40_heavy",
                                  "json_visc300"])
def test_full_frames_with_viscosity(port_lib, gpu_lib, name):
    """Whole frames in FP64 parity mode with viscosity on: same substeps and
    particle count as the oracle, positions within 1e-3 cells, viscosity
    iterations of the last substep within ITER_SLACK, particle viscosities
    bit-exact."""
    sc = SCENES[name]()
    o = fo.OracleSolver(sc, "port")
    g = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_FP64, pool_threads=POOL_THREADS)
    worst = 0.0
    for f in range(4):
        o.step_frame()
        g.step_frame()
        assert o.stat(2) == g.stat(2), f"frame {f}: substeps"
        a, b = o.get_particles(), g.get_particles()
        assert a["pos"].shape == b["pos"].shape, f"frame {f}: particle count"
        err = float(np.max(np.abs(a["pos"] - b["pos"]))) if len(a["pos"]) else 0.0
        worst = max(worst, err)
        assert err < 1e-3, f"frame {f}: positions differ by {err}"
        assert abs(o.stat(fo.S_VISCOSITY_ITERS) - g.stat(gpu.FS_STAT_VISCOSITY_ITERS)) <= ITER_SLACK
        assert np.array_equal(a["visc"], b["visc"]), f"frame {f}: particle viscosity"
    print(f"\n{name}: worst position difference over 4 frames {worst:.3e} cells")
    assert o.particle_count() > 0
    g.close()
    o.close()


def test_production_mode_runs_viscous_frames(gpu_lib):
    """The FP32 production solves with viscosity on: frames complete with
    finite velocities and converging viscosity solves."""
    sc = SCENES["dam48_obstacle_heavy"]()
    g = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_FP32, pool_threads=POOL_THREADS)
    for _ in range(3):
        g.step_frame()
        assert g.stat(gpu.FS_STAT_VISCOSITY_ITERS) > 0
    p = g.get_particles()
    assert len(p["pos"]) > 0 and np.all(np.isfinite(p["vel"]))
    g.close()


def test_stage_times_include_viscosity(gpu_lib):
    """The per-stage timers attribute the viscosity model and the second
    projection to SolverStage VISCOSITY (8) and REPRESSURE (9)."""
    sc = SCENES["dam40_heavy"]()
    g = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_FP32, pool_threads=POOL_THREADS)
    g.enable_timers(True)
    g.step_frame()
    t = g.stage_times()
    # with viscosity the density correction and its endStage(DENSITY) are
    # skipped (flipsolver2d.cpp:425-430)
    assert t[8] > 0 and t[9] > 0 and t[2] == 0.0
    g.close()


def test_batch_refuses_viscous_members(gpu_lib):
    """fs_batch_add refuses a handle with viscosity on: its solve reads the
    stopping flag on the host between iteration batches."""
    sc = SCENES["dam40_light"]()
    g = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_SPEC, pool_threads=POOL_THREADS)
    b = gpu.Batch()
    with pytest.raises(gpu.FsError) as e:
        b.add(g)
    assert e.value.status == gpu.FS_ERR_UNSUPPORTED
    b.close()
    g.close()
