"""Edge-case scenes shared by the oracle pin tests (test_oracle.py) and the
GPU parity tests (test_gpu_edges.py):

  * ragged_dam   -- a 1.0 x 0.6 m domain, so gridSizeI != gridSizeJ
                    (jsonscenereader.cpp:103-118 sizes the grid from the
                    longer side), with walls and a dam block;
  * sink_dam     -- a dam break whose block falls into a sink
                    (FlipSolver::addSink, sink.h): particles in SINK cells
                    are killed during advection (flipsolver2d.cpp:305-338);
  * empty_box    -- walls and an obstacle, no fluid: zero particles from the
                    first frame on;
  * nb_ragged_dam -- the ragged dam stepped by NBFlipSolver.
"""
from flipsolver2d_gb300 import scenes
from flipsolver2d_gb300.scenes import FlipSolverParameters, Scene, SceneObject


def _params(res: int, seed: int, **kw) -> FlipSolverParameters:
    return FlipSolverParameters(resolution=res, fluidDensity=1000.0, seed=seed,
                                particlesPerCell=4, globalAcceleration=(9.81, 0.0), fps=30,
                                maxSubsteps=10, picRatio=0.03, cflNumber=5.0,
                                particleScale=0.8, pcgIterLimit=200, **kw)


def ragged_dam(res: int = 40, seed: int = 11) -> Scene:
    p = _params(res, seed, domainSizeI=1.0, domainSizeJ=0.6)
    dx, _, _ = p.grid()
    objs = scenes.walls(dx, 1.0, 0.6)
    objs.append(SceneObject("fluid", scenes.rect(0.45, dx, 1.0 - dx, 0.3)))
    return Scene(f"ragged_dam_{res}", p, objs)


def sink_dam(res: int = 36, seed: int = 12) -> Scene:
    sc = scenes.dam_break(res, seed=seed)
    dx, _, _ = sc.params.grid()
    # a sink on the floor (gravity points to +I) ahead of the spreading
    # front: the block's own cells would be reclassified as fluid
    sc.objects.append(SceneObject("sink", scenes.rect(1.0 - 4 * dx, 0.45, 1.0 - dx, 0.8)))
    sc.name = f"sink_dam_{res}"
    return sc


def empty_box(res: int = 32, seed: int = 13) -> Scene:
    p = _params(res, seed)
    dx, _, _ = p.grid()
    objs = scenes.walls(dx)
    objs.append(SceneObject("solid", scenes.rect(0.4, 0.4, 0.6, 0.6), friction=0.1))
    return Scene(f"empty_box_{res}", p, objs)


def nb_ragged_dam(res: int = 40, seed: int = 14) -> Scene:
    """ragged_dam stepped by NBFlipSolver, with nb_dam_break's settings."""
    sc = ragged_dam(res, seed)
    sc.params.particlesPerCell = 8
    sc.params.pcgIterLimit = 1000
    for o in sc.objects:
        if o.kind == "fluid":
            o.viscosity = 10.0
    sc.sim_type = scenes.SIM_NBFLIP
    sc.name = f"nb_ragged_dam_{res}"
    return sc


EDGE_SCENES = {"ragged_dam40": ragged_dam, "sink_dam36": sink_dam, "empty_box32": empty_box,
               "nb_ragged_dam40": nb_ragged_dam}
