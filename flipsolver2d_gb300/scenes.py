"""Scene descriptions for the FLIP substep workloads (plain data, no compute).

A scene is the parameter block the reference fills from a JSON `settings`
object (Utils/jsonscenereader.cpp:79-136) plus the list of polygonal objects it
adds through FlipSolver::addGeometry / addInitialFluid / addSink
(flipsolver2d.cpp:602-620).  Vertices are in scene units (metres); the solver
converts to cell units with dx.

Workloads (sizes as used by the tests and the benchmark):
  * dam_break(128)            -- 1x1 m, 128^2 cells, 1-cell solid walls, fluid
                                 block I in [0.4, 1-dx], J in [dx, 0.4], 4
                                 particles per cell, seed 42.
  * dam_break(1024, obstacle) -- same layout at 1024^2, seed 7, plus one convex
                                 6-vertex solid (friction 0.1) drawn in the
                                 central 30 % of the domain.
The fluid block is inset by one cell so that it does not overwrite the wall
cells: FlipSolver::updateInitialFluid (flipsolver2d.cpp:573-590) runs after
updateSolids and would otherwise turn wall cells into fluid.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

SIMULATION_LIQUID = 0
PARAM_PARTICLE, PARAM_HYBRID, PARAM_GRID = 0, 1, 2


class FlipSolverParametersC(ctypes.Structure):
    """C layout shared by `fs_params` (include/fs_gpu.h) and `fso_params`
    (oracle/fsoracle.h); field-for-field FlipSolverParameters
    (flipsolver2d.h:33-56)."""

    _fields_ = [
        ("fluidDensity", ctypes.c_double),
        ("seed", ctypes.c_uint),
        ("dx", ctypes.c_double),
        ("particlesPerCell", ctypes.c_int),
        ("globalAccelerationI", ctypes.c_float),
        ("globalAccelerationJ", ctypes.c_float),
        ("resolution", ctypes.c_float),
        ("fps", ctypes.c_int),
        ("maxSubsteps", ctypes.c_int),
        ("picRatio", ctypes.c_float),
        ("cflNumber", ctypes.c_float),
        ("particleScale", ctypes.c_float),
        ("pcgIterLimit", ctypes.c_int),
        ("domainSizeI", ctypes.c_float),
        ("domainSizeJ", ctypes.c_float),
        ("gridSizeI", ctypes.c_int),
        ("gridSizeJ", ctypes.c_int),
        ("sceneScale", ctypes.c_float),
        ("viscosityEnabled", ctypes.c_int),
        ("useHeavyViscosity", ctypes.c_int),
        ("simulationMethod", ctypes.c_int),
        ("parameterHandlingMethod", ctypes.c_int),
    ]


@dataclass
class FlipSolverParameters:
    """Python mirror of FlipSolverParameters with the JSON defaults of
    JsonSceneReader::populateFlipSolverParamsFromJson
    (jsonscenereader.cpp:79-136)."""

    resolution: int = 128
    domainSizeI: float = 1.0
    domainSizeJ: float = 1.0
    fluidDensity: float = 1.0
    seed: int = 0
    particlesPerCell: int = 4
    globalAcceleration: Tuple[float, float] = (9.8, 0.0)
    fps: int = 30
    maxSubsteps: int = 30
    picRatio: float = 0.03
    cflNumber: float = 10.0
    particleScale: float = 0.8
    pcgIterLimit: int = 200
    sceneScale: float = 1.0
    viscosityEnabled: bool = False
    useHeavyViscosity: bool = False
    parameterHandlingMethod: int = PARAM_PARTICLE

    def grid(self) -> Tuple[float, int, int]:
        """dx and grid sizes exactly as jsonscenereader.cpp:103-118 computes
        them (float arithmetic, truncating conversion to int)."""
        f32 = np.float32
        dI = f32(self.domainSizeI) * f32(self.sceneScale)
        dJ = f32(self.domainSizeJ) * f32(self.sceneScale)
        res = f32(self.resolution)
        if dI > dJ:
            dx = f32(dI) / res
            return float(dx), int(self.resolution), int(f32(f32(dJ) / f32(dI)) * res)
        dx = f32(dJ) / res
        return float(dx), int(f32(f32(dI) / f32(dJ)) * res), int(self.resolution)

    def to_c(self) -> FlipSolverParametersC:
        dx, gi, gj = self.grid()
        c = FlipSolverParametersC()
        c.fluidDensity = float(self.fluidDensity)
        c.seed = int(self.seed)
        c.dx = dx
        c.particlesPerCell = int(self.particlesPerCell)
        c.globalAccelerationI = float(self.globalAcceleration[0])
        c.globalAccelerationJ = float(self.globalAcceleration[1])
        c.resolution = float(self.resolution)
        c.fps = int(self.fps)
        c.maxSubsteps = int(self.maxSubsteps)
        c.picRatio = float(self.picRatio)
        c.cflNumber = float(self.cflNumber)
        c.particleScale = float(self.particleScale)
        c.pcgIterLimit = int(self.pcgIterLimit)
        c.domainSizeI = float(np.float32(self.domainSizeI) * np.float32(self.sceneScale))
        c.domainSizeJ = float(np.float32(self.domainSizeJ) * np.float32(self.sceneScale))
        c.gridSizeI = gi
        c.gridSizeJ = gj
        c.sceneScale = float(self.sceneScale)
        c.viscosityEnabled = int(bool(self.viscosityEnabled))
        c.useHeavyViscosity = int(bool(self.useHeavyViscosity))
        c.simulationMethod = SIMULATION_LIQUID
        c.parameterHandlingMethod = int(self.parameterHandlingMethod)
        return c


@dataclass
class SceneObject:
    kind: str  # "solid" | "fluid" | "sink" | "source"
    verts: np.ndarray  # (n, 2) float32, metres
    friction: float = 0.0
    viscosity: float = 0.0
    divergence: float = 0.0
    # sources (Emitter): velocity in scene units per second, applied to the
    # grid and the new particles only when transfer_velocity is set
    velocity: Tuple[float, float] = (0.0, 0.0)
    transfer_velocity: bool = False


SIM_FLIP, SIM_NBFLIP = "flip", "nbflip"


@dataclass
class Scene:
    name: str
    params: FlipSolverParameters
    objects: List[SceneObject] = field(default_factory=list)
    # the solver class the reference's scene reader picks from "simType":
    # FlipSolver ("flip" / "fluid") or NBFlipSolver ("nbflip")
    sim_type: str = SIM_FLIP


def rect(i0: float, j0: float, i1: float, j1: float) -> np.ndarray:
    return np.array([[i0, j0], [i1, j0], [i1, j1], [i0, j1]], dtype=np.float32)


def _convex_hull(pts: np.ndarray) -> np.ndarray:
    """Andrew's monotone chain; returns hull vertices counter-clockwise."""
    p = sorted(map(tuple, pts.tolist()))

    def cross(o, a, b):
        return (a[0] - o[0]) * (b[1] - o[1]) - (a[1] - o[1]) * (b[0] - o[0])

    lower, upper = [], []
    for q in p:
        while len(lower) >= 2 and cross(lower[-2], lower[-1], q) <= 0:
            lower.pop()
        lower.append(q)
    for q in reversed(p):
        while len(upper) >= 2 and cross(upper[-2], upper[-1], q) <= 0:
            upper.pop()
        upper.append(q)
    return np.array(lower[:-1] + upper[:-1], dtype=np.float64)


def convex_polygon(rng: np.random.Generator, n_verts: int, lo: float, hi: float) -> np.ndarray:
    """Draw n_verts points uniformly in [lo, hi]^2 and redraw until their
    convex hull has exactly n_verts vertices."""
    while True:
        pts = rng.uniform(lo, hi, size=(n_verts, 2))
        hull = _convex_hull(pts)
        if len(hull) == n_verts:
            return hull.astype(np.float32)


def walls(dx: float, size_i: float = 1.0, size_j: float = 1.0) -> List[SceneObject]:
    """Four one-cell-thick solid walls around the domain, friction 0."""
    return [
        SceneObject("solid", rect(0.0, 0.0, dx, size_j)),
        SceneObject("solid", rect(size_i - dx, 0.0, size_i, size_j)),
        SceneObject("solid", rect(0.0, 0.0, size_i, dx)),
        SceneObject("solid", rect(0.0, size_j - dx, size_i, size_j)),
    ]


def dam_break(resolution: int = 128, seed: int = 42, obstacle: bool = False,
              obstacle_seed: Optional[int] = None, fluid_box=(0.4, 1.0, 0.0, 0.4),
              **overrides) -> Scene:
    """Plain-FLIP dam break: density 1000, g = (9.81, 0), 30 fps,
    maxSubsteps 10, picRatio 0.03, cflNumber 5, pcgIterLimit 200, 4 ppc."""
    p = FlipSolverParameters(resolution=resolution, fluidDensity=1000.0, seed=seed,
                             particlesPerCell=4, globalAcceleration=(9.81, 0.0), fps=30,
                             maxSubsteps=10, picRatio=0.03, cflNumber=5.0,
                             particleScale=0.8, pcgIterLimit=200)
    for k, v in overrides.items():
        setattr(p, k, v)
    dx, _, _ = p.grid()
    objs = walls(dx)
    i0, i1, j0, j1 = fluid_box
    # inset by one cell wherever the block touches a wall
    i0 = max(i0, dx)
    i1 = min(i1, 1.0 - dx)
    j0 = max(j0, dx)
    j1 = min(j1, 1.0 - dx)
    objs.append(SceneObject("fluid", rect(i0, j0, i1, j1)))
    if obstacle:
        rng = np.random.default_rng(seed if obstacle_seed is None else obstacle_seed)
        objs.append(SceneObject("solid", convex_polygon(rng, 6, 0.35, 0.65), friction=0.1))
    name = f"dam_break_{resolution}" + ("_obstacle" if obstacle else "")
    return Scene(name, p, objs)


def nb_dam_break(resolution: int = 128, seed: int = 0, obstacle: bool = False,
                 viscosity: float = 10.0, **overrides) -> Scene:
    """NB-FLIP dam break (NBFlipSolver): the dam_break layout with 8
    particles per cell, particle viscosity `viscosity` and an iteration limit
    of 1000, stepped by the narrow-band solver.  NB-FLIP seeds no particles
    at start; its first substep fills the band below the fluid surface."""
    kw = dict(particlesPerCell=8, pcgIterLimit=1000)
    kw.update(overrides)
    sc = dam_break(resolution, seed=seed, obstacle=obstacle, **kw)
    for o in sc.objects:
        if o.kind == "fluid":
            o.viscosity = float(viscosity)
    sc.name = "nb_" + sc.name
    sc.sim_type = SIM_NBFLIP
    return sc


def with_source(sc: Scene, box=(0.15, 0.3, 0.45, 0.6), velocity=(2.0, -1.0),
                transfer: bool = True, viscosity: float = 0.0) -> Scene:
    """The scene plus one rectangular source (FlipSolver::addSource) of the
    given box (I0, I1, J0, J1 in metres), emitter velocity (metres per
    second) and viscosity."""
    i0, i1, j0, j1 = box
    sc.objects.append(SceneObject("source", rect(i0, j0, i1, j1), viscosity=float(viscosity),
                                  velocity=(float(velocity[0]), float(velocity[1])),
                                  transfer_velocity=bool(transfer)))
    sc.name += "_source"
    return sc


def with_viscosity(sc: Scene, viscosity: float = 5.0, heavy: bool = False) -> Scene:
    """The scene with viscosity on (FlipSolverParameters::viscosityEnabled and
    useHeavyViscosity, flipsolver2d.h:51-52): its initial fluid carries the
    particle viscosity `viscosity`, and each substep applies the light or the
    heavy model (viscositymodel.cpp) after the pressure projection and
    projects again."""
    sc.params.viscosityEnabled = True
    sc.params.useHeavyViscosity = bool(heavy)
    for o in sc.objects:
        if o.kind == "fluid":
            o.viscosity = float(viscosity)
    sc.name += "_viscous_heavy" if heavy else "_viscous"
    return sc


def random_scene(side: int, seed: int, ppc: int = 4, **overrides) -> Scene:
    """Randomised scene used by the parity tests and the batched workload:
    fluid box corners uniform in [0.1, 0.9] m, 1-3 convex solids of 4-8
    vertices inside the walls, all drawn from default_rng(seed)."""
    rng = np.random.default_rng(seed)
    p = FlipSolverParameters(resolution=side, fluidDensity=1000.0, seed=seed,
                             particlesPerCell=ppc, globalAcceleration=(9.81, 0.0), fps=30,
                             maxSubsteps=10, picRatio=0.03, cflNumber=5.0,
                             particleScale=0.8, pcgIterLimit=200)
    for k, v in overrides.items():
        setattr(p, k, v)
    dx, _, _ = p.grid()
    objs = walls(dx)
    ci = np.sort(rng.uniform(0.1, 0.9, size=2))
    cj = np.sort(rng.uniform(0.1, 0.9, size=2))
    objs.append(SceneObject("fluid", rect(ci[0], cj[0], ci[1], cj[1])))
    for _ in range(int(rng.integers(1, 4))):
        nv = int(rng.integers(4, 9))
        # vertices at sorted random angles on a circle are always in convex
        # position, so no redraw loop is needed for up to 8 vertices
        ang = np.sort(rng.uniform(0.0, 2.0 * np.pi, size=nv))
        rad = float(rng.uniform(0.04, 0.12))
        c = rng.uniform(0.2, 0.8, size=2)
        verts = np.stack([c[0] + rad * np.cos(ang), c[1] + rad * np.sin(ang)], axis=1)
        objs.append(SceneObject("solid", verts.astype(np.float32),
                                friction=float(rng.uniform(0.0, 0.3))))
    return Scene(f"random_{side}_{seed}", p, objs)


def poisson_case(n: int, seed: int = 0, target: float = 0.55, dt: float = 1.0 / 30,
                 density: float = 1000.0):
    """A standalone pressure problem of the mixed-precision configuration:
    an n x n grid with a 1-cell SOLID border, a seeded star-shaped polygon of
    16 vertices (angles sorted, radii scaled until 55 % +- 1 % of the cells
    are FLUID by the cell-centre inside test) and EMPTY elsewhere (Dirichlet
    0); the right-hand side is the reference's calcPressureRhs
    (flipsolver2d.cpp:962-991) applied to a face-velocity field with i.i.d.
    N(0, 1) FP32 values.  Returns (material int8 [n, n], rhs float64 [n, n],
    dx)."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / n
    ang = np.sort(rng.uniform(0.0, 2.0 * np.pi, 16))
    rad = rng.uniform(0.5, 1.0, 16)
    yy, xx = np.mgrid[0:n, 0:n]
    cy, cx = (yy + 0.5) / n - 0.5, (xx + 0.5) / n - 0.5
    theta = np.mod(np.arctan2(cy, cx), 2.0 * np.pi)
    rr = np.hypot(cy, cx)
    # polygon radius along each cell's direction (linear between vertices)
    a_ext = np.concatenate([ang, ang[:1] + 2.0 * np.pi])
    r_ext = np.concatenate([rad, rad[:1]])
    t = np.where(theta < ang[0], theta + 2.0 * np.pi, theta)
    k = np.clip(np.searchsorted(a_ext, t) - 1, 0, 15)
    w = (t - a_ext[k]) / (a_ext[k + 1] - a_ext[k])
    prad = r_ext[k] * (1.0 - w) + r_ext[k + 1] * w
    lo, hi = 0.0, 1.0
    m = None
    for _ in range(60):
        s = 0.5 * (lo + hi)
        inside = rr < s * prad
        frac = inside[1:-1, 1:-1].mean() * (n - 2) ** 2 / n ** 2
        if abs(frac - target) <= 0.01:
            m = inside
            break
        if frac < target:
            lo = s
        else:
            hi = s
    if m is None:
        m = rr < 0.5 * (lo + hi) * prad
    mat = np.full((n, n), 0x10, np.int8)
    mat[m] = 0x40
    mat[0, :] = mat[-1, :] = mat[:, 0] = mat[:, -1] = 0x20
    u = rng.standard_normal((n + 1, n)).astype(np.float32)
    v = rng.standard_normal((n, n + 1)).astype(np.float32)
    fluid = (mat & 0x40) != 0
    solid = (mat & 0x20) != 0
    pad = np.pad(solid, 1, mode="edge")
    scale = 1.0 / dx
    div = (u[1:, :] - u[:-1, :] + v[:, 1:] - v[:, :-1]).astype(np.float64)
    rhs = -scale * div
    rhs -= pad[0:n, 1:n + 1] * scale * u[:-1, :].astype(np.float64)      # solid at i-1
    rhs += pad[2:n + 2, 1:n + 1] * scale * u[1:, :].astype(np.float64)   # solid at i+1
    rhs -= pad[1:n + 1, 0:n] * scale * v[:, :-1].astype(np.float64)      # solid at j-1
    rhs += pad[1:n + 1, 2:n + 2] * scale * v[:, 1:].astype(np.float64)   # solid at j+1
    rhs[~fluid] = 0.0
    return mat, rhs, dx


class UnsupportedScene(ValueError):
    """A scene file that needs a solver or object this GPU path does not have
    (NB-FLIP, smoke, fire, or emitting sources)."""


def scene_from_json(source, name: str = "json") -> Scene:
    """JsonSceneReader::loadJson (Utils/jsonscenereader.cpp:8-77) for the
    plain liquid solver: `source` is a path, a JSON text or an already parsed
    dict in the reference's scene format ({"settings": {...}, "solver":
    {"objects": [...]}}).  Settings take the reference's defaults
    (populateFlipSolverParamsFromJson, :79-136); objects are added in file
    order as addObjectFromJson does (:255-287): "solid" -> addGeometry with
    its friction, "fluid" -> addInitialFluid with its viscosity, "sink" ->
    addSink with its divergence, "source" -> addSource with its viscosity,
    divergence, velocity and transferVelocity (emitterFromJson, :197-225);
    disabled objects are skipped and vertices are multiplied by the scene
    scale.  "nbflip" selects NBFlipSolver (jsonscenereader.cpp creates it for
    that simType).  Solver types other than "flip" / "fluid" / "nbflip" raise
    UnsupportedScene."""
    import json
    import os

    if isinstance(source, dict):
        doc = source
    elif isinstance(source, str) and source.lstrip().startswith("{"):
        doc = json.loads(source)
    else:
        with open(source) as f:
            doc = json.load(f)
        name = os.path.splitext(os.path.basename(str(source)))[0]
    st = doc["settings"]
    sim = st["simType"]
    if sim not in ("flip", "fluid", "nbflip"):
        raise UnsupportedScene(f"simType {sim!r}: only the FLIP and NB-FLIP liquid solvers are on this path")

    def get(key, default):
        return st[key] if key in st else default

    s = float(get("scale", 1.0))
    handling = {"particle": PARAM_PARTICLE, "hybrid": PARAM_HYBRID, "grid": PARAM_GRID}
    g = get("globalAcceleration", (9.8, 0.0))
    p = FlipSolverParameters(
        resolution=int(st["resolution"]),
        domainSizeI=float(st["domainSizeI"]),
        domainSizeJ=float(st["domainSizeJ"]),
        fluidDensity=float(get("density", 1.0)),
        seed=int(get("seed", 0)),
        particlesPerCell=int(st["particlesPerCell"]),
        globalAcceleration=(float(g[0]), float(g[1])),
        fps=int(st["fps"]),
        maxSubsteps=int(get("maxSubsteps", 30)),
        picRatio=float(get("picRatio", 0.03)),
        cflNumber=float(get("cflNumber", 10.0)),
        particleScale=float(get("particleScale", 0.8)),
        pcgIterLimit=int(get("pcgIterLimit", 200)),
        sceneScale=s,
        viscosityEnabled=bool(get("viscosityEnabled", False)),
        useHeavyViscosity=bool(get("heavyViscosity", False)),
        parameterHandlingMethod=handling.get(get("parameterHandlingMethod", "particle"), PARAM_PARTICLE),
    )
    objs: List[SceneObject] = []
    for o in doc["solver"]["objects"]:
        if not o.get("enabled", True):
            continue
        verts = (np.float32(s) * np.asarray(o["verts"], dtype=np.float32)).astype(np.float32)
        kind = o["type"]
        if kind == "solid":
            objs.append(SceneObject("solid", verts, friction=float(o.get("friction", 0.0))))
        elif kind == "fluid":
            objs.append(SceneObject("fluid", verts, viscosity=float(o.get("viscosity", 0.0))))
        elif kind == "sink":
            objs.append(SceneObject("sink", verts, divergence=float(o.get("divergence", 0.0))))
        elif kind == "source":
            vel = o.get("velocity", (0.0, 0.0))
            objs.append(SceneObject("source", verts, viscosity=float(o.get("viscosity", 0.0)),
                                    divergence=float(o.get("divergence", 0.0)),
                                    velocity=(float(vel[0]), float(vel[1])),
                                    transfer_velocity=bool(o.get("transferVelocity", False))))
        else:
            raise UnsupportedScene(f"object type {kind!r}")
    return Scene(name, p, objs, sim_type=SIM_NBFLIP if sim == "nbflip" else SIM_FLIP)
