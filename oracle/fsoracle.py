"""ctypes driver for the CPU oracles of the FLIP substep (see fsoracle.h).

TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline / reference arm import this module, and only as the checker or the
timed CPU baseline.  The product package never imports it.

Two libraries implement the interface:
  * ``ref``  -- oracle/_ref/libfsref.so, the reference sources built in place
               (oracle/Makefile.ref); present only where the reference is.
  * ``port`` -- oracle/_build/libfsoracle.so, the plain-C restatement
               (oracle/fsoracle.c), built by oracle/build.py everywhere.
"""
from __future__ import annotations

import ctypes
import os
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "_ref", "libfsref.so")
PORT_LIB = os.path.join(HERE, "_build", "libfsoracle.so")

# stage ids (fsoracle.h enum fso_stage)
ADVECT, DECOMPOSITION, REBIN, DENSITY, P2G, SDF, MATERIALS, AFTER_TRANSFER, LEVELSET, \
    VEL_EXTRAP, SAVE_GRID, BODY_FORCES, PROJECT, FRICTION, G2P, COUNT, RESEED, \
    DENSITY_GRID, LEVELSET_OUTSIDE, VISCOSITY = range(20)

# statistic ids (fsoracle.h enum fso_stat)
S_DENSITY_ITERS, S_PRESSURE_ITERS, S_SUBSTEPS, S_FRAME, S_POOL_THREADS, S_VISCOSITY_ITERS = range(6)

# the order in which FlipSolver::step() (flipsolver2d.cpp:412-462) runs them
STEP_STAGES = [ADVECT, DECOMPOSITION, REBIN, DENSITY, P2G, SDF, MATERIALS, AFTER_TRANSFER,
               LEVELSET, VEL_EXTRAP, SAVE_GRID, BODY_FORCES, PROJECT, FRICTION, VEL_EXTRAP,
               G2P, COUNT, RESEED]

# NBFlipSolver::step (nbflipsolver.cpp:26-64) with gridUpdate (:213-225)
NB_STEP_STAGES = [ADVECT, REBIN, P2G, VEL_EXTRAP, SAVE_GRID, SDF, LEVELSET_OUTSIDE,
                  AFTER_TRANSFER, LEVELSET, MATERIALS, BODY_FORCES, DECOMPOSITION, PROJECT,
                  FRICTION, VEL_EXTRAP, G2P, COUNT, RESEED]

# grid ids and numpy dtypes (fsoracle.h enum fso_grid)
GRIDS: Dict[str, tuple] = {
    "material": (0, np.int8, "c"), "solid_sdf": (1, np.float32, "c"),
    "fluid_sdf": (2, np.float32, "c"), "u": (3, np.float32, "u"), "v": (4, np.float32, "v"),
    "u_valid": (5, np.uint8, "u"), "v_valid": (6, np.uint8, "v"),
    "saved_u": (7, np.float32, "u"), "saved_v": (8, np.float32, "v"),
    "viscosity": (9, np.float32, "c"), "known_centered": (10, np.uint8, "c"),
    "density": (11, np.float32, "c"), "particle_counts": (12, np.int32, "c"),
    "solid_id": (13, np.int32, "c"), "div_control": (14, np.float32, "c"),
    "density_rhs": (15, np.float64, "c"), "density_pressure": (16, np.float64, "c"),
    "pressure": (17, np.float64, "c"), "pressure_rhs": (18, np.float64, "c"),
    "emitter_id": (19, np.int32, "c"),
    "advected_u": (20, np.float32, "u"), "advected_v": (21, np.float32, "v"),
    "advected_sdf": (22, np.float32, "c"), "advected_viscosity": (23, np.float32, "c"),
}
STATE_GRIDS = ["material", "solid_sdf", "fluid_sdf", "u", "v", "u_valid", "v_valid",
               "saved_u", "saved_v", "viscosity", "known_centered", "density",
               "particle_counts", "solid_id", "div_control", "density_rhs",
               "density_pressure", "emitter_id"]
NB_GRIDS = ["advected_u", "advected_v", "advected_sdf", "advected_viscosity"]

_libs: Dict[str, ctypes.CDLL] = {}


def _bind(lib: ctypes.CDLL) -> ctypes.CDLL:
    vp, c_int, c_float, c_double = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double
    sz = ctypes.c_size_t
    sig = {
        "fso_create": (vp, [vp]), "fso_create_nbflip": (vp, [vp]), "fso_destroy": (None, [vp]),
        "fso_get_rng": (c_int, [vp, vp]), "fso_set_rng": (c_int, [vp, vp]),
        "fso_add_geometry": (c_int, [vp, c_float, vp, c_int]),
        "fso_add_initial_fluid": (c_int, [vp, c_float, vp, c_int]),
        "fso_add_sink": (c_int, [vp, c_float, vp, c_int]),
        "fso_add_source": (c_int, [vp, vp, c_int, c_float, c_float, c_float, c_float, c_int]),
        "fso_first_frame_init": (None, [vp]), "fso_step_frame": (None, [vp]),
        "fso_set_step_dt": (None, [vp, c_float]), "fso_step_dt": (c_float, [vp]),
        "fso_step": (None, [vp]), "fso_run_stage": (c_int, [vp, c_int]),
        "fso_max_particle_velocity": (c_float, [vp]),
        "fso_bin_count": (sz, [vp]), "fso_particle_count": (sz, [vp]),
        "fso_get_particles": (None, [vp, vp, vp, vp, vp, vp]),
        "fso_set_particles": (None, [vp, vp, vp, vp, vp, vp]),
        "fso_grid_bytes": (sz, [vp, c_int]), "fso_get_grid": (c_int, [vp, c_int, vp]),
        "fso_set_grid": (c_int, [vp, c_int, vp]), "fso_stat": (c_int, [vp, c_int]),
        "fso_pcg_solve": (c_int, [c_int, c_int, vp, c_float, c_double, c_double, vp, vp,
                                  c_int, c_double]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if hasattr(lib, "fso_hardware_concurrency"):
        lib.fso_hardware_concurrency.restype = c_int
        lib.fso_hardware_concurrency.argtypes = []
    # the spec-mode FP64 oracle exists in the C restatement only (the
    # reference has no such solve on its hot path)
    if hasattr(lib, "fso_spec_solve"):
        lib.fso_spec_solve.restype = c_int
        lib.fso_spec_solve.argtypes = [c_int, c_int, vp, c_float, c_double, c_double, vp, vp,
                                       c_double, c_int, vp]
    return lib


def load(kind: str = "port") -> ctypes.CDLL:
    """Load the oracle library `kind` ("port" or "ref")."""
    if kind in _libs:
        return _libs[kind]
    path = REF_LIB if kind == "ref" else PORT_LIB
    if not os.path.exists(path):
        raise FileNotFoundError(f"oracle library {path} is not built")
    lib = _bind(ctypes.CDLL(path))
    _libs[kind] = lib
    return lib


def available(kind: str) -> bool:
    return os.path.exists(REF_LIB if kind == "ref" else PORT_LIB)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleSolver:
    """One FlipSolver instance inside an oracle library."""

    def __init__(self, scene, kind: str = "port"):
        self.lib = load(kind)
        self.kind = kind
        self.scene = scene
        self._cp = scene.params.to_c()
        self.ni, self.nj = self._cp.gridSizeI, self._cp.gridSizeJ
        self.nb = getattr(scene, "sim_type", "flip") == "nbflip"
        create = self.lib.fso_create_nbflip if self.nb else self.lib.fso_create
        self.h = create(ctypes.byref(self._cp))
        for o in scene.objects:
            v = np.ascontiguousarray(o.verts, dtype=np.float32)
            if o.kind == "solid":
                self.lib.fso_add_geometry(self.h, o.friction, _ptr(v), len(v))
            elif o.kind == "fluid":
                self.lib.fso_add_initial_fluid(self.h, o.viscosity, _ptr(v), len(v))
            elif o.kind == "sink":
                self.lib.fso_add_sink(self.h, o.divergence, _ptr(v), len(v))
            elif o.kind == "source":
                self.lib.fso_add_source(self.h, _ptr(v), len(v), o.viscosity, o.divergence,
                                        float(o.velocity[0]), float(o.velocity[1]),
                                        int(o.transfer_velocity))
            else:
                raise ValueError(o.kind)

    def close(self):
        if self.h:
            self.lib.fso_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # driving
    def first_frame_init(self):
        self.lib.fso_first_frame_init(self.h)

    def step_frame(self):
        self.lib.fso_step_frame(self.h)

    def set_dt(self, dt: float):
        self.lib.fso_set_step_dt(self.h, float(dt))

    @property
    def dt(self) -> float:
        return float(self.lib.fso_step_dt(self.h))

    def step(self):
        self.lib.fso_step(self.h)

    def stage(self, s: int):
        assert self.lib.fso_run_stage(self.h, int(s)) == 0

    def max_particle_velocity(self) -> float:
        return float(self.lib.fso_max_particle_velocity(self.h))

    def stat(self, which: int) -> int:
        return int(self.lib.fso_stat(self.h, which))

    # state
    def particle_count(self) -> int:
        return int(self.lib.fso_particle_count(self.h))

    def bin_count(self) -> int:
        return int(self.lib.fso_bin_count(self.h))

    def get_particles(self) -> dict:
        n = self.particle_count()
        nb = self.bin_count()
        counts = np.zeros(nb, np.int32)
        pos = np.zeros((n, 2), np.float32)
        vel = np.zeros((n, 2), np.float32)
        visc = np.zeros(n, np.float32)
        dead = np.zeros(n, np.uint8)
        self.lib.fso_get_particles(self.h, _ptr(counts), _ptr(pos), _ptr(vel), _ptr(visc),
                                   _ptr(dead))
        return {"bin_counts": counts, "pos": pos, "vel": vel, "visc": visc, "dead": dead}

    def set_particles(self, p: dict):
        c = np.ascontiguousarray(p["bin_counts"], np.int32)
        assert len(c) == self.bin_count()
        pos = np.ascontiguousarray(p["pos"], np.float32)
        vel = np.ascontiguousarray(p["vel"], np.float32)
        visc = np.ascontiguousarray(p["visc"], np.float32)
        dead = np.ascontiguousarray(p["dead"], np.uint8)
        self.lib.fso_set_particles(self.h, _ptr(c), _ptr(pos), _ptr(vel), _ptr(visc),
                                   _ptr(dead))

    def grid_shape(self, name: str):
        kind = GRIDS[name][2]
        return {"c": (self.ni, self.nj), "u": (self.ni + 1, self.nj),
                "v": (self.ni, self.nj + 1)}[kind]

    def get_grid(self, name: str) -> np.ndarray:
        gid, dt, _ = GRIDS[name]
        out = np.zeros(self.grid_shape(name), dt)
        assert self.lib.fso_grid_bytes(self.h, gid) == out.nbytes
        assert self.lib.fso_get_grid(self.h, gid, _ptr(out)) == 0
        return out

    def set_grid(self, name: str, a: np.ndarray):
        gid, dt, _ = GRIDS[name]
        a = np.ascontiguousarray(a, dtype=dt).reshape(self.grid_shape(name))
        assert self.lib.fso_set_grid(self.h, gid, _ptr(a)) == 0

    def get_rng(self) -> np.ndarray:
        """The std::mt19937 state: 624 words and the index of the next one."""
        st = np.zeros(625, np.uint32)
        assert self.lib.fso_get_rng(self.h, _ptr(st)) == 0
        return st

    def set_rng(self, st: np.ndarray):
        st = np.ascontiguousarray(st, np.uint32)
        assert st.shape == (625,) and self.lib.fso_set_rng(self.h, _ptr(st)) == 0

    def state_grids(self):
        return STATE_GRIDS + (NB_GRIDS if self.nb else [])

    def snapshot(self) -> dict:
        s = {"particles": self.get_particles(), "dt": self.dt, "rng": self.get_rng()}
        for g in self.state_grids():
            s[g] = self.get_grid(g)
        return s

    def restore(self, snap: dict):
        self.set_particles(snap["particles"])
        for g in self.state_grids():
            if g in snap:
                self.set_grid(g, snap[g])
        if "rng" in snap:
            self.set_rng(snap["rng"])
        self.set_dt(snap["dt"])


def pcg_solve(material: np.ndarray, rhs: np.ndarray, dt: float, density: float, dx: float,
              iter_limit: int, tol: float, kind: str = "port"):
    """LinearSolver::solve on the A/IPP that the solver builds from `material`.
    Returns (iterations, solution)."""
    lib = load(kind)
    ni, nj = material.shape
    m = np.ascontiguousarray(material, np.int8)
    b = np.ascontiguousarray(rhs, np.float64).reshape(ni, nj)
    x = np.zeros((ni, nj), np.float64)
    it = lib.fso_pcg_solve(ni, nj, _ptr(m), float(dt), float(density), float(dx), _ptr(b),
                           _ptr(x), int(iter_limit), float(tol))
    return int(it), x


def spec_solve(material: np.ndarray, rhs: np.ndarray, dt: float, density: float, dx: float,
               rel_tol: float = 1e-6, max_iter: int = 100000):
    """Full-FP64 PCG with the textbook IPP to a true relative residual.
    Returns (iterations, solution, final relative residual)."""
    lib = load("port")
    ni, nj = material.shape
    m = np.ascontiguousarray(material, np.int8)
    b = np.ascontiguousarray(rhs, np.float64).reshape(ni, nj)
    x = np.zeros((ni, nj), np.float64)
    rr = ctypes.c_double(0.0)
    it = lib.fso_spec_solve(ni, nj, _ptr(m), float(dt), float(density), float(dx), _ptr(b), _ptr(x),
                            float(rel_tol), int(max_iter), ctypes.byref(rr))
    return int(it), x, float(rr.value)
