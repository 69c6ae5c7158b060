"""ctypes binding of libfsgpu.so (include/fs_gpu.h) and a Python mirror of the
reference's FlipSolver / LinearSolver interface on top of it.

The CUDA library is required: importing this module does not build it, and
every call fails loudly (FsError / OSError) when it is missing or when no CUDA
device is present.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import re
from typing import Dict, Optional

import numpy as np

from . import scenes as _scenes

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfsgpu.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "fs_gpu.h")

FS_OK = 0
# fs_status codes (include/fs_gpu.h)
FS_ERR_BAD_ARG, FS_ERR_CUDA, FS_ERR_OOM, FS_ERR_TIMEOUT, FS_ERR_UNSUPPORTED, FS_ERR_STATE, \
    FS_ERR_NONFINITE = range(1, 8)
FS_PCG_FP32, FS_PCG_FP64, FS_PCG_SPEC = 0, 1, 2
# fs_stat ids (FS_STAT_*)
FS_STAT_DENSITY_ITERS, FS_STAT_PRESSURE_ITERS, FS_STAT_SUBSTEPS, FS_STAT_FRAME, \
    FS_STAT_POOL_THREADS, FS_STAT_SUBSTEPS_TOTAL, FS_STAT_VISCOSITY_ITERS = range(7)

# stage ids (FS_STAGE_*), identical to the oracle's
ADVECT, DECOMPOSITION, REBIN, DENSITY, P2G, SDF, MATERIALS, AFTER_TRANSFER, LEVELSET, \
    VEL_EXTRAP, SAVE_GRID, BODY_FORCES, PROJECT, FRICTION, G2P, COUNT, RESEED, \
    DENSITY_GRID, LEVELSET_OUTSIDE, VISCOSITY = range(20)

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
NB_GRIDS = ["advected_u", "advected_v", "advected_sdf", "advected_viscosity"]


class FsError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__(f"{where} failed with status {status}: {msg}")
        self.status = status


class ExecParams(ctypes.Structure):
    _fields_ = [("pcg_precision", ctypes.c_int), ("pool_threads", ctypes.c_int),
                ("device", ctypes.c_int), ("wait_polls", ctypes.c_int), ("reserved", ctypes.c_int * 4)]


_lib: Optional[ctypes.CDLL] = None

_SIGS = {
    "fs_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "fs_last_error": (ctypes.c_char_p, []),
    "fs_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fs_create_nbflip": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fs_get_rng_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fs_set_rng_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fs_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "fs_add_geometry": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p, ctypes.c_int]),
    "fs_add_initial_fluid": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p, ctypes.c_int]),
    "fs_add_sink": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p, ctypes.c_int]),
    "fs_add_source": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_float,
                                     ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_int]),
    "fs_first_frame_init": (ctypes.c_int, [ctypes.c_void_p]),
    "fs_step_frame": (ctypes.c_int, [ctypes.c_void_p]),
    "fs_step": (ctypes.c_int, [ctypes.c_void_p]),
    "fs_set_step_dt": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_float]),
    "fs_get_step_dt": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fs_run_stage": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "fs_max_particle_velocity": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fs_particle_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fs_bin_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fs_get_particles": (ctypes.c_int, [ctypes.c_void_p] * 6),
    "fs_set_particles": (ctypes.c_int, [ctypes.c_void_p] * 6),
    "fs_grid_bytes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "fs_get_grid": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]),
    "fs_set_grid": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]),
    "fs_get_stat": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "fs_enable_timers": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "fs_reset_timers": (ctypes.c_int, [ctypes.c_void_p]),
    "fs_get_timer": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "fs_get_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fs_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "fs_pcg_solve": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_float,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_void_p, ctypes.c_void_p]),
    "fs_pcg_solve_device": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.c_float, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]),
    "fs_pcg_solve_operator": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_double,
                                             ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                             ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]),
    "fs_pcg_solve_spec": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_float,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fs_device_bytes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fs_get_stage_time": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "fs_cluster_autotune": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_void_p, ctypes.c_void_p]),
    "fs_batch_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "fs_batch_add": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fs_batch_remove": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fs_batch_begin_frame": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fs_batch_round": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fs_batch_run_frames": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "fs_batch_in_frame": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fs_batch_submit_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fs_batch_solve_done": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_void_p]),
    "fs_batch_take_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_void_p]),
    "fs_batch_step_frame": (ctypes.c_int, [ctypes.c_void_p]),
    "fs_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "fs_batch_timer": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "fs_pcg_solve_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                          ctypes.c_void_p]),
    "fs_resident_autotune": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_void_p]),
    "fs_server_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_int, ctypes.c_void_p]),
    "fs_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fs_server_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_void_p]),
    "fs_server_take": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p]),
    "fs_server_clusters": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fs_server_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "fs_pcg_solve_device_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                                   ctypes.c_float, ctypes.c_double, ctypes.c_double,
                                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                                   ctypes.c_double, ctypes.c_void_p,
                                                   ctypes.c_void_p]),
}


def header_symbols() -> list:
    """Function names declared in include/fs_gpu.h."""
    with open(HEADER) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(fs_\w+)\s*\(", text, re.M)))


def load() -> ctypes.CDLL:
    """Load the in-tree CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OSError(f"{LIB_PATH} is missing: build it with "
                      "`python -m flipsolver2d_gb300.build` (no CPU fallback exists)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _check(st: int, where: str):
    if st != FS_OK:
        lib = load()
        raise FsError(st, where, lib.fs_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def exec_params(precision: int = FS_PCG_FP32, pool_threads: int = 0, device: int = 0,
                wait_polls: int = 0) -> ExecParams:
    e = ExecParams()
    e.pcg_precision = precision
    e.pool_threads = pool_threads
    e.device = device
    e.wait_polls = wait_polls
    return e


class GpuFlipSolver:
    """FlipSolver (flipsolver2d.h:183-432) with its substep on the GPU, or
    NBFlipSolver (nbflipsolver.h:12-78) for scenes of simType "nbflip"."""

    def __init__(self, scene, precision: int = FS_PCG_FP32, pool_threads: int = 0,
                 device: int = 0, wait_polls: int = 0):
        self.lib = load()
        self.scene = scene
        self._cp = scene.params.to_c()
        self.ni, self.nj = self._cp.gridSizeI, self._cp.gridSizeJ
        self._ex = exec_params(precision, pool_threads, device, wait_polls)
        h = ctypes.c_void_p()
        self.nb = getattr(scene, "sim_type", "flip") == "nbflip"
        create = "fs_create_nbflip" if self.nb else "fs_create"
        _check(getattr(self.lib, create)(ctypes.byref(self._cp), ctypes.byref(self._ex),
                                         ctypes.byref(h)), create)
        self.h = h
        for o in scene.objects:
            v = np.ascontiguousarray(o.verts, dtype=np.float32)
            if o.kind == "solid":
                _check(self.lib.fs_add_geometry(self.h, o.friction, _ptr(v), len(v)), "fs_add_geometry")
            elif o.kind == "fluid":
                _check(self.lib.fs_add_initial_fluid(self.h, o.viscosity, _ptr(v), len(v)),
                       "fs_add_initial_fluid")
            elif o.kind == "sink":
                _check(self.lib.fs_add_sink(self.h, o.divergence, _ptr(v), len(v)), "fs_add_sink")
            elif o.kind == "source":
                _check(self.lib.fs_add_source(self.h, _ptr(v), len(v), o.viscosity, o.divergence,
                                              float(o.velocity[0]), float(o.velocity[1]),
                                              int(o.transfer_velocity)), "fs_add_source")
            else:
                raise ValueError(o.kind)

    def close(self):
        if getattr(self, "h", None):
            self.lib.fs_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # driving (names follow the oracle driver so tests read alike)
    def first_frame_init(self):
        _check(self.lib.fs_first_frame_init(self.h), "fs_first_frame_init")

    def step_frame(self):
        _check(self.lib.fs_step_frame(self.h), "fs_step_frame")

    def step(self):
        _check(self.lib.fs_step(self.h), "fs_step")

    def set_dt(self, dt: float):
        _check(self.lib.fs_set_step_dt(self.h, float(dt)), "fs_set_step_dt")

    @property
    def dt(self) -> float:
        x = ctypes.c_float()
        _check(self.lib.fs_get_step_dt(self.h, ctypes.byref(x)), "fs_get_step_dt")
        return float(x.value)

    def stage(self, s: int):
        _check(self.lib.fs_run_stage(self.h, int(s)), f"fs_run_stage({s})")

    def max_particle_velocity(self) -> float:
        x = ctypes.c_float()
        _check(self.lib.fs_max_particle_velocity(self.h, ctypes.byref(x)), "fs_max_particle_velocity")
        return float(x.value)

    def stage_times(self):
        """Milliseconds per SolverStage (12 entries) since reset_timers."""
        out = []
        for k in range(12):
            x = ctypes.c_double()
            _check(self.lib.fs_get_stage_time(self.h, k, ctypes.byref(x)), "fs_get_stage_time")
            out.append(float(x.value))
        return out

    def device_bytes(self) -> int:
        x = ctypes.c_size_t()
        _check(self.lib.fs_device_bytes(self.h, ctypes.byref(x)), "fs_device_bytes")
        return int(x.value)

    def stat(self, which: int) -> int:
        x = ctypes.c_int()
        _check(self.lib.fs_get_stat(self.h, which, ctypes.byref(x)), "fs_get_stat")
        return int(x.value)

    def particle_count(self) -> int:
        x = ctypes.c_size_t()
        _check(self.lib.fs_particle_count(self.h, ctypes.byref(x)), "fs_particle_count")
        return int(x.value)

    def bin_count(self) -> int:
        x = ctypes.c_size_t()
        _check(self.lib.fs_bin_count(self.h, ctypes.byref(x)), "fs_bin_count")
        return int(x.value)

    def get_particles(self, out: Optional[dict] = None) -> dict:
        """The particles in bin order.  `out` may hold preallocated arrays
        (e.g. in pinned memory) with room for at least particle_count()
        particles: bin_counts [nbins], pos [cap, 2], vel [cap, 2], visc [cap],
        dead [cap]; the result then views them."""
        n = self.particle_count()
        if out is None:
            counts = np.zeros(self.bin_count(), np.int32)
            pos = np.zeros((n, 2), np.float32)
            vel = np.zeros((n, 2), np.float32)
            visc = np.zeros(n, np.float32)
            dead = np.zeros(n, np.uint8)
        else:
            counts, pos, vel = out["bin_counts"], out["pos"][:n], out["vel"][:n]
            visc, dead = out["visc"][:n], out["dead"][:n]
        _check(self.lib.fs_get_particles(self.h, _ptr(counts), _ptr(pos), _ptr(vel), _ptr(visc),
                                         _ptr(dead)), "fs_get_particles")
        return {"bin_counts": counts, "pos": pos, "vel": vel, "visc": visc, "dead": dead}

    def set_particles(self, p: dict):
        c = np.ascontiguousarray(p["bin_counts"], np.int32)
        pos = np.ascontiguousarray(p["pos"], np.float32)
        vel = np.ascontiguousarray(p["vel"], np.float32)
        visc = np.ascontiguousarray(p["visc"], np.float32)
        dead = np.ascontiguousarray(p.get("dead", np.zeros(len(pos), np.uint8)), np.uint8)
        _check(self.lib.fs_set_particles(self.h, _ptr(c), _ptr(pos), _ptr(vel), _ptr(visc),
                                         _ptr(dead)), "fs_set_particles")

    def grid_shape(self, name: str):
        kind = GRIDS[name][2]
        return {"c": (self.ni, self.nj), "u": (self.ni + 1, self.nj),
                "v": (self.ni, self.nj + 1)}[kind]

    def get_grid(self, name: str, out: Optional[np.ndarray] = None) -> np.ndarray:
        gid, dt, _ = GRIDS[name]
        if out is None:
            out = np.zeros(self.grid_shape(name), dt)
        _check(self.lib.fs_get_grid(self.h, gid, _ptr(out), out.nbytes), f"fs_get_grid({name})")
        return out

    def set_grid(self, name: str, a: np.ndarray):
        gid, dt, _ = GRIDS[name]
        a = np.ascontiguousarray(a, dtype=dt).reshape(self.grid_shape(name))
        _check(self.lib.fs_set_grid(self.h, gid, _ptr(a), a.nbytes), f"fs_set_grid({name})")

    def get_rng(self) -> np.ndarray:
        """The std::mt19937 state: 624 words and the index of the next one."""
        st = np.zeros(625, np.uint32)
        _check(self.lib.fs_get_rng_state(self.h, _ptr(st)), "fs_get_rng_state")
        return st

    def set_rng(self, st: np.ndarray):
        st = np.ascontiguousarray(st, np.uint32)
        assert st.shape == (625,)
        _check(self.lib.fs_set_rng_state(self.h, _ptr(st)), "fs_set_rng_state")

    def restore(self, snap: dict, grids=None):
        """Load an oracle snapshot (particles + grids + dt, and the engine
        state when the snapshot has one)."""
        self.set_particles(snap["particles"])
        names = grids or [k for k in GRIDS if k in snap and (self.nb or k not in NB_GRIDS)]
        for g in names:
            self.set_grid(g, snap[g])
        if "rng" in snap:
            self.set_rng(snap["rng"])
        self.set_dt(snap["dt"])

    # timing
    def enable_timers(self, on: bool = True):
        _check(self.lib.fs_enable_timers(self.h, int(on)), "fs_enable_timers")

    def reset_timers(self):
        _check(self.lib.fs_reset_timers(self.h), "fs_reset_timers")

    def timer(self, which: int) -> float:
        x = ctypes.c_double()
        _check(self.lib.fs_get_timer(self.h, which, ctypes.byref(x)), "fs_get_timer")
        return float(x.value)

    def stream_ptr(self) -> int:
        x = ctypes.c_void_p()
        _check(self.lib.fs_get_stream(self.h, ctypes.byref(x)), "fs_get_stream")
        return int(x.value or 0)

    def synchronize(self):
        _check(self.lib.fs_synchronize(self.h), "fs_synchronize")


class GpuLinearSolver:
    """LinearSolver (linearsolver.h:9-23): solve() keeps the reference's
    arguments and return convention (iteration count; == iterLimit means the
    solve failed)."""

    def __init__(self, precision: int = FS_PCG_FP32, pool_threads: int = 0, device: int = 0,
                 wait_polls: int = 0):
        self.lib = load()
        self._ex = exec_params(precision, pool_threads, device, wait_polls)

    def solve(self, material: np.ndarray, dt: float, density: float, dx: float,
              result: np.ndarray, vec: np.ndarray, iter_limit: int = 20, tol: float = 1e-6) -> int:
        ni, nj = material.shape
        m = np.ascontiguousarray(material, np.int8)
        b = np.ascontiguousarray(vec, np.float64).reshape(ni, nj)
        x = np.zeros((ni, nj), np.float64)
        it = ctypes.c_int()
        _check(self.lib.fs_pcg_solve(ni, nj, _ptr(m), float(dt), float(density), float(dx), _ptr(b),
                                     _ptr(x), int(iter_limit), float(tol), ctypes.byref(self._ex),
                                     ctypes.byref(it)), "fs_pcg_solve")
        result[...] = x.reshape(result.shape)
        return int(it.value)


def pcg_solve(material: np.ndarray, rhs: np.ndarray, dt: float, density: float, dx: float,
              iter_limit: int, tol: float, precision: int = FS_PCG_FP32, pool_threads: int = 8,
              wait_polls: int = 0):
    """Functional form returning (iterations, solution)."""
    x = np.zeros(material.shape, np.float64)
    it = GpuLinearSolver(precision, pool_threads, wait_polls=wait_polls).solve(
        material, dt, density, dx, x, rhs, iter_limit, tol)
    return it, x


def pcg_solve_operator(cell_info: np.ndarray, rhs: np.ndarray, scale: float, iter_limit: int,
                       tol: float, precision: int = FS_PCG_FP32, pool_threads: int = 8, device: int = 0):
    """fs_pcg_solve_operator: LinearSolver::solve on an operator given as one
    byte per cell (unit bit 7, non-solid count bits 4-6, fluid-neighbour mask
    bits 0-3) and its scale.  Returns (iterations, solution float64)."""
    lib = load()
    ni, nj = cell_info.shape
    info = np.ascontiguousarray(cell_info, np.uint8)
    b = np.ascontiguousarray(rhs, np.float64).reshape(ni, nj)
    x = np.zeros((ni, nj), np.float64)
    it = ctypes.c_int()
    ex = exec_params(precision, pool_threads, device)
    _check(lib.fs_pcg_solve_operator(ni, nj, _ptr(info), scale, _ptr(b), _ptr(x), iter_limit, tol,
                                     ctypes.byref(ex), ctypes.byref(it)), "fs_pcg_solve_operator")
    return int(it.value), x


def resident_autotune(ni: int, nj: int, device: int = 0):
    """fs_resident_autotune: (tile rows, tile columns, us per iteration) of
    the fastest resident tile shape, recorded for this grid shape."""
    lib = load()
    r, c, us = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
    _check(lib.fs_resident_autotune(int(ni), int(nj), int(device), ctypes.byref(r), ctypes.byref(c),
                                    ctypes.byref(us)), "fs_resident_autotune")
    return int(r.value), int(c.value), float(us.value)


class Server:
    """fs_server: the device-resident request loop for spec-mode solves (a
    persistent launch that takes requests from a ring in mapped memory)."""

    def __init__(self, max_ni: int, max_nj: int, slots: int = 64, rel_tol: float = 1e-6,
                 max_iter: int = 100000, device: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        _check(self.lib.fs_server_create(int(device), int(max_ni), int(max_nj), int(slots), float(rel_tol),
                                         int(max_iter), ctypes.byref(h)), "fs_server_create")
        self.h = h
        self._shapes = {}

    def submit(self, material, rhs, dt, density, dx) -> int:
        ni, nj = material.shape
        m = np.ascontiguousarray(material, np.int8)
        b = np.ascontiguousarray(rhs, np.float64).reshape(ni, nj)
        sysd = PoissonSystem(ni, nj, m.ctypes.data, float(dt), float(density), float(dx),
                             b.ctypes.data, None, 0, 0.0)
        t = ctypes.c_ulonglong()
        _check(self.lib.fs_server_submit(self.h, ctypes.byref(sysd), ctypes.byref(t)), "fs_server_submit")
        self._shapes[int(t.value)] = (ni, nj)
        return int(t.value)

    def poll(self, ticket: int) -> bool:
        x = ctypes.c_int()
        _check(self.lib.fs_server_poll(self.h, ctypes.c_ulonglong(ticket), ctypes.byref(x)), "fs_server_poll")
        return bool(x.value)

    def take(self, ticket: int):
        """(inner iterations, solution float64 [ni, nj], relative residual)."""
        ni, nj = self._shapes.get(ticket, (1, 1))  # an unknown ticket: the library reports it
        x = np.zeros((ni, nj), np.float64)
        it = ctypes.c_int()
        rr = ctypes.c_double()
        _check(self.lib.fs_server_take(self.h, ctypes.c_ulonglong(ticket), x.ctypes.data, ctypes.byref(it),
                                       ctypes.byref(rr)), "fs_server_take")
        del self._shapes[ticket]
        return int(it.value), x, float(rr.value)

    def clusters(self) -> int:
        x = ctypes.c_int()
        _check(self.lib.fs_server_clusters(self.h, ctypes.byref(x)), "fs_server_clusters")
        return int(x.value)

    def close(self):
        if getattr(self, "h", None):
            st = self.lib.fs_server_destroy(self.h)
            self.h = None
            _check(st, "fs_server_destroy")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """fs_batch: GpuFlipSolver handles (FS_PCG_SPEC) stepped together; each
    handle's results equal those of stepping it alone.  Members join and
    leave between their frames; standalone systems can ride along."""

    def __init__(self, solvers=()):
        self.lib = load()
        self.solvers = list(solvers)
        arr = (ctypes.c_void_p * max(len(self.solvers), 1))(*[g.h.value for g in self.solvers])
        h = ctypes.c_void_p()
        _check(self.lib.fs_batch_create(arr, len(self.solvers), ctypes.byref(h)), "fs_batch_create")
        self.h = h
        self._solves = {}

    def step_frame(self):
        _check(self.lib.fs_batch_step_frame(self.h), "fs_batch_step_frame")

    def run_frames(self, frames: int):
        """`frames` frames of every member, pipelined across members."""
        _check(self.lib.fs_batch_run_frames(self.h, int(frames)), "fs_batch_run_frames")

    def add(self, g):
        _check(self.lib.fs_batch_add(self.h, g.h), "fs_batch_add")
        self.solvers.append(g)

    def remove(self, g):
        _check(self.lib.fs_batch_remove(self.h, g.h), "fs_batch_remove")
        self.solvers.remove(g)

    def begin_frame(self, g):
        _check(self.lib.fs_batch_begin_frame(self.h, g.h), "fs_batch_begin_frame")

    def in_frame(self, g) -> bool:
        x = ctypes.c_int()
        _check(self.lib.fs_batch_in_frame(self.h, g.h, ctypes.byref(x)), "fs_batch_in_frame")
        return bool(x.value)

    def round(self) -> int:
        """One round; returns the members still inside a frame."""
        x = ctypes.c_int()
        _check(self.lib.fs_batch_round(self.h, ctypes.byref(x)), "fs_batch_round")
        return int(x.value)

    def submit_solve(self, material, rhs, dt, density, dx) -> int:
        ni, nj = material.shape
        m = np.ascontiguousarray(material, np.int8)
        b = np.ascontiguousarray(rhs, np.float64).reshape(ni, nj)
        sysd = PoissonSystem(ni, nj, m.ctypes.data, float(dt), float(density), float(dx),
                             b.ctypes.data, None, 0, 0.0)
        t = ctypes.c_ulonglong()
        _check(self.lib.fs_batch_submit_solve(self.h, ctypes.byref(sysd), ctypes.byref(t)),
               "fs_batch_submit_solve")
        self._solves[int(t.value)] = (ni, nj)
        return int(t.value)

    def solve_done(self, ticket: int) -> bool:
        x = ctypes.c_int()
        _check(self.lib.fs_batch_solve_done(self.h, ctypes.c_ulonglong(ticket), ctypes.byref(x)),
               "fs_batch_solve_done")
        return bool(x.value)

    def take_solve(self, ticket: int):
        """(inner iterations, solution float64 [ni, nj], relative residual)."""
        ni, nj = self._solves.pop(ticket)
        x = np.zeros((ni, nj), np.float64)
        sysd = PoissonSystem(ni, nj, None, 0.0, 0.0, 0.0, None, x.ctypes.data, 0, 0.0)
        _check(self.lib.fs_batch_take_solve(self.h, ctypes.c_ulonglong(ticket), ctypes.byref(sysd)),
               "fs_batch_take_solve")
        return int(sysd.iterations), x, float(sysd.rel_residual)

    def timer(self, which: int) -> float:
        """0 merged-solve device ms, 1 round wall ms, 2 rounds; 3 resets."""
        x = ctypes.c_double()
        _check(self.lib.fs_batch_timer(self.h, int(which), ctypes.byref(x)), "fs_batch_timer")
        return float(x.value)

    def close(self):
        if getattr(self, "h", None):
            self.lib.fs_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cluster_autotune(ni: int, nj: int, objective: int = 0, device: int = 0):
    """fs_cluster_autotune: (chosen CTAs per cluster, microseconds per inner
    iteration).  objective 0 = throughput (batches), 1 = latency."""
    lib = load()
    c = ctypes.c_int()
    us = ctypes.c_float()
    _check(lib.fs_cluster_autotune(int(ni), int(nj), int(objective), int(device), ctypes.byref(c),
                                   ctypes.byref(us)), "fs_cluster_autotune")
    return int(c.value), float(us.value)


class PoissonSystem(ctypes.Structure):
    """fs_poisson_system (include/fs_gpu.h)."""
    _fields_ = [("ni", ctypes.c_int), ("nj", ctypes.c_int), ("material", ctypes.c_void_p),
                ("dt", ctypes.c_float), ("density", ctypes.c_double), ("dx", ctypes.c_double),
                ("rhs", ctypes.c_void_p), ("result", ctypes.c_void_p),
                ("iterations", ctypes.c_int), ("rel_residual", ctypes.c_double)]


def pcg_solve_batch(problems, rel_tol: float = 1e-6, max_iter: int = 100000, device: int = 0):
    """Batched spec-mode solve (fs_pcg_solve_batch): `problems` is a list of
    (material int8 [ni, nj], rhs float64 [ni, nj], dt, density, dx).  Returns a
    list of (inner iterations, solution float64 [ni, nj], relative residual)."""
    lib = load()
    n = len(problems)
    arr = (PoissonSystem * max(n, 1))()
    keep = []
    for k, (mat, rhs, dt, density, dx) in enumerate(problems):
        ni, nj = mat.shape
        m = np.ascontiguousarray(mat, np.int8)
        b = np.ascontiguousarray(rhs, np.float64).reshape(ni, nj)
        x = np.zeros((ni, nj), np.float64)
        keep.append((m, b, x))
        arr[k] = PoissonSystem(ni, nj, m.ctypes.data, float(dt), float(density), float(dx),
                               b.ctypes.data, x.ctypes.data, 0, 0.0)
    ex = ExecParams(FS_PCG_FP32, 0, device)
    st = lib.fs_pcg_solve_batch(ctypes.addressof(arr), n, float(rel_tol), int(max_iter),
                                ctypes.byref(ex))
    _check(st, "fs_pcg_solve_batch")
    return [(int(arr[k].iterations), keep[k][2], float(arr[k].rel_residual)) for k in range(n)]


def pcg_solve_spec(material: np.ndarray, rhs: np.ndarray, dt: float, density: float, dx: float,
                   rel_tol: float = 1e-6, max_iter: int = 100000, device: int = 0):
    """Spec-mode solve to a true relative residual (FP32 inner PCG with the
    textbook IPP, FP64 refinement).  Returns (inner iterations, solution,
    final relative residual)."""
    lib = load()
    ni, nj = material.shape
    m = np.ascontiguousarray(material, np.int8)
    b = np.ascontiguousarray(rhs, np.float64).reshape(ni, nj)
    x = np.zeros((ni, nj), np.float64)
    ex = ExecParams(FS_PCG_FP32, 0, device)
    it = ctypes.c_int(0)
    rr = ctypes.c_double(0.0)
    st = lib.fs_pcg_solve_spec(ni, nj, m.ctypes.data, float(dt), float(density), float(dx),
                               b.ctypes.data, x.ctypes.data, float(rel_tol), int(max_iter),
                               ctypes.byref(ex), ctypes.byref(it), ctypes.byref(rr))
    _check(st, "fs_pcg_solve_spec")
    return int(it.value), x, float(rr.value)
