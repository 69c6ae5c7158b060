"""Benchmark of the FLIP substep on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

Workload: the large plain-FLIP dam break -- 1x1 m at 1024^2 cells, 1-cell
solid walls, fluid block I in [0.4, 1-dx], J in [dx, 0.4], 4 particles per
cell jittered from seed 7 (~1.0 M particles), one convex 6-vertex solid
(friction 0.1) drawn in the central 30 % from seed 7; density 1000, g = 9.81,
30 fps, CFL 5, picRatio 0.03, pcgIterLimit 200 with the reference's absolute
1e-2 max-abs stopping test, FP32 PCG vectors with float-pair (hi + lo)
reductions and scalars.  Synthetic seeded data.  --res picks a smaller grid
of the same scene (parity-size runs and profiler captures).  A step is one substep (FlipSolver::step) with the CFL dt the
reference's frame loop would choose; the scene is first advanced by two
frames so the fluid is moving.

One JSON line is printed.  `value` is device-timed (CUDA events on the
solver's stream, L2 flushed by a 256 MiB write between steps, outside the
events); `e2e` goes through the C ABI with host-resident state uploaded and
downloaded every step; `roofline` is for the PCG kernel, which dominates the
substep; `cpu_baseline` is the CPU oracle on this host's cores on a bounded
sample of the same workload.  `fp64_check` steps the final state once more
in FP32 and in the FP64 parity mode from identical inputs and reports the
FP32 error.  Unless --no-batch, sub-objects beside it: `spec_single`, the
same scene with every solve to a 1e-6 true residual (FS_PCG_SPEC);
`poisson_2048`, one 2048^2 standalone spec-mode solve; `batch`, the batched
form of the path: 64 scenes of the batched-scenes workload stepped together
at a 1e-6 pressure residual, and the same scenes one at a time; `nbflip`,
the same scene stepped by the narrow-band solver (NB-FLIP); `serve`, 120
requests of the seeded serving stream (requests/s, p50/p99 latency, worst
solve residual).
With --impl reference only the CPU
implementation is timed (the reference's sources are not present on GPU
hosts, so its plain-C restatement, pinned bit for bit to it, stands in).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

RES = 1024
SEED = 7
WARM_FRAMES = 2
METRIC = "particle-substeps/s"
WORKLOAD = "dam_break_1024_obstacle"
# DRAM bytes (read + write) of one k_pcg_resident launch at 1024^2, measured
# by ncu (dram__bytes_read.sum + dram__bytes_write.sum) on this workload; the
# solve keeps its vectors on chip, so this is little more than b and the
# operator in, x out
PCG_TRAFFIC_BYTES = 9078784


def set_resolution(res: int):
    global RES, WORKLOAD
    RES = res
    WORKLOAD = f"dam_break_{res}_obstacle"


def scene():
    from flipsolver2d_gb300 import scenes

    return scenes.dam_break(RES, seed=SEED, obstacle=True)


def cfl_dt(vel: float, p) -> float:
    """First substep size of FlipSolver::stepFrame (flipsolver2d.cpp:478-489)."""
    f32 = np.float32
    frame_dt = f32(1.0) / f32(p.fps)
    m = f32(p.cflNumber) / (f32(vel) + f32(1e-15))
    if m >= frame_dt or p.maxSubsteps == 1:
        return float(frame_dt)
    if f32(2.0) * m >= frame_dt:
        return float(f32(0.5) * frame_dt)
    return float(m)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.pre = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
            return
        # nvidia-smi takes a moment to start: wait for its first sample, so
        # that the samples kept are the ones taken inside the timed region
        t0 = time.time()
        while not self.lines and self.proc.poll() is None and time.time() - t0 < 5:
            time.sleep(0.01)
        self.pre, self.lines = self.lines, []

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # a region shorter than the sampling period: the sample just before it
        in_region = len(self.lines)
        for ln in self.lines if in_region else self.pre[-1:]:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sms) if sms else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sms), "samples_in_region": in_region}


def combine_replicas(ms: float, work: float, dist=None, device: str = "cpu"):
    """Whole-job figures of independent replicas (one scene per rank, no
    collective on the data path): the slowest rank's time and the sum of the
    particle-substeps all ranks processed."""
    if dist is None:
        return ms, work
    import torch

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    w = torch.tensor([float(work)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    return float(t.item()), float(w.item())


def executed_iters(ret: int, limit: int) -> int:
    """LinearSolver::solve returns the loop index on convergence."""
    return limit if ret >= limit else ret + 1


def cpu_info():
    """What the CPU baseline ran on: the CPU model (lscpu), the processors
    the OS reports and this process may use, and the count the reference's
    thread pool would take (std::thread::hardware_concurrency())."""
    import platform

    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                model = ln.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    info = {"cpu_model": model, "machine": platform.machine(), "nproc": os.cpu_count(),
            "affinity_cpus": len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else None}
    try:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import fsoracle as fo

        info["hardware_concurrency"] = int(fo.load("port").fso_hardware_concurrency())
    except Exception:
        info["hardware_concurrency"] = None
    return info


def run_cpu_sample(threads: int, substeps: int = 2, snapshot=None, warmup: int = 3):
    """The CPU implementation on a bounded sample of the work the GPU arm
    times: the workload after WARM_FRAMES frames and `warmup` CFL substeps,
    then `substeps` timed substeps, each with the CFL dt of the frame loop.
    The warm state is `snapshot` (the GPU's state at that point, in the
    oracle's layout) when given, else the oracle steps it itself; either way
    it is untimed.  The reference build runs where its sources are present,
    else the pinned plain-C port, on `threads` host threads with the
    reference's pool size for its chunked reductions."""
    os.environ["FSO_HOST_THREADS"] = str(threads)
    os.environ["FSO_REF_THREADS"] = str(threads)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build as oracle_build

    oracle_build.build_port()
    import fsoracle as fo

    kind = "reference" if fo.available("ref") else "port"
    sc = scene()
    o = fo.OracleSolver(sc, "ref" if kind == "reference" else "port")
    o.first_frame_init()
    t_warm = time.perf_counter()
    if snapshot is not None:
        o.restore(snapshot)
        start = "the GPU's state"
    else:
        for _ in range(WARM_FRAMES):
            o.step_frame()
        for _ in range(warmup):
            o.set_dt(cfl_dt(o.max_particle_velocity(), sc.params))
            o.step()
        start = "its own state"
    t_warm = time.perf_counter() - t_warm
    work, t_total, times, iters = 0, 0.0, [], []
    for _ in range(substeps):
        n = o.particle_count()
        o.set_dt(cfl_dt(o.max_particle_velocity(), sc.params))
        t0 = time.perf_counter()
        o.step()
        dt = time.perf_counter() - t0
        times.append(dt)
        t_total += dt
        work += n
        iters.append([executed_iters(o.stat(0), sc.params.pcgIterLimit),
                      executed_iters(o.stat(1), sc.params.pcgIterLimit)])
    o.close()
    info = cpu_info()
    return {"value": work / t_total, "unit": METRIC, "cores": threads, "kind": kind,
            "sample": f"{substeps} substeps of {WORKLOAD} from {start} after {WARM_FRAMES} frames "
                      f"and {warmup} substeps ({work} particle-substeps, {t_total:.1f} s; "
                      f"warm-up {t_warm:.1f} s untimed)",
            "pcg_iterations_per_step": iters, "step_s": times, **info}


def bench_config(warmup: int):
    """`config` of both arms: the workload and the point it is timed at."""
    return {"workload": WORKLOAD, "grid": RES, "seed": SEED, "warm_frames": WARM_FRAMES,
            "warm_substeps": warmup, "pcg_iter_limit": 200,
            "stopping": "reference absolute 1e-2 max-abs test"}


CPU_KEYS = ("value", "unit", "cores", "kind", "sample", "cpu_model", "machine", "nproc",
            "affinity_cpus", "hardware_concurrency", "pcg_iterations_per_step")


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    steps = max(1, min(args.steps, 3))
    cb = run_cpu_sample(threads, substeps=steps, warmup=args.warmup)
    line = {"metric": METRIC, "value": cb["value"], "unit": METRIC, "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(cb["step_s"])),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded dam-break scene)", "config": bench_config(args.warmup),
            "pcg": "reference PCG+IPP, FP64, limit 200, abs tol 1e-2",
            "impl": "reference",
            "cpu_baseline": {k: cb[k] for k in CPU_KEYS if k in cb},
            "e2e": {"value": cb["value"], "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def apply_operator(mat, x, dt, density, dx):
    """The reference's pressure operator (IndexedPressureParameterUnit::
    multiply, pressuredata.h:132-146, rows as getPressureProjectionMatrix
    builds them, flipsolver2d.cpp:797-887) applied in float64 on the host:
    scale (count x_c - sum of fluid neighbours) on fluid rows, identity on the
    others.  Used only to measure residuals outside any timed region."""
    ni, nj = mat.shape
    scale = np.float64(np.float32(dt)) / (density * dx * dx)
    fl = (mat & 0x40) != 0
    solid = (mat & 0x20) != 0
    pad_s = np.pad(solid, 1, mode="edge")
    pad_f = np.pad(fl, 1, mode="edge")
    xp = np.pad(x, 1)
    cnt = np.zeros_like(x)
    acc = np.zeros_like(x)
    for di, dj in ((-1, 0), (1, 0), (0, -1), (0, 1)):
        cnt += ~pad_s[1 + di:ni + 1 + di, 1 + dj:nj + 1 + dj]
        acc += pad_f[1 + di:ni + 1 + di, 1 + dj:nj + 1 + dj] * xp[1 + di:ni + 1 + di, 1 + dj:nj + 1 + dj]
    out = x.copy()
    out[fl] = (scale * (cnt * x - acc))[fl]
    return out


# the FP32 production mode's bar against the FP64 parity mode on one substep
# from identical inputs (the 200-iteration solve does not converge, so the
# bar is on residuals, velocities and the recurrence's own spread)
FP64_CHECK_VEL_BAR = 1e-2
FP64_CHECK_SPREAD_FACTOR = 10.0


def fp64_check(s, sc, p):
    """One substep from identical state in the measured FP32 mode and in the
    FP64 parity mode (the reference's own arithmetic): the FP32 error and the
    bar it is held to.  Outside any timed region.

    * pressure_rel_l2: FP32 pressure against FP64;
    * true_rel_residual_fp32 / _fp64: ||b - A p|| / ||b|| of each mode's
      pressure on its own right-hand side, with the reference's operator;
    * fp64_spread_rel_l2: how far the FP64 solve itself moves when b moves by
      1e-7 relative (about one FP32 rounding): the recurrence's sensitivity;
    * grid_velocity_rel_l2, particle_vel_rel_l2: the projected velocities.
    The bar: FP32 residual <= 1.05 x FP64 residual + 1e-6, velocities within
    1e-2, pressure within max(1e-2, 10 x spread)."""
    from flipsolver2d_gb300 import gpu

    snap = s.get_particles()
    grids = {g: s.get_grid(g) for g in ("u", "v", "material")}
    dt = cfl_dt(s.max_particle_velocity(), p)
    d = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_FP64)
    d.first_frame_init()  # the solid data; the fluid state is replaced below
    out = []
    for g in (s, d):
        g.set_particles(snap)
        for k, a in grids.items():
            g.set_grid(k, a)
        g.set_dt(dt)
        g.step()
        out.append((g.get_particles(), g.get_grid("pressure"), g.get_grid("pressure_rhs"),
                    g.get_grid("u"), g.get_grid("v"), [g.stat(0), g.stat(1)]))
    d.close()
    (a, pa, ba, ua, va, ia), (b, pb, bb, ub, vb, ib) = out

    def rel(x, y):
        n = float(np.linalg.norm(y))
        return float(np.linalg.norm(np.asarray(x, np.float64) - np.asarray(y, np.float64)) / n) if n else 0.0

    mat = grids["material"]  # the operator of this substep's solves
    dx = 1.0 / RES

    def rel_residual(x, rhs):
        n = float(np.linalg.norm(rhs))
        return float(np.linalg.norm(rhs - apply_operator(mat, x, dt, p.fluidDensity, dx)) / n) if n else 0.0

    _, p0 = gpu.pcg_solve(mat, bb, dt, p.fluidDensity, dx, p.pcgIterLimit, 1e-2,
                          precision=gpu.FS_PCG_FP64)
    xi = np.random.default_rng(5).standard_normal(bb.shape)
    _, p1 = gpu.pcg_solve(mat, bb * (1.0 + 1e-7 * xi), dt, p.fluidDensity, dx, p.pcgIterLimit, 1e-2,
                          precision=gpu.FS_PCG_FP64)
    spread = rel(p1, p0)
    rr32, rr64 = rel_residual(pa, ba), rel_residual(pb, bb)
    res = {"dt": dt, "particles": int(len(b["pos"])), "pressure_rel_l2": rel(pa, pb),
           "true_rel_residual_fp32": rr32, "true_rel_residual_fp64": rr64,
           "fp64_spread_rel_l2": spread,
           "grid_velocity_rel_l2": max(rel(ua, ub), rel(va, vb)),
           # iterations of the density and pressure solves in each mode: a
           # different stopping iteration under the absolute max-abs test
           # tells a branch apart from rounding in the unconverged solve
           "pcg_iters_fp32": ia, "pcg_iters_fp64": ib}
    if a["pos"].shape == b["pos"].shape:
        res["particle_vel_rel_l2"] = rel(a["vel"], b["vel"])
        res["particle_pos_max_abs_cells"] = float(np.max(np.abs(a["pos"] - b["pos"])))
    else:
        res["particle_count_difference"] = int(len(a["pos"]) - len(b["pos"]))
    res["bar"] = {"residual": rr32 <= 1.05 * rr64 + 1e-6,
                  "velocity": res["grid_velocity_rel_l2"] <= FP64_CHECK_VEL_BAR
                  and res.get("particle_vel_rel_l2", 1.0) <= FP64_CHECK_VEL_BAR,
                  "pressure": res["pressure_rel_l2"] <= max(1e-2, FP64_CHECK_SPREAD_FACTOR * spread),
                  "stated": "residual <= 1.05 x FP64 + 1e-6; velocities <= 1e-2 rel-L2; "
                            "pressure <= max(1e-2, 10 x FP64 spread under a 1e-7 change of b)"}
    res["bar"]["pass"] = res["bar"]["residual"] and res["bar"]["velocity"] and res["bar"]["pressure"]
    return res


def gpu_snapshot(s):
    """The handle's state in the oracle's snapshot layout (the CPU sample
    starts from it)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import fsoracle as fo

    snap = {"particles": s.get_particles(), "dt": s.dt, "rng": s.get_rng()}
    for g in fo.STATE_GRIDS:
        snap[g] = s.get_grid(g)
    return snap


def spec_single_measure(local: int, steps: int):
    """The bench scene alone in FS_PCG_SPEC mode: every density and pressure
    solve to a 1e-6 true relative residual (FP32 inner PCG, FP64 refinement);
    after the same warm frames and 3 warm-up substeps, `steps` substeps
    device-timed like the main line (L2 flushed between them)."""
    import torch
    from flipsolver2d_gb300 import gpu

    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")
    sc = scene()
    p = sc.params
    s = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_SPEC, device=local)
    for _ in range(WARM_FRAMES):
        s.step_frame()

    def one_step():
        n = s.particle_count()
        s.set_dt(cfl_dt(s.max_particle_velocity(), p))
        s.step()
        return n

    for _ in range(3):
        one_step()
    s.enable_timers(True)
    work, step_ms = 0, []
    for _ in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        s.reset_timers()
        work += one_step()
        step_ms.append(s.timer(0))
    s.enable_timers(False)
    s.close()
    total = float(sum(step_ms))
    return {"workload": f"{WORKLOAD}, FS_PCG_SPEC", "value": work / (total / 1e3), "unit": METRIC,
            "ms_per_step": total / steps, "steps": steps,
            "step_latency_ms": {"p50": float(np.percentile(step_ms, 50)),
                                "p99": float(np.percentile(step_ms, 99))},
            "pcg": "every solve to a 1e-6 true relative residual: FP32 inner PCG, textbook IPP, "
                   "FP64 refinement"}


def poisson_measure(n: int, warmup: int, steps: int):
    """The mixed-precision configuration: fs_pcg_solve_spec on the seeded
    n x n star mask (55 % fluid) with the divergence of N(0, 1) faces, to a
    1e-6 true relative residual; host arrays, so the time includes the
    uploads and the download."""
    from flipsolver2d_gb300 import gpu, scenes

    m, b, dx = scenes.poisson_case(n, seed=0)
    for _ in range(warmup):
        gpu.pcg_solve_spec(m, b, 1.0 / 30, 1000.0, dx, 1e-6)
    times, iters, rr = [], [], 0.0
    for _ in range(steps):
        t0 = time.perf_counter()
        it, x, rr = gpu.pcg_solve_spec(m, b, 1.0 / 30, 1000.0, dx, 1e-6)
        times.append(time.perf_counter() - t0)
        iters.append(it)
    total = sum(times)
    return {"workload": f"poisson_{n}_spec", "value": n * n * sum(iters) / total,
            "unit": "cell-iter/s", "ms_per_solve": 1e3 * total / steps, "inner_iterations": iters,
            "rel_residual": rr, "path": "fs_pcg_solve_spec with host arrays (uploads included)"}


def gpu_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    from flipsolver2d_gb300 import build, gpu

    build.build()
    torch.cuda.set_device(local)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")

    def l2_flush():
        flush.fill_(1.0)
        torch.cuda.synchronize()

    sc = scene()
    p = sc.params
    s = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_FP32, device=local)
    for _ in range(WARM_FRAMES):
        s.step_frame()
    ncell = s.ni * s.nj
    limit = p.pcgIterLimit

    def one_step():
        n = s.particle_count()
        s.set_dt(cfl_dt(s.max_particle_velocity(), p))
        s.step()
        return n

    for _ in range(args.warmup):
        one_step()
    # the state the timed substeps start from, for the CPU sample
    cpu_start = gpu_snapshot(s) if (rank == 0 and not args.no_cpu) else None
    s.enable_timers(True)
    sampler = ClockSampler(local)
    sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    if args.profile_timed:  # ncu --profile-from-start off sees the timed substeps only
        torch.cuda.profiler.start()
    work, step_ms, pcg_ms, iters, bytes_pcg = 0, [], 0.0, [], 0.0
    launches = 0.0
    for _ in range(args.steps):
        l2_flush()
        s.reset_timers()
        n = one_step()
        work += n
        step_ms.append(s.timer(0))
        pcg_ms += s.timer(1)
        launches += s.timer(2)
        itd = executed_iters(s.stat(0), limit)
        itp = executed_iters(s.stat(1), limit)
        iters.append((itd, itp))
        # algorithmic bytes of one solve: setup 16 B/cell (read b, write x, r, s)
        # + 34 B per cell-iteration (FP32 x, r, s and the u8 operator row)
        bytes_pcg += ncell * (2 * 16 + 34 * (itd + itp))
    torch.cuda.synchronize()
    if args.profile_timed:
        torch.cuda.profiler.stop()
    clocks = sampler.stop()
    s.enable_timers(False)
    total_ms, work = combine_replicas(float(sum(step_ms)), work, dist, f"cuda:{local}")
    value = work / (total_ms / 1e3)

    # end to end through the C ABI with host-resident state: upload particles
    # and the carried grids, one substep, download them again
    e2e_steps = max(1, min(args.steps, 5))
    # host state in pinned memory, room for twice the particles
    cap = 2 * s.particle_count() + 1024

    def pinned(shape, dtype):
        return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()

    hp = {"bin_counts": pinned((s.bin_count(),), torch.int32), "pos": pinned((cap, 2), torch.float32),
          "vel": pinned((cap, 2), torch.float32), "visc": pinned((cap,), torch.float32),
          "dead": pinned((cap,), torch.uint8)}
    carried = ["u", "v", "material"]
    tdt = {"u": torch.float32, "v": torch.float32, "material": torch.int8}
    hg = {g: pinned(s.grid_shape(g), tdt[g]) for g in carried}
    snap_p = s.get_particles(out=hp)
    snap_g = {g: s.get_grid(g, out=hg[g]) for g in carried}
    h2d = sum(v.nbytes for k, v in snap_p.items() if k != "dead") + snap_p["dead"].nbytes
    h2d += sum(a.nbytes for a in snap_g.values())
    d2h = h2d
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_work = 0
    for _ in range(e2e_steps):
        s.set_particles(snap_p)
        for g, a in snap_g.items():
            s.set_grid(g, a)
        e2e_work += len(snap_p["pos"])
        s.set_dt(cfl_dt(s.max_particle_velocity(), p))
        s.step()
        snap_p = s.get_particles(out=hp)
        snap_g = {g: s.get_grid(g, out=hg[g]) for g in carried}
    e2e_s = time.perf_counter() - t0
    e2e_ms, e2e_work = combine_replicas(1e3 * e2e_s, e2e_work, dist, f"cuda:{local}")
    e2e_value = e2e_work / (e2e_ms / 1e3)

    peak, peak_kind = measured_peaks()
    achieved = bytes_pcg / (pcg_ms / 1e3) / 1e9 if pcg_ms > 0 else None
    n_pcg = 2 * args.steps
    cell_iters = sum(ncell * (a + b) for a, b in iters)
    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            cpu = run_cpu_sample(os.cpu_count() or 1, substeps=2, snapshot=cpu_start,
                                 warmup=args.warmup)
            cpu = {k: cpu[k] for k in CPU_KEYS if k in cpu}
        except Exception as e:  # reported, never fatal for the GPU line
            cpu = {"value": None, "unit": METRIC, "cores": 0, "kind": "port",
                   "sample": f"failed: {e}"}
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded dam-break scene)",
        "config": bench_config(args.warmup),
        "particles": int(work / args.steps),
        "pcg": "PCG+IPP FP32 vectors, float-pair reductions and scalars, reference stopping "
               "(limit 200, abs tol 1e-2 max-abs)",
        "l2": "flushed between steps (256 MiB write)",
        "parallelism": "replicas" if world > 1 else "single GPU",
        "pcg_cell_iter_per_s": cell_iters / (pcg_ms / 1e3) if pcg_ms > 0 else None,
        "pcg_iterations_per_step": [list(x) for x in iters],
        "step_latency_ms": {"p50": float(np.percentile(step_ms, 50)),
                            "p99": float(np.percentile(step_ms, 99))},
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
                "path": "fs_set_particles + fs_set_grid(u, v, material) + fs_step + "
                        "fs_get_particles + fs_get_grid, pinned host buffers"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "k_pcg_resident",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "traffic": PCG_TRAFFIC_BYTES if RES == 1024 else None,
                     "peak_source": peak_kind,
                     "bytes_model": "per solve 16 B/cell + 34 B/cell-iteration",
                     "launches": n_pcg, "avg_launch_ms": pcg_ms / n_pcg},
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    if rank == 0:
        try:
            line["fp64_check"] = fp64_check(s, sc, p)
        except Exception as e:  # reported, never fatal for the main line
            line["fp64_check"] = {"error": str(e)}
    s.close()
    if rank == 0 and world == 1 and not args.no_batch:
        # the plain single-scene path at a 1e-6 pressure residual: the same
        # scene in FS_PCG_SPEC mode (the figure the batched form divides by)
        try:
            line["spec_single"] = spec_single_measure(local, 5)
        except Exception as e:  # reported, never fatal for the main line
            line["spec_single"] = {"error": str(e)}
        # the mixed-precision configuration: one 2048^2 standalone solve
        try:
            line["poisson_2048"] = poisson_measure(2048, 1, 3)
        except Exception as e:  # reported, never fatal for the main line
            line["poisson_2048"] = {"error": str(e)}
    if rank == 0 and world == 1 and not args.no_batch:
        # the batched form of the same path beside the single-scene line: the
        # batched-scenes workload at its configured size, 256 scenes stepped
        # together, and 16 of them one at a time, both at a 1e-6 pressure
        # residual
        try:
            r = batch_measure(BATCH_SCENES, 2, 3, 16)
            bv = r["work"] / (r["total_ms"] / 1e3)
            ss = line.get("spec_single", {}).get("value")
            line["batch"] = {"workload": f"batch_{BATCH_SCENES}_scenes (sides 64-512, seeds "
                                         f"1000..{1000 + BATCH_SCENES - 1})",
                             "value": bv, "unit": METRIC, "frames": 3,
                             "vs_spec_single_1024": bv / ss if ss else None,
                             "ms_per_frame": r["total_ms"] / 3,
                             "single_scene": r["single"], "vs_single_scene": bv / r["single"],
                             "merged_solve_share": r["solve_ms"] / max(r["rounds_ms"], 1e-9),
                             "pcg": "FS_PCG_SPEC, 1e-6 true relative residual"}
        except Exception as e:  # reported, never fatal for the main line
            line["batch"] = {"error": str(e)}
    if rank == 0 and world == 1 and not args.no_batch:
        # the narrow-band variant of the same scene beside it (NBFlipSolver)
        try:
            r = nb_measure(RES, 3, 5, local, with_e2e=False)
            line["nbflip"] = {"workload": f"nb_dam_break_{RES}_obstacle (NBFlipSolver, 8 per cell, "
                                          "limit 1000, tolerance 1e-6)",
                              "value": r["work"] / (r["total_ms"] / 1e3), "unit": METRIC,
                              "ms_per_step": r["total_ms"] / 5, "steps": 5,
                              "cell_substeps_per_s": r["cells"] * 5 / (r["total_ms"] / 1e3),
                              "particles": int(r["work"] / 5)}
        except Exception as e:  # reported, never fatal for the main line
            line["nbflip"] = {"error": str(e)}
    if rank == 0 and world == 1 and not args.no_batch:
        # the serving loop on a short stretch of the request stream
        try:
            r = serve_measure(SERVE_SUBOBJECT_REQUESTS)
            line["serve"] = {"workload": f"serve_{r['requests']}_requests (Poisson 2000/s, "
                                         f"{r['scenes']} resident scenes of sides 64-1024, "
                                         "20 % standalone solves of sides 256-2048)",
                             "value": r["frame_work"] / r["elapsed_s"], "unit": METRIC,
                             "requests_per_s": r["requests_per_s"], "latency_ms": r["latency_ms"],
                             "worst_solve_rel_residual": r["worst_solve_rel_residual"],
                             "rounds": r["rounds"], "elapsed_s": r["elapsed_s"],
                             "pcg": "FS_PCG_SPEC, 1e-6 true relative residual"}
        except Exception as e:  # reported, never fatal for the main line
            line["serve"] = {"error": str(e)}
        # the device-resident request loop on solve requests
        try:
            r = serve_device_measure(SERVE_DEVICE_REQUESTS)
            line["serve_device"] = {
                "workload": f"serve_device_{r['requests']}_solves (Poisson 2000/s, sides 64-512, "
                            "masks of the Poisson case)",
                "value": r["requests_per_s"], "unit": "requests/s", "latency_ms": r["latency_ms"],
                "cell_iter_per_s": r["cell_iter_per_s"], "clusters": r["clusters"],
                "worst_rel_residual": r["worst_rel_residual"], "elapsed_s": r["elapsed_s"],
                "h2d_bytes": r["h2d_bytes"], "d2h_bytes": r["d2h_bytes"],
                "path": "fs_server_submit / fs_server_poll / fs_server_take: one persistent cluster-solve "
                        "launch fed from a ring in mapped pinned memory",
                "pcg": "FS_PCG_SPEC cluster solve, 1e-6 true relative residual"}
        except Exception as e:  # reported, never fatal for the main line
            line["serve_device"] = {"error": str(e)}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


NB_WARM_FRAMES = 4
BATCH_SCENES = 256
SERVE_SUBOBJECT_REQUESTS = 120
SERVE_DEVICE_REQUESTS = 400


def serve_device_measure(n_requests: int, rate: float = 2000.0, sides=(64, 512), slots: int = 256):
    """Serves n_requests spec-mode solve requests through the device-resident
    loop (fs_server_*): Poisson arrivals at `rate` per second
    (default_rng(19)), sides log-uniform in `sides`, the masks and
    right-hand sides of scenes.poisson_case.  The problems are built before
    the clock starts; a request is submitted at its arrival time (or when a
    slot frees), and completes when its result is back in host memory.
    Latencies run from arrival to that point."""
    import math
    from flipsolver2d_gb300 import gpu, scenes

    rng = np.random.default_rng(19)
    reqs, t = [], 0.0
    for _ in range(n_requests):
        t += rng.exponential(1.0 / rate)
        side = int(round(math.exp(rng.uniform(math.log(sides[0]), math.log(sides[1])))))
        side = max(sides[0], min(sides[1], side))
        m, b, dx = scenes.poisson_case(side, seed=int(rng.integers(1 << 30)))
        reqs.append({"arrival": t, "m": m, "b": b, "dx": dx})
    srv = gpu.Server(sides[1], sides[1], slots=slots)
    # warm-up: the first launch and its module load stay outside the clock
    w = [srv.submit(reqs[k]["m"], reqs[k]["b"], 1.0 / 30, 1000.0, reqs[k]["dx"]) for k in range(4)]
    while not all(srv.poll(x) for x in w):
        time.sleep(0.0002)
    for x in w:
        srv.take(x)
    pending, inflight, done = 0, {}, []
    t0 = time.perf_counter()
    while len(done) < len(reqs):
        now = time.perf_counter() - t0
        while pending < len(reqs) and reqs[pending]["arrival"] <= now:
            q = reqs[pending]
            try:
                inflight[srv.submit(q["m"], q["b"], 1.0 / 30, 1000.0, q["dx"])] = q
            except gpu.FsError as e:
                if e.status != 6:  # every slot busy: submit it after the next take
                    raise
                break
            pending += 1
        for tk in [x for x in inflight if srv.poll(x)]:
            it, x, rel = srv.take(tk)
            q = inflight.pop(tk)
            q.update(done=time.perf_counter() - t0, it=it, rel=rel)
            done.append(q)
        if now > 120.0:
            raise RuntimeError("device serving did not finish within 120 s")
    elapsed = time.perf_counter() - t0
    clusters = srv.clusters()
    srv.close()
    lat = [1e3 * (q["done"] - q["arrival"]) for q in done]
    return {
        "requests": len(done), "elapsed_s": elapsed, "requests_per_s": len(done) / elapsed,
        "latency_ms": {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))},
        "cell_iter_per_s": sum(q["m"].size * q["it"] for q in done) / elapsed,
        "worst_rel_residual": max(q["rel"] for q in done), "clusters": clusters,
        "h2d_bytes": sum(q["m"].nbytes + q["b"].nbytes for q in done),
        "d2h_bytes": sum(q["b"].nbytes for q in done),
    }


def nb_scene(res: int):
    from flipsolver2d_gb300 import scenes

    return scenes.nb_dam_break(res, seed=SEED, obstacle=True)


def nb_measure(res: int, warmup: int, steps: int, local: int = 0, with_e2e: bool = True,
               want_snapshot: bool = False):
    """NB-FLIP substeps of the narrow-band dam break at res^2 (FP32 PCG),
    device-timed like the FLIP line; e2e through the C ABI with the state a
    substep carries (particles, u, v, material, fluid SDF, viscosity, counts,
    engine state) uploaded and downloaded every step."""
    import torch

    from flipsolver2d_gb300 import gpu

    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")
    sc = nb_scene(res)
    p = sc.params
    s = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_FP32, device=local)
    for _ in range(NB_WARM_FRAMES):
        s.step_frame()

    def one_step():
        n = s.particle_count()
        s.set_dt(cfl_dt(s.max_particle_velocity(), p))
        s.step()
        return n

    for _ in range(warmup):
        one_step()
    s.enable_timers(True)
    torch.cuda.synchronize()
    work, step_ms, pcg_ms, launches, iters = 0, [], 0.0, 0.0, []
    stages = np.zeros(12)
    for _ in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        s.reset_timers()
        work += one_step()
        step_ms.append(s.timer(0))
        pcg_ms += s.timer(1)
        launches += s.timer(2)
        stages += np.array(s.stage_times())
        iters.append(executed_iters(s.stat(1), p.pcgIterLimit))
    s.enable_timers(False)
    out = {"work": work, "total_ms": float(sum(step_ms)), "pcg_ms": pcg_ms, "launches": launches,
           "cells": s.ni * s.nj, "pressure_iters": iters, "step_ms": step_ms,
           "stage_ms": (stages / steps).tolist()}
    if with_e2e:
        carried = ["u", "v", "material", "fluid_sdf", "viscosity", "particle_counts"]
        e2e_steps = max(1, min(steps, 5))
        cap = 2 * p.particlesPerCell * s.ni * s.nj

        def pinned(shape, dtype):
            return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()

        tdt = {np.float32: torch.float32, np.int8: torch.int8, np.int32: torch.int32}
        hp = {"bin_counts": pinned((s.bin_count(),), torch.int32), "pos": pinned((cap, 2), torch.float32),
              "vel": pinned((cap, 2), torch.float32), "visc": pinned((cap,), torch.float32),
              "dead": pinned((cap,), torch.uint8)}
        hg = {g: pinned(s.grid_shape(g), tdt[gpu.GRIDS[g][1]]) for g in carried}
        snap_p = s.get_particles(out=hp)
        snap_g = {g: s.get_grid(g, out=hg[g]) for g in carried}
        rng = s.get_rng()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_work, h2d = 0, 0
        for _ in range(e2e_steps):
            s.set_particles(snap_p)
            for g, a in snap_g.items():
                s.set_grid(g, a)
            s.set_rng(rng)
            h2d = sum(v.nbytes for v in snap_p.values()) + sum(a.nbytes for a in snap_g.values())
            e2e_work += len(snap_p["pos"])
            s.set_dt(cfl_dt(s.max_particle_velocity(), p))
            s.step()
            snap_p = s.get_particles(out=hp)
            snap_g = {g: s.get_grid(g, out=hg[g]) for g in carried}
            rng = s.get_rng()
        e2e_s = time.perf_counter() - t0
        out["e2e"] = {"value": e2e_work / e2e_s, "unit": METRIC, "h2d_bytes_per_step": int(h2d),
                      "d2h_bytes_per_step": int(h2d), "steps": e2e_steps,
                      "path": "fs_set_particles + fs_set_grid(u, v, material, fluid_sdf, "
                              "viscosity, particle_counts) + fs_set_rng_state + fs_step + the "
                              "matching gets, pinned host buffers"}
    if want_snapshot:
        # the state the CPU sample starts from (the oracle's snapshot layout)
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import fsoracle as fo

        snap = {"particles": s.get_particles(), "dt": s.dt, "rng": s.get_rng()}
        for g in fo.STATE_GRIDS + fo.NB_GRIDS:
            snap[g] = s.get_grid(g)
        out["snapshot"] = snap
    s.close()
    return out


def nb_cpu_sample(res: int, threads: int, substeps: int = 1, snapshot=None):
    """The CPU oracle on the NB-FLIP workload: `substeps` timed substeps
    from `snapshot` (the GPU's state after the warm frames; stepping the warm
    frames on the CPU would take minutes), else from the oracle's own warm
    frames."""
    os.environ["FSO_HOST_THREADS"] = str(threads)
    os.environ.setdefault("FSO_REF_THREADS", str(threads))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build as oracle_build

    oracle_build.build_port()
    import fsoracle as fo

    kind = "reference" if fo.available("ref") else "port"
    sc = nb_scene(res)
    o = fo.OracleSolver(sc, "ref" if kind == "reference" else "port")
    o.first_frame_init()
    if snapshot is not None:
        o.restore(snapshot)
    else:
        for _ in range(NB_WARM_FRAMES):
            o.step_frame()
    work, t_total, times = 0, 0.0, []
    for _ in range(substeps):
        n = o.particle_count()
        o.set_dt(cfl_dt(o.max_particle_velocity(), sc.params))
        t0 = time.perf_counter()
        o.step()
        dt = time.perf_counter() - t0
        times.append(dt)
        t_total += dt
        work += n
    o.close()
    return {"value": work / t_total, "unit": METRIC, "cores": threads, "kind": kind,
            "sample": f"{substeps} substep(s) of nb_dam_break_{res}_obstacle from "
                      f"{'the GPU state' if snapshot is not None else 'the oracle state'} after "
                      f"{NB_WARM_FRAMES} frames ({work} particle-substeps, {t_total:.1f} s)",
            "step_s": times}


def nbflip_arm(args):
    """NB-FLIP (NBFlipSolver) substeps of the narrow-band dam break."""
    from flipsolver2d_gb300 import build

    build.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    sampler = ClockSampler(local)
    sampler.start()
    r = nb_measure(args.res, args.warmup, args.steps, local, want_snapshot=not args.no_cpu)
    clocks = sampler.stop()
    value = r["work"] / (r["total_ms"] / 1e3)
    cpu = None
    if not args.no_cpu:
        try:
            cpu = nb_cpu_sample(args.res, os.cpu_count() or 1, 1, r.get("snapshot"))
            cpu = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
        except Exception as e:  # reported, never fatal for the GPU line
            cpu = {"value": None, "unit": METRIC, "cores": 0, "kind": "port", "sample": f"failed: {e}"}
    peak, peak_kind = measured_peaks()
    cell_iters = sum(r["cells"] * it for it in r["pressure_iters"])
    bytes_pcg = sum(r["cells"] * (16 + 34 * it) for it in r["pressure_iters"])
    achieved = bytes_pcg / (r["pcg_ms"] / 1e3) / 1e9 if r["pcg_ms"] > 0 else None
    names = ["advection", "decomposition", "density", "rebin", "particle_to_grid", "grid_update",
             "after_transfer", "pressure", "viscosity", "repressure", "particle_update", "reseed"]
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["total_ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded NB-FLIP dam-break scene)",
        "config": {"workload": f"nb_dam_break_{args.res}_obstacle", "solver": "NBFlipSolver",
                   "grid": args.res, "seed": SEED, "particles": int(r["work"] / args.steps),
                   "pcg": "PCG+IPP FP32, reference stopping (limit 1000, abs tol 1e-6 max-abs)",
                   "l2": "flushed between steps (256 MiB write)", "warm_frames": NB_WARM_FRAMES},
        "cell_substeps_per_s": r["cells"] * args.steps / (r["total_ms"] / 1e3),
        "pcg_cell_iter_per_s": cell_iters / (r["pcg_ms"] / 1e3) if r["pcg_ms"] > 0 else None,
        "pressure_iterations_per_step": r["pressure_iters"],
        "stage_ms_per_step": {n: round(v, 4) for n, v in zip(names, r["stage_ms"]) if v > 0},
        "e2e": r["e2e"], "gpu_launches": int(r["launches"]),
        "roofline": {"bound": "hbm", "kernel": "k_pcg_resident", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                     "traffic": None, "peak_source": peak_kind,
                     "bytes_model": "per solve 16 B/cell + 34 B/cell-iteration",
                     "launches": args.steps, "avg_launch_ms": r["pcg_ms"] / args.steps},
        "cpu_baseline": cpu, "clocks": clocks,
    }
    print(json.dumps(line))
    return 0


def poisson_arm(args):
    """Standalone mixed-precision pressure solves (--poisson N): the spec-mode
    solve to a 1e-6 true relative residual on a seeded 55 %-fluid star mask
    with the divergence of N(0, 1) face velocities as right-hand side.  Each
    step is one whole solve through fs_pcg_solve_spec with host arrays, so the
    time includes the uploads and the download."""
    from flipsolver2d_gb300 import build, gpu, scenes

    build.build()
    n = args.poisson
    m, b, dx = scenes.poisson_case(n, seed=0)
    for _ in range(args.warmup):
        gpu.pcg_solve_spec(m, b, 1.0 / 30, 1000.0, dx, 1e-6)
    times, iters, rr = [], [], 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        it, x, rr = gpu.pcg_solve_spec(m, b, 1.0 / 30, 1000.0, dx, 1e-6)
        times.append(time.perf_counter() - t0)
        iters.append(it)
    total = sum(times)
    cells = n * n
    line = {"metric": "pcg-cell-iter/s", "value": cells * sum(iters) / total, "unit": "cell-iter/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded star mask, N(0,1) face velocities)",
            "config": {"workload": f"poisson_{n}_spec", "grid": n, "rel_tol": 1e-6,
                       "solver": "FP32 PCG, textbook IPP, FP64 refinement"},
            "inner_iterations": iters, "rel_residual": rr,
            "e2e": {"value": cells * sum(iters) / total, "unit": "cell-iter/s",
                    "h2d_bytes_per_step": int(m.nbytes + b.nbytes), "d2h_bytes_per_step": int(b.nbytes)}}
    print(json.dumps(line))
    return 0


BATCH_SIDES = (64, 96, 128, 192, 256, 384, 512)


def batch_scenes(n: int):
    """The batched-scenes workload: scene k has its grid side drawn uniformly
    from BATCH_SIDES with default_rng(1000 + k) and the randomised layout of
    scenes.random_scene (fluid box corners in [0.1, 0.9] m, 1-3 convex solids
    of 4-8 vertices, 4 particles per cell) from seed 1000 + k."""
    from flipsolver2d_gb300 import scenes

    out = []
    for k in range(n):
        side = BATCH_SIDES[int(np.random.default_rng(1000 + k).integers(0, len(BATCH_SIDES)))]
        out.append(scenes.random_scene(side, 1000 + k))
    return out


def batch_measure(n: int, warm: int, frames: int, single_sample: int):
    """Steps `n` scenes of the batched workload together: `warm` untimed
    frames, then `frames` timed ones run pipelined (fs_batch_run_frames: a
    scene whose frame ends starts its next one in the next round; host wall
    clock around the blocking call), then `single_sample` of the same scenes
    one at a time through fs_step_frame.  The work is the particles each
    scene holds when the timed frames start times the substeps it runs.
    Returns a dict of the figures."""
    import torch
    from flipsolver2d_gb300 import gpu

    scs = batch_scenes(n)
    # the autotuner picks each grid shape's cluster size for throughput
    # before any handle exists, so every handle of a shape shares the plan
    plans = {}
    for sc in scs:
        _, ni, nj = sc.params.grid()
        if (ni, nj) not in plans:
            plans[(ni, nj)] = gpu.cluster_autotune(ni, nj, 0)
    hs = [gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_SPEC) for sc in scs]
    b = gpu.Batch(hs)
    b.run_frames(warm)
    hs[0].reset_timers()
    b.timer(3)
    counts = [g.particle_count() for g in hs]
    sub0 = [g.stat(5) for g in hs]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.run_frames(frames)  # returns after the device finished
    total_ms = 1e3 * (time.perf_counter() - t0)
    subs = [g.stat(5) - a for g, a in zip(hs, sub0)]
    rounds = b.timer(2)
    out = {"work": sum(c * k for c, k in zip(counts, subs)), "total_ms": total_ms,
           "cells": sum(g.ni * g.nj * k for g, k in zip(hs, subs)),
           # per round the dt table (4 B per scene) and the systems of the two
           # merged solves (72 B each) go up, the scalars (32 B each) come down
           "h2d": 4 * len(hs) * rounds + 2 * 72 * sum(subs), "d2h": 32 * sum(subs),
           "launches": hs[0].timer(2), "solve_ms": b.timer(0), "rounds_ms": b.timer(1),
           "rounds": rounds, "total_cells": int(sum(g.ni * g.nj for g in hs)),
           "particles": int(sum(counts)),
           "plans": {f"{k[0]}x{k[1]}": {"ctas_per_cluster": v[0], "us_per_iteration": round(v[1], 2)}
                     for k, v in sorted(plans.items())}}
    b.close()
    m = min(len(hs), single_sample)
    single_work, single_s = 0, 0.0
    for g in hs[:m]:
        k = g.particle_count()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.step_frame()
        single_s += time.perf_counter() - t0
        single_work += k * g.stat(2)
    out["single"] = single_work / single_s if single_s > 0 else None
    out["single_scenes"] = m
    for g in hs:
        g.close()
    return out


def batch_arm(args):
    """Batched scenes (--batch N): N independent scenes in FS_PCG_SPEC mode
    (every density and pressure solve to a 1e-6 true relative residual)
    advanced together by fs_batch_step_frame.  A step is one frame of every
    scene; the work is the sum over scenes of live particles x substeps.
    The same scenes stepped one at a time through fs_step_frame (same mode,
    same residual) give the single-scene figure beside it."""
    import torch
    from flipsolver2d_gb300 import build

    build.build()
    torch.cuda.set_device(0)
    sampler = ClockSampler(0)
    sampler.start()
    r = batch_measure(args.batch, args.warmup, args.steps, args.single_sample)
    clocks = sampler.stop()
    total_s = r["total_ms"] / 1e3
    value = r["work"] / total_s
    single = r["single"]
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["total_ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded random scenes)",
        "config": {"workload": f"batch_{args.batch}_scenes", "sides": list(BATCH_SIDES),
                   "scene_seeds": f"1000..{1000 + args.batch - 1}", "cells": r["total_cells"],
                   "particles": r["particles"],
                   "pcg": "FS_PCG_SPEC: FP32 PCG, textbook IPP, FP64 refinement to 1e-6, "
                          "one thread-block cluster per system",
                   "l2": "working set of all scenes far above L2",
                   "step": "one frame of every scene, the frames run pipelined (fs_batch_run_frames)",
                   "autotuned_plans": r["plans"],
                   "parallelism": "single GPU"},
        "cell_substeps_per_s": r["cells"] / total_s,
        "merged_solves": {"device_ms_per_step": r["solve_ms"] / args.steps,
                          "rounds_ms_per_step": r["rounds_ms"] / args.steps,
                          "rounds_per_step": r["rounds"] / args.steps},
        "single_scene": {"value": single, "unit": METRIC, "scenes": r["single_scenes"],
                         "path": "fs_step_frame per scene, FS_PCG_SPEC, one scene at a time"},
        "vs_single_scene": (value / single) if single else None,
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": int(r["h2d"] / args.steps),
                "d2h_bytes_per_step": int(r["d2h"] / args.steps),
                "path": "value itself is host-timed around the public call fs_batch_step_frame on "
                        "resident scenes; per round the dt table and solve lists go up and the "
                        "scalars come down"},
        "gpu_launches": int(r["launches"]),
        "clocks": clocks,
    }
    print(json.dumps(line))
    return 0


def solve_batch_arm(args):
    """Batched standalone solves (--solve-batch N): N pressure systems of the
    mixed-precision configuration (scenes.poisson_case, side --res, seeds
    0..N-1) submitted to a batch and solved in one round, i.e. one
    k_pcg_cluster launch per plan, to a 1e-6 true relative residual.  The
    uploads happen at submission, outside the timed region; the device time
    of the merged launch comes from CUDA events on the batch's solve stream.
    `value` is cell-iterations per second of device time."""
    import torch
    from flipsolver2d_gb300 import build, gpu, scenes

    build.build()
    torch.cuda.set_device(0)
    n, side = args.solve_batch, args.res
    probs = []
    for k in range(n):
        m, b, dx = scenes.poisson_case(side, seed=k)
        probs.append((m, b, 1.0 / 30, 1000.0, dx))
    bt = gpu.Batch()

    def one_round():
        tickets = [bt.submit_solve(*p) for p in probs]
        bt.timer(3)
        bt.round()
        ms = bt.timer(0)
        res = [bt.take_solve(t) for t in tickets]
        return ms, res

    for _ in range(args.warmup):
        one_round()
    sampler = ClockSampler(0)
    sampler.start()
    total_ms, cell_iters, worst = 0.0, 0, 0.0
    iters = []
    for _ in range(args.steps):
        ms, res = one_round()
        total_ms += ms
        cell_iters += sum(side * side * r[0] for r in res)
        worst = max(worst, max(r[2] for r in res))
        iters.append([r[0] for r in res])
    clocks = sampler.stop()
    peak, peak_kind = measured_peaks()
    achieved = 34.0 * cell_iters / (total_ms / 1e3) / 1e9
    line = {
        "metric": "pcg-cell-iter/s", "value": cell_iters / (total_ms / 1e3), "unit": "cell-iter/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded star masks, N(0,1) face velocities)",
        "config": {"workload": f"solve_batch_{n}x{side}", "systems": n, "grid": side, "rel_tol": 1e-6,
                   "solver": "k_pcg_cluster: FP32 PCG, textbook IPP, FP64 refinement, one "
                             "thread-block cluster per system",
                   "l2": "vectors on chip; b, x and the operator bytes stream once per solve",
                   "parallelism": "single GPU"},
        "inner_iterations": iters[-1][:8], "worst_rel_residual": worst,
        "e2e": {"value": None, "unit": "cell-iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "path": "device time only; fs_pcg_solve_batch is the host-array call"},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "kernel": "k_pcg_cluster", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": None, "peak_source": peak_kind,
                     "bytes_model": "34 B/cell-iteration (the HBM-streaming model; the kernel keeps "
                                    "its vectors on chip, so this is a speed figure)"},
        "clocks": clocks,
    }
    print(json.dumps(line))
    bt.close()
    return 0


def serve_measure(n_requests: int, pool: int = 32):
    """Serves n_requests of the seeded request stream: Poisson arrivals at
    2000 per second (default_rng(9)), 80 % frame requests to `pool` resident
    scenes with sides log-uniform in [64, 1024] and 20 % standalone solves of
    sides log-uniform in [256, 2048], by continuous batching under a 150 GB
    device-memory budget (flipsolver2d_gb300/serve.py).  Every scene first
    gets one warm-up frame, so its creation, seeding and graph capture are
    outside the measurement.  Latencies run from arrival to completion."""
    import torch
    from flipsolver2d_gb300 import serve

    specs, reqs = serve.serving_workload(n_requests, rate=2000.0, seed=9, pool=pool,
                                         frame_sides=(64, 1024), solve_sides=(256, 2048))
    srv = serve.Server(budget_bytes=150e9)
    for k, sc in specs.items():
        srv.register_scene(k, sc)
    warm = [serve.Request("frame", 0.0, scene=k) for k in specs]
    srv.run(warm)
    srv.finished = []
    srv.rounds = 0
    srv.batch.timer(3)
    sampler = ClockSampler(0)
    sampler.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    done = srv.run(reqs)
    elapsed = time.perf_counter() - t0
    clocks = sampler.stop()
    out = {
        "requests": len(reqs), "warm": len(warm), "scenes": len(specs), "elapsed_s": elapsed,
        "frame_work": sum(r.work for r in done if r.kind == "frame"),
        "solve_work": sum(r.work for r in done if r.kind == "solve"),
        "requests_per_s": len(done) / elapsed,
        "latency_ms": serve.latency_summary(done),
        "rounds": srv.rounds, "merged_solve_device_ms": srv.batch.timer(0),
        "worst_solve_rel_residual": max((r.result[2] for r in done if r.kind == "solve"), default=None),
        "h2d_bytes": sum(r.problem[0].nbytes + r.problem[1].nbytes for r in done if r.kind == "solve"),
        "d2h_bytes": sum(r.problem[1].nbytes for r in done if r.kind == "solve"),
        "clocks": clocks,
    }
    srv.close()
    return out


def serve_arm(args):
    """Serving loop (--serve R): R requests of the seeded request stream
    (serve_measure).  `value` is frame work served per second of the run
    (particle-substeps/s)."""
    import torch
    from flipsolver2d_gb300 import build

    build.build()
    torch.cuda.set_device(0)
    r = serve_measure(args.serve)
    n = r["requests"]
    line = {
        "metric": METRIC, "value": r["frame_work"] / r["elapsed_s"], "unit": METRIC, "n_gpus": 1,
        "steps": n, "warmup": r["warm"], "ms_per_step": 1e3 * r["elapsed_s"] / n,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded request stream, random scenes and star masks)",
        "config": {"workload": f"serve_{n}_requests", "rate_per_s": 2000.0, "seed": 9,
                   "scenes": r["scenes"], "frame_sides": [64, 1024], "solve_sides": [256, 2048],
                   "solve_fraction": 0.2, "budget_bytes": 150e9,
                   "pcg": "FS_PCG_SPEC, 1e-6 true relative residual",
                   "step": "one request", "parallelism": "single GPU"},
        "requests_per_s": r["requests_per_s"],
        "solve_cell_iter_per_s": r["solve_work"] / r["elapsed_s"],
        "latency_ms": r["latency_ms"],
        "rounds": r["rounds"], "merged_solve_device_ms": r["merged_solve_device_ms"],
        "worst_solve_rel_residual": r["worst_solve_rel_residual"],
        "e2e": {"value": r["frame_work"] / r["elapsed_s"], "unit": METRIC,
                "h2d_bytes_per_step": int(r["h2d_bytes"] / n), "d2h_bytes_per_step": int(r["d2h_bytes"] / n),
                "path": "value itself is host-timed around the serving loop on the public API"},
        "clocks": r["clocks"],
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the batched-scenes figure of the default line")
    ap.add_argument("--res", type=int, default=RES, help="grid side of the dam break (default 1024)")
    ap.add_argument("--poisson", type=int, default=0,
                    help="time standalone spec-mode pressure solves on an N x N grid instead")
    ap.add_argument("--batch", type=int, default=0,
                    help="time N scenes stepped together (fs_batch) instead")
    ap.add_argument("--solve-batch", type=int, default=0,
                    help="time N standalone systems of side --res solved in one merged launch")
    ap.add_argument("--nbflip", action="store_true",
                    help="NB-FLIP (NBFlipSolver) substeps of the narrow-band dam break at --res")
    ap.add_argument("--serve", type=int, default=0,
                    help="serve R requests of the seeded request stream instead")
    ap.add_argument("--profile-timed", action="store_true",
                    help="bracket the timed substeps with cudaProfilerStart/Stop, for "
                         "ncu --profile-from-start off")
    ap.add_argument("--single-sample", type=int, default=32,
                    help="scenes stepped one at a time for the single-scene figure of --batch")
    args = ap.parse_args()
    if args.solve_batch and "--res" not in sys.argv:
        args.res = 128
    set_resolution(args.res)
    if args.warmup < 3:
        args.warmup = 3
    if args.poisson:
        return poisson_arm(args)
    if args.batch:
        return batch_arm(args)
    if args.serve:
        return serve_arm(args)
    if args.solve_batch:
        return solve_batch_arm(args)
    if args.nbflip:
        return nbflip_arm(args)
    if args.impl == "reference":
        return reference_arm(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
