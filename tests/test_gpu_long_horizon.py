"""Long runs of the plain dam break at 128^2 (4 particles per cell, seed 42):
60 frames on the GPU, in the FP32 production mode and the FP64 parity mode,
against the oracle port (oracle/fsoracle.c, pinned bit for bit to the
reference build), compared statistically frame by frame: particle count,
kinetic energy (sum of |v|^2 over particles) and fluid volume (cells marked
FLUID).

The reference's own dynamics are chaotic at this size.  An ensemble of oracle
runs, the unperturbed one and ENSEMBLE - 1 runs whose particle velocities
were moved by one ulp (every 97th particle, a different offset each) after
the first frame, measures that: by frame 50 a one-ulp change moves the
particle count by about 40 % and the kinetic energy by more than 100 %.  So
the bars are:

* early frames (2-6, before the trajectories separate): the GPU's particle
  count and fluid volume within EARLY_FACTOR times the ensemble's largest
  deviation from the unperturbed run, plus EARLY_FLOOR relative.  The
  kinetic energy is left to the mean bar: a one-ulp perturbation moves it by
  up to 40 % as early as frame 5, so a per-frame bar would need a far larger
  ensemble to mean anything;
* the whole run: the GPU's mean over frames 20-60 of each statistic within
  MEAN_SIGMAS ensemble standard deviations (of the members' own means) of the
  ensemble mean, plus MEAN_FLOOR relative.
"""
import numpy as np
import pytest

import fsoracle as fo
from flipsolver2d_gb300 import gpu, scenes

from conftest import POOL_THREADS

pytestmark = pytest.mark.gpu

FRAMES = 60
ENSEMBLE = 4
EARLY = range(1, 6)       # frame indices 1..5 (frames 2-6)
LATE = slice(19, FRAMES)  # frames 20-60
EARLY_FACTOR, EARLY_FLOOR = 3.0, 0.01
MEAN_SIGMAS, MEAN_FLOOR = 3.0, 0.05
NAMES = ("particles", "kinetic energy", "fluid cells")
EARLY_STATS = (0, 2)  # particle count and fluid volume


def stats(particles, material):
    v = particles["vel"].astype(np.float64)
    return (len(particles["pos"]), float(np.sum(v * v)), int(np.sum((material & 0x40) != 0)))


def oracle_run(member):
    o = fo.OracleSolver(scenes.dam_break(128, seed=42), "port")
    out = []
    for f in range(FRAMES):
        o.step_frame()
        if f == 0 and member > 0:
            p = o.get_particles()
            v = p["vel"].copy()
            v[member::97] = np.nextafter(v[member::97], np.float32(np.inf))
            o.set_particles(dict(p, vel=v))
        out.append(stats(o.get_particles(), o.get_grid("material")))
    o.close()
    return np.array(out, np.float64)


def gpu_run(precision):
    g = gpu.GpuFlipSolver(scenes.dam_break(128, seed=42), precision=precision, pool_threads=POOL_THREADS)
    out = []
    for _ in range(FRAMES):
        g.step_frame()
        out.append(stats(g.get_particles(), g.get_grid("material")))
    g.close()
    return np.array(out, np.float64)


@pytest.fixture(scope="module")
def ensemble(port_lib):
    return np.stack([oracle_run(m) for m in range(ENSEMBLE)])


@pytest.mark.parametrize("precision", [gpu.FS_PCG_FP32, gpu.FS_PCG_FP64])
def test_c1_sixty_frames_statistics(gpu_lib, ensemble, precision):
    g = gpu_run(precision)
    base = ensemble[0]
    spread = np.max(np.abs(ensemble[1:] - base), axis=0)  # per frame, per statistic
    tag = "FP32" if precision == gpu.FS_PCG_FP32 else "FP64"
    for f in EARLY:
        print(f"\n{tag} frame {f + 1}: GPU {g[f].tolist()} oracle {base[f].tolist()} "
              f"ensemble spread {spread[f].tolist()}")
        for k in EARLY_STATS:
            bar = EARLY_FACTOR * spread[f, k] + EARLY_FLOOR * abs(base[f, k])
            dev = abs(g[f, k] - base[f, k])
            assert dev <= bar, f"{tag} frame {f + 1} {NAMES[k]}: {g[f, k]} vs oracle {base[f, k]} (bar {bar})"
    member_means = ensemble[:, LATE, :].mean(axis=1)  # ENSEMBLE x 3
    mu, sd = member_means.mean(axis=0), member_means.std(axis=0, ddof=1)
    gm = g[LATE].mean(axis=0)
    for k, name in enumerate(NAMES):
        bar = MEAN_SIGMAS * sd[k] + MEAN_FLOOR * abs(mu[k])
        print(f"\n{tag} {name}: GPU mean over frames 20-60 {gm[k]:.4g}, ensemble {mu[k]:.4g} "
              f"+- {sd[k]:.3g} (bar {bar:.3g}); frame 60 {g[-1, k]:.4g} vs {base[-1, k]:.4g}")
        assert abs(gm[k] - mu[k]) <= bar, f"{tag} {name}"
