"""NB-FLIP (NBFlipSolver, nbflipsolver.cpp) on the GPU against the CPU oracle
(oracle/fsoracle.c, pinned bit for bit to the reference in test_oracle.py).

Bar, as for the FLIP substep (test_gpu_parity.py):
  * bit-exact: first-frame SDF, materials and engine state; narrow-band
    pruning, semi-Lagrangian grids, P2G with NB-FLIP's centred weights, the
    outside and inside level sets, the grid combination, materials, body
    forces, friction, G2P, counting, and the band reseeding (positions,
    storage order, viscosities, engine state) -- each stage fed the same
    snapshot;
  * PCG in FP64 mode: same iteration count, relative-L2 <= 1e-9 on the
    pressure (the dot products sum in another order);
  * whole frames in FP64 mode: the oracle's trajectory within 1e-3 cells.
"""
import numpy as np
import pytest

import fsoracle as fo
from flipsolver2d_gb300 import gpu, scenes

from conftest import POOL_THREADS
from test_gpu_parity import assert_grid_equal, assert_particles_equal, rel_l2

pytestmark = pytest.mark.gpu

SCENES = {
    "nb_dam48_obstacle": lambda: scenes.nb_dam_break(48, seed=7, obstacle=True),
    "nb_dam61": lambda: scenes.nb_dam_break(61, seed=2),
}

STATE = ["material", "fluid_sdf", "u", "v", "u_valid", "v_valid", "saved_u", "saved_v",
         "viscosity", "known_centered", "particle_counts", "div_control"] + gpu.NB_GRIDS


@pytest.fixture(params=sorted(SCENES))
def scene(request, port_lib, gpu_lib):
    return SCENES[request.param]()


def warm(scene, frames):
    o = fo.OracleSolver(scene, "port")
    for _ in range(frames):
        o.step_frame()
    return o


def same_all(o, g, what, skip=()):
    assert_particles_equal(o.get_particles(), g.get_particles(), what=what)
    for name in STATE:
        if name not in skip:
            assert_grid_equal(o, g, name, what)
    assert np.array_equal(o.get_rng(), g.get_rng()), f"{what}: engine state"


def test_first_frame_init(scene):
    o = fo.OracleSolver(scene, "port")
    g = gpu.GpuFlipSolver(scene, pool_threads=POOL_THREADS)
    o.first_frame_init()
    g.first_frame_init()
    assert g.particle_count() == o.particle_count() == 0
    for name in ["material", "solid_sdf", "solid_id", "fluid_sdf", "viscosity", "particle_counts"]:
        assert_grid_equal(o, g, name, "first frame")
    assert np.array_equal(o.get_rng(), g.get_rng())


def test_stages_from_identical_snapshots(scene):
    """Every stage of NBFlipSolver::step in its order, both sides continuing
    from the same state; the state is re-synchronised after the projection."""
    o = warm(scene, 4)
    assert o.particle_count() > 0
    o.set_dt(o.dt * 0.9)
    g = gpu.GpuFlipSolver(scene, precision=gpu.FS_PCG_FP64, pool_threads=POOL_THREADS)
    g.restore(o.snapshot())
    same_all(o, g, "restore")

    o.stage(fo.ADVECT)
    g.stage(gpu.ADVECT)
    assert_particles_equal(o.get_particles(), g.get_particles(), what="advect + narrow band")
    for name in gpu.NB_GRIDS:
        assert_grid_equal(o, g, name, "semi-Lagrangian advection")
    o.stage(fo.REBIN)
    g.stage(gpu.REBIN)
    same_all(o, g, "narrow band + rebin")
    o.stage(fo.P2G)
    g.stage(gpu.P2G)  # fused with updateSdf
    same_all(o, g, "p2g", skip=("fluid_sdf",))
    for s in (fo.VEL_EXTRAP, fo.SAVE_GRID, fo.SDF):
        o.stage(s)
        g.stage(s)
    same_all(o, g, "extrapolation, saved grid, SDF")
    o.stage(fo.LEVELSET_OUTSIDE)
    g.stage(gpu.LEVELSET_OUTSIDE)
    same_all(o, g, "outside level set")
    o.stage(fo.AFTER_TRANSFER)
    g.stage(gpu.AFTER_TRANSFER)
    same_all(o, g, "combination")
    for s in (fo.LEVELSET, fo.MATERIALS, fo.BODY_FORCES, fo.DECOMPOSITION):
        o.stage(s)
        g.stage(s)
        same_all(o, g, f"stage {s}")
    o.stage(fo.PROJECT)
    g.stage(gpu.PROJECT)
    assert o.stat(1) == g.stat(1)
    assert rel_l2(g.get_grid("pressure"), o.get_grid("pressure")) <= 1e-9
    # continue bit for bit from the oracle's projected state
    g.restore(o.snapshot())
    for s in (fo.FRICTION, fo.VEL_EXTRAP, fo.G2P, fo.COUNT, fo.RESEED):
        o.stage(s)
        g.stage(s)
        same_all(o, g, f"stage {s}")
    assert g.particle_count() > 0


def _untemper(y):
    """Inverse of MT19937's output tempering (for crafting engine states)."""
    y = int(y)
    y ^= y >> 18
    y ^= (y << 15) & 0xEFC60000
    t = y
    for _ in range(5):
        t = y ^ ((t << 7) & 0x9D2C5680)
    y = t & 0xFFFFFFFF
    t = y
    for _ in range(3):
        t = y ^ (t >> 11)
    return t & 0xFFFFFFFF


def _temper(y):
    y ^= y >> 11
    y ^= (y << 7) & 0x9D2C5680
    y ^= (y << 15) & 0xEFC60000
    y ^= y >> 18
    return y & 0xFFFFFFFF


def test_untemper_inverts_temper():
    rng = np.random.default_rng(0)
    for w in rng.integers(0, 2**32, size=200, dtype=np.uint64):
        assert _temper(_untemper(int(w))) == int(w)


@pytest.mark.parametrize("mode", ["round_up", "mixed"])
def test_reseed_with_crafted_draws(port_lib, gpu_lib, mode):
    """Reseeding with an engine state whose next 624 words are chosen: words
    near 2^32 make i + U(0,1) round up into the next cell, so candidates
    leave their cell's bin and the reference's viscosity store through the
    cell's bin (nbflipsolver.cpp:190-194) overwrites other particles.  Both
    sides must agree on every particle and on the engine state."""
    sc = scenes.nb_dam_break(48, seed=7, obstacle=True)
    o = warm(sc, 4)
    o.stage(fo.ADVECT)
    for s in fo.NB_STEP_STAGES[1:-1]:
        o.stage(s)
    rng = np.random.default_rng(11)
    words = np.full(624, 0xFFFFFFFF, np.uint64)
    if mode == "mixed":
        words = np.where(rng.random(624) < 0.5, words,
                         rng.integers(0, 2**32, size=624, dtype=np.uint64))
    st = np.zeros(625, np.uint32)
    st[:624] = [_untemper(int(w)) for w in words]
    st[624] = 0
    o.set_rng(st)
    g = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_FP64, pool_threads=POOL_THREADS)
    g.restore(o.snapshot())
    before = o.particle_count()
    o.stage(fo.RESEED)
    g.stage(gpu.RESEED)
    same_all(o, g, f"crafted reseed ({mode})")
    assert o.particle_count() > before


def test_full_frames_fp64(scene):
    """Whole NB-FLIP frames in FP64-PCG mode follow the oracle: same
    substeps and particle count, positions within 1e-3 cells, engine states
    equal (the same draws were taken)."""
    o = fo.OracleSolver(scene, "port")
    g = gpu.GpuFlipSolver(scene, precision=gpu.FS_PCG_FP64, pool_threads=POOL_THREADS)
    for f in range(6):
        o.step_frame()
        g.step_frame()
        assert o.stat(2) == g.stat(2), f"frame {f}: substeps"
        a, b = o.get_particles(), g.get_particles()
        assert a["pos"].shape == b["pos"].shape, f"frame {f}: particle count"
        if len(a["pos"]):
            assert np.max(np.abs(a["pos"] - b["pos"])) < 1e-3, f"frame {f}"
        assert np.array_equal(o.get_rng(), g.get_rng()), f"frame {f}: engine state"
        m = np.mean(o.get_grid("material") == g.get_grid("material"))
        assert m >= 0.999, f"frame {f}: material agreement {m}"


def test_full_frames_fp32(scene):
    """FP32-PCG production mode: the trajectory stays close to the FP64
    oracle's (particle count within 2 %, materials on >= 98 % of cells)."""
    o = fo.OracleSolver(scene, "port")
    g = gpu.GpuFlipSolver(scene, precision=gpu.FS_PCG_FP32, pool_threads=POOL_THREADS)
    for _ in range(4):
        o.step_frame()
        g.step_frame()
    na, nb = o.particle_count(), g.particle_count()
    assert abs(na - nb) <= max(4, na // 50)
    m = np.mean(o.get_grid("material") == g.get_grid("material"))
    assert m >= 0.98


def test_rng_state_roundtrip_and_batch_refusal(gpu_lib):
    sc = scenes.nb_dam_break(32, seed=1)
    g = gpu.GpuFlipSolver(sc)
    st = g.get_rng()
    assert st[624] == 624  # freshly seeded: the next draw regenerates
    st2 = st.copy()
    st2[624] = 17
    g.set_rng(st2)
    assert np.array_equal(g.get_rng(), st2)
    with pytest.raises(gpu.FsError):
        gpu.Batch([g])
    f = gpu.GpuFlipSolver(scenes.dam_break(32, seed=1))
    fs = f.get_rng()
    assert fs[624] == 624 and fs[0] == 1  # std::mt19937(1) before any draw


@pytest.mark.parametrize("shape", [(900, 1000), (1024, 1024)])
def test_level_sets_on_large_grids(port_lib, gpu_lib, shape):
    """The inside and outside level sets at sizes where the 86 x 86 tiles
    (one wave a pass) are used: a synthetic field with a particle-SDF-like
    band, deep unknown regions (values above NI * NJ) and fluid pockets,
    bit-exact against the oracle's FIFO BFS."""
    ni, nj = shape
    sc = scenes.nb_dam_break(max(ni, nj), seed=4)
    sc.params.domainSizeI, sc.params.domainSizeJ = ni / max(ni, nj), nj / max(ni, nj)
    o = fo.OracleSolver(sc, "port")
    g = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_FP64, pool_threads=POOL_THREADS)
    assert (o.ni, o.nj) == (g.ni, g.nj) == (ni, nj)
    rng = np.random.default_rng(ni)
    ii, jj = np.meshgrid(np.arange(ni), np.arange(nj), indexing="ij")
    sdf = np.full((ni, nj), 1.8446743e19, np.float32)  # no particle nearby
    for _ in range(6):  # rings of known values around random centres
        ci, cj, r = rng.uniform(0, ni), rng.uniform(0, nj), rng.uniform(20, 200)
        d = np.sqrt((ii - ci) ** 2 + (jj - cj) ** 2) - r
        band = np.abs(d) < 2.5
        sdf[band] = np.minimum(sdf[band], (d[band] * 0.7).astype(np.float32))
    for stage, field in ((fo.LEVELSET_OUTSIDE, sdf),
                         (fo.LEVELSET, np.where(sdf > 1e6, rng.uniform(-1, 1, sdf.shape), sdf))):
        f = np.ascontiguousarray(field, np.float32)
        o.set_grid("fluid_sdf", f)
        g.set_grid("fluid_sdf", f)
        o.stage(stage)
        g.stage(stage)
        assert_grid_equal(o, g, "fluid_sdf", f"level set stage {stage} at {shape}")


def test_spec_mode_runs_the_nbflip_step(port_lib, gpu_lib):
    """FS_PCG_SPEC (every solve to a 1e-6 true relative residual) drives the
    NB-FLIP step too: frames run, the band fills, and the pressure solve's
    iterations stay within the spec-mode limit."""
    sc = scenes.nb_dam_break(64, seed=5)
    g = gpu.GpuFlipSolver(sc, precision=gpu.FS_PCG_SPEC)
    for _ in range(4):
        g.step_frame()
    assert g.particle_count() > 0
    assert 0 < g.stat(1) < 20000
    assert np.all(np.isfinite(g.get_grid("u"))) and np.all(np.isfinite(g.get_grid("fluid_sdf")))
