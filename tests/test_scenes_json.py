"""Scene files in the reference's JSON format (Utils/jsonscenereader.cpp):
settings with the reference's defaults, objects in file order, the scene
scale applied to vertices, unsupported solver and object types refused."""
import os

import numpy as np
import pytest

from flipsolver2d_gb300 import scenes

# a small dam break written in the reference's scene format (units of the
# scene scale; the disabled object must be skipped)
DAM_JSON = """
{
  "settings": {
    "simType": "flip", "domainSizeI": 10, "domainSizeJ": 10, "resolution": 36,
    "fps": 30, "density": 1000, "maxSubsteps": 10, "pcgIterLimit": 200, "seed": 3,
    "particlesPerCell": 4, "picRatio": 0.03, "cflNumber": 5, "scale": 0.1,
    "globalAcceleration": [9.81, 0]
  },
  "solver": {
    "objects": [
      {"type": "solid", "verts": [[0, 0], [0, 10], [0.3, 10], [0.3, 0]]},
      {"type": "solid", "verts": [[9.7, 0], [9.7, 10], [10, 10], [10, 0]]},
      {"type": "solid", "verts": [[0, 0], [0, 0.3], [10, 0.3], [10, 0]]},
      {"type": "solid", "verts": [[0, 9.7], [0, 10], [10, 10], [10, 9.7]]},
      {"type": "solid", "friction": 0.1, "verts": [[4, 4], [4, 6], [6, 6], [6, 4]]},
      {"type": "solid", "enabled": false, "verts": [[1, 1], [1, 2], [2, 2], [2, 1]]},
      {"type": "fluid", "verts": [[4.5, 0.3], [4.5, 3.8], [9.7, 3.8], [9.7, 0.3]]}
    ]
  }
}
"""


def test_settings_and_objects():
    sc = scenes.scene_from_json(DAM_JSON, "dam36")
    p = sc.params
    assert (p.resolution, p.fps, p.seed, p.particlesPerCell) == (36, 30, 3, 4)
    assert p.fluidDensity == 1000 and p.cflNumber == 5 and p.maxSubsteps == 10
    assert p.sceneScale == pytest.approx(0.1)
    dx, gi, gj = p.grid()
    assert (gi, gj) == (36, 36) and dx == pytest.approx(np.float32(1.0) / np.float32(36))
    kinds = [o.kind for o in sc.objects]
    assert kinds == ["solid"] * 5 + ["fluid"]  # the disabled solid is gone
    assert sc.objects[4].friction == pytest.approx(0.1)
    np.testing.assert_allclose(sc.objects[5].verts[0], [0.45, 0.03], rtol=1e-6)


def test_defaults_follow_the_reference():
    doc = {"settings": {"simType": "fluid", "domainSizeI": 1, "domainSizeJ": 2, "resolution": 64,
                        "fps": 24, "particlesPerCell": 8},
           "solver": {"objects": []}}
    p = scenes.scene_from_json(doc).params
    assert p.fluidDensity == 1.0 and p.seed == 0 and p.maxSubsteps == 30
    assert p.cflNumber == 10.0 and p.pcgIterLimit == 200 and p.picRatio == pytest.approx(0.03)
    assert p.globalAcceleration == (9.8, 0.0)
    dx, gi, gj = p.grid()
    assert (gi, gj) == (32, 64)  # the longer side gets the resolution


@pytest.mark.parametrize("doc,what", [
    ({"settings": {"simType": "smoke"}, "solver": {"objects": []}}, "simType"),
    ({"settings": {"simType": "fire"}, "solver": {"objects": []}}, "simType"),
])
def test_unsupported_solvers(doc, what):
    with pytest.raises(scenes.UnsupportedScene, match=what):
        scenes.scene_from_json(doc)


def test_nbflip_selects_the_narrow_band_solver():
    doc = {"settings": {"simType": "nbflip", "domainSizeI": 5, "domainSizeJ": 5, "resolution": 32,
                        "fps": 30, "particlesPerCell": 8},
           "solver": {"objects": [{"type": "fluid", "viscosity": 10,
                                   "verts": [[2, 0.3], [2, 1.3], [4.7, 1.3], [4.7, 0.3]]}]}}
    sc = scenes.scene_from_json(doc)
    assert sc.sim_type == scenes.SIM_NBFLIP and sc.objects[0].viscosity == 10
    assert scenes.scene_from_json(DAM_JSON).sim_type == scenes.SIM_FLIP


def test_sources_follow_emitter_from_json():
    doc = {"settings": {"simType": "flip", "domainSizeI": 1, "domainSizeJ": 1, "resolution": 16,
                        "fps": 30, "particlesPerCell": 4},
           "solver": {"objects": [{"type": "source", "verts": [[0, 0], [0, 1], [1, 1]],
                                   "velocity": [-7, 2], "viscosity": 4, "transferVelocity": True},
                                  {"type": "source", "verts": [[0, 0], [0, 1], [1, 1]]}]}}
    a, b = scenes.scene_from_json(doc).objects
    assert a.kind == b.kind == "source"
    assert a.velocity == (-7.0, 2.0) and a.viscosity == 4.0 and a.transfer_velocity
    assert b.velocity == (0.0, 0.0) and b.viscosity == 0.0 and not b.transfer_velocity


import build as oracle_build  # noqa: E402  (oracle/ is on sys.path via conftest)

REF_SCENES = os.path.join(oracle_build.reference_dir(), "Liquid2dRender", "scenes")


@pytest.mark.skipif(not os.path.isdir(REF_SCENES), reason="reference scene files not present")
def test_reference_scene_files_parse_or_are_refused():
    loaded, refused, nb = 0, 0, 0
    for fn in sorted(os.listdir(REF_SCENES)):
        if not fn.endswith(".json"):
            continue
        try:
            sc = scenes.scene_from_json(os.path.join(REF_SCENES, fn))
        except scenes.UnsupportedScene:
            refused += 1
            continue
        dx, gi, gj = sc.params.grid()
        assert gi > 0 and gj > 0 and dx > 0 and sc.objects
        loaded += 1
        nb += sc.sim_type == scenes.SIM_NBFLIP
    assert loaded >= 1 and loaded + refused >= 10
    assert nb >= 2  # dam_break.json and level_eq.json: NB-FLIP without sources


@pytest.mark.skipif(not os.path.isdir(REF_SCENES), reason="reference scene files not present")
def test_reference_scene_files_run_the_same_on_both_oracles(port_lib, ref_lib):
    """The reference's NB-FLIP dam break and its scenes with sources (NB-FLIP
    glass pour and waterfall, the FLIP test scene), at a reduced resolution,
    on the reference build and on the C restatement: identical particles,
    grids and engine state frame by frame."""
    import fsoracle as fo

    for fn in ("dam_break.json", "glass_pour.json", "waterfall.json", "test_scene.json"):
        sc = scenes.scene_from_json(os.path.join(REF_SCENES, fn))
        sc.params.resolution = 64
        _same_on_both(fo, sc)


@pytest.mark.skipif(not os.path.isdir(REF_SCENES), reason="reference scene files not present")
def test_reference_viscosity_scenes_run_the_same_on_both_oracles(port_lib, ref_lib):
    """The reference's scene files with viscosity on (the light model; FLIP
    and NB-FLIP), at a reduced resolution, on the reference build (its own
    viscositymodel.cpp) and on the C restatement: identical frame by frame."""
    import fsoracle as fo

    for fn in ("double_dam_break.json", "viscosity_bar.json", "viscosity_test.json", "bounds_check.json"):
        sc = scenes.scene_from_json(os.path.join(REF_SCENES, fn))
        assert sc.params.viscosityEnabled, fn
        sc.params.resolution = 48
        _same_on_both(fo, sc, frames=3)


def test_viscosity_settings_from_json():
    doc = {"settings": {"simType": "flip", "domainSizeI": 1, "domainSizeJ": 1, "resolution": 16,
                        "fps": 30, "particlesPerCell": 4, "viscosityEnabled": True,
                        "heavyViscosity": True},
           "solver": {"objects": [{"type": "fluid", "viscosity": 25,
                                   "verts": [[0.2, 0.2], [0.2, 0.6], [0.6, 0.6], [0.6, 0.2]]}]}}
    sc = scenes.scene_from_json(doc)
    assert sc.params.viscosityEnabled and sc.params.useHeavyViscosity
    assert sc.objects[0].viscosity == 25.0
    assert not scenes.scene_from_json(DAM_JSON).params.viscosityEnabled


def _same_on_both(fo, sc, frames=6):
    r, p = fo.OracleSolver(sc, "ref"), fo.OracleSolver(sc, "port")
    for _ in range(frames):
        r.step_frame()
        p.step_frame()
        pr, pp = r.get_particles(), p.get_particles()
        for k in pr:
            assert np.array_equal(pr[k], pp[k]), k
        for g in r.state_grids():
            assert np.array_equal(r.get_grid(g), p.get_grid(g), equal_nan=True), g
        assert np.array_equal(r.get_rng(), p.get_rng())
    assert r.particle_count() > 0
