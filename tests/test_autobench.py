"""The AutoBench-layout statistics (flipsolver2d_gb300/autobench.py): the
column headers of the reference's bench table (AutoBench/benchruntable.cpp
getColumnHeader, read from the reference tree when it is present), the CSV
writer, and -- on the GPU -- per-stage device times that add up to the timed
substeps."""
import csv
import os
import re

import numpy as np
import pytest

import build as oracle_build  # noqa: E402  (oracle/ is on sys.path via conftest)
from flipsolver2d_gb300 import autobench, scenes


def test_columns_match_reference_headers():
    path = os.path.join(oracle_build.reference_dir(), "AutoBench", "benchruntable.cpp")
    if not os.path.exists(path):
        pytest.skip("reference tree not present")
    src = open(path).read()
    body = src[src.index("getColumnHeader"):]
    heads = re.findall(r'return "([^"]+)";', body)
    heads = [h for h in heads if not h.startswith("INVALID")]
    assert heads == autobench.COLUMNS


def test_csv_layout(tmp_path):
    rows = [[0, 2, 10.0] + [1.0] * 12 + [200, 200, 0], [1, 3, 11.0] + [2.0] * 12 + [150, 0, 0]]
    out = tmp_path / "t.csv"
    autobench.write_csv(str(out), [("dam", rows)])
    got = list(csv.reader(open(out)))
    assert got[0] == ["Scene"] + autobench.COLUMNS
    assert len(got) == 3 and got[1][0] == "dam" and got[2][2] == "3"


@pytest.mark.gpu
def test_stage_times_add_up(gpu_lib):
    rows = autobench.run_scene(scenes.dam_break(96, seed=3), 2)
    assert len(rows) == 2
    for r in rows:
        assert len(r) == len(autobench.COLUMNS)
        stages = np.array(r[3:15])
        assert np.all(stages >= 0.0) and stages[1] > 0 and stages[7] > 0
        assert stages[4] == 0.0 and stages[8] == 0.0 and stages[9] == 0.0
        assert r[2] >= 0.9 * stages.sum()  # the wall time covers the device stages


@pytest.mark.gpu
def test_nbflip_stage_times(gpu_lib):
    """NB-FLIP ends its stages differently (nbflipsolver.cpp:26-64): particle
    to grid has its own time, there is no density correction, and the level
    sets count in after transfer."""
    rows = autobench.run_scene(scenes.nb_dam_break(96, seed=3), 3)
    for r in rows[1:]:
        stages = np.array(r[3:15])
        assert np.all(stages >= 0.0)
        assert stages[4] > 0 and stages[6] > 0 and stages[7] > 0 and stages[11] > 0
        assert stages[2] == 0.0 and stages[8] == 0.0 and stages[9] == 0.0
        assert r[2] >= 0.9 * stages.sum()
