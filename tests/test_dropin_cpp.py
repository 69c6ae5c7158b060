"""The C++ drop-ins (include/fs_gpu_flipsolver.hpp) compile and link against
the reference's own headers and objects, and the LinearSolver adapter packs
the reference's operator rows into exactly the operator bytes that the GPU's
own decomposition derives from the material grid.

Runs where the reference sources are present (it compiles
tests/dropin/dropin_check.cpp against FlipSolver2dLib/ and links the
reference build oracle/_ref/libfsref.so and libfsgpu.so); no device is needed:
without one, the GPU step must fail with FS_ERR_CUDA (there is no CPU
fallback)."""
import os
import platform
import subprocess

import numpy as np
import pytest

import build as oracle_build  # oracle/build.py
from flipsolver2d_gb300 import build as gpu_build
from operator_bytes import decomposition_bytes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def dropin_binary(tmp_path_factory, ref_lib):
    ref = oracle_build.reference_dir()
    src = os.path.join(ref, "FlipSolver2dLib")
    gpu_build.build()
    out = str(tmp_path_factory.mktemp("dropin") / "dropin_check")
    shim = ["-I", os.path.join(ROOT, "oracle", "refshim")]
    if platform.machine() != "x86_64":
        shim += ["-I", os.path.join(ROOT, "oracle", "refshim", "arm64")]
    ref_dir = os.path.join(ROOT, "oracle", "_ref")
    gpu_dir = os.path.dirname(gpu_build.LIB)
    cmd = (["g++", "-std=c++20", "-O1", "-DENQUEUE_IS_RUN", "-DNUMPY_LOGGING", "-w"] + shim +
           ["-I", src, "-I", os.path.join(src, "threading"), "-I", os.path.join(ROOT, "include"),
            os.path.join(ROOT, "tests", "dropin", "dropin_check.cpp"), "-o", out,
            "-L", ref_dir, "-lfsref", "-L", gpu_dir, "-lfsgpu",
            f"-Wl,-rpath,{ref_dir}", f"-Wl,-rpath,{gpu_dir}"])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return out


def test_dropin_compiles_links_and_packs_the_operator(dropin_binary):
    r = subprocess.run([dropin_binary], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = {ln.split(" ", 1)[0]: ln.split(" ", 1)[1] for ln in r.stdout.splitlines() if " " in ln}
    n = 24
    mat = np.array([int(v) for v in lines["material"].split()], np.int8).reshape(n, n)
    got = np.array([int(v) for v in lines["operator"].split()], np.uint8).reshape(n, n)
    want = decomposition_bytes(mat)
    unit = (want & 0x80) != 0
    assert unit.sum() > 50, "the scene has fluid"
    assert np.array_equal(got[unit], want[unit]), "unit rows"
    # the counts of the unit rows' linear neighbours select the IPP rows
    flat_u = np.flatnonzero(unit.ravel())
    nbrs = np.unique(np.concatenate([flat_u - n, flat_u + n, flat_u - 1, flat_u + 1]))
    nbrs = nbrs[(nbrs >= 0) & (nbrs < n * n)]
    assert np.array_equal((got.ravel()[nbrs] >> 4) & 7, (want.ravel()[nbrs] >> 4) & 7), "neighbour counts"
    # the GPU step: FS_ERR_CUDA without a device, a stepped frame with one
    step = lines.get("step", "")
    assert step.startswith("ok") or step.startswith("error 2 "), step
