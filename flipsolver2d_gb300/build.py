"""Build recipe for libfsgpu.so, the CUDA extension behind include/fs_gpu.h.

    python -m flipsolver2d_gb300.build

Compiles the translation units in parallel with nvcc for sm_103a only
and links them into flipsolver2d_gb300/_build/libfsgpu.so (in-tree, git
ignored).  The particle and grid kernels and the host driver are built with
-fmad=false (and the host compiler with -ffp-contract=off) so that every float
expression rounds exactly like the reference CPU build; the PCG file keeps
fused multiply-add for its FP32 arithmetic.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libfsgpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = {
    "fs_particles.cu": ["-fmad=false"],
    "fs_grid.cu": ["-fmad=false"],
    "fs_nbflip.cu": ["-fmad=false"],
    "fs_api.cu": ["-fmad=false"],
    "fs_pcg.cu": ["-fmad=true"],
    "fs_pcg_tma.cu": ["-fmad=true"],
    "fs_spec.cu": ["-fmad=true"],
    "fs_cluster.cu": ["-fmad=true"],
    "fs_viscosity.cu": ["-fmad=false"],
}


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "fs_gpu.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(verbose: bool = False, force: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-ffp-contract=off", "-I", CSRC, "-I", INCLUDE] + ARCH
    procs = []
    objs = []
    for unit, flags in UNITS.items():
        obj = os.path.join(OUT_DIR, unit.replace(".cu", ".o"))
        cmd = [nvcc(), "-c", os.path.join(CSRC, unit), "-o", obj] + common + flags
        if verbose:
            print(" ".join(cmd))
        procs.append((unit, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    failed = []
    for unit, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((unit, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if failed:
        msg = "\n".join(f"--- {u}\n{o}" for u, o in failed)
        raise RuntimeError(f"nvcc failed:\n{msg}")
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
