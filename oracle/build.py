"""Build recipe for the CPU oracles (test infrastructure).

    python oracle/build.py            # port always; reference when its sources exist

* oracle/_build/libfsoracle.so -- fsoracle.c, the plain-C restatement.
  Flags: -O2 -ffp-contract=off (no fused multiply-add, matching the
  reference oracle build), no -ffast-math, portable (no -march).
* oracle/_ref/libfsref.so -- the reference sources compiled in place by
  Makefile.ref, only when the reference tree is present (FS_REFERENCE_DIR,
  default /root/reference).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def build_port(verbose: bool = False) -> str:
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libfsoracle.so")
    src = os.path.join(HERE, "fsoracle.c")
    hdr = os.path.join(HERE, "fsoracle.h")
    if (os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src)
            and os.path.getmtime(out) >= os.path.getmtime(hdr)):
        return out
    cmd = [os.environ.get("CC", "gcc"), "-std=c11", "-O2", "-ffp-contract=off", "-fPIC",
           "-shared", "-Wall", "-Wno-unused-function", "-o", out, src, "-lpthread", "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return out


def reference_dir() -> str:
    return os.environ.get("FS_REFERENCE_DIR", "/root/reference")


def build_ref(verbose: bool = False) -> str | None:
    ref = reference_dir()
    if not os.path.isdir(os.path.join(ref, "FlipSolver2dLib")):
        return None
    nproc = str(os.cpu_count() or 4)
    cmd = ["make", "-s", "-f", "Makefile.ref", f"REF={ref}", "-j", nproc]
    subprocess.run(cmd, check=True, cwd=HERE,
                   stdout=None if verbose else subprocess.DEVNULL)
    return os.path.join(HERE, "_ref", "libfsref.so")


def main() -> int:
    print(build_port(verbose=True))
    r = build_ref(verbose=True)
    print(r if r else "reference sources absent: oracle/_ref not built")
    return 0


if __name__ == "__main__":
    sys.exit(main())
