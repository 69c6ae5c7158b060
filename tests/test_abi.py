"""The C ABI library builds for sm_103a, loads, and exports every entry point
that include/fs_gpu.h declares.  No compute call is made (no GPU needed)."""
import ctypes
import subprocess

from flipsolver2d_gb300 import build, gpu


def test_library_exports_header(gpu_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    declared = gpu.header_symbols()
    assert len(declared) >= 25
    missing = [s for s in declared if s not in exported]
    assert not missing, f"declared in fs_gpu.h but not exported: {missing}"


def test_status_strings(gpu_lib):
    assert gpu_lib.fs_status_string(0) == b"ok"
    assert gpu_lib.fs_status_string(4) == b"device wait timed out"


def test_bad_arguments_rejected_without_device(gpu_lib):
    # argument validation happens before any device work
    h = ctypes.c_void_p()
    assert gpu_lib.fs_create(None, None, ctypes.byref(h)) == 1
    assert gpu_lib.fs_pcg_solve(0, 0, None, 0.0, 1.0, 1.0, None, None, 1, 1e-2, None, None) == 1
    assert b"invalid" in gpu_lib.fs_last_error()
    srv = ctypes.c_void_p()
    assert gpu_lib.fs_server_create(0, 0, 64, 4, ctypes.c_double(1e-6), 100, ctypes.byref(srv)) == 1
    assert gpu_lib.fs_server_submit(None, None, None) == 1
