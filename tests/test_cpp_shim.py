"""The header-only C++ layer (include/klshell_gb300.hpp) compiles against the C-ABI, links the
built library, and reports ABI errors as klsa::Error; without a device, creating a problem fails
with the library's CUDA error code instead of crashing."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_driver_builds_and_handles_errors(lib, tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    libdir = os.path.join(ROOT, "gsstructuralanalysis_gb300", "_lib")
    exe = str(tmp_path / "shim_driver")
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "shim_driver.cpp"), "-o", exe,
           "-L", libdir, "-lklshell_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    env = dict(os.environ)
    cuda_lib = "/usr/local/cuda/lib64"
    env["LD_LIBRARY_PATH"] = cuda_lib + (":" + env["LD_LIBRARY_PATH"] if env.get("LD_LIBRARY_PATH") else "")
    r = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=120)
    out = r.stdout.strip()
    assert r.returncode == 0, (out, r.stderr)
    assert out.startswith("no-device code=-2") or out.startswith("ok status=0"), out
