"""The header-only C++ layer (include/klshell_gb300.hpp) compiles against the C-ABI, links the
built library, and reports ABI errors as klsa::Error.  Without a device, creating a problem fails
with the library's CUDA error code instead of crashing; with one (the gpu-marked test), the C++
StaticNewton solves the plate and its solution matches the FP64 oracle's gsStaticNewton."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build_and_run(tmp_path):
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
    return out


def test_cpp_driver_builds_and_handles_errors(lib, tmp_path):
    out = _build_and_run(tmp_path)
    assert out.startswith("no-device code=-2") or out.startswith("ok status=0"), out


@pytest.mark.gpu
def test_cpp_driver_solves_on_the_gpu(lib, oracle_mod, tmp_path):
    import numpy as np
    from gsstructuralanalysis_gb300 import problems as P
    out = _build_and_run(tmp_path)
    lines = out.splitlines()
    assert lines[0].startswith("ok status=0"), out
    U = np.array([float(v) for v in lines[1].split()[1:]])
    prob = P.flat_plate(m=2, p=2, bc="simply", pressure=1.0)
    oa = oracle_mod.OracleAssembler(prob)
    ref = oracle_mod.StaticNewton(oa.linear(), oa.force(), oa.jacobian, oa.residual, dict(tol=1e-10, maxIt=20))
    assert ref.solve() == 0
    assert U.shape == ref.U.shape
    assert np.linalg.norm(U - ref.U) <= 1e-6 * np.linalg.norm(ref.U)
