"""The native gsAPALMData restatement (klsa::APALMData in csrc/apalm.cpp, host code of the built
library) against the oracle's independent Python restatement (oracle/apalm.py), and the oracle
against the reference's own gsAPALMData compiled unchanged (oracle/ref_apalm_data.cpp, built
where the reference tree exists), all driven by the same scripted jobs: every popped job
(interval length, start, previous and reference points, level) and the final flat solutions
(curve times, points, levels) agree."""
import os
import shutil
import subprocess

import pytest

import apalm as AP

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _oracle_lines():
    out = []
    d = AP.APALMData(max_level=2, tolerance=0.05)
    d.set_data([0.0, 1.0, 2.0, 3.0], [0.0, 1.0, 2.0, 3.0])
    d.init()
    for _ in range(12):
        if d.empty():
            break
        ID, dt, start, prev = d.pop()
        ref = d.reference(ID)
        level = d.job_level(ID)
        out.append(("job", ID, dt, start, prev, ref, level))
        dist = [0.5 * dt, 0.5 * dt, 0.2 * dt / (1 + level) * (1 + 0.1 * ID)]
        d.submit(ID, dist, [100.0 + 10 * ID, 101.0 + 10 * ID], dt * (1.0 + 0.03 * ID), dt * (1.0 - 0.04 * (ID % 3)))
        d.finish_job(ID)
    for t, s, lv in zip(*d.flat()):
        out.append(("flat", t, s, lv))
    b = AP.APALMData(max_level=1, tolerance=0.05)
    b.add_start_point(0.0, 0.0)
    b.dt = 0.25
    for it in range(10):
        if b.empty():
            break
        ID, dt, start, _ = b.pop()
        level = b.job_level(ID)
        out.append(("bjob", ID, dt, start, level))
        if level == 0:
            t = b.job_start_time(ID) + dt * (1.0 + 0.01 * ID)
            b.append_data(t, 1000.0 + ID)
            b.finish_job(ID)
            if it < 4:
                b.append_point(True)
        else:
            b.submit(ID, [0.5 * dt, 0.5 * dt, 0.3 * dt], [2000.0 + ID, 2001.0 + ID], dt * 1.05, dt * 0.9)
            b.finish_job(ID)
    for t, s, lv in zip(*b.flat()):
        out.append(("bflat", t, s, lv))
    return out


def _compare(lines, expected):
    assert len(lines) == len(expected) and len(lines) > 15
    for a, b in zip(lines, expected):
        assert a[0] == b[0] and len(a) == len(b), (a, b)
        for x, y in zip(a[1:], b[1:]):
            assert float(x) == pytest.approx(float(y), rel=1e-13, abs=1e-15), (a, b)


def test_oracle_apalm_data_matches_reference():
    RS = pytest.importorskip("refsolvers")
    if not RS.available() or not os.path.exists(RS.APALM_DATA_DRIVER):
        pytest.skip("reference tree not present: gsAPALMData not built")
    r = subprocess.run([RS.APALM_DATA_DRIVER], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    _compare([ln.split() for ln in r.stdout.strip().splitlines()], _oracle_lines())


def test_native_apalm_data_matches_oracle(lib, tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    cuda_inc = "/usr/local/cuda/include"
    libdir = os.path.join(ROOT, "gsstructuralanalysis_gb300", "_lib")
    exe = str(tmp_path / "apalm_data_driver")
    cmd = [gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "gsstructuralanalysis_gb300", "csrc"), "-I", cuda_inc,
           os.path.join(ROOT, "tests", "cpp", "apalm_data_driver.cpp"), "-o", exe, "-L", libdir, "-lklshell_gb300",
           f"-Wl,-rpath,{libdir}", "-L", "/usr/local/cuda/lib64", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    env = dict(os.environ)
    env["LD_LIBRARY_PATH"] = "/usr/local/cuda/lib64" + (":" + env["LD_LIBRARY_PATH"] if env.get("LD_LIBRARY_PATH") else "")
    r = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0, r.stderr
    _compare([ln.split() for ln in r.stdout.strip().splitlines()], _oracle_lines())
