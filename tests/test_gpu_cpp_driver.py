"""The C++ host layer: examples/dambreak_2d.cpp (the reference driver's call sites on the
CUDA policy) compiles against sphinxsys_cuda.h and agrees with the oracle."""
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from sphinxsys_gb300 import build, cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def compile_example(tmp_path, name="dambreak_2d"):
    lib = build.build()
    exe = str(tmp_path / name)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "sphinxsys_gb300", "host"),
           os.path.join(ROOT, "examples", name + ".cpp"), "-o", exe, "-L", os.path.dirname(lib), "-lsphx_cuda",
           f"-Wl,-rpath,{os.path.dirname(lib)}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


@pytest.mark.parametrize("name", ["dambreak_2d", "taylor_green_2d", "dambreak_sycl_3d"])
def test_example_compiles(tmp_path, name):
    assert os.path.exists(compile_example(tmp_path, name))


@pytest.mark.gpu
def test_cpp_driver_matches_oracle(tmp_path):
    exe = compile_example(tmp_path)
    iters = 201
    res = subprocess.run([exe, "20", str(iters)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    out = res.stdout.split("\n")
    rows = [ln.split() for ln in out if ln.startswith(("observe", "final"))]
    oc = O.OracleCase(cases.dambreak_2d())
    expect = [(0, 0.0, oc.observe_pressure()[0], oc.total_mechanical_energy())]
    for it in range(iters):
        observe = it % 200 == 0 and it != 0
        _, _, obs, en = oc.advection_step(observe=observe)
        if observe:
            expect.append((it, oc.physical_time.value, obs[0], en))
    obs_rows = [r for r in rows if r[0] == "observe"]
    assert len(obs_rows) == len(expect)
    for r, e in zip(obs_rows, expect):
        assert int(r[1]) == e[0]
        assert abs(float(r[2]) - e[1]) <= 1e-12 * max(1.0, e[1])
        assert abs(float(r[3]) - e[2]) <= 1e-8 * max(1.0, abs(e[2]))
        assert abs(float(r[4]) - e[3]) <= 1e-10 * abs(e[3])
    final = [r for r in rows if r[0] == "final"][0]
    assert int(final[1]) == iters
    assert abs(float(final[4]) / oc.total_mechanical_energy() - 1) < 1e-10


@pytest.mark.gpu
def test_cpp_taylor_green_matches_oracle(tmp_path):
    """examples/taylor_green_2d.cpp (taylor_green.cpp's call sites) at 50 x 50 for 40
    advection steps against the oracle: same physical time, kinetic energy within 1e-10."""
    exe = compile_example(tmp_path, "taylor_green_2d")
    steps = 40
    res = subprocess.run([exe, "5", str(steps), "50"], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    final = [ln.split() for ln in res.stdout.split("\n") if ln.startswith("final")][0]
    o = O.OracleTGV(cases.taylor_green_2d(50))
    for _ in range(steps):
        o.advection_step()
    assert int(final[1]) == steps
    assert abs(float(final[2]) / o.physical_time.value - 1) < 1e-12
    assert abs(float(final[3]) / o.kinetic_energy() - 1) < 1e-10
    assert abs(float(final[4]) / o.maximum_speed() - 1) < 1e-10


@pytest.mark.gpu
def test_cpp_sycl_3d_driver_matches_oracle(tmp_path):
    """examples/dambreak_sycl_3d.cpp (the 3D SYCL driver's CK call sites on the CUDA
    policy) for 110 advection steps, through the particle sort at step 100, against the
    oracle's nested CK loop: same physical time, mechanical energy within 1e-10."""
    exe = compile_example(tmp_path, "dambreak_sycl_3d")
    steps = 110
    res = subprocess.run([exe, "20", str(steps)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    lines = [ln.split() for ln in res.stdout.split("\n") if ln]
    probes = [ln for ln in lines if ln[0] == "probe"]
    energy = [ln for ln in lines if ln[0] == "energy"]
    assert len(probes) == steps + 1 and int(probes[-1][1]) == steps
    oc = O.OracleCase(cases.dambreak_3d_reference())
    assert abs(float(energy[0][3]) / oc.total_mechanical_energy() - 1) < 1e-12
    for _ in range(steps):
        oc.ck_nested_advection_step()
    assert abs(float(probes[-1][2]) / oc.physical_time.value - 1) < 1e-12
    assert int(energy[-1][1]) == steps
    assert abs(float(energy[-1][3]) / oc.total_mechanical_energy() - 1) < 1e-10
    np.testing.assert_allclose([float(v) for v in probes[-1][3:]], oc.ck_observe_pressure(), rtol=1e-8, atol=1e-10)
