"""The C++ host layer's dynamic-time-warping regression test (testDTWRegression, the
testResult of the CK drivers' addReduceRegression / addObserveRegression) against the
Python restatement, on the stored runs of the reference written in its own file layout:
a stored run passes, a shifted copy fails, and both restatements give the same outcome."""
import os
import subprocess

import numpy as np
import pytest

from sphinxsys_gb300 import build, regression

import regression_files as RF

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    lib = build.build()
    exe = str(tmp_path_factory.mktemp("dtw") / "dtw_regression_check")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "sphinxsys_gb300", "host"),
                    os.path.join(ROOT, "tests", "cpp", "dtw_regression_check.cpp"), "-o", exe, "-L",
                    os.path.dirname(lib), "-lsphx_cuda", f"-Wl,-rpath,{os.path.dirname(lib)}"],
                   check=True, capture_output=True, text=True)
    return exe


CASES = [("dambreak2d_ck", "WaterBody_TotalMechanicalEnergy"), ("dambreak2d_ck", "FluidObserver_Pressure"),
         ("dambreak2d", "FluidObserver_Pressure"), ("dambreak3d", "FluidObserver_Pressure"),
         ("taylor_green2d", "WaterBody_MaximumSpeed")]


@pytest.mark.parametrize("prefix,group", CASES, ids=lambda x: str(x))
def test_cpp_dtw_regression_matches_python(tmp_path, golden, checker, prefix, group):
    folder = str(tmp_path / "input")
    identifier, quantity = RF.write_input_folder(folder, golden, prefix, group)
    runs = RF.stored_runs(golden, prefix, group)
    stored = [np.atleast_2d(golden[f"{prefix}/{group}/Run_{n}"]) for n in sorted(runs)]
    dtw = np.atleast_1d(golden[f"{prefix}/{group}/dtw"])
    first = runs[min(runs)]
    length = min(len(s) for s in first)
    for shift, expect in ((0.0, True), (2.0 * float(dtw.max()), False)):
        current = np.array([s[:length] for s in first]) + shift  # observations x snapshots
        series = str(tmp_path / f"series_{shift}.txt")
        np.savetxt(series, current.T)
        res = subprocess.run([checker, folder, identifier, quantity, series], capture_output=True, text=True)
        ok_py, _ = regression.passes(stored, current, dtw)
        assert res.returncode in (0, 1), res.stdout + res.stderr
        assert (res.returncode == 0) == ok_py == expect, (shift, res.stdout)


def test_cpp_dtw_regression_reports_missing_database(tmp_path, checker):
    series = str(tmp_path / "s.txt")
    np.savetxt(series, np.ones((5, 1)))
    res = subprocess.run([checker, str(tmp_path / "nothing"), "WaterBody", "TotalMechanicalEnergy", series],
                         capture_output=True, text=True)
    assert res.returncode == 1 and "missing" in res.stdout
