"""Regenerates tests/golden/regression_series.npz from the SPHinXsys source tree.

Reads, as text, the regression databases the reference keeps for the weakly-compressible
dam-break examples (observer pressure, total mechanical energy and free-surface height
time series written by RegressionTestDynamicTimeWarping, plus the stored DTW distances)
and the exclusive-scan known answer of the reference's unit test.  Run it where the
reference tree is available:

    python tests/golden/make_golden.py /path/to/SPHinXsys

Each series is stored as an array of shape (observations, snapshots) under the key
``<case>/<Body>_<Quantity>/Run_<n>``; DTW distances under ``<case>/<Body>_<Quantity>/dtw``.
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

CASES = {
    "dambreak2d": "tests/2d_examples/test_2d_dambreak/regression_test_tool",
    "dambreak3d": "tests/3d_examples/test_3d_dambreak/regression_test_tool",
    "dambreak2d_ck": "tests/tests_sycl/2d_examples/test_2d_dambreak_sycl/regression_test_tool",
    "dambreak3d_ck": "tests/tests_sycl/3d_examples/test_3d_dambreak_sycl/regression_test_tool",
    "stlw2d": "tests/2d_examples/test_2d_stlw/regression_test_tool",
    "still_water2d_ck": "tests/tests_sycl/2d_examples/test_2d_still_water_sycl/regression_test_tool",
    "taylor_green2d": "tests/2d_examples/test_2d_taylor_green/regression_test_tool",
}
SKIP = set()
SCAN_TEST = ("tests/tests_sycl/unit_test_src/shared/particle_dynamics/configuration_dynamics/"
             "test_exclusive_scan_sycl/test_exclusive_scan.cpp")

_ATTR = re.compile(r'snapshot_(\d+)="([^"]+)"')
_PART = re.compile(r"<Particle_(\d+)([^>]*)/>")
_DTW = re.compile(r'(\w+)_(\d+)="([^"]+)"')


def parse_result(text: str) -> np.ndarray:
    rows = {}
    for m in _PART.finditer(text):
        vals = {int(k): float(v) for k, v in _ATTR.findall(m.group(2))}
        rows[int(m.group(1))] = [vals[k] for k in sorted(vals)]
    n = max(len(r) for r in rows.values())
    return np.array([rows[k] + [np.nan] * (n - len(rows[k])) for k in sorted(rows)])


def parse_dtw(text: str) -> np.ndarray:
    vals = {}
    for name, k, v in _DTW.findall(text.split("<DTWDistance", 1)[1]):
        vals[int(k)] = float(v)
    return np.array([vals[k] for k in sorted(vals)])


def parse_scan(text: str):
    arrays = re.findall(r"\{([0-9,\s]+)\}", text)
    return [np.array([int(x) for x in a.split(",") if x.strip()], dtype=np.int64) for a in arrays[:2]]


def main(root: str) -> None:
    out = {}
    for case, rel in CASES.items():
        d = os.path.join(root, rel)
        for fn in sorted(os.listdir(d)):
            m = re.match(r"(.+)_Run_(\d+)_result\.xml$", fn)
            if m and (case, m.group(1)) in SKIP:
                continue
            if m:
                with open(os.path.join(d, fn)) as f:
                    out[f"{case}/{m.group(1)}/Run_{m.group(2)}"] = parse_result(f.read())
            m = re.match(r"(.+)_dtwdistance\.xml$", fn)
            if m:
                with open(os.path.join(d, fn)) as f:
                    out[f"{case}/{m.group(1)}/dtw"] = parse_dtw(f.read())
    with open(os.path.join(root, SCAN_TEST)) as f:
        inp, expect = parse_scan(f.read())
    out["exclusive_scan/input"] = inp
    out["exclusive_scan/expected"] = expect
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "regression_series.npz")
    np.savez_compressed(dst, **out)
    for k, v in out.items():
        print(k, v.shape)


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPHINXSYS_REFERENCE")
    if not src:
        sys.exit("usage: python make_golden.py <SPHinXsys source tree> (or set SPHINXSYS_REFERENCE)")
    main(src)
