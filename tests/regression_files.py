"""Writes stored regression runs (tests/golden/regression_series.npz) as the reference's
regression_test_tool files, the input folder of RegressionTestDynamicTimeWarping::testResult:
<identifier>_<quantity>_runtimes.dat (converged flag, number of runs, repeat label),
_dtwdistance.xml (the stored maximum distance per observation) and one
_Run_<n>_result.xml per stored run (Particle_<k> elements with snapshot_<s> attributes),
in the layout of src/shared/regression_test/regression_test_base.hpp and
dynamic_time_warping_method.hpp."""
import os

import numpy as np


def groups(golden, prefix):
    """{"<identifier>_<quantity>": [run indices]} of one case."""
    out = {}
    for k in golden.files:
        parts = k.split("/")
        if parts[0] == prefix and parts[2].startswith("Run_"):
            out.setdefault(parts[1], []).append(int(parts[2][4:]))
    return {g: sorted(v) for g, v in out.items()}


def stored_runs(golden, prefix, group):
    """Stored runs as lists of per-observation series (padding removed)."""
    runs = {}
    for n in groups(golden, prefix)[group]:
        a = np.atleast_2d(golden[f"{prefix}/{group}/Run_{n}"])
        runs[n] = [row[~np.isnan(row)] for row in a]
    return runs


def write_input_folder(folder, golden, prefix, group):
    identifier, quantity = group.split("_", 1)
    os.makedirs(folder, exist_ok=True)
    base = os.path.join(folder, group)
    runs = stored_runs(golden, prefix, group)
    with open(base + "_runtimes.dat", "w") as f:
        f.write(f"true\n{max(runs) + 1}\n0\n")
    dtw = np.atleast_1d(golden[f"{prefix}/{group}/dtw"])
    attrs = " ".join(f'{quantity}_{k}="{float(v)!r}"' for k, v in enumerate(dtw))
    with open(base + "_dtwdistance.xml", "w") as f:
        f.write(f'<?xml version="1.0" encoding="UTF-8" ?>\n<dtw_distance>\n    <DTWDistance {attrs} />\n'
                "</dtw_distance>\n")
    for n, series in runs.items():
        lines = ['<?xml version="1.0" encoding="UTF-8" ?>', "<result>", "    <Snapshot_Element>",
                 f'        <Snapshot number_of_snapshot_for_local_result_="{len(series[0])}" />',
                 "    </Snapshot_Element>", "    <Result_Element>"]
        for k, s in enumerate(series):
            a = " ".join(f'snapshot_{i}="{float(v)!r}"' for i, v in enumerate(s))
            lines.append(f"        <Particle_{k} {a} />")
        lines += ["    </Result_Element>", "</result>"]
        with open(f"{base}_Run_{n}_result.xml", "w") as f:
            f.write("\n".join(lines) + "\n")
    return identifier, quantity
